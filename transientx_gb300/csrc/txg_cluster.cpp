/*
 * txg_cluster.cpp -- candidate clustering on the host, the Cluster<double>::run step
 * (src/singlepulse/cluster.cpp:63-161 with include/clustering.h:26-100).
 *
 * Input: the S > thre points of one block in row-major (idm, isamp) order, as the threshold
 * scan of cluster.cpp:91-112 produces them.  Each point sits at
 * (dmdelay(dms+idm*ddm, fmax, fmin)/2, isamp*tsamp); two points are neighbours when their
 * squared distance is <= radius^2, radius raised to 1.5*tsamp at least (cluster.cpp:117).
 * Clusters are grown from the highest-S remaining point (earliest index on ties, the index
 * passing through a float as clustering.h:264-270 stores it) over the neighbour relation, at
 * most maxncand of them.  Each cluster reports its highest-S member (first on ties).  The
 * final filter (drop / minpts) reproduces cluster.cpp:145-158, whose size test reads
 * candcluster[k] while entries are being erased from that vector: after an erase the test
 * sees the following cluster's entry, a moved-from entry reads as empty and an erased last
 * entry keeps its size.
 *
 * Below 2^24 points (where the float index is exact) the clusters are found as connected
 * components with a union-find (a sweep over DM rows, or a grid when many DM rows lie within
 * one radius); from 2^24 points on, the breadth-first growth itself runs over a grid with
 * cells slightly wider than the radius, so every neighbour lies in the 3x3 cells around a
 * point.
 */
#include <algorithm>
#include <cmath>
#include <cstring>
#include <unordered_map>
#include <vector>

#include "txg_internal.h"

namespace txg {

namespace {

struct Grid {
    double cell;
    std::unordered_map<uint64_t, std::vector<long>> cells;
    static uint64_t key(int64_t cx, int64_t cy)
    {
        return ((uint64_t)(cx + (1LL << 31)) << 32) ^ (uint64_t)(cy + (1LL << 31));
    }
};

} // namespace

/* Reported candidates (cluster.cpp:124-158): per cluster its highest-S member (first on
 * ties); drop / minpts tested against candcluster[k] while erasing from it, so after an erase
 * the test sees the following cluster's entry, a moved-from entry reads as empty and an erased
 * last entry keeps its size. */
static long select_report(const txg_cand *c, long n, const std::vector<int> &cid, int ncluster,
                          int minpts, int drop, int maxwn, txg_cand *out, long cap)
{
    std::vector<long> mxi(ncluster, -1);
    std::vector<float> mxs(ncluster, 0.f);
    std::vector<size_t> size(ncluster, 0);
    for (long i = 0; i < n; i++) {
        if (cid[i] == 0) continue;
        const int k = cid[i] - 1;
        size[k]++;
        if (c[i].S > mxs[k]) {
            mxs[k] = c[i].S;
            mxi[k] = i;
        }
    }
    std::vector<size_t> slot(size);
    long len = ncluster, nout = 0;
    for (long k = 0; k < ncluster; k++) {
        const long m = mxi[k];
        if (m < 0) continue;
        const int wn = c[m].wn;
        if ((!drop || wn != maxwn) && slot[k] >= (size_t)minpts) {
            if (nout < cap) out[nout] = c[m];
            nout++;
        } else {
            if (k + 1 < len) {
                for (long q = k; q < len - 1; q++) slot[q] = slot[q + 1];
                slot[len - 1] = 0;
            }
            len--;
        }
    }
    return nout;
}

/* Breadth-first growth from each seed, as clustering.h does (used when the seed index can
 * round through the float, i.e. 2^24 points or more). */
static long cluster_bfs(const txg_cand *c, long n, double dms, double ddm, double fmax, double fmin,
                        double tsamp, double radius, int maxncand, int minpts, int drop, int maxwn,
                        txg_cand *out, long cap)
{
    if (n <= 0) return 0;
    std::vector<double> px(n), py(n);
    for (long i = 0; i < n; i++) {
        double dm = dms + c[i].idm * ddm;
        px[i] = dmdelay(dm, fmax, fmin) * 0.5;
        py[i] = c[i].isamp * tsamp;
    }
    if (radius < 1.5 * tsamp) radius = 1.5 * tsamp;
    const double r2 = radius * radius;

    Grid grid;
    grid.cell = radius * 1.0000001;
    std::vector<int64_t> cx(n), cy(n);
    for (long i = 0; i < n; i++) {
        cx[i] = (int64_t)std::floor(px[i] / grid.cell);
        cy[i] = (int64_t)std::floor(py[i] / grid.cell);
        grid.cells[Grid::key(cx[i], cy[i])].push_back(i);
    }
    auto neighbours = [&](long p, std::vector<long> &dst) {
        for (int64_t dx = -1; dx <= 1; dx++)
            for (int64_t dy = -1; dy <= 1; dy++) {
                auto it = grid.cells.find(Grid::key(cx[p] + dx, cy[p] + dy));
                if (it == grid.cells.end()) continue;
                for (long q : it->second) {
                    double ex = px[q] - px[p], ey = py[q] - py[p];
                    if (ex * ex + ey * ey <= r2) dst.push_back(q);
                }
            }
    };

    /* seed order: S descending, index ascending; removed points are skipped */
    std::vector<long> order(n);
    for (long i = 0; i < n; i++) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](long a, long b) { return c[a].S > c[b].S; });
    std::vector<char> removed(n, 0), visited(n, 0), mark(n, 0);
    std::vector<int> cid(n, 0);
    long cursor = 0;
    int icluster = 0;
    std::vector<long> front, next, nb, reached;
    while (icluster++ < maxncand) {
        while (cursor < n && removed[order[cursor]]) cursor++;
        if (cursor >= n) break;
        /* a point with S <= -1 is never chosen (the scan starts from maxsnr = -1) */
        if (!(c[order[cursor]].S > -1.f)) break;
        long seed = (long)(float)order[cursor];
        front.clear();
        neighbours(seed, front);
        reached.clear();
        while (!front.empty()) {
            next.clear();
            for (long idx : front) {
                cid[idx] = icluster;
                visited[idx] = 1;
                nb.clear();
                neighbours(idx, nb);
                for (long q : nb)
                    if (!mark[q]) {
                        mark[q] = 1;
                        next.push_back(q);
                    }
                reached.push_back(idx);
            }
            front.clear();
            for (long q : next) {
                mark[q] = 0;
                if (!visited[q]) front.push_back(q);
            }
        }
        for (long q : reached) removed[q] = 1;
    }
    return select_report(c, n, cid, icluster - 1, minpts, drop, maxwn, out, cap);
}

/* Union-find over point indices; roots are the smaller index of a merge. */
struct Forest {
    std::vector<long> parent;
    explicit Forest(long n) : parent(n)
    {
        for (long i = 0; i < n; i++) parent[i] = i;
    }
    long find(long a)
    {
        while (parent[a] != a) {
            parent[a] = parent[parent[a]];
            a = parent[a];
        }
        return a;
    }
    void unite(long a, long b)
    {
        a = find(a);
        b = find(b);
        if (a != b) parent[a < b ? b : a] = a < b ? a : b;
    }
};

/* Components by grid: cells of side radius/sqrt(2) (any two points of one cell are
 * neighbours), cells up to two apart linked by the first pair within the radius.  Used when
 * many DM rows lie within one radius of each other. */
static void components_grid(long n, const double *px, const double *py, double radius, double r2,
                            Forest &F)
{
    const double side = radius / std::sqrt(2.) * (1. - 1e-6);
    std::vector<int64_t> cx(n), cy(n);
    for (long i = 0; i < n; i++) {
        cx[i] = (int64_t)std::floor(px[i] / side);
        cy[i] = (int64_t)std::floor(py[i] / side);
    }
    std::vector<long> byc(n);
    for (long i = 0; i < n; i++) byc[i] = i;
    std::sort(byc.begin(), byc.end(), [&](long a, long b) {
        return cx[a] != cx[b] ? cx[a] < cx[b] : (cy[a] != cy[b] ? cy[a] < cy[b] : a < b);
    });
    struct Cell {
        int64_t x, y;
        long beg, end;
    };
    std::vector<Cell> cells;
    for (long k = 0; k < n;) {
        long e = k;
        while (e < n && cx[byc[e]] == cx[byc[k]] && cy[byc[e]] == cy[byc[k]]) e++;
        cells.push_back({cx[byc[k]], cy[byc[k]], k, e});
        k = e;
    }
    for (const Cell &q : cells)
        for (long k = q.beg + 1; k < q.end; k++) F.unite(byc[q.beg], byc[k]);
    auto locate = [&](int64_t x, int64_t y) -> long {
        long lo = 0, hi = (long)cells.size();
        while (lo < hi) {
            long mid = (lo + hi) / 2;
            if (cells[mid].x < x || (cells[mid].x == x && cells[mid].y < y)) lo = mid + 1;
            else hi = mid;
        }
        return (lo < (long)cells.size() && cells[lo].x == x && cells[lo].y == y) ? lo : -1;
    };
    for (long ci = 0; ci < (long)cells.size(); ci++) {
        const Cell &a = cells[ci];
        for (int64_t dx = 0; dx <= 2; dx++)
            for (int64_t dy = -2; dy <= 2; dy++) {
                if (dx == 0 && dy <= 0) continue; /* each pair of cells once */
                const long cj = locate(a.x + dx, a.y + dy);
                if (cj < 0) continue;
                const Cell &b = cells[cj];
                if (F.find(byc[a.beg]) == F.find(byc[b.beg])) continue;
                bool linked = false;
                for (long p = a.beg; p < a.end && !linked; p++)
                    for (long q = b.beg; q < b.end; q++) {
                        const double ex = px[byc[q]] - px[byc[p]], ey = py[byc[q]] - py[byc[p]];
                        if (ex * ex + ey * ey <= r2) {
                            F.unite(byc[p], byc[q]);
                            linked = true;
                            break;
                        }
                    }
            }
    }
}

/* Clusters are the connected components of the neighbour graph (every point a breadth-first
 * growth reaches from its seed), numbered in the seed order of clustering.h:262-272: a
 * component's seed is its highest-S point (earliest index on ties, S > -1), and components
 * are taken by seed S descending, earlier seed first on ties.
 *
 * Components by DM-row sweep: with the points ordered by (idm, isamp), px is monotone in idm
 * and py in isamp, so (i) within one DM row a point's neighbours are contiguous and linking
 * consecutive neighbours is enough, and (ii) for two rows within one radius in px, the
 * neighbours of each point of the first row form a contiguous window of the second whose
 * ends never move back; linking each point to the new part of its window (or to one point of
 * the part shared with the previous window) costs O(n_a + n_b) per pair of rows. */
long cluster_run(const txg_cand *c, long n, double dms, double ddm, double fmax, double fmin,
                 double tsamp, double radius, int maxncand, int minpts, int drop, int maxwn,
                 txg_cand *out, long cap)
{
    if (n <= 0) return 0;
    if (n >= (1L << 24))
        return cluster_bfs(c, n, dms, ddm, fmax, fmin, tsamp, radius, maxncand, minpts, drop, maxwn,
                           out, cap);
    if (radius < 1.5 * tsamp) radius = 1.5 * tsamp;
    const double r2 = radius * radius;

    /* (idm, isamp) order; the threshold scan already delivers it */
    std::vector<long> ord(n);
    for (long i = 0; i < n; i++) ord[i] = i;
    bool sorted = true;
    for (long i = 1; i < n && sorted; i++)
        sorted = c[i - 1].idm < c[i].idm || (c[i - 1].idm == c[i].idm && c[i - 1].isamp <= c[i].isamp);
    if (!sorted)
        std::stable_sort(ord.begin(), ord.end(), [&](long a, long b) {
            return c[a].idm != c[b].idm ? c[a].idm < c[b].idm : c[a].isamp < c[b].isamp;
        });
    /* coordinates in sweep order */
    std::vector<double> px(n), py(n);
    struct Row {
        long beg, end;
    };
    std::vector<Row> rows;
    for (long k = 0; k < n;) {
        long e = k;
        const int32_t idm = c[ord[k]].idm;
        const double x = dmdelay(dms + idm * ddm, fmax, fmin) * 0.5;
        while (e < n && c[ord[e]].idm == idm) {
            px[e] = x;
            py[e] = c[ord[e]].isamp * tsamp;
            e++;
        }
        rows.push_back({k, e});
        k = e;
    }
    const long nrow = (long)rows.size();
    /* rows within one radius in px: a prefix of the following rows, ending at reach[a] */
    std::vector<long> reach(nrow);
    double work = 0.;
    for (long a = 0, b = 1; a < nrow; a++) {
        if (b < a + 1) b = a + 1;
        while (b < nrow) {
            const double ex = px[rows[b].beg] - px[rows[a].beg];
            if (!(ex * ex <= r2)) break;
            b++;
        }
        reach[a] = b;
        for (long q = a + 1; q < b && work < 1e18; q++)
            work += (double)(rows[a].end - rows[a].beg + rows[q].end - rows[q].beg);
        if (work > 64. * (double)n + 4e6) break;
    }
    Forest F(n); /* over sweep positions */
    if (work > 64. * (double)n + 4e6) {
        components_grid(n, px.data(), py.data(), radius, r2, F);
    } else {
        for (long a = 0; a < nrow; a++) {
            const Row A = rows[a];
            for (long k = A.beg + 1; k < A.end; k++) {
                const double ey = py[k] - py[k - 1];
                if (0. * 0. + ey * ey <= r2) F.unite(k - 1, k);
            }
            for (long bi = a + 1; bi < reach[a]; bi++) {
                const Row B = rows[bi];
                const double ex = px[B.beg] - px[A.beg];
                const double ex2 = ex * ex;
                auto nb = [&](long p, long q) {
                    const double ey = py[q] - py[p];
                    return ex2 + ey * ey <= r2;
                };
                long lo = B.beg, hi = B.beg, shared = B.beg; /* [lo, hi): window; < shared: linked */
                for (long p = A.beg; p < A.end; p++) {
                    while (lo < B.end && py[lo] <= py[p] && !nb(p, lo)) lo++;
                    if (lo >= B.end) break;
                    if (!nb(p, lo)) continue; /* empty window: the next row point is ahead */
                    if (hi < lo + 1) hi = lo + 1;
                    while (hi < B.end && nb(p, hi)) hi++;
                    long from = lo;
                    if (shared > lo) { /* overlaps the previous window, whose points are linked */
                        F.unite(p, lo);
                        from = shared;
                    }
                    for (long q = from; q < hi; q++) F.unite(p, q);
                    shared = hi;
                }
            }
        }
    }
    /* seeds per component, in input-index terms */
    std::vector<long> pos(n);
    for (long k = 0; k < n; k++) pos[ord[k]] = k;
    std::vector<float> best(n, -1.f);
    std::vector<long> seed(n, -1);
    for (long i = 0; i < n; i++) {
        const long r = F.find(pos[i]);
        if (c[i].S > best[r]) {
            best[r] = c[i].S;
            seed[r] = i;
        }
    }
    std::vector<long> roots;
    for (long k = 0; k < n; k++)
        if (F.parent[k] == k && seed[k] >= 0) roots.push_back(k);
    std::sort(roots.begin(), roots.end(), [&](long a, long b) {
        return best[a] != best[b] ? best[a] > best[b] : seed[a] < seed[b];
    });
    const long ncl = std::min<long>((long)roots.size(), maxncand > 0 ? maxncand : 0);
    std::vector<int> rid(n, 0);
    for (long k = 0; k < ncl; k++) rid[roots[k]] = (int)(k + 1);
    std::vector<int> cid(n, 0);
    for (long i = 0; i < n; i++) cid[i] = rid[F.find(pos[i])];
    return select_report(c, n, cid, (int)ncl, minpts, drop, maxwn, out, cap);
}

} // namespace txg
