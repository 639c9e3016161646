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
 * Neighbour search: uniform grid with cells slightly wider than the radius, so every
 * neighbour lies in the 3x3 cells around a point.
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

long cluster_run(const txg_cand *c, long n, double dms, double ddm, double fmax, double fmin,
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
    const int ncluster = icluster - 1;

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

} // namespace txg
