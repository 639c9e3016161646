/*
 * kdtree.h -- stand-in for XLibs' KDtree<T>, with the interface include/clustering.h:56-99
 * and src/singlepulse/cluster.cpp:114-124 use (build, findNeighbors, findNeighborsAdd,
 * ncluster, KDnode{index, point}).  A neighbour of p is any point q with
 * sum_d (q_d - p_d)^2 <= radius2.  Search: points sorted by their first coordinate, a
 * binary search bounds the candidate slab.  Test infrastructure only.
 */
#ifndef TXREF_KDTREE_H
#define TXREF_KDTREE_H
#include <algorithm>
#include <cmath>
#include <vector>

template <typename T>
struct KDnode
{
    long int index;
    std::vector<T> point;
};

template <typename T>
class KDtree
{
public:
    explicit KDtree(int nd) : ndim(nd), ncluster(0) {}

    void build(std::vector<std::vector<T>> &points)
    {
        nodes.resize(points.size());
        order.resize(points.size());
        for (size_t i = 0; i < points.size(); i++)
        {
            nodes[i].index = (long int)i;
            nodes[i].point = points[i];
            order[i] = (long int)i;
        }
        std::sort(order.begin(), order.end(), [this](long int a, long int b) {
            if (nodes[a].point[0] != nodes[b].point[0]) return nodes[a].point[0] < nodes[b].point[0];
            return a < b;
        });
    }

    void findNeighbors(const std::vector<T> &p, T radius2, std::vector<KDnode<T> *> &out)
    {
        out.clear();
        findNeighborsAdd(p, radius2, out);
    }

    void findNeighborsAdd(const std::vector<T> &p, T radius2, std::vector<KDnode<T> *> &out)
    {
        T r = std::sqrt(radius2) * (T)1.000001 + (T)1e-300;
        T xmin = p[0] - r, xmax = p[0] + r;
        auto lo = std::lower_bound(order.begin(), order.end(), xmin,
                                   [this](long int a, T v) { return nodes[a].point[0] < v; });
        for (auto it = lo; it != order.end() && nodes[*it].point[0] <= xmax; ++it)
        {
            const std::vector<T> &q = nodes[*it].point;
            T d2 = 0;
            for (int d = 0; d < ndim; d++) d2 = d2 + (q[d] - p[d]) * (q[d] - p[d]);
            if (d2 <= radius2) out.push_back(&nodes[*it]);
        }
    }

    int ndim;
    long int ncluster;

private:
    std::vector<KDnode<T>> nodes;
    std::vector<long int> order;
};
#endif
