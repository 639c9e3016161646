/*
 * cluster.h -- Cluster<T> with the public interface of the reference's include/cluster.h:
 * run() clusters the S > thre points of the last block of the boxcar's GPU row with
 * Cluster<double>::run's rule (txg_cluster, cluster.cpp:63-161, clustering.h:26-100) and fills
 * candlist (idm, isamp, wn, S) and candcluster (each reported candidate's cluster bounds as
 * (idm, isamp) pairs: its lowest and highest DM index and sample).  candstate is not kept.
 */
#ifndef TXG_COMPAT_CLUSTER_H
#define TXG_COMPAT_CLUSTER_H

#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include "boxcar.h"
#include "compat_common.h"

template <typename T>
class Cluster {
public:
    Cluster() = default;
    Cluster(const Cluster &) = default;
    Cluster &operator=(const Cluster &) = default;
    ~Cluster() = default;

    bool run(Boxcar &boxcar, float threS, double radius_smearing, int kvalue, int maxncand,
             int minpts, bool remove_cand_with_maxwidth)
    {
        (void)threS;  /* the row's threshold selected the points on the GPU */
        (void)kvalue; /* the neighbour count of the reference's KD-tree search is not used
                         by its clustering rule either */
        counter = boxcar.counter;
        if (counter <= 0) return false;
        tsamp = boxcar.tsamp;
        nsamples = boxcar.nsamples;
        dms = boxcar.dms;
        ddm = boxcar.ddm;
        ndm = boxcar.ndm;
        candlist.clear();
        candcluster.clear();
        const txg_compat::Binding &g = boxcar.gpu();
        int64_t n = 0;
        txg_compat::check(txg_get_candidates(g.h, g.beam, g.row, nullptr, 0, &n), "Cluster::run");
        std::vector<txg_cand> pts((size_t)n);
        txg_compat::check(txg_get_candidates(g.h, g.beam, g.row, pts.data(), n, &n), "Cluster::run");
        std::vector<txg_cand> out((size_t)(maxncand > 0 ? maxncand : 1));
        int64_t nout = 0;
        txg_compat::check(txg_cluster(pts.data(), n, boxcar.dms, boxcar.ddm, boxcar.fmax,
                                      boxcar.fmin, boxcar.tsamp, radius_smearing, maxncand,
                                      minpts, remove_cand_with_maxwidth ? 1 : 0, boxcar.maxwn,
                                      out.data(), (int64_t)out.size(), &nout),
                          "Cluster::run");
        for (int64_t k = 0; k < nout; k++) {
            candlist.emplace_back((long int)out[k].idm, (long int)out[k].isamp, out[k].wn, out[k].S);
            candcluster.push_back({{(long int)out[k].idm, (long int)out[k].isamp}});
        }
        return true;
    }
    void dumpstate2txt(const std::string fname)
    {
        FILE *f = std::fopen(fname.c_str(), "w");
        if (!f) return;
        for (auto &c : candlist)
            std::fprintf(f, "%ld %ld %d %f\n", std::get<0>(c), std::get<1>(c), std::get<2>(c),
                         (double)std::get<3>(c));
        std::fclose(f);
    }

public:
    long int counter = 0;
    double tsamp = 0.;
    long int nsamples = 0;
    double dms = 0.;
    double ddm = 0.;
    long int ndm = 0;
    std::vector<std::tuple<long int, long int, int, float>> candlist;
    std::vector<std::vector<std::pair<long int, long int>>> candcluster;
    std::vector<std::tuple<T, T, long int, long int>> candstate;
};

#endif
