/*
 * ref_harness.cpp -- extern "C" entry points around the reference's own Boxcar
 * (src/singlepulse/boxcar.cpp) and Cluster<double> (src/singlepulse/cluster.cpp), compiled
 * in place from the reference tree by oracle/Makefile (target `ref`) into oracle/_ref/.
 * Used only to pin the oracle restatement and to generate tests/golden fixtures.
 */
#include <cstring>
#include <vector>

#include "boxcar.h"
#include "cluster.h"

/* globals the reference declares in include/dedisperse.h:25-29 and defines in
 * src/singlepulse/dedisperse_fil.cpp:34-39 */
unsigned int num_threads = 1;
unsigned int dbscan_radius = 0;
unsigned int dbscan_k = 0;
bool repeater = false;
bool dumptim = false;

static void setup(RealTime::SubbandDedispersion &dd, const float *tim, long ndm, long n,
                  double dms, double ddm, double tsamp, double fmin, double fmax)
{
    dd.ndump = n;
    dd.noverlap = 0;
    dd.ndm = ndm;
    dd.dms = dms;
    dd.ddm = ddm;
    dd.tsamp = tsamp;
    dd.nchans = 2;
    dd.frequencies = {fmax, fmin};
    dd.counter = n; /* passes the gate of boxcar.cpp:161 with offset 0 */
    dd.offset = 0;
    dd.series = tim;
}

extern "C" int ref_boxcar_run(const float *tim, long ndm, long n, const int *vwn, int nw,
                              int iqr, float *mxS, int *mxwn, int nthreads)
{
    RealTime::SubbandDedispersion dd;
    setup(dd, tim, ndm, n, 0., 1., 1e-3, 1000., 1500.);
    Boxcar b;
    b.prepare(dd);
    std::vector<int> w(vwn, vwn + nw);
    num_threads = nthreads > 0 ? nthreads : 1;
    bool ok = b.run(dd, w, iqr != 0);
    std::memcpy(mxS, b.mxS, sizeof(float) * ndm * n);
    std::memcpy(mxwn, b.mxwn, sizeof(int) * ndm * n);
    return ok ? 1 : 0;
}

extern "C" long ref_cluster_run(const float *mxS, const int *mxwn, long ndm, long n,
                                double dms, double ddm, double tsamp, double fmin,
                                double fmax, int maxwn, float thre, double radius_smearing,
                                int kvalue, int maxncand, int minpts, int drop, long counter,
                                long *out_idm, long *out_isamp, int *out_wn, float *out_S,
                                long cap)
{
    RealTime::SubbandDedispersion dd;
    setup(dd, nullptr, ndm, n, dms, ddm, tsamp, fmin, fmax);
    Boxcar b;
    b.prepare(dd);
    std::memcpy(b.mxS, mxS, sizeof(float) * ndm * n);
    std::memcpy(b.mxwn, mxwn, sizeof(int) * ndm * n);
    b.counter = counter;
    b.maxwn = maxwn;
    Cluster<double> c;
    if (!c.run(b, thre, radius_smearing, kvalue, maxncand, minpts, drop != 0)) return -1;
    long m = (long)c.candlist.size();
    for (long i = 0; i < m && i < cap; i++)
    {
        out_idm[i] = std::get<0>(c.candlist[i]);
        out_isamp[i] = std::get<1>(c.candlist[i]);
        out_wn[i] = std::get<2>(c.candlist[i]);
        out_S[i] = std::get<3>(c.candlist[i]);
    }
    return m;
}
