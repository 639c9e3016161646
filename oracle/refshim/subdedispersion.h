/*
 * subdedispersion.h -- stand-in for XLibs' RealTime::SubbandDedispersion, reduced to the
 * members that src/singlepulse/boxcar.cpp (:142-183) and cluster.cpp (:102) read.  The
 * parity harness points `series` at dedispersed data it generated; get_timdata returns
 * row idm of it.  Test infrastructure only.
 */
#ifndef TXREF_SUBDEDISPERSION_H
#define TXREF_SUBDEDISPERSION_H
#include <vector>
#include "utils.h"

namespace RealTime
{
class SubbandDedispersion
{
public:
    struct Sub
    {
        long int nchans = 0;
        double tsamp = 0.;
        std::vector<double> frequencies;
    } sub;

    long int counter = 0, offset = 0, noverlap = 0, ndump = 0, ndm = 0, nchans = 0;
    double dms = 0., ddm = 0., tsamp = 0.;
    std::vector<double> frequencies;
    const float *series = nullptr; /* [ndm][ndump+noverlap] */

    void get_timdata(std::vector<float> &tim, int idm, bool = true) const
    {
        long int n = ndump + noverlap;
        tim.assign(series + (long int)idm * n, series + ((long int)idm + 1) * n);
    }
    void get_subdata(std::vector<float> &s, int, bool = false) const { s.clear(); }

    /* dispersion delay with the constant of include/candidate.h:116-119 */
    static double dmdelay(double dm, double fh, double fl)
    {
        return 4.148741601e3 * dm * (1. / (fl * fl) - 1. / (fh * fh));
    }
};
} // namespace RealTime
#endif
