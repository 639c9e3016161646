/*
 * ref_rfi.cpp -- extern "C" entry around the reference's own Candidate::zdot and
 * Candidate::kadaneF (src/singlepulse/candidate.cpp:710-897, compiled in place), run on a
 * channel-major block [nchan][nbin], so that the oracle's main-path restatements (txo_zdot,
 * txo_kadaneF) can be compared with the in-tree code they follow.  Test infrastructure only.
 *
 * op 0: zdot on the block as given.
 * op 1: get_stats + normalize (Candidate::kadaneF refuses unnormalised data,
 *       candidate.cpp:712-716), the normalised block copied to `normalized`, then
 *       kadaneF(td, fd, threshold, nwidth) with the candidate width `width` and bin `tbin`.
 * The block is overwritten with the result.  ref_candidate_downsample runs
 * Candidate::downsample(td, fd) (candidate.cpp:381-427) on a block and its frequencies;
 * ref_dmdelay is Candidate::dmdelay (include/candidate.h:116-119).
 */
#include <cstring>

#include "candidate.h"

extern unsigned int num_threads;

extern "C" int ref_candidate_rfi(float *data, int nchan, long nbin, double tbin, float width, int op,
                                 int td, int fd, float threshold, int nwidth, float *normalized)
{
    num_threads = 1;
    Candidate c;
    c.npol = 1;
    c.nchan = nchan;
    c.nbin = nbin;
    c.tbin = tbin;
    c.width = c.width_orig = width;
    c.data.assign(data, data + (size_t)nchan * nbin);
    if (op == 0) {
        c.zdot();
    } else if (op == 1) {
        c.get_stats();
        c.normalize();
        if (normalized) std::memcpy(normalized, c.data.data(), sizeof(float) * (size_t)nchan * nbin);
        c.kadaneF(td, fd, threshold, nwidth);
    } else {
        return -1;
    }
    std::memcpy(data, c.data.data(), sizeof(float) * (size_t)nchan * nbin);
    return 0;
}

extern "C" int ref_candidate_downsample(const float *data, int nchan, long nbin, const double *freqs,
                                        int td, int fd, float *out, double *fout)
{
    num_threads = 1;
    Candidate c;
    c.npol = 1;
    c.nchan = nchan;
    c.nbin = nbin;
    c.tbin = 1.;
    c.frequencies.assign(freqs, freqs + nchan);
    c.data.assign(data, data + (size_t)nchan * nbin);
    c.downsample(td, fd);
    std::memcpy(out, c.data.data(), sizeof(float) * (size_t)c.nchan * c.nbin);
    std::memcpy(fout, c.frequencies.data(), sizeof(double) * (size_t)c.nchan);
    return 0;
}

extern "C" double ref_dmdelay(double dm, double fh, double fl) { return Candidate::dmdelay(dm, fh, fl); }
