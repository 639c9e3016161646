/*
 * ref_replot.cpp -- extern "C" entry around the reference's own Candidate class
 * (src/singlepulse/candidate.cpp compiled in place) running the per-candidate chain of
 * replot_fil (src/singlepulse/replot_fil.cpp:409-457): [zdot] -> get_stats -> dedisperse
 * (incoherent) -> shrink_to_fit -> azap -> zap -> get_stats -> normalize -> [clip] ->
 * [kadaneF] -> downsample(1, fd) -> optimize + matched_filter, or peak_search (nopt).
 * Steps are numbered 1..12 in that order; `upto` stops after a step, so that each stage can
 * be compared.  Test infrastructure only.
 */
#include <cstring>
#include <utility>
#include <vector>

#include "candidate.h"

/* the reference's thread-count global (defined in ref_harness.cpp).  Candidate::peak_search
 * adds channels into the shared profile inside an OpenMP loop over channels
 * (candidate.cpp:1113-1121), a data race with more than one thread: the chain runs with one. */
extern unsigned int num_threads;

extern "C" int ref_replot(const float *data, int nchan, long nbin, double tbin, const double *freqs,
                          double dm, double width, int zdot, const int *kadane, const int *clip,
                          float zapthre, const double *zap, int nzap, int fd, float snrloss,
                          int nwidth, int pow2bin, int nopt, int upto, float *data_out,
                          long data_cap, long *nbin_out, int *nchan_out, float *snr, float *width_out,
                          double *dm_maxsnr, double *mjd, float *snrmap, long snrmap_cap,
                          int *ndm_out)
{
    num_threads = 1;
    Candidate c;
    c.npol = 1;
    c.nchan = nchan;
    c.nbin = nbin;
    c.tbin = tbin;
    c.frequencies.assign(freqs, freqs + nchan);
    c.data.assign(data, data + (size_t)nchan * nbin);
    c.dm = dm;
    c.width = c.width_orig = (float)width;
    c.mjd_start = 0.;
    std::vector<std::pair<double, double>> zaplist;
    for (int z = 0; z < nzap; z++) zaplist.emplace_back(zap[2 * z], zap[2 * z + 1]);
    int step = 0;
    if (zdot) c.zdot();
    if (++step < upto) c.get_stats();
    if (++step < upto) c.dedisperse(false);
    if (++step < upto) c.shrink_to_fit(2 * nwidth, pow2bin != 0, kadane ? kadane[0] : 1);
    if (++step < upto) c.azap(zapthre);
    if (++step < upto) c.zap(zaplist);
    if (++step < upto) c.get_stats();
    if (++step < upto) c.normalize();
    if (++step < upto && clip) c.clip(clip[0], clip[1], (float)clip[2]);
    if (++step < upto && kadane) c.kadaneF(kadane[0], kadane[1], (float)kadane[2]);
    if (++step < upto) c.downsample(1, fd);
    if (++step < upto) {
        if (!nopt) {
            c.optimize();
            c.matched_filter(snrloss);
        } else {
            c.peak_search(snrloss);
        }
        *snr = c.snr;
        *width_out = c.width;
        *dm_maxsnr = c.dm_maxsnr;
        *mjd = (double)c.mjd;
        *ndm_out = nopt ? 1 : c.ndm;
        const long m = (long)c.dmtsnrmap.size();
        if (snrmap) std::memcpy(snrmap, c.dmtsnrmap.data(), sizeof(float) * (m < snrmap_cap ? m : snrmap_cap));
    }
    *nbin_out = c.nbin;
    *nchan_out = c.nchan;
    const long n = (long)c.data.size();
    if (data_out) std::memcpy(data_out, c.data.data(), sizeof(float) * (n < data_cap ? n : data_cap));
    return 0;
}
