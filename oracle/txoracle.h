/*
 * txoracle.h -- CPU restatement of the TransientX per-block single-pulse hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the oracle the CUDA path is compared against in
 * the tests and the timed CPU baseline of bench.py.  The product library (transientx_gb300) never
 * links, loads or calls it.
 *
 * What is restated from where (paths relative to the TransientX source tree):
 *   - stage order of one ddplan row ........ src/singlepulse/singlepulse.cpp:287-341
 *   - skewness/kurtosis channel zap ........ dedisperse_fil.cpp:264-276,329 (PreprocessLite),
 *                                            outlier rule as candidate.cpp:622-652
 *   - boxcar width ladder .................. src/singlepulse/singlepulse.cpp:242-254
 *   - time/frequency sum-downsample ......... src/singlepulse/candidate.cpp:381-427
 *   - kadaneF zapping ...................... src/singlepulse/candidate.cpp:710-829,
 *                                            main-path arguments singlepulse.cpp:305-308
 *   - zero-DM matched filter (zdot) ........ src/singlepulse/candidate.cpp:831-897
 *   - dispersion delay ..................... include/candidate.h:116-119, rounding as
 *                                            src/singlepulse/candidate.cpp:113
 *   - boxcar matched filter ................ src/singlepulse/boxcar.cpp:158-296
 *   - threshold scan + clustering .......... src/singlepulse/cluster.cpp:63-161,
 *                                            include/clustering.h:26-100
 * Equalize, BaseLine, RFI::zdot/kadaneF of the main path and RealTime::SubbandDedispersion
 * live in the external XLibs library, which is not part of the reference tree: their
 * definitions here follow the reference documentation (the rst files of docs/pipeline) and the
 * in-tree candidate.cpp versions; parity for those stages is "unpinned" against XLibs.  The
 * zdot and kadaneF restatements are compared with the reference's own Candidate::zdot and
 * Candidate::kadaneF compiled in place (ref_rfi.cpp).
 */
#ifndef TXORACLE_H
#define TXORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- scalar helpers ------------------------------------------------------------------ */
double txo_dmdelay(double dm, double fh, double fl);
int txo_width_ladder(float minw, float maxw, float snrloss, double tsamp, int *vwn, int cap);
float txo_kadane(const float *y, long n, long *start, long *end);
double txo_red32(const float *x, const float *y, long n, int mode);

/* ---- preprocessing of one block, channel-major x[j*ldx + i] --------------------------- */
void txo_sk_moments(const uint8_t *raw, long n0, int nchan, double *skew, double *kurt);
int txo_skzap(const uint8_t *raw, long n0, int nchan, float thr, uint8_t *mask);
void txo_unpack_downsample(const uint8_t *raw, long n0, int nchan, int td, int fd,
                           float *x, long ldx, const uint8_t *mask);
void txo_downsample_freqs(const double *f, int nchan, int fd, double *out);
void txo_equalize(float *x, int nchan, long n, long ldx, uint8_t *live);
void txo_baseline(float *x, int nchan, long n, long ldx, long nw, const uint8_t *live);
void txo_zap_channels(float *x, int nchan, long n, long ldx, const double *freqs,
                      const double *zap, int nzap);
int txo_kadaneF(float *x, int nchan, long n, long ldx, int tdk, int fdk, float thr,
                long wnlimit, int32_t *ranges);
void txo_zdot(float *x, int nchan, long n, long ldx);
int txo_kadaneT(float *x, int nchan, long n, long ldx, int tdk, int fdk, float thr, long bwlimit,
                int32_t *ranges);
int txo_mask(float *x, int nchan, long n, long ldx, int tdk, int fdk, float thr, float *quart);
void txo_zero(float *x, int nchan, long n, long ldx, const uint8_t *live);

/* ---- boxcar over dedispersed series (boxcar.cpp:180-296) ------------------------------ */
void txo_boxcar_match(const float *tim, long n, const int *vwn, int nw, int iqr,
                      int avx2_tail, float *vS, int *vwnmax);
void txo_boxcar_run(const float *tim, long ndm, long n, const int *vwn, int nw, int iqr,
                    int avx2_tail, float *mxS, int *mxwn);
void txo_boxcar_match_f64(const double *tim, long n, const int *vwn, int nw, float *vS,
                          int *vwnmax);

/* ---- threshold scan + clustering (cluster.cpp:63-161, clustering.h:26-100) ------------ */
typedef struct {
    int64_t idm;
    int64_t isamp;
    int32_t wn;
    float S;
} txo_cand;

long txo_threshold_scan(const float *mxS, const int *mxwn, long ndm, long n, float thre,
                        txo_cand *out, long cap);
long txo_cluster(const txo_cand *cands, long ncand, double dms, double ddm, double fmax,
                 double fmin, double tsamp, double radius_smearing, int maxncand, int minpts,
                 int drop, int maxwn, txo_cand *out, int32_t *cluster_size_out);

/* ---- two-stage subband dedispersion (streaming) --------------------------------------- */
typedef struct txo_dedisp txo_dedisp;
typedef struct {
    int nchan, nsub, group, ngroup;
    long ndm, ndump, maxd1, maxd2, noverlap, offset, ring, nout, counter;
    double tsamp, fmax, fmin;
} txo_dedisp_info;

txo_dedisp *txo_dedisp_create(int nchan, const double *freqs, double tsamp, long ndump,
                              double dms, double ddm, long ndm, double overlap, int nsub,
                              int group);
void txo_dedisp_destroy(txo_dedisp *dd);
void txo_dedisp_get_info(const txo_dedisp *dd, txo_dedisp_info *info);
void txo_dedisp_tables(const txo_dedisp *dd, int32_t *d1, int32_t *d2, int32_t *sub_start,
                       double *fref);
int txo_dedisp_run(txo_dedisp *dd, const float *x, long ldx);
const float *txo_dedisp_timdata(const txo_dedisp *dd);
void txo_dedisp_set_fp64(txo_dedisp *dd);
const double *txo_dedisp_timdata64(const txo_dedisp *dd);
int txo_dedisp_subdata(const txo_dedisp *dd, long idm, float *out);
void txo_cand_band(const float *sub, int nsub, long nout, const int32_t *sub_start,
                   const double *fsub, long isamp, int wn, float *fl, float *fh);

/* ---- one ddplan row, the SinglePulse::run chain --------------------------------------- */
enum { TXO_RFI_KADANEF = 1, TXO_RFI_ZDOT = 2, TXO_RFI_MASK = 3, TXO_RFI_KADANET = 4, TXO_RFI_ZERO = 5 };

typedef struct {
    int td, fd;
    float bswidth;
    int nrfi;
    int rfi_kind[8], rfi_td[8], rfi_fd[8];
    int nzap;
    double zap[16][2];
    float threKadaneF;
    double widthlimit;
    double dms, ddm;
    long ndm;
    double overlap;
    int nsub, group;
    float minw, maxw, snrloss;
    int iqr, avx2_tail;
    float thre;
    float zapthre;
    int fp64; /* dedispersion sums and boxcar in double: the FP64 reference */
    float threMask, threKadaneT;
    double bandlimitKT;
} txo_row;

typedef struct txo_sp txo_sp;
txo_sp *txo_sp_create(const txo_row *row, int nchan, const double *freqs, double tsamp,
                      long ndump);
void txo_sp_destroy(txo_sp *sp);
int txo_sp_run(txo_sp *sp, const uint8_t *raw);
/* SinglePulse::run on a preprocessed float block [ndump][nchan] (time-major): the caller's
 * DataBuffer<float> after PreprocessLite (dedisperse_fil.cpp:329, singlepulse.cpp:287-341). */
int txo_sp_run_f32(txo_sp *sp, const float *blk);
void txo_unpack_downsample_f32(const float *blk, long n0, int nchan, int td, int fd, float *x,
                               long ldx);
void txo_equalize_f32(float *x, int nchan, long n, long ldx, uint8_t *live);
int txo_sp_nwidths(const txo_sp *sp, int *vwn, int cap);
void txo_sp_dedisp_info(const txo_sp *sp, txo_dedisp_info *info);
const float *txo_sp_block(const txo_sp *sp, long *ldx, int *nchan, long *n);
const int32_t *txo_sp_zap_ranges(const txo_sp *sp, int irfi, int *nrows);
const float *txo_sp_timdata(const txo_sp *sp);
const uint8_t *txo_sp_mask(const txo_sp *sp);
const float *txo_sp_mxS(const txo_sp *sp);
const int *txo_sp_mxwn(const txo_sp *sp);
void txo_sp_freqs(const txo_sp *sp, double *out);
const txo_dedisp *txo_sp_dedisp(const txo_sp *sp);

void txo_set_threads(int n);

#ifdef __cplusplus
}
#endif

#endif /* TXORACLE_H */
