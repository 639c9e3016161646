/*
 * txg_internal.h -- internal declarations shared by the host planner, the C ABI and the
 * CUDA kernels of the GB300 single-pulse search.
 */
#ifndef TXG_INTERNAL_H
#define TXG_INTERNAL_H

#include <stdint.h>
#include <string>
#include <vector>

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "../../include/transientx_gb300.h"

namespace txg {

/* Host-side plan of one ddplan row (beam independent). */
struct RowPlan {
    txg_row cfg;
    int C = 0;            /* channels after fd */
    long N = 0;           /* block samples after td */
    double tsamp = 0.;    /* sampling time after td */
    std::vector<double> freqs;
    double fmax = 0., fmin = 0.;
    /* subband dedispersion geometry */
    int nsub = 0, G = 0, ng = 0;
    long maxd1 = 0, maxd2 = 0, noverlap = 0, offset = 0, nout = 0;
    long R = 0;           /* ring modulus (>= offset + N, multiple of 32) */
    long H = 0;           /* history columns kept in front of each block (>= maxd1) */
    long s2_span = 0;     /* largest d2 spread inside one stage-2 DM chunk */
    int maxch = 0;        /* channels in the widest subband */
    long ldh = 0;         /* row stride of the channel buffer */
    std::vector<int32_t> sub_start; /* nsub+1 */
    std::vector<double> fref;       /* nsub */
    std::vector<double> fsub;       /* nsub: mean frequency of each subband's channels */
    std::vector<int32_t> d1;        /* [ng][C] */
    std::vector<int32_t> d2;        /* [ndm][nsub] */
    std::vector<int32_t> vwn;
    int maxwn = 0;
    long bl_nw = 0;       /* baseline window in samples, 0 = off */
    std::vector<int32_t> zap_chan;
    long kad_wnlimit[8] = {0}; /* kadaneF: minimum window (samples); kadaneT: minimum band
                                * (channels), both downsampled */
    float kad_thr = 0.f;       /* threKadaneF^2 */
    float kadT_thr = 0.f;      /* threKadaneT^2 */
    float mask_thr = 0.f;      /* threMask (IQR units) */
    /* dedispersion launch shapes */
    int s1_var = 0;   /* resident stage-1 launch shape, 0 = default */
    int s2_var = 0;   /* stage-2 threads per CTA, 0 = default (see txg_dedisp.cu) */
    int s2_kb = 0;    /* stage-2 shared memory per CTA, KB (0 = the kernel's default) */
};

/* Deterministic planning helpers (txg_plan.cpp). */
double dmdelay(double dm, double fh, double fl);
int width_ladder(float minw, float maxw, float snrloss, double tsamp, int32_t *vwn, int cap);
int plan_row(const txg_row &cfg, int nchans_raw, const double *freqs_raw, double tsamp_raw,
             long ndump_raw, RowPlan &out, std::string &err);
int auto_nsub(int C, const std::vector<double> &freqs, double tsamp, double ddm, long ndm);
int auto_group(int C, int nsub, const std::vector<double> &freqs, double tsamp, double ddm,
               long ndm);

/* Host clustering (txg_cluster.cpp). */
long cluster_run(const txg_cand *c, long n, double dms, double ddm, double fmax, double fmin,
                 double tsamp, double radius, int maxncand, int minpts, int drop, int maxwn,
                 txg_cand *out, long cap);

/* ---- kernel launchers (txg_pre.cu, txg_dedisp.cu, txg_boxcar.cu) -------------------- */
void launch_skzap(const uint8_t *raw, int C_raw, long n0, float thr, unsigned long long *sums,
                  double *stats, uint8_t *mask, cudaStream_t st);
size_t skzap_max_channels();
/* Unpack + downsample.  With `part` (eq_part_tiles(N) x C pairs of 64-bit words) the unpack
 * also writes equalize's per-tile integer sums; returns whether it did (some unpack shapes
 * do not, and launch_eq_params then reads the block). */
long eq_part_tiles(long N);
bool launch_unpack(const uint8_t *raw, int C_raw, long n0, int td, int fd, float *x, long ldx,
                   int C, long N, const uint8_t *mask, unsigned long long *part, cudaStream_t st);
/* equalize: per-channel (mean, 1/sd) and live flags; the apply is fused into the next pass */
void launch_eq_params(const unsigned long long *part, const float *x, long ldx, int C, long N,
                      float2 *eqp, uint8_t *live, cudaStream_t st);
/* Float blocks: transpose + sum-downsample of a time-major float block, and equalize's
 * (mean, 1/sd) pairs and live flags from FP64 sums in the fixed red32 pattern. */
void launch_unpack_f32(const float *blk, int C_raw, long n0, int td, int fd, float *x, long ldx,
                       int C, long N, cudaStream_t st);
void launch_eq_params_f32(const float *x, long ldx, int C, long N, float2 *eqp, uint8_t *live,
                          cudaStream_t st);
/* x <- standardised x, minus b on live channels when b is given */
void launch_eq_apply(float *x, long ldx, int C, long N, const float2 *eqp, const float *b,
                     const uint8_t *live, cudaStream_t st);
/* column mean (tp: of the standardised block, tp[j] = (mean, 1/sd) of channel j) */
void launch_colmean(const float *x, long ldx, int C, long N, const uint8_t *live, const float2 *tp,
                    float *out, cudaStream_t st);
void launch_smooth(const float *z, long N, long nw, float *b, cudaStream_t st);
void launch_sub_series(float *x, long ldx, int C, long N, const float *b, const uint8_t *live,
                       cudaStream_t st);
void launch_zero_rows(float *x, long ldx, const int32_t *rows, int nrows, long N,
                      cudaStream_t st);
void launch_kadane(float *x, long ldx, int C, long N, int tdk, int fdk, float thr,
                   long wnlimit, float *ds, int32_t *ranges, cudaStream_t st);
/* kadaneT: maximum-sum band along frequency per downsampled sample; ranges [Nds][4]
 * (channel start,end of the positive and negative band, -1 if not zapped). */
void launch_kadaneT(float *x, long ldx, int C, long N, int tdk, int fdk, float thr,
                    long bwlimit, float *ds, int32_t *ranges, cudaStream_t st);
/* mask: pixels of the td x fd downsampled block outside [Q1 - t*R, Q3 + t*R] are zapped;
 * sel: device scratch of MASK_SEL_WORDS words (selection state, then Q1, Q3 and the two
 * limits as float bits); nzap: device int receiving the number of zapped pixels. */
constexpr int MASK_SEL_WORDS = 2 * 256 + 8;
void launch_mask(float *x, long ldx, int C, long N, int tdk, int fdk, float thr, float *ds,
                 uint32_t *sel, int32_t *nzap, cudaStream_t st);
/* zp: C (mean, 1/sd) pairs of scratch */
void launch_zdot(float *x, long ldx, int C, long N, float *s, double *sstats, float2 *zp,
                 cudaStream_t st);
/* Every precision reads the FP32 channel buffer and accumulates in FP32; the ring stores
 * FP32, BF16 or FP16 (prec).  var: resident launch shape (0 = default; see txg_dedisp.cu). */
void launch_stage1(const float *xh, long ldh, long col0, int C, long N, int nsub,
                   int ng, const int32_t *sub_start, const int32_t *d1, long maxd1, int maxch,
                   void *ring, long R, long tbase_mod, int prec, int var, int *err, cudaStream_t st);
long stage2_span(const int32_t *d2h, int nsub, int G, long ndm);
long stage2_window(long span);
/* s2_var: threads per CTA (0 = 32, 1 = 64, 2 = 128; 3-5 the same with half a group's DMs per
 * CTA); s2_kb: shared-memory budget of one stage-2 CTA in KB, 0 = the kernel's default (CTAs
 * per SM follow from it) */
void launch_stage2(const void *ring, long R, int nsub, int G, long ndm, long nout,
                   const int32_t *d2, long span, long t0_mod, int prec, int s2_var, int s2_kb,
                   float *tim, long ldt, int *err, cudaStream_t st);
/* the bounded wait of the window copies on a copy that completes (extra = 0) or on a barrier
 * expecting extra bytes more than arrive; status[0]: 0 completed, 1 gave up */
void launch_wait_selftest(const uint8_t *src, int extra, long limit_ms, int *status, cudaStream_t st);
/* the subband series of fine DM k ([nsub][nout] floats) and, per candidate, the per-subband
 * sums over its window (vpf [n][nsub]) from the subband ring */
void launch_subdata(const void *ring, long R, int nsub, int G, const int32_t *d2, long k,
                    long t0_mod, long nout, int prec, float *out, cudaStream_t st);
void launch_cand_vpf(const void *ring, long R, int nsub, int G, const int32_t *d2,
                     const int32_t *sub_start, long t0_mod, long nout, const txg_cand *c, long n,
                     int prec, float *vpf, cudaStream_t st);
/* Boxcar::run on [ndm][n] series.  Rows longer than boxcar_max_samples() use the segmented
 * kernels and need scratch (boxcar_scratch_doubles(ndm) doubles); maxwn bounds the halo. */
size_t boxcar_scratch_doubles(long ndm);
bool boxcar_supported(long n, int maxwn, int nw);
int launch_boxcar(const float *tim, long ldt, long ndm, long n, const int32_t *vwn, int nw,
                  int maxwn, int iqr, int avx2_tail, float thre, txg_cand *cand, int *ncand,
                  long cap, float *mxS, int32_t *mxwn, double *scratch, int *err, cudaStream_t st);
size_t boxcar_max_samples();

} // namespace txg

#define TXG_CUDA_TRY(expr)                                                                  \
    do {                                                                                    \
        cudaError_t e_ = (expr);                                                            \
        if (e_ != cudaSuccess) return txg::set_cuda_error(e_, #expr, __FILE__, __LINE__);   \
    } while (0)

namespace txg {
int set_cuda_error(cudaError_t e, const char *expr, const char *file, int line);
int set_arg_error(const std::string &msg);
const char *last_error_text();
} // namespace txg

#endif
