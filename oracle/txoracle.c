/*
 * txoracle.c -- CPU restatement of the TransientX per-block single-pulse hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle of the tests and the timed CPU baseline).  The product never
 * links or calls this file.  Build with -ffp-contract=off: every floating-point operation
 * below is meant to round exactly once, as written.
 *
 * Conventions shared with the CUDA path (they make the two bit-comparable):
 *   - block data are channel-major, x[j*ldx + i], j = channel, i = time sample;
 *   - every float sum runs in the order written here, starting from 0.0f;
 *   - per-row reductions that need FP64 use txo_red32() (lane-strided FP32 runs of 32,
 *     FP64 lane accumulators, 32-lane xor butterfly), which a warp computes identically.
 * See txoracle.h for the reference file:line each function follows.
 */
#include "txoracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static int g_threads = 0;

void txo_set_threads(int n) { g_threads = n; }

static int nthr(void)
{
#ifdef _OPENMP
    return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
    return 1;
#endif
}

/* include/candidate.h:116-119 */
double txo_dmdelay(double dm, double fh, double fl)
{
    return 4.148741601e3 * dm * (1. / (fl * fl) - 1. / (fh * fh));
}

/* src/singlepulse/singlepulse.cpp:242-254, with the reference's int/float/double mixing. */
int txo_width_ladder(float minw, float maxw, float snrloss, double tsamp, int *vwn, int cap)
{
    float mw = (double)minw < tsamp ? (float)tsamp : minw;
    float wfactor = (float)(1. / ((1. - (double)snrloss) * (1. - (double)snrloss)));
    int n = 0;
    if (cap <= 0) return 0;
    vwn[n++] = (int)round((double)mw / tsamp);
    while (n < cap) {
        int w1 = vwn[n - 1];
        int w2 = (int)((float)w1 * wfactor);
        w2 = w2 < w1 + 1 ? w1 + 1 : w2;
        if ((double)w2 * tsamp > (double)maxw) break;
        vwn[n++] = w2;
    }
    return n;
}

/* Maximum-sum window (the kadane<float> of XLibs utils.h is not in the reference tree; this
 * is the definition both implementations use): a new maximum needs a strictly larger sum
 * (earliest window wins), and the running sum restarts after it drops below zero. */
float txo_kadane(const float *y, long n, long *start, long *end)
{
    float best = -INFINITY, cur = 0.f;
    long cs = 0;
    *start = 0;
    *end = -1;
    if (n <= 0) return 0.f;
    for (long i = 0; i < n; i++) {
        cur = cur + y[i];
        if (cur > best) {
            best = cur;
            *start = cs;
            *end = i;
        }
        if (cur < 0.f) {
            cur = 0.f;
            cs = i + 1;
        }
    }
    return best;
}

/* Deterministic row reduction: mode 0 sums x, mode 1 sums x*x, mode 2 sums x*y (products
 * rounded to float).  Lane l (0..31) takes i = l, l+32, l+64, ... in runs of TXO_RED_RUN
 * summed in FP32; each run total is added to the lane's FP64 accumulator; the 32
 * accumulators are combined by an xor butterfly (offsets 16, 8, 4, 2, 1). */
#define TXO_RED_RUN 32
double txo_red32(const float *x, const float *y, long n, int mode)
{
    double acc[32], tmp[32];
    for (int l = 0; l < 32; l++) {
        double a = 0.;
        long i = l;
        while (i < n) {
            float run = 0.f;
            for (int r = 0; r < TXO_RED_RUN && i < n; r++, i += 32) {
                float v = mode == 0 ? x[i] : (mode == 1 ? x[i] * x[i] : x[i] * y[i]);
                run = run + v;
            }
            a = a + (double)run;
        }
        acc[l] = a;
    }
    for (int off = 16; off >= 1; off >>= 1) {
        for (int l = 0; l < 32; l++) tmp[l] = acc[l] + acc[l ^ off];
        memcpy(acc, tmp, sizeof(acc));
    }
    return acc[0];
}

/* Skewness-kurtosis channel zap of the raw block (the PreprocessLite filter of
 * dedisperse_fil.cpp:264-276,329, method of docs/pipeline/rfi_mitigation.rst "Skewness-Kurtosis
 * filter"; outlier rule as Candidate::azap, candidate.cpp:622-652).  Per channel the central
 * moments come from exact integer sums of (v-128)^p; skewness m3/m2^1.5 and excess kurtosis
 * m4/m2^2-3 (0 for constant channels); a channel is zapped when either lies outside
 * [Q1 - thr*R, Q3 + thr*R] with Q1 = sorted[n/4], Q3 = sorted[n-1-n/4], R = Q3-Q1.
 * mask[c] = 1 marks a zapped channel.  thr <= 0 disables the filter. */
static int cmp_double(const void *a, const void *b)
{
    double x = *(const double *)a, y = *(const double *)b;
    return (x > y) - (x < y);
}

void txo_sk_moments(const uint8_t *raw, long n0, int nchan, double *skew, double *kurt)
{
#pragma omp parallel for num_threads(nthr())
    for (int c = 0; c < nchan; c++) {
        int64_t s1 = 0, s2 = 0, s3 = 0, s4 = 0;
        for (long t = 0; t < n0; t++) {
            int64_t v = (int64_t)raw[t * (long)nchan + c] - 128;
            int64_t v2 = v * v;
            s1 += v;
            s2 += v2;
            s3 += v2 * v;
            s4 += v2 * v2;
        }
        const double n = (double)n0;
        const double a = (double)s1 / n, b = (double)s2 / n, cc = (double)s3 / n, d = (double)s4 / n;
        const double aa = a * a;
        const double m2 = b - aa;
        const double m3 = (cc - 3. * a * b) + 2. * aa * a;
        const double m4 = ((d - 4. * a * cc) + 6. * aa * b) - 3. * aa * aa;
        if (m2 > 0.) {
            skew[c] = m3 / (m2 * sqrt(m2));
            kurt[c] = m4 / (m2 * m2) - 3.;
        } else {
            skew[c] = 0.;
            kurt[c] = 0.;
        }
    }
}

int txo_skzap(const uint8_t *raw, long n0, int nchan, float thr, uint8_t *mask)
{
    memset(mask, 0, nchan);
    if (!(thr > 0.f) || nchan < 1 || n0 < 1) return 0;
    double *sk = (double *)malloc(sizeof(double) * nchan), *ku = (double *)malloc(sizeof(double) * nchan);
    double *srt = (double *)malloc(sizeof(double) * nchan);
    txo_sk_moments(raw, n0, nchan, sk, ku);
    double lo[2], hi[2];
    for (int q = 0; q < 2; q++) {
        memcpy(srt, q == 0 ? sk : ku, sizeof(double) * nchan);
        qsort(srt, nchan, sizeof(double), cmp_double);
        double q1 = srt[nchan / 4], q3 = srt[nchan - 1 - nchan / 4], R = q3 - q1;
        lo[q] = q1 - (double)thr * R;
        hi[q] = q3 + (double)thr * R;
    }
    int nz = 0;
    for (int c = 0; c < nchan; c++) {
        if (sk[c] < lo[0] || sk[c] > hi[0] || ku[c] < lo[1] || ku[c] > hi[1]) {
            mask[c] = 1;
            nz++;
        }
    }
    free(sk);
    free(ku);
    free(srt);
    return nz;
}

/* uint8 time-major raw block [n0][nchan] -> channel-major sums of td x fd neighbours
 * (src/singlepulse/candidate.cpp:395-407: k over fd outer, n over td inner); channels with
 * mask[c] != 0 contribute 0 (weight 0 as in candidate.cpp:603-618). */
void txo_unpack_downsample(const uint8_t *raw, long n0, int nchan, int td, int fd, float *x,
                           long ldx, const uint8_t *mask)
{
    int nc = nchan / fd;
    long nn = n0 / td;
#pragma omp parallel for num_threads(nthr())
    for (int j = 0; j < nc; j++) {
        for (long i = 0; i < nn; i++) {
            float acc = 0.f;
            for (int k = 0; k < fd; k++) {
                const long c = (long)j * fd + k;
                for (int t = 0; t < td; t++)
                    acc = acc + (mask && mask[c] ? 0.f : (float)raw[(i * td + t) * (long)nchan + c]);
            }
            x[(long)j * ldx + i] = acc;
        }
    }
}

/* The same downsample of a float block (time-major [n0][nchan]) that the caller already
 * preprocessed: the order of the 8-bit path (fd outer, td inner), no channel mask. */
void txo_unpack_downsample_f32(const float *blk, long n0, int nchan, int td, int fd, float *x,
                               long ldx)
{
    int nc = nchan / fd;
    long nn = n0 / td;
#pragma omp parallel for num_threads(nthr())
    for (int j = 0; j < nc; j++) {
        for (long i = 0; i < nn; i++) {
            float acc = 0.f;
            for (int k = 0; k < fd; k++) {
                const long c = (long)j * fd + k;
                for (int t = 0; t < td; t++) acc = acc + blk[(i * td + t) * (long)nchan + c];
            }
            x[(long)j * ldx + i] = acc;
        }
    }
}

/* src/singlepulse/candidate.cpp:410-418 */
void txo_downsample_freqs(const double *f, int nchan, int fd, double *out)
{
    int nc = nchan / fd;
    for (int j = 0; j < nc; j++) {
        double s = 0.;
        for (int k = 0; k < fd; k++) s += f[j * fd + k];
        out[j] = s / fd;
    }
}

/* Per-channel zero mean / unit variance (docs/pipeline/preprocess.rst:15-18).  The input is
 * the integer-valued sum-downsample of uint8 data, so the sums are exact in int64; the
 * standard deviation falls back to 1 when the variance is not positive (as
 * candidate.cpp:850 does for zdot). */
void txo_equalize(float *x, int nchan, long n, long ldx, uint8_t *live)
{
    if (n <= 0) return;
#pragma omp parallel for num_threads(nthr())
    for (int j = 0; j < nchan; j++) {
        float *r = x + (long)j * ldx;
        int64_t s1 = 0, s2 = 0;
        for (long i = 0; i < n; i++) {
            int64_t v = (int64_t)llrintf(r[i]);
            s1 += v;
            s2 += v * v;
        }
        double mean = (double)s1 / (double)n;
        double var = (double)s2 / (double)n - mean * mean;
        double sd = var > 0. ? sqrt(var) : 1.;
        float mf = (float)mean, inv = (float)(1. / sd);
        for (long i = 0; i < n; i++) r[i] = (r[i] - mf) * inv;
        if (live) live[j] = var > 0. ? 1 : 0;
    }
}

/* Equalize of a float block: the sums of the values and of their squares in the fixed FP64
 * pattern of txo_red32 instead of exact integer sums, then the same mean, variance, standard
 * deviation (1 when the variance is not positive) and apply as txo_equalize. */
void txo_equalize_f32(float *x, int nchan, long n, long ldx, uint8_t *live)
{
    if (n <= 0) return;
#pragma omp parallel for num_threads(nthr())
    for (int j = 0; j < nchan; j++) {
        float *r = x + (long)j * ldx;
        double s1 = txo_red32(r, 0, n, 0), s2 = txo_red32(r, 0, n, 1);
        double mean = s1 / (double)n;
        double var = s2 / (double)n - mean * mean;
        double sd = var > 0. ? sqrt(var) : 1.;
        float mf = (float)mean, inv = (float)(1. / sd);
        for (long i = 0; i < n; i++) r[i] = (r[i] - mf) * inv;
        if (live) live[j] = var > 0. ? 1 : 0;
    }
}

/* Channel sum at sample i in the fixed order both implementations use: 32 consecutive
 * channel blocks of ceil(nchan/32), each summed from 0.0f, block sums (empty blocks
 * included) added in order. */
#define COLSUM_BLK 32
static float colsum(const float *x, int nchan, long ldx, long i)
{
    const int cb = (nchan + COLSUM_BLK - 1) / COLSUM_BLK;
    float t = 0.f;
    for (int q = 0; q < COLSUM_BLK; q++) {
        float acc = 0.f;
        const int j1 = (q + 1) * cb < nchan ? (q + 1) * cb : nchan;
        for (int j = q * cb; j < j1; j++) acc = acc + x[(long)j * ldx + i];
        t = t + acc;
    }
    return t;
}

/* Subtract the smoothed zero-DM series (docs/pipeline/preprocess.rst:26-29): z[i] is the
 * mean over live channels at sample i, b[i] the mean of z over [i-nw/2, i+nw/2] clipped to
 * the block; b is subtracted from live channels only.  A channel is live when its block had
 * non-zero variance at Equalize (dead and zapped channels are exactly 0 there and stay 0). */
void txo_baseline(float *x, int nchan, long n, long ldx, long nw, const uint8_t *live)
{
    if (nw <= 0 || n <= 0) return;
    float *z = (float *)malloc(sizeof(float) * n);
    float *b = (float *)malloc(sizeof(float) * n);
    long h = nw / 2;
    int nlive = 0;
    for (int j = 0; j < nchan; j++) nlive += live[j] ? 1 : 0;
    if (nlive == 0) {
        free(z);
        free(b);
        return;
    }
#pragma omp parallel for num_threads(nthr())
    for (long i = 0; i < n; i++) z[i] = colsum(x, nchan, ldx, i) / (float)nlive;
#pragma omp parallel for num_threads(nthr())
    for (long i = 0; i < n; i++) {
        long lo = i - h < 0 ? 0 : i - h;
        long hi = i + h > n - 1 ? n - 1 : i + h;
        float acc = 0.f;
        for (long u = lo; u <= hi; u++) acc = acc + z[u];
        b[i] = acc / (float)(hi - lo + 1);
    }
#pragma omp parallel for num_threads(nthr())
    for (int j = 0; j < nchan; j++)
        if (live[j])
            for (long i = 0; i < n; i++) x[(long)j * ldx + i] = x[(long)j * ldx + i] - b[i];
    free(z);
    free(b);
}

/* Manual frequency zapping (docs/pipeline/rfi_mitigation.rst "Manually zap"): channels whose
 * frequency lies in [fl, fh] are filled with the channel mean, which is 0 after Equalize. */
void txo_zap_channels(float *x, int nchan, long n, long ldx, const double *freqs,
                      const double *zap, int nzap)
{
    for (int j = 0; j < nchan; j++) {
        int hit = 0;
        for (int z = 0; z < nzap; z++) {
            double lo = zap[2 * z] < zap[2 * z + 1] ? zap[2 * z] : zap[2 * z + 1];
            double hi = zap[2 * z] < zap[2 * z + 1] ? zap[2 * z + 1] : zap[2 * z];
            if (freqs[j] >= lo && freqs[j] <= hi) hit = 1;
        }
        if (hit)
            for (long i = 0; i < n; i++) x[(long)j * ldx + i] = 0.f;
    }
}

/* kadaneF (src/singlepulse/candidate.cpp:710-829) with the main-path arguments of
 * singlepulse.cpp:305-308: thr is the squared S/N threshold, wnlimit the minimum window in
 * downsampled samples, zapped samples are filled with the mean (0).  ranges[4*j + 0..3]
 * receives [start, end) in block samples of the positive and of the negative window of
 * downsampled channel j, or -1,-1 when that window is not zapped.  Returns the number of
 * zapped windows. */
int txo_kadaneF(float *x, int nchan, long n, long ldx, int tdk, int fdk, float thr,
                long wnlimit, int32_t *ranges)
{
    long nds = n / tdk;
    int cds = nchan / fdk;
    int nzapped = 0;
    float var = (float)(tdk * fdk);
#pragma omp parallel num_threads(nthr()) reduction(+ : nzapped)
    {
        float *d = (float *)malloc(sizeof(float) * (nds > 0 ? nds : 1));
        float *y = (float *)malloc(sizeof(float) * (nds > 0 ? nds : 1));
#pragma omp for
        for (int j = 0; j < cds; j++) {
            for (long i = 0; i < nds; i++) {
                float acc = 0.f;
                for (int k = 0; k < fdk; k++)
                    for (int t = 0; t < tdk; t++)
                        acc = acc + x[((long)j * fdk + k) * ldx + i * tdk + t];
                d[i] = acc;
            }
            for (int p = 0; p < 2; p++) {
                for (long i = 0; i < nds; i++) y[i] = p == 0 ? d[i] : -d[i];
                long start, end;
                float boxsum = txo_kadane(y, nds, &start, &end);
                long wn = end - start + 1;
                float snr2 = 0.f;
                if (wn > wnlimit) snr2 = boxsum * boxsum / ((float)wn * var);
                if (nds > 0 && snr2 > thr) {
                    ranges[4 * j + 2 * p] = (int32_t)(start * tdk);
                    ranges[4 * j + 2 * p + 1] = (int32_t)((end + 1) * tdk);
                    nzapped++;
                } else {
                    ranges[4 * j + 2 * p] = -1;
                    ranges[4 * j + 2 * p + 1] = -1;
                }
            }
        }
        free(d);
        free(y);
    }
#pragma omp parallel for num_threads(nthr())
    for (int j = 0; j < cds; j++)
        for (int p = 0; p < 2; p++) {
            int32_t a = ranges[4 * j + 2 * p], b = ranges[4 * j + 2 * p + 1];
            if (a < 0) continue;
            for (int k = 0; k < fdk; k++)
                for (long i = a; i < b; i++) x[((long)j * fdk + k) * ldx + i] = 0.f;
        }
    return nzapped;
}

static int cmp_float(const void *a, const void *b);

/* Sum-downsample of kadaneF (candidate.cpp:727-739): d[j*nds + i] = sum over k < fdk (outer)
 * and t < tdk (inner) of x[j*fdk + k][i*tdk + t], from 0.0f. */
static void ds_sum(const float *x, long ldx, int cds, long nds, int tdk, int fdk, float *d)
{
#pragma omp parallel for num_threads(nthr())
    for (int j = 0; j < cds; j++)
        for (long i = 0; i < nds; i++) {
            float acc = 0.f;
            for (int k = 0; k < fdk; k++)
                for (int t = 0; t < tdk; t++) acc = acc + x[((long)j * fdk + k) * ldx + i * tdk + t];
            d[(long)j * nds + i] = acc;
        }
}

/* kadaneT, the rfilist entry `kadaneT td fd` (singlepulse.cpp:310-313; the XLibs source is
 * not in the reference tree, the CLI describes a band limit in MHz and an S/N threshold,
 * dedisperse_fil.cpp:79,83).  Defined here as kadaneF with time and frequency exchanged:
 * on the td x fd sum-downsampled block, each downsampled sample i scans its channels in
 * ascending order for the maximum-sum band (txo_kadane), positive and negated; the band is
 * zapped (set to the mean, 0) when it spans more than bwlimit downsampled channels and
 * boxsum^2/(wn*td*fd) > thr (the squared threshold).  ranges[4*i + 0..3] receives the
 * [start, end) channels of the positive and negative band, or -1,-1.  Returns the number of
 * zapped bands. */
int txo_kadaneT(float *x, int nchan, long n, long ldx, int tdk, int fdk, float thr, long bwlimit,
                int32_t *ranges)
{
    const long nds = n / tdk;
    const int cds = nchan / fdk;
    if (nds <= 0 || cds <= 0) return 0;
    float *d = (float *)malloc(sizeof(float) * (size_t)cds * nds);
    ds_sum(x, ldx, cds, nds, tdk, fdk, d);
    const float var = (float)(tdk * fdk);
    int nzapped = 0;
#pragma omp parallel num_threads(nthr()) reduction(+ : nzapped)
    {
        float *y = (float *)malloc(sizeof(float) * cds);
#pragma omp for
        for (long i = 0; i < nds; i++)
            for (int p = 0; p < 2; p++) {
                for (int j = 0; j < cds; j++) y[j] = p == 0 ? d[(long)j * nds + i] : -d[(long)j * nds + i];
                long start, end;
                float boxsum = txo_kadane(y, cds, &start, &end);
                long wn = end - start + 1;
                float snr2 = 0.f;
                if (wn > bwlimit) snr2 = boxsum * boxsum / ((float)wn * var);
                if (snr2 > thr) {
                    ranges[4 * i + 2 * p] = (int32_t)(start * fdk);
                    ranges[4 * i + 2 * p + 1] = (int32_t)((end + 1) * fdk);
                    nzapped++;
                } else {
                    ranges[4 * i + 2 * p] = -1;
                    ranges[4 * i + 2 * p + 1] = -1;
                }
            }
        free(y);
    }
#pragma omp parallel for num_threads(nthr())
    for (long i = 0; i < nds; i++)
        for (int p = 0; p < 2; p++) {
            int32_t a = ranges[4 * i + 2 * p], b = ranges[4 * i + 2 * p + 1];
            if (a < 0) continue;
            for (int c = a; c < b; c++)
                for (int t = 0; t < tdk; t++) x[(long)c * ldx + i * tdk + t] = 0.f;
        }
    free(d);
    return nzapped;
}

/* Mask filter, the rfilist entry `mask td fd` (singlepulse.cpp:300-303; docs
 * pipeline/rfi_mitigation.rst "Mask filter" and its diagram: downsample by td x fd, remove
 * pixel outliers by IQR; the XLibs source is not in the reference tree).  Defined here with
 * the quartile rule of the channel zap (candidate.cpp:622-652): over all pixels d of the
 * sum-downsampled block, Q1 = sorted[n/4], Q3 = sorted[n-1-n/4], R = Q3 - Q1; pixels below
 * Q1 - thr*R or above Q3 + thr*R are zapped (their td x fd cells set to the mean, 0).
 * quart (4 floats, may be NULL) receives Q1, Q3 and the two limits.  Returns the number of
 * zapped pixels. */
int txo_mask(float *x, int nchan, long n, long ldx, int tdk, int fdk, float thr, float *quart)
{
    const long nds = n / tdk;
    const int cds = nchan / fdk;
    if (nds <= 0 || cds <= 0) return 0;
    const long np = (long)cds * nds;
    float *d = (float *)malloc(sizeof(float) * np);
    float *srt = (float *)malloc(sizeof(float) * np);
    ds_sum(x, ldx, cds, nds, tdk, fdk, d);
    memcpy(srt, d, sizeof(float) * np);
    qsort(srt, np, sizeof(float), cmp_float);
    const float q1 = srt[np / 4], q3 = srt[np - 1 - np / 4];
    const float r = q3 - q1;
    const float lo = q1 - thr * r, hi = q3 + thr * r;
    if (quart) {
        quart[0] = q1;
        quart[1] = q3;
        quart[2] = lo;
        quart[3] = hi;
    }
    int nz = 0;
#pragma omp parallel for num_threads(nthr()) reduction(+ : nz)
    for (int j = 0; j < cds; j++)
        for (long i = 0; i < nds; i++) {
            const float v = d[(long)j * nds + i];
            if (v < lo || v > hi) {
                nz++;
                for (int k = 0; k < fdk; k++)
                    for (int t = 0; t < tdk; t++) x[((long)j * fdk + k) * ldx + i * tdk + t] = 0.f;
            }
        }
    free(d);
    free(srt);
    return nz;
}

/* Zero-DM filter, the rfilist entry `zero` (singlepulse.cpp:320-323; docs usage: "zero
 * (zero-DM filter)"): the live-channel mean series is subtracted from every live channel,
 * i.e. BaseLine with a one-sample window. */
void txo_zero(float *x, int nchan, long n, long ldx, const uint8_t *live)
{
    txo_baseline(x, nchan, n, ldx, 1, live);
}

/* Zero-DM matched filter (src/singlepulse/candidate.cpp:831-897): normalise every channel,
 * form the channel-mean series s, remove each channel's least-squares fit alpha*s+beta. */
void txo_zdot(float *x, int nchan, long n, long ldx)
{
    if (n <= 0 || nchan <= 0) return;
    float *s = (float *)malloc(sizeof(float) * n);
#pragma omp parallel for num_threads(nthr())
    for (int j = 0; j < nchan; j++) {
        float *r = x + (long)j * ldx;
        double s1 = txo_red32(r, 0, n, 0), s2 = txo_red32(r, 0, n, 1);
        double mean = s1 / (double)n;
        double var = s2 / (double)n - mean * mean;
        double sd = var > 0. ? sqrt(var) : 1.;
        float mf = (float)mean, inv = (float)(1. / sd);
        for (long i = 0; i < n; i++) r[i] = (r[i] - mf) * inv;
    }
#pragma omp parallel for num_threads(nthr())
    for (long i = 0; i < n; i++) s[i] = colsum(x, nchan, ldx, i) / (float)nchan;
    double se = txo_red32(s, 0, n, 0), ss = txo_red32(s, 0, n, 1);
    double tmp = se * se - ss * (double)n;
#pragma omp parallel for num_threads(nthr())
    for (int j = 0; j < nchan; j++) {
        float *r = x + (long)j * ldx;
        double xe = txo_red32(r, 0, n, 0), xs = txo_red32(r, s, n, 2);
        double alpha = 0., beta = 0.;
        if (tmp != 0.) {
            alpha = (xe * se - xs * (double)n) / tmp;
            beta = (xs * se - xe * ss) / tmp;
        }
        float af = (float)alpha, bf = (float)beta;
        for (long i = 0; i < n; i++) r[i] = r[i] - (af * s[i] + bf);
    }
    free(s);
}

/* ---------------------------------------------------------------------------------------
 * Boxcar matched filter, restated from src/singlepulse/boxcar.cpp:180-296.
 * avx2_tail != 0 reproduces the -mavx2 build, which only visits
 * i in [wl, wl + 8*floor((n-wl-wh)/8)) for each width (boxcar.cpp:264-279).
 * ------------------------------------------------------------------------------------- */
static int cmp_float(const void *a, const void *b)
{
    float x = *(const float *)a, y = *(const float *)b;
    return (x > y) - (x < y);
}

void txo_boxcar_match(const float *tim, long n, const int *vwn, int nw, int iqr,
                      int avx2_tail, float *vS, int *vwnmax)
{
    float *csump = (float *)malloc(sizeof(float) * (n > 0 ? n : 1));
    memset(vS, 0, sizeof(float) * n);
    memset(vwnmax, 0, sizeof(int) * n);
    float mean = 0.f, var = 0.f;
    if (!iqr) {
        for (long i = 0; i < n; i++) {
            mean = mean + tim[i];
            var = var + tim[i] * tim[i];
        }
        mean = mean / (float)n;
        var = var / (float)n;
        var = var - mean * mean;
    } else {
        float *c = (float *)malloc(sizeof(float) * (n > 0 ? n : 1));
        memcpy(c, tim, sizeof(float) * n);
        qsort(c, n, sizeof(float), cmp_float);
        float q1 = c[n / 4], q2 = c[n / 2], q3 = c[n - 1 - n / 4];
        mean = q2;
        var = (float)(((double)(q3 - q1) / 1.349) * ((double)(q3 - q1) / 1.349));
        free(c);
    }
    float csum = 0.f;
    for (long i = 0; i < n; i++) {
        csum = csum + (tim[i] - mean);
        csump[i] = csum;
    }
    if (var > 0.f) {
        for (int k = 0; k < nw; k++) {
            int wn = vwn[k];
            int wl = wn / 2 + 1;
            int wh = (wn - 1) / 2;
            float temp = (float)sqrt(1. / (double)((float)wn * var));
            long lo = wl, hi = n - wh;
            if (avx2_tail) {
                int len = (int)(n - wh - wl);
                long nv = len / 8;
                hi = nv > 0 ? wl + 8 * nv : wl;
            }
            for (long i = lo; i < hi; i++) {
                float boxsum = csump[i + wh] - csump[i - wl];
                float S = boxsum * temp;
                if (S >= vS[i]) {
                    vS[i] = S;
                    vwnmax[i] = wn;
                } else if (avx2_tail && !(S < vS[i])) {
                    /* unordered compare: both AVX masks are zero and the blend yields 0 */
                    vS[i] = 0.f;
                    vwnmax[i] = 0;
                }
            }
        }
    }
    free(csump);
}

/* FP64 reference of the boxcar: the same search with mean, variance, running sum and S in
 * double (used to state the error of the float paths). */
void txo_boxcar_match_f64(const double *tim, long n, const int *vwn, int nw, float *vS,
                          int *vwnmax)
{
    double *c = (double *)malloc(sizeof(double) * (n > 0 ? n : 1));
    double *best = (double *)calloc(n > 0 ? n : 1, sizeof(double));
    memset(vwnmax, 0, sizeof(int) * n);
    double mean = 0., var = 0.;
    for (long i = 0; i < n; i++) {
        mean += tim[i];
        var += tim[i] * tim[i];
    }
    mean /= (double)n;
    var = var / (double)n - mean * mean;
    double acc = 0.;
    for (long i = 0; i < n; i++) {
        acc += tim[i] - mean;
        c[i] = acc;
    }
    if (var > 0.)
        for (int k = 0; k < nw; k++) {
            int wn = vwn[k], wl = wn / 2 + 1, wh = (wn - 1) / 2;
            double temp = sqrt(1. / ((double)wn * var));
            for (long i = wl; i < n - wh; i++) {
                double S = (c[i + wh] - c[i - wl]) * temp;
                if (S >= best[i]) {
                    best[i] = S;
                    vwnmax[i] = wn;
                }
            }
        }
    for (long i = 0; i < n; i++) vS[i] = (float)best[i];
    free(c);
    free(best);
}

void txo_boxcar_run(const float *tim, long ndm, long n, const int *vwn, int nw, int iqr,
                    int avx2_tail, float *mxS, int *mxwn)
{
#pragma omp parallel for num_threads(nthr()) schedule(dynamic, 4)
    for (long k = 0; k < ndm; k++)
        txo_boxcar_match(tim + k * n, n, vwn, nw, iqr, avx2_tail, mxS + k * n, mxwn + k * n);
}

/* ---------------------------------------------------------------------------------------
 * Threshold scan (cluster.cpp:89-112) and clustering (clustering.h:26-100 +
 * cluster.cpp:114-158).  Neighbours are points whose squared distance in
 * (dmdelay(dm,fmax,fmin)/2, isamp*tsamp) is <= radius^2.
 * ------------------------------------------------------------------------------------- */
long txo_threshold_scan(const float *mxS, const int *mxwn, long ndm, long n, float thre,
                        txo_cand *out, long cap)
{
    long c = 0;
    for (long j = 0; j < ndm; j++)
        for (long i = 0; i < n; i++) {
            float S = mxS[j * n + i];
            if (S > thre) {
                if (c < cap) {
                    out[c].idm = j;
                    out[c].isamp = i;
                    out[c].wn = mxwn[j * n + i];
                    out[c].S = S;
                }
                c++;
            }
        }
    return c;
}

typedef struct {
    double x, y;
    long idx;
} pt_t;

static int cmp_pt(const void *a, const void *b)
{
    const pt_t *p = (const pt_t *)a, *q = (const pt_t *)b;
    if (p->x != q->x) return p->x < q->x ? -1 : 1;
    return (p->idx > q->idx) - (p->idx < q->idx);
}

/* all points within radius^2 of (px, py), by scanning the x-sorted list */
static long neighbours(const pt_t *sorted, long n, double px, double py, double r2, double r,
                       long *out)
{
    long lo = 0, hi = n, m = 0;
    double xmin = px - r * 1.000001 - 1e-300;
    while (lo < hi) {
        long mid = (lo + hi) / 2;
        if (sorted[mid].x < xmin) lo = mid + 1;
        else hi = mid;
    }
    double xmax = px + r * 1.000001 + 1e-300;
    for (long i = lo; i < n && sorted[i].x <= xmax; i++) {
        double dx = sorted[i].x - px, dy = sorted[i].y - py;
        if (dx * dx + dy * dy <= r2) out[m++] = sorted[i].idx;
    }
    return m;
}

long txo_cluster(const txo_cand *cands, long ncand, double dms, double ddm, double fmax,
                 double fmin, double tsamp, double radius_smearing, int maxncand, int minpts,
                 int drop, int maxwn, txo_cand *out, int32_t *cluster_size_out)
{
    long n = ncand;
    pt_t *pts = (pt_t *)malloc(sizeof(pt_t) * (n > 0 ? n : 1));
    pt_t *sorted = (pt_t *)malloc(sizeof(pt_t) * (n > 0 ? n : 1));
    for (long i = 0; i < n; i++) {
        double dm = dms + cands[i].idm * ddm;
        pts[i].x = txo_dmdelay(dm, fmax, fmin) * 0.5;
        pts[i].y = cands[i].isamp * tsamp;
        pts[i].idx = i;
    }
    memcpy(sorted, pts, sizeof(pt_t) * n);
    qsort(sorted, n, sizeof(pt_t), cmp_pt);
    if (radius_smearing < 1.5 * tsamp) radius_smearing = 1.5 * tsamp;
    double r2 = radius_smearing * radius_smearing;
    double r = sqrt(r2);

    long *cid = (long *)calloc(n > 0 ? n : 1, sizeof(long));     /* states[i][1] */
    char *visited = (char *)calloc(n > 0 ? n : 1, 1);             /* states[i][2] == 2 */
    char *inset = (char *)calloc(n > 0 ? n : 1, 1);
    long *idxs1 = (long *)malloc(sizeof(long) * (n > 0 ? n : 1));
    long *front = (long *)malloc(sizeof(long) * (n > 0 ? n : 1));
    long *next = (long *)malloc(sizeof(long) * (n > 0 ? n : 1));
    long *nb = (long *)malloc(sizeof(long) * (n > 0 ? n : 1));
    long *reached = (long *)malloc(sizeof(long) * (n > 0 ? n : 1));
    long n1 = n;
    for (long i = 0; i < n; i++) idxs1[i] = i;

    int icluster = 0;
    while ((icluster++ < maxncand) && n1 > 0) {
        float maxsnr = -1.f, maxsnr_idx = -1.f; /* the seed index is held in a float */
        for (long q = 0; q < n1; q++)
            if (cands[idxs1[q]].S > maxsnr) {
                maxsnr = cands[idxs1[q]].S;
                maxsnr_idx = (float)idxs1[q];
            }
        long seed = (long)maxsnr_idx;
        long nf = neighbours(sorted, n, pts[seed].x, pts[seed].y, r2, r, front);
        long nreached = 0;
        while (nf > 0) {
            long nn = 0;
            for (long q = 0; q < nf; q++) {
                long idx = front[q];
                cid[idx] = icluster;
                visited[idx] = 1;
                long m = neighbours(sorted, n, pts[idx].x, pts[idx].y, r2, r, nb);
                for (long t = 0; t < m; t++)
                    if (!inset[nb[t]]) {
                        inset[nb[t]] = 1;
                        next[nn++] = nb[t];
                    }
                reached[nreached++] = idx;
            }
            long nf2 = 0;
            for (long t = 0; t < nn; t++) {
                inset[next[t]] = 0;
                if (!visited[next[t]]) front[nf2++] = next[t];
            }
            nf = nf2;
        }
        /* idxs1 = idxs1 \ reached (both as sets; idxs1 stays sorted) */
        for (long t = 0; t < nreached; t++) inset[reached[t]] = 1;
        long w = 0;
        for (long q = 0; q < n1; q++)
            if (!inset[idxs1[q]]) idxs1[w++] = idxs1[q];
        for (long t = 0; t < nreached; t++) inset[reached[t]] = 0;
        n1 = w;
    }
    int ncluster = icluster - 1;

    long *mxi = (long *)malloc(sizeof(long) * (ncluster > 0 ? ncluster : 1));
    float *mxs = (float *)malloc(sizeof(float) * (ncluster > 0 ? ncluster : 1));
    size_t *size = (size_t *)calloc(ncluster > 0 ? ncluster : 1, sizeof(size_t));
    size_t *slot = (size_t *)calloc(ncluster > 0 ? ncluster : 1, sizeof(size_t));
    for (int k = 0; k < ncluster; k++) {
        mxi[k] = -1;
        mxs[k] = 0.f;
    }
    for (long i = 0; i < n; i++) {
        if (cid[i] == 0) continue;
        long c = cid[i] - 1;
        size[c]++;
        if (cands[i].S > mxs[c]) {
            mxs[c] = cands[i].S;
            mxi[c] = i;
        }
    }
    /* cluster.cpp:145-158 checks candcluster[k] while erasing from it, so after the first
     * erase the size test reads the next cluster's entry; slot[] follows the vector's
     * contents (a moved-from element reads as empty, a destroyed one keeps its size). */
    memcpy(slot, size, sizeof(size_t) * (ncluster > 0 ? ncluster : 1));
    long len = ncluster, nout = 0;
    for (long k = 0; k < ncluster; k++) {
        long m = mxi[k];
        if (m < 0) continue; /* no member above 0: the reference indexes candleft[-1] here */
        int wn = cands[m].wn;
        if (((!drop) || (wn != maxwn)) && slot[k] >= (size_t)minpts) {
            out[nout] = cands[m];
            if (cluster_size_out) cluster_size_out[nout] = (int32_t)size[k];
            nout++;
        } else {
            if (k + 1 < len) {
                for (long q = k; q < len - 1; q++) slot[q] = slot[q + 1];
                slot[len - 1] = 0;
            }
            len--;
        }
    }
    free(pts); free(sorted); free(cid); free(visited); free(inset); free(idxs1);
    free(front); free(next); free(nb); free(reached); free(mxi); free(mxs); free(size);
    free(slot);
    return nout;
}

/* ---------------------------------------------------------------------------------------
 * Two-stage subband dedispersion.  RealTime::SubbandDedispersion is XLibs code that is not in
 * the reference tree; the interface it must satisfy is fixed by its call sites
 * (singlepulse.cpp:230-238,328,338; boxcar.cpp:144-161,183; dedisperse_fil.cpp:347), the
 * algorithm by docs/pipeline/dedispersion.rst (subband dedispersion).  Definition:
 *   subband s holds channels j with j*nsub/nchan == s; fref[s] is its highest frequency;
 *   fine DM k: dm_k = dms + k*ddm; DM group g = k/group, coarse DM = mean of the group's
 *   first and last fine DM;
 *   d1[g][j] = round(dmdelay(dmc_g, fref[s(j)], f_j)/tsamp)   (within-subband delay)
 *   d2[k][s] = round(dmdelay(dm_k, fmax, fref[s])/tsamp)      (subband delay)
 *   stage 1: sub[g][s][t] = sum_{j in s, ascending} x_j[t + d1[g][j]]
 *   stage 2: tim[k][i]    = sum_{s ascending} sub[g(k)][s][t0 + i + d2[k][s]]
 *   noverlap = (long)(overlap*ndump); offset = ndump*ceil((maxd1+maxd2+noverlap)/ndump);
 *   after each block counter += ndump; output exists once
 *   counter >= offset - noverlap + ndump (the Boxcar::run gate, boxcar.cpp:161) and covers
 *   t0 = counter - ndump - offset .. t0 + ndump + noverlap - 1.
 * ------------------------------------------------------------------------------------- */
struct txo_dedisp {
    txo_dedisp_info info;
    double dms, ddm;
    double *freqs, *fref;
    int32_t *sub_start, *d1, *d2;
    float *hist, *ring, *tim;
    double *ring64, *tim64; /* FP64 mode: sums kept in double */
    long ldh;
};

txo_dedisp *txo_dedisp_create(int nchan, const double *freqs, double tsamp, long ndump,
                              double dms, double ddm, long ndm, double overlap, int nsub,
                              int group)
{
    if (nchan <= 0 || ndump <= 0 || ndm <= 0 || nsub <= 0 || nsub > nchan || group <= 0 ||
        dms < 0. || ddm < 0. || tsamp <= 0.)
        return NULL;
    txo_dedisp *dd = (txo_dedisp *)calloc(1, sizeof(txo_dedisp));
    txo_dedisp_info *in = &dd->info;
    in->nchan = nchan;
    in->nsub = nsub;
    in->group = group;
    in->ngroup = (int)((ndm + group - 1) / group);
    in->ndm = ndm;
    in->ndump = ndump;
    in->tsamp = tsamp;
    dd->dms = dms;
    dd->ddm = ddm;
    dd->freqs = (double *)malloc(sizeof(double) * nchan);
    memcpy(dd->freqs, freqs, sizeof(double) * nchan);
    dd->fref = (double *)malloc(sizeof(double) * nsub);
    dd->sub_start = (int32_t *)malloc(sizeof(int32_t) * (nsub + 1));
    for (int s = 0; s <= nsub; s++)
        dd->sub_start[s] = (int32_t)(((long)s * nchan + nsub - 1) / nsub);
    in->fmax = freqs[0];
    in->fmin = freqs[0];
    for (int j = 0; j < nchan; j++) {
        in->fmax = freqs[j] > in->fmax ? freqs[j] : in->fmax;
        in->fmin = freqs[j] < in->fmin ? freqs[j] : in->fmin;
    }
    for (int s = 0; s < nsub; s++) {
        double m = freqs[dd->sub_start[s]];
        for (int j = dd->sub_start[s]; j < dd->sub_start[s + 1]; j++) m = freqs[j] > m ? freqs[j] : m;
        dd->fref[s] = m;
    }
    int ng = in->ngroup;
    dd->d1 = (int32_t *)malloc(sizeof(int32_t) * (size_t)ng * nchan);
    dd->d2 = (int32_t *)malloc(sizeof(int32_t) * (size_t)ndm * nsub);
    long maxd1 = 0, maxd2 = 0;
    for (int g = 0; g < ng; g++) {
        long first = (long)g * group;
        long last = first + group < ndm ? first + group - 1 : ndm - 1;
        double dmc = dms + ddm * 0.5 * (double)(first + last);
        for (int s = 0; s < nsub; s++)
            for (int j = dd->sub_start[s]; j < dd->sub_start[s + 1]; j++) {
                int32_t d = (int32_t)round(txo_dmdelay(dmc, dd->fref[s], freqs[j]) / tsamp);
                dd->d1[(size_t)g * nchan + j] = d;
                maxd1 = d > maxd1 ? d : maxd1;
            }
    }
    for (long k = 0; k < ndm; k++) {
        double dm = dms + (double)k * ddm;
        for (int s = 0; s < nsub; s++) {
            int32_t d = (int32_t)round(txo_dmdelay(dm, in->fmax, dd->fref[s]) / tsamp);
            dd->d2[(size_t)k * nsub + s] = d;
            maxd2 = d > maxd2 ? d : maxd2;
        }
    }
    in->maxd1 = maxd1;
    in->maxd2 = maxd2;
    in->noverlap = (long)(overlap * (double)ndump);
    in->offset = (maxd1 + maxd2 + in->noverlap + ndump - 1) / ndump * ndump;
    in->ring = in->offset + ndump;
    in->nout = ndump + in->noverlap;
    in->counter = 0;
    dd->ldh = maxd1 + ndump;
    dd->hist = (float *)calloc((size_t)nchan * dd->ldh, sizeof(float));
    dd->ring = (float *)calloc((size_t)ng * nsub * in->ring, sizeof(float));
    dd->tim = (float *)calloc((size_t)ndm * in->nout, sizeof(float));
    return dd;
}

void txo_dedisp_destroy(txo_dedisp *dd)
{
    if (!dd) return;
    free(dd->freqs); free(dd->fref); free(dd->sub_start); free(dd->d1); free(dd->d2);
    free(dd->hist); free(dd->ring); free(dd->tim); free(dd->ring64); free(dd->tim64); free(dd);
}

/* Switch the dedispersion sums to double (both stages); txo_dedisp_run then fills the double
 * series returned by txo_dedisp_timdata64. */
void txo_dedisp_set_fp64(txo_dedisp *dd)
{
    txo_dedisp_info *in = &dd->info;
    if (dd->ring64) return;
    dd->ring64 = (double *)calloc((size_t)in->ngroup * in->nsub * in->ring, sizeof(double));
    dd->tim64 = (double *)calloc((size_t)in->ndm * in->nout, sizeof(double));
}

const double *txo_dedisp_timdata64(const txo_dedisp *dd) { return dd->tim64; }

void txo_dedisp_get_info(const txo_dedisp *dd, txo_dedisp_info *info) { *info = dd->info; }

void txo_dedisp_tables(const txo_dedisp *dd, int32_t *d1, int32_t *d2, int32_t *sub_start,
                       double *fref)
{
    const txo_dedisp_info *in = &dd->info;
    if (d1) memcpy(d1, dd->d1, sizeof(int32_t) * (size_t)in->ngroup * in->nchan);
    if (d2) memcpy(d2, dd->d2, sizeof(int32_t) * (size_t)in->ndm * in->nsub);
    if (sub_start) memcpy(sub_start, dd->sub_start, sizeof(int32_t) * (in->nsub + 1));
    if (fref) memcpy(fref, dd->fref, sizeof(double) * in->nsub);
}

static inline long pmod(long a, long m)
{
    long r = a % m;
    return r < 0 ? r + m : r;
}

int txo_dedisp_run(txo_dedisp *dd, const float *x, long ldx)
{
    txo_dedisp_info *in = &dd->info;
    long N = in->ndump, H = in->maxd1, R = in->ring, ldh = dd->ldh;
    int nchan = in->nchan, nsub = in->nsub, ng = in->ngroup;
    for (int j = 0; j < nchan; j++)
        memcpy(dd->hist + (long)j * ldh + H, x + (long)j * ldx, sizeof(float) * N);
    in->counter += N;
    long tbase = in->counter - N - H; /* absolute time of stage-1 output column 0 */
    int gated = in->counter >= in->offset - in->noverlap + N;
    if (dd->ring64) {
        /* FP64 reference: the same sums in double */
#pragma omp parallel num_threads(nthr())
        {
            double *acc = (double *)malloc(sizeof(double) * N);
#pragma omp for collapse(2) schedule(static)
            for (int g = 0; g < ng; g++)
                for (int s = 0; s < nsub; s++) {
                    double *out = dd->ring64 + ((size_t)g * nsub + s) * R;
                    const int32_t *d1 = dd->d1 + (size_t)g * nchan;
                    for (long u = 0; u < N; u++) acc[u] = 0.;
                    for (int j = dd->sub_start[s]; j < dd->sub_start[s + 1]; j++) {
                        const float *src = dd->hist + (long)j * ldh + d1[j];
                        for (long u = 0; u < N; u++) acc[u] += (double)src[u];
                    }
                    for (long u = 0; u < N; u++) out[pmod(tbase + u, R)] = acc[u];
                }
            free(acc);
        }
        if (gated) {
            long t0 = in->counter - N - in->offset, nout = in->nout;
#pragma omp parallel for num_threads(nthr()) schedule(static)
            for (long k = 0; k < in->ndm; k++) {
                int g = (int)(k / in->group);
                const int32_t *d2 = dd->d2 + (size_t)k * nsub;
                double *o = dd->tim64 + (size_t)k * nout;
                for (long i = 0; i < nout; i++) o[i] = 0.;
                for (int s = 0; s < nsub; s++) {
                    const double *row = dd->ring64 + ((size_t)g * nsub + s) * R;
                    for (long i = 0; i < nout; i++) o[i] += row[pmod(t0 + i + d2[s], R)];
                }
                float *of = dd->tim + (size_t)k * nout;
                for (long i = 0; i < nout; i++) of[i] = (float)o[i];
            }
        }
    } else {
        /* Loops run channel (subband) outermost and time innermost so they vectorise; every
         * output still sums its terms in ascending channel (subband) order from 0.0f. */
    #pragma omp parallel num_threads(nthr())
        {
            float *acc = (float *)malloc(sizeof(float) * (N > in->nout ? N : in->nout));
    #pragma omp for collapse(2) schedule(static)
            for (int g = 0; g < ng; g++)
                for (int s = 0; s < nsub; s++) {
                    float *out = dd->ring + ((size_t)g * nsub + s) * R;
                    const int32_t *d1 = dd->d1 + (size_t)g * nchan;
                    for (long u = 0; u < N; u++) acc[u] = 0.f;
                    for (int j = dd->sub_start[s]; j < dd->sub_start[s + 1]; j++) {
                        const float *src = dd->hist + (long)j * ldh + d1[j];
                        for (long u = 0; u < N; u++) acc[u] = acc[u] + src[u];
                    }
                    for (long u = 0; u < N; u++) out[pmod(tbase + u, R)] = acc[u];
                }
            free(acc);
        }
        if (gated) {
            long t0 = in->counter - N - in->offset, nout = in->nout;
    #pragma omp parallel for num_threads(nthr()) schedule(static)
            for (long k = 0; k < in->ndm; k++) {
                int g = (int)(k / in->group);
                const int32_t *d2 = dd->d2 + (size_t)k * nsub;
                float *o = dd->tim + (size_t)k * nout;
                for (long i = 0; i < nout; i++) o[i] = 0.f;
                for (int s = 0; s < nsub; s++) {
                    const float *row = dd->ring + ((size_t)g * nsub + s) * R;
                    long t = pmod(t0 + d2[s], R), i = 0;
                    while (i < nout) { /* contiguous runs up to the ring end */
                        long run = R - t < nout - i ? R - t : nout - i;
                        for (long q = 0; q < run; q++) o[i + q] = o[i + q] + row[t + q];
                        i += run;
                        t = 0;
                    }
                }
            }
        }
    }
    for (int j = 0; j < nchan; j++)
        memmove(dd->hist + (long)j * ldh, dd->hist + (long)j * ldh + N, sizeof(float) * H);
    return gated;
}

const float *txo_dedisp_timdata(const txo_dedisp *dd) { return dd->tim; }

/* SubbandDedispersion::get_subdata(sub, idm, true) (candplot.cpp:123) after a gated block:
 * the nsub subband series of fine DM idm aligned at that DM, out[s*nout + i] =
 * ring[g][s][t0 + i + d2[idm][s]], the sums of each subband's channels (FP32 ring). */
int txo_dedisp_subdata(const txo_dedisp *dd, long idm, float *out)
{
    const txo_dedisp_info *in = &dd->info;
    if (idm < 0 || idm >= in->ndm || !dd->ring) return -1;
    const long N = in->ndump, R = in->ring, nout = in->nout;
    const long t0 = in->counter - N - in->offset;
    const int nsub = in->nsub;
    const long g = idm / in->group;
    for (int s = 0; s < nsub; s++) {
        const float *row = dd->ring + ((size_t)g * nsub + s) * R;
        const int32_t d = dd->d2[(size_t)idm * nsub + s];
        for (long i = 0; i < nout; i++) out[(size_t)s * nout + i] = row[pmod(t0 + i + d, R)];
    }
    return 0;
}

/* The fl/fh of a candidate's .cands line (candplot.cpp:143-231): per subband j the sum over
 * samples i in (isamp-wn, isamp+wn) of sub[j][i]/fcnt[j] (ascending i, from 0), the
 * maximum-sum run of subbands (txo_kadane), and fl, fh = the ends of that run on the linear
 * frequency axis vfnorm[j] = f[0] + j/(nsub-1.)*(f[nsub-1] - f[0]) of the subband
 * frequencies f (here the mean frequency of each subband's channels). */
void txo_cand_band(const float *sub, int nsub, long nout, const int32_t *sub_start,
                   const double *fsub, long isamp, int wn, float *fl, float *fh)
{
    float *vpf = (float *)malloc(sizeof(float) * nsub);
    const long lo = isamp - wn + 1 < 0 ? 0 : isamp - wn + 1;
    const long hi = isamp + wn < nout ? isamp + wn : nout;
    for (int j = 0; j < nsub; j++) {
        const float cnt = (float)(sub_start[j + 1] - sub_start[j]);
        float acc = 0.f;
        for (long i = lo; i < hi; i++) acc = acc + sub[(size_t)j * nout + i] / cnt;
        vpf[j] = acc;
    }
    long fs = 0, fe = 0;
    txo_kadane(vpf, nsub, &fs, &fe);
    if (fe < 0) fe = 0;
    const double den = nsub > 1 ? nsub - 1. : 1.;
    *fl = (float)(fsub[0] + fs / den * (fsub[nsub - 1] - fsub[0]));
    *fh = (float)(fsub[0] + fe / den * (fsub[nsub - 1] - fsub[0]));
    free(vpf);
}

/* ---------------------------------------------------------------------------------------
 * One ddplan row: SinglePulse::prepare/run (singlepulse.cpp:206-254, 287-341) without the
 * plotting; the rfilist ops run in their listed order.
 * ------------------------------------------------------------------------------------- */
struct txo_sp {
    txo_row row;
    uint8_t *mask, *live;
    int nchan_raw, nchan;
    long ndump_raw, n;
    double tsamp;
    double *freqs;
    float *x;
    long ldx;
    int32_t *ranges[8];
    int vwn[256];
    int nw;
    txo_dedisp *dd;
    float *mxS;
    int *mxwn;
};

txo_sp *txo_sp_create(const txo_row *row, int nchan, const double *freqs, double tsamp,
                      long ndump)
{
    if (row->td <= 0 || row->fd <= 0 || ndump % row->td != 0 || nchan % row->fd != 0)
        return NULL;
    txo_sp *sp = (txo_sp *)calloc(1, sizeof(txo_sp));
    sp->row = *row;
    sp->nchan_raw = nchan;
    sp->ndump_raw = ndump;
    sp->nchan = nchan / row->fd;
    sp->n = ndump / row->td;
    sp->tsamp = tsamp * row->td;
    sp->freqs = (double *)malloc(sizeof(double) * sp->nchan);
    txo_downsample_freqs(freqs, nchan, row->fd, sp->freqs);
    sp->ldx = sp->n;
    sp->x = (float *)calloc((size_t)sp->nchan * sp->ldx, sizeof(float));
    sp->mask = (uint8_t *)calloc(nchan, 1);
    sp->live = (uint8_t *)calloc(sp->nchan, 1);
    for (int r = 0; r < row->nrfi && r < 8; r++) {
        if (row->rfi_kind[r] == TXO_RFI_KADANEF)
            sp->ranges[r] = (int32_t *)calloc((size_t)4 * (sp->nchan / row->rfi_fd[r] + 1), 4);
        else if (row->rfi_kind[r] == TXO_RFI_KADANET)
            sp->ranges[r] = (int32_t *)calloc((size_t)4 * (sp->n / row->rfi_td[r] + 1), 4);
        else if (row->rfi_kind[r] == TXO_RFI_MASK)
            sp->ranges[r] = (int32_t *)calloc(4, 4);
    }
    sp->dd = txo_dedisp_create(sp->nchan, sp->freqs, sp->tsamp, sp->n, row->dms, row->ddm,
                               row->ndm, row->overlap, row->nsub, row->group);
    if (!sp->dd) {
        txo_sp_destroy(sp);
        return NULL;
    }
    if (row->fp64) txo_dedisp_set_fp64(sp->dd);
    sp->nw = txo_width_ladder(row->minw, row->maxw, row->snrloss, sp->tsamp, sp->vwn, 256);
    long nout = sp->dd->info.nout;
    sp->mxS = (float *)calloc((size_t)row->ndm * nout, sizeof(float));
    sp->mxwn = (int *)calloc((size_t)row->ndm * nout, sizeof(int));
    return sp;
}

void txo_sp_destroy(txo_sp *sp)
{
    if (!sp) return;
    free(sp->freqs);
    free(sp->x);
    free(sp->mask);
    free(sp->live);
    for (int r = 0; r < 8; r++) free(sp->ranges[r]);
    txo_dedisp_destroy(sp->dd);
    free(sp->mxS);
    free(sp->mxwn);
    free(sp);
}

static int sp_rest(txo_sp *sp);

int txo_sp_run(txo_sp *sp, const uint8_t *raw)
{
    const txo_row *row = &sp->row;
    txo_skzap(raw, sp->ndump_raw, sp->nchan_raw, row->zapthre, sp->mask);
    txo_unpack_downsample(raw, sp->ndump_raw, sp->nchan_raw, row->td, row->fd, sp->x, sp->ldx,
                          sp->mask);
    txo_equalize(sp->x, sp->nchan, sp->n, sp->ldx, sp->live);
    return sp_rest(sp);
}

/* SinglePulse::run on a float block the caller preprocessed: no channel zap, float downsample
 * and float equalize, then the same chain. */
int txo_sp_run_f32(txo_sp *sp, const float *blk)
{
    const txo_row *row = &sp->row;
    memset(sp->mask, 0, (size_t)sp->nchan_raw);
    txo_unpack_downsample_f32(blk, sp->ndump_raw, sp->nchan_raw, row->td, row->fd, sp->x, sp->ldx);
    txo_equalize_f32(sp->x, sp->nchan, sp->n, sp->ldx, sp->live);
    return sp_rest(sp);
}

/* baseline, zaplist, rfilist, dedispersion and boxcar of one block (singlepulse.cpp:291-330) */
static int sp_rest(txo_sp *sp)
{
    const txo_row *row = &sp->row;
    long nw = row->bswidth > 0.f ? (long)round((double)row->bswidth / sp->tsamp) : 0;
    txo_baseline(sp->x, sp->nchan, sp->n, sp->ldx, nw, sp->live);
    if (row->nzap > 0)
        txo_zap_channels(sp->x, sp->nchan, sp->n, sp->ldx, sp->freqs, &row->zap[0][0], row->nzap);
    for (int r = 0; r < row->nrfi && r < 8; r++) {
        if (row->rfi_kind[r] == TXO_RFI_KADANEF) {
            float thr = row->threKadaneF * row->threKadaneF;
            long wnlimit = (long)(row->widthlimit / (sp->tsamp * row->rfi_td[r]));
            txo_kadaneF(sp->x, sp->nchan, sp->n, sp->ldx, row->rfi_td[r], row->rfi_fd[r], thr,
                        wnlimit, sp->ranges[r]);
        } else if (row->rfi_kind[r] == TXO_RFI_ZDOT) {
            txo_zdot(sp->x, sp->nchan, sp->n, sp->ldx);
        } else if (row->rfi_kind[r] == TXO_RFI_KADANET) {
            const double chbw = sp->nchan > 1 ? fabs(sp->freqs[1] - sp->freqs[0]) : 0.;
            const long bwlimit = chbw > 0. ? (long)(row->bandlimitKT / (chbw * row->rfi_fd[r])) : 0;
            txo_kadaneT(sp->x, sp->nchan, sp->n, sp->ldx, row->rfi_td[r], row->rfi_fd[r],
                        row->threKadaneT * row->threKadaneT, bwlimit, sp->ranges[r]);
        } else if (row->rfi_kind[r] == TXO_RFI_MASK) {
            sp->ranges[r][0] = txo_mask(sp->x, sp->nchan, sp->n, sp->ldx, row->rfi_td[r],
                                        row->rfi_fd[r], row->threMask, NULL);
        } else if (row->rfi_kind[r] == TXO_RFI_ZERO) {
            txo_zero(sp->x, sp->nchan, sp->n, sp->ldx, sp->live);
        }
    }
    int gated = txo_dedisp_run(sp->dd, sp->x, sp->ldx);
    if (gated && row->fp64) {
        const long nout = sp->dd->info.nout;
#pragma omp parallel for num_threads(nthr()) schedule(dynamic, 4)
        for (long k = 0; k < row->ndm; k++)
            txo_boxcar_match_f64(sp->dd->tim64 + k * nout, nout, sp->vwn, sp->nw, sp->mxS + k * nout,
                                 sp->mxwn + k * nout);
    } else if (gated) {
        txo_boxcar_run(sp->dd->tim, row->ndm, sp->dd->info.nout, sp->vwn, sp->nw, row->iqr,
                       row->avx2_tail, sp->mxS, sp->mxwn);
    }
    return gated;
}

int txo_sp_nwidths(const txo_sp *sp, int *vwn, int cap)
{
    for (int k = 0; k < sp->nw && k < cap; k++) vwn[k] = sp->vwn[k];
    return sp->nw;
}

void txo_sp_dedisp_info(const txo_sp *sp, txo_dedisp_info *info) { *info = sp->dd->info; }

const float *txo_sp_block(const txo_sp *sp, long *ldx, int *nchan, long *n)
{
    *ldx = sp->ldx;
    *nchan = sp->nchan;
    *n = sp->n;
    return sp->x;
}

const int32_t *txo_sp_zap_ranges(const txo_sp *sp, int irfi, int *nrows)
{
    if (irfi < 0 || irfi >= 8 || !sp->ranges[irfi]) return NULL;
    const int kind = sp->row.rfi_kind[irfi];
    *nrows = kind == TXO_RFI_KADANEF ? sp->nchan / sp->row.rfi_fd[irfi]
             : kind == TXO_RFI_KADANET ? (int)(sp->n / sp->row.rfi_td[irfi]) : 1;
    return sp->ranges[irfi];
}

const float *txo_sp_timdata(const txo_sp *sp) { return sp->dd->tim; }
const txo_dedisp *txo_sp_dedisp(const txo_sp *sp) { return sp->dd; }
const uint8_t *txo_sp_mask(const txo_sp *sp) { return sp->mask; }
const float *txo_sp_mxS(const txo_sp *sp) { return sp->mxS; }
const int *txo_sp_mxwn(const txo_sp *sp) { return sp->mxwn; }
void txo_sp_freqs(const txo_sp *sp, double *out)
{
    memcpy(out, sp->freqs, sizeof(double) * sp->nchan);
}
