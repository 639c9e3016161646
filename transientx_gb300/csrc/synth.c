/*
 * synth.c -- seeded synthetic 8-bit filterbank generator (time-major [t][chan] uint8).
 *
 * Sample (t, c) = clip(floor(mean + sigma*z + A(t,c) + 0.5), 0, 255) with
 *   z = inverse normal CDF of a uniform drawn from a counter-based hash of (seed, t, c),
 *   A = sum of injected signals at (t, c):
 *     dispersed boxcar pulses (delay round(dmdelay(dm, fmax, f_c)/tsamp), constant
 *     4.148741601e3 s MHz^2 / (pc cm^-3)), amplitude snr*sigma/sqrt(nchan*width),
 *     narrow-band sinusoids on chosen channels, zero-DM broadband impulses.
 * Samples with A == 0 take a table path that yields the same value as the formula.
 * Any time range can be generated independently, so blocks can be produced on demand.
 *
 * Inverse normal CDF: P. J. Acklam's rational approximation (relative error < 1.15e-9).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
    double t0;      /* arrival time at the highest frequency (s) */
    double dm;      /* pc cm^-3 */
    double width;   /* s */
    double snr;
} txs_pulse;

typedef struct {
    int32_t chan;
    double amp;     /* in units of sigma */
    double period;  /* s */
    double phase;   /* rad */
} txs_sine;

typedef struct {
    double t0;      /* s */
    int64_t nsamp;
    double amp;     /* in units of sigma */
} txs_impulse;

typedef struct {
    int32_t nchan;
    double tsamp;
    const double *freqs;
    double mean, sigma;
    uint64_t seed;
    int32_t npulse;
    const txs_pulse *pulses;
    int32_t nsine;
    const txs_sine *sines;
    int32_t nimp;
    const txs_impulse *imps;
} txs_cfg;

static inline uint64_t mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

static inline uint32_t draw(uint64_t seed, uint64_t idx)
{
    return (uint32_t)(mix64(seed + 0x9E3779B97F4A7C15ULL * (idx + 1)) >> 32);
}

static double inv_norm(double p)
{
    static const double a[6] = {-3.969683028665376e+01, 2.209460984245205e+02,
                                -2.759285104469687e+02, 1.383577518672690e+02,
                                -3.066479806614716e+01, 2.506628277459239e+00};
    static const double b[5] = {-5.447609879822406e+01, 1.615858368580409e+02,
                                -1.556989798598866e+02, 6.680131188771972e+01,
                                -1.328068155288572e+01};
    static const double c[6] = {-7.784894002430293e-03, -3.223964580411365e-01,
                                -2.400758277161838e+00, -2.549732539343734e+00,
                                4.374664141464968e+00, 2.938163982698783e+00};
    static const double d[4] = {7.784695709041462e-03, 3.224671290700398e-01,
                                2.445134137142996e+00, 3.754408661907416e+00};
    const double plow = 0.02425, phigh = 1. - plow;
    if (p < plow) {
        double q = sqrt(-2. * log(p));
        return (((((c[0] * q + c[1]) * q + c[2]) * q + c[3]) * q + c[4]) * q + c[5]) /
               ((((d[0] * q + d[1]) * q + d[2]) * q + d[3]) * q + 1.);
    }
    if (p <= phigh) {
        double q = p - 0.5, r = q * q;
        return (((((a[0] * r + a[1]) * r + a[2]) * r + a[3]) * r + a[4]) * r + a[5]) * q /
               (((((b[0] * r + b[1]) * r + b[2]) * r + b[3]) * r + b[4]) * r + 1.);
    }
    double q = sqrt(-2. * log(1. - p));
    return -(((((c[0] * q + c[1]) * q + c[2]) * q + c[3]) * q + c[4]) * q + c[5]) /
           ((((d[0] * q + d[1]) * q + d[2]) * q + d[3]) * q + 1.);
}

static inline int quant(double mean, double sigma, uint32_t u, double A)
{
    double z = inv_norm(((double)u + 0.5) * (1. / 4294967296.));
    double v = floor(mean + sigma * z + A + 0.5);
    return v < 0. ? 0 : (v > 255. ? 255 : (int)v);
}

/* thr[v] = smallest u with quant(u) >= v (thr[0] = 0, 2^32 when v is never reached);
 * quant is monotone in u */
static void make_table(double mean, double sigma, uint64_t *thr)
{
    thr[0] = 0;
    for (int v = 1; v < 256; v++) {
        uint64_t lo = 0, hi = 0x100000000ULL;
        while (lo < hi) {
            uint64_t mid = (lo + hi) / 2;
            if (quant(mean, sigma, (uint32_t)mid, 0.) >= v) hi = mid;
            else lo = mid + 1;
        }
        thr[v] = lo;
    }
}

static inline int table_quant(const uint64_t *thr, uint32_t u)
{
    int lo = 0, hi = 255; /* largest v with thr[v] <= u */
    while (lo < hi) {
        int mid = (lo + hi + 1) / 2;
        if (thr[mid] <= (uint64_t)u) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

static double dmdelay(double dm, double fh, double fl)
{
    return 4.148741601e3 * dm * (1. / (fl * fl) - 1. / (fh * fh));
}

int txs_generate(const txs_cfg *cfg, int64_t tbeg, int64_t n, uint8_t *out, int nthreads)
{
    int C = cfg->nchan;
    if (C <= 0 || n < 0 || cfg->tsamp <= 0.) return -1;
    uint64_t thr[256];
    make_table(cfg->mean, cfg->sigma, thr);
    double fmax = cfg->freqs[0];
    for (int c = 0; c < C; c++) fmax = cfg->freqs[c] > fmax ? cfg->freqs[c] : fmax;

    /* per pulse: first sample at fmax, width in samples, amplitude, per-channel delays */
    int np = cfg->npulse;
    int64_t *pstart = (int64_t *)malloc(sizeof(int64_t) * (np > 0 ? np : 1));
    int64_t *pw = (int64_t *)malloc(sizeof(int64_t) * (np > 0 ? np : 1));
    double *pamp = (double *)malloc(sizeof(double) * (np > 0 ? np : 1));
    int64_t *pdelay = (int64_t *)malloc(sizeof(int64_t) * (size_t)(np > 0 ? np : 1) * C);
    for (int p = 0; p < np; p++) {
        const txs_pulse *P = &cfg->pulses[p];
        int64_t w = (int64_t)llround(P->width / cfg->tsamp);
        if (w < 1) w = 1;
        pw[p] = w;
        pstart[p] = (int64_t)llround(P->t0 / cfg->tsamp) - w / 2;
        pamp[p] = P->snr * cfg->sigma / sqrt((double)C * (double)w);
        for (int c = 0; c < C; c++)
            pdelay[(size_t)p * C + c] = (int64_t)llround(dmdelay(P->dm, fmax, cfg->freqs[c]) / cfg->tsamp);
    }
    const int64_t TT = 256;
    int64_t ntile = (n + TT - 1) / TT;
#ifdef _OPENMP
    int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#else
    int nt = 1;
    (void)nthreads;
#endif
#pragma omp parallel num_threads(nt)
    {
        float *A = (float *)malloc(sizeof(float) * TT * C);
        unsigned char *any = (unsigned char *)malloc(TT);
#pragma omp for schedule(dynamic, 4)
        for (int64_t tile = 0; tile < ntile; tile++) {
            int64_t a = tbeg + tile * TT, b = a + TT;
            if (b > tbeg + n) b = tbeg + n;
            int64_t m = b - a;
            memset(A, 0, sizeof(float) * TT * C);
            memset(any, 0, TT);
            for (int p = 0; p < np; p++)
                for (int c = 0; c < C; c++) {
                    int64_t s = pstart[p] + pdelay[(size_t)p * C + c], e = s + pw[p];
                    if (e <= a || s >= b) continue;
                    for (int64_t t = (s > a ? s : a); t < (e < b ? e : b); t++) {
                        A[(t - a) * C + c] += (float)pamp[p];
                        any[t - a] = 1;
                    }
                }
            for (int q = 0; q < cfg->nsine; q++) {
                const txs_sine *S = &cfg->sines[q];
                if (S->chan < 0 || S->chan >= C) continue;
                for (int64_t t = a; t < b; t++) {
                    double ph = 2. * M_PI * ((double)t * cfg->tsamp) / S->period + S->phase;
                    A[(t - a) * C + S->chan] += (float)(S->amp * cfg->sigma * sin(ph));
                    any[t - a] = 1;
                }
            }
            for (int q = 0; q < cfg->nimp; q++) {
                const txs_impulse *I = &cfg->imps[q];
                int64_t s = (int64_t)llround(I->t0 / cfg->tsamp), e = s + I->nsamp;
                if (e <= a || s >= b) continue;
                for (int64_t t = (s > a ? s : a); t < (e < b ? e : b); t++) {
                    for (int c = 0; c < C; c++) A[(t - a) * C + c] += (float)(I->amp * cfg->sigma);
                    any[t - a] = 1;
                }
            }
            for (int64_t r = 0; r < m; r++) {
                int64_t t = a + r;
                uint8_t *o = out + (size_t)(t - tbeg) * C;
                const float *Ar = A + r * C;
                for (int c = 0; c < C; c++) {
                    uint32_t u = draw(cfg->seed, (uint64_t)t * (uint64_t)C + (uint64_t)c);
                    if (any[r] && Ar[c] != 0.f)
                        o[c] = (uint8_t)quant(cfg->mean, cfg->sigma, u, (double)Ar[c]);
                    else
                        o[c] = (uint8_t)table_quant(thr, u);
                }
            }
        }
        free(A);
        free(any);
    }
    free(pstart);
    free(pw);
    free(pamp);
    free(pdelay);
    return 0;
}
