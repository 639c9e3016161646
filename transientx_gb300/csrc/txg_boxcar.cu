/*
 * txg_boxcar.cu -- boxcar matched filter over dedispersed series, the Boxcar::match /
 * Boxcar::run step (src/singlepulse/boxcar.cpp:158-296), fused with the S/N threshold and
 * candidate compaction that feed Cluster::run (cluster.cpp:89-112).
 *
 * One CTA per DM row.  The row is staged in shared memory, its mean/variance reduced
 * (FP32 runs combined in FP64), then the running sum of (x - mean) is formed in place by a
 * block scan (per-thread FP32 chunks, FP64 chunk offsets added as a float pair) and every
 * sample i keeps the
 * largest S = (c[i+wh] - c[i-wl]) * sqrt(1/(wn*var)) over the width ladder, later widths
 * winning ties (S >= best, best starting at 0) as in boxcar.cpp:253-262.  Rows with
 * var <= 0 yield zeros (boxcar.cpp:242).  The IQR statistics (boxcar.cpp:215-227) come from
 * an exact radix selection of the three order statistics.  Points with S > thre are appended
 * to the candidate list with a warp-aggregated atomic; dense mxS/mxwn are optional.
 */
#include <algorithm>
#include <cfloat>
#include <cstdlib>

#include "txg_internal.h"

namespace txg {

namespace {

constexpr int BX_THREADS = 512;
constexpr int BX_U = 4;  /* samples per thread per pass, tracked search: width parameters
                          * loaded once for all */
constexpr int BX_UF = 8; /* the same for the maximum-only search */
constexpr unsigned FULL = 0xffffffffu;
constexpr size_t BX_SMEM_MAX = 200 * 1024; /* + ~10 KB static stays under 227 KB */
constexpr int BX_RUN = 32; /* row statistics: FP32 runs per thread before each FP64 addition */

__device__ __forceinline__ double block_sum_d(double v, double *red)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) v = __dadd_rn(v, __shfl_xor_sync(FULL, v, off));
    __syncthreads();
    if (lane == 0) red[w] = v;
    __syncthreads();
    double t = 0.;
    if (threadIdx.x < 32) {
        t = threadIdx.x < (BX_THREADS / 32) ? red[threadIdx.x] : 0.;
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) t = __dadd_rn(t, __shfl_xor_sync(FULL, t, off));
        if (threadIdx.x == 0) red[0] = t;
    }
    __syncthreads();
    return red[0];
}

/* float -> unsigned key with the same ordering */
__device__ __forceinline__ unsigned fkey(float f)
{
    unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float fkey_inv(unsigned k)
{
    unsigned u = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
    return __uint_as_float(u);
}

/* Exact k-th smallest (0-based) of row[0..n) by 4 rounds of 8-bit radix selection. */
__device__ float select_kth(const float *row, long n, long k, unsigned *hist)
{
    unsigned prefix = 0, mask = 0;
    long kk = k;
    for (int shift = 24; shift >= 0; shift -= 8) {
        for (int b = threadIdx.x; b < 256; b += BX_THREADS) hist[b] = 0;
        __syncthreads();
        for (long i = threadIdx.x; i < n; i += BX_THREADS) {
            unsigned key = fkey(row[i]);
            if ((key & mask) == prefix) atomicAdd(&hist[(key >> shift) & 255u], 1u);
        }
        __syncthreads();
        __shared__ unsigned sel_bin;
        __shared__ long sel_rem;
        if (threadIdx.x == 0) {
            long acc = 0;
            unsigned b = 0;
            for (; b < 256; b++) {
                if (acc + (long)hist[b] > kk) break;
                acc += hist[b];
            }
            sel_bin = b;
            sel_rem = kk - acc;
        }
        __syncthreads();
        prefix |= sel_bin << shift;
        mask |= 255u << shift;
        kk = sel_rem;
        __syncthreads();
    }
    return fkey_inv(prefix);
}

/* Best S over the width ladder for U samples i = i0 + u*BX_THREADS, with its width (later
 * widths win ties).  CHECK selects the per-width range test (needed near the row ends); AVX2
 * reproduces the unordered-compare blend of the -mavx2 build. */
template <bool CHECK, bool AVX2, int U>
__device__ __forceinline__ void widths_pass(const float *__restrict__ c, int coff, int i0, int iend,
                                            int nw, const int4 *__restrict__ wpar,
                                            const float *__restrict__ temp_w, float *best, int *bw)
{
    /* c[j - coff] holds the running sum at sample j; samples at or past iend are skipped */
    for (int w = 0; w < nw; w++) {
        const int4 p = wpar[w];
        const float tw = temp_w[w];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int i = i0 + u * BX_THREADS;
            if (!CHECK || (i >= p.x && i < p.z && i < iend)) {
                const float S = __fmul_rn(__fsub_rn(c[i - coff + p.y], c[i - coff - p.x]), tw);
                if (S >= best[u]) {
                    best[u] = S;
                    bw[u] = p.w;
                } else if (AVX2 && !(S < best[u])) {
                    best[u] = 0.f;
                    bw[u] = 0;
                }
            }
        }
    }
}

/* The same search keeping only the best S (S is never NaN: var > 0 and the sums are finite,
 * so the maximum is that of the tracked search). */
template <bool CHECK, int U>
__device__ __forceinline__ void widths_max(const float *__restrict__ c, int coff, int i0, int iend,
                                           int nw, const int4 *__restrict__ wpar,
                                           const float *__restrict__ temp_w, float *best)
{
    for (int w = 0; w < nw; w++) {
        const int4 p = wpar[w];
        const float tw = temp_w[w];
        const int hz = min(p.z, iend);
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int i = i0 + u * BX_THREADS;
            if (!CHECK || (i >= p.x && i < hz)) {
                const float S = __fmul_rn(__fsub_rn(c[i - coff + p.y], c[i - coff - p.x]), tw);
                best[u] = fmaxf(best[u], S);
            }
        }
    }
}

/* Width search over samples [s_lo, iend) of row k, the running sum at c[j - coff]; every
 * width is in range for samples in [lo_all, hi_all).  Points with S > thre are appended to
 * the candidate list (warp-aggregated atomic), dense mxS/mxwn written when given.  TRACK keeps
 * the best width at every step (the dense output and the AVX2 blend need it); otherwise the
 * pass keeps only the maximum S and the width of each point above the threshold is found
 * afterwards with the same arithmetic. */
template <bool AVX2, bool TRACK>
__device__ __forceinline__ void search_row(const float *__restrict__ c, int coff, int s_lo, int iend,
                                           int lo_all, int hi_all, int nw, const int4 *__restrict__ wpar,
                                           const float *__restrict__ temp_w, bool active, float thre,
                                           long k, long n, txg_cand *__restrict__ cand,
                                           int *__restrict__ ncand, long cap, float *__restrict__ mxS,
                                           int32_t *__restrict__ mxwn)
{
    constexpr int U = TRACK ? BX_U : BX_UF;
    const int tid = threadIdx.x, lane = tid & 31;
    for (int base = s_lo; base < iend; base += BX_THREADS * U) {
        float best[U];
        int bw[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            best[u] = 0.f;
            bw[u] = 0;
        }
        if (active) {
            const int i0 = base + tid;
            const bool inner = base >= lo_all && base + BX_THREADS * U <= hi_all && base + BX_THREADS * U <= iend;
            if (TRACK) {
                if (inner)
                    widths_pass<false, AVX2, U>(c, coff, i0, iend, nw, wpar, temp_w, best, bw);
                else
                    widths_pass<true, AVX2, U>(c, coff, i0, iend, nw, wpar, temp_w, best, bw);
            } else {
                if (inner)
                    widths_max<false, U>(c, coff, i0, iend, nw, wpar, temp_w, best);
                else
                    widths_max<true, U>(c, coff, i0, iend, nw, wpar, temp_w, best);
            }
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int i = base + tid + u * BX_THREADS;
            if (TRACK && i < iend && mxS) {
                mxS[k * n + i] = best[u];
                mxwn[k * n + i] = bw[u];
            }
            const bool hit = i < iend && best[u] > thre;
            if (!TRACK) {
                /* the tracked search keeps the last width whose S reaches the final best (>= with
                 * best starting at 0): the largest w with S_w == best, or width 0 when none
                 * equals it (best stayed 0).  The warp finds it for each hit in turn, one width
                 * per lane, with the same arithmetic as the search. */
                unsigned hm = __ballot_sync(FULL, hit);
                while (hm) {
                    const int src = __ffs(hm) - 1;
                    hm &= hm - 1;
                    const int is = __shfl_sync(FULL, i, src);
                    const float bs = __shfl_sync(FULL, best[u], src);
                    int wf = -1;
                    for (int w0 = 0; w0 < nw; w0 += 32) {
                        const int w = w0 + lane;
                        bool eq = false;
                        if (w < nw) {
                            const int4 p = wpar[w];
                            if (is >= p.x && is < min(p.z, iend))
                                eq = __fmul_rn(__fsub_rn(c[is - coff + p.y], c[is - coff - p.x]), temp_w[w]) == bs;
                        }
                        const unsigned e = __ballot_sync(FULL, eq);
                        if (e) wf = w0 + 31 - __clz(e);
                    }
                    if (lane == src) bw[u] = wf >= 0 ? wpar[wf].w : 0;
                }
            }
            const unsigned m = __ballot_sync(FULL, hit);
            if (m) {
                int basei = 0;
                if (lane == __ffs(m) - 1) basei = atomicAdd(ncand, __popc(m));
                basei = __shfl_sync(FULL, basei, __ffs(m) - 1);
                if (hit) {
                    const long slot = basei + __popc(m & ((1u << lane) - 1u));
                    if (slot < cap) cand[slot] = txg_cand{(int32_t)k, (int32_t)i, bw[u], best[u]};
                }
            }
        }
    }
}

template <bool AVX2, bool TRACK>
__global__ void __launch_bounds__(BX_THREADS, 4)
k_boxcar(const float *__restrict__ tim, long ldt, long n, const int32_t *__restrict__ vwn,
         int nw, int iqr, float thre, txg_cand *__restrict__ cand,
         int *__restrict__ ncand, long cap, float *__restrict__ mxS, int32_t *__restrict__ mxwn)
{
    const int avx2_tail = AVX2 ? 1 : 0;
    extern __shared__ __align__(16) float c[];
    __shared__ double red[BX_THREADS / 32];
    __shared__ double chunk_off[BX_THREADS];
    __shared__ float temp_w[256];
    __shared__ int4 wpar[256]; /* wl, wh, end of the visited range, wn */
    __shared__ int lo_all, hi_all; /* samples where every width is in range */
    __shared__ unsigned hist[256];
    __shared__ float mean_sh, var_sh;
    const long k = blockIdx.x;
    const int tid = threadIdx.x;
    const float *row = tim + k * ldt;

    for (long i = tid; i < n; i += BX_THREADS) c[i] = row[i];
    __syncthreads();

    if (!iqr) {
        double s1 = 0., s2 = 0.;
        long i = tid;
        while (i < n) {
            float r1 = 0.f, r2 = 0.f;
            for (int r = 0; r < BX_RUN && i < n; r++, i += BX_THREADS) {
                float v = c[i];
                r1 = __fadd_rn(r1, v);
                r2 = __fadd_rn(r2, __fmul_rn(v, v));
            }
            s1 = __dadd_rn(s1, (double)r1);
            s2 = __dadd_rn(s2, (double)r2);
        }
        s1 = block_sum_d(s1, red);
        s2 = block_sum_d(s2, red);
        if (tid == 0) {
            double m = __ddiv_rn(s1, (double)n);
            double v = __dsub_rn(__ddiv_rn(s2, (double)n), __dmul_rn(m, m));
            mean_sh = __double2float_rn(m);
            var_sh = __double2float_rn(v);
        }
    } else {
        float q1 = select_kth(c, n, n / 4, hist);
        float q2 = select_kth(c, n, n / 2, hist);
        float q3 = select_kth(c, n, n - 1 - n / 4, hist);
        if (tid == 0) {
            double d = __ddiv_rn((double)__fsub_rn(q3, q1), 1.349);
            mean_sh = q2;
            var_sh = __double2float_rn(__dmul_rn(d, d));
        }
    }
    __syncthreads();
    const float mean = mean_sh, var = var_sh;

    /* running sum of (x - mean): thread t owns the contiguous chunk [t*L, (t+1)*L) */
    const long L = (n + BX_THREADS - 1) / BX_THREADS;
    const long a = (long)tid * L, b = a + L < n ? a + L : n;
    float loc = 0.f;
    for (long i = a; i < b; i++) loc = __fadd_rn(loc, __fsub_rn(c[i], mean));
    chunk_off[tid] = (double)loc;
    __syncthreads();
    if (tid < 32) { /* exclusive scan of the chunk totals in FP64 by one warp */
        const int per = BX_THREADS / 32;
        double run = 0.;
        for (int q = 0; q < per; q++) run = __dadd_rn(run, chunk_off[tid * per + q]);
        double incl = run;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            double y = __shfl_up_sync(FULL, incl, off);
            if (tid >= off) incl = __dadd_rn(incl, y);
        }
        /* exclusive prefix = the left neighbour's inclusive sum */
        const double left = __shfl_up_sync(FULL, incl, 1);
        double ex = tid == 0 ? 0. : left;
        for (int q = 0; q < per; q++) {
            const double v = chunk_off[tid * per + q];
            chunk_off[tid * per + q] = ex;
            ex = __dadd_rn(ex, v);
        }
    }
    __syncthreads();
    {
        /* the chunk's FP64 offset as a float pair: c[i] = (hi + run) + lo, two FP32 adds per
         * sample (the FP64 pipe is a small fraction of the FP32 one on this part) */
        const double off = chunk_off[tid];
        const float oh = __double2float_rn(off), ol = __double2float_rn(__dsub_rn(off, (double)oh));
        float run = 0.f;
        for (long i = a; i < b; i++) {
            run = __fadd_rn(run, __fsub_rn(c[i], mean));
            c[i] = __fadd_rn(__fadd_rn(oh, run), ol);
        }
    }
    for (int w = tid; w < nw; w += BX_THREADS) {
        const int wn = vwn[w];
        const int wl = wn / 2 + 1, wh = (wn - 1) / 2;
        temp_w[w] = __double2float_rn(__dsqrt_rn(__ddiv_rn(1., (double)__fmul_rn((float)wn, var))));
        long hi = n - wh;
        if (avx2_tail) {
            long len = n - wh - wl;
            long nv = len >= 0 ? len / 8 : 0; /* C division truncates toward zero */
            hi = nv > 0 ? wl + 8 * nv : wl;
        }
        wpar[w] = make_int4(wl, wh, (int)hi, wn);
    }
    __syncthreads();

    if (tid == 0) {
        int lo = 0, hi = (int)n;
        for (int w = 0; w < nw; w++) {
            lo = max(lo, wpar[w].x);
            hi = min(hi, wpar[w].z);
        }
        lo_all = lo;
        hi_all = hi;
    }
    __syncthreads();

    search_row<AVX2, TRACK>(c, 0, 0, (int)n, lo_all, hi_all, nw, wpar, temp_w, var > 0.f, thre, k, n,
                            cand, ncand, cap, mxS, mxwn);
}

/* ---- rows longer than one CTA's shared memory ------------------------------------------ */
/* The single-CTA kernel's arithmetic depends only on n: statistics by the fixed run pattern,
 * and the running sum over BX_THREADS chunks of L = ceil(n/BX_THREADS) samples (FP32 inside a
 * chunk, FP64 chunk offsets added as a float pair).  k_boxcar_prep computes, per row, the same
 * statistics and chunk offsets from global memory; k_boxcar_seg rebuilds the running sum of a
 * segment of chunks plus a halo of the widest boxcar and runs the same width passes: results
 * are identical to k_boxcar's.  scratch row k: [0, BX_THREADS) chunk offsets, [BX_THREADS] mean and var. */
constexpr int SEG_CHUNKS = 32; /* chunks per segment CTA */

__global__ void __launch_bounds__(BX_THREADS)
k_boxcar_prep(const float *__restrict__ tim, long ldt, long n, int iqr, double *__restrict__ scratch)
{
    __shared__ double red[BX_THREADS / 32];
    __shared__ double chunk_off[BX_THREADS];
    __shared__ unsigned hist[256];
    __shared__ float mean_sh, var_sh;
    const long k = blockIdx.x;
    const int tid = threadIdx.x;
    const float *row = tim + k * ldt;
    if (!iqr) {
        double s1 = 0., s2 = 0.;
        long i = tid;
        while (i < n) {
            float r1 = 0.f, r2 = 0.f;
            for (int r = 0; r < BX_RUN && i < n; r++, i += BX_THREADS) {
                float v = row[i];
                r1 = __fadd_rn(r1, v);
                r2 = __fadd_rn(r2, __fmul_rn(v, v));
            }
            s1 = __dadd_rn(s1, (double)r1);
            s2 = __dadd_rn(s2, (double)r2);
        }
        s1 = block_sum_d(s1, red);
        s2 = block_sum_d(s2, red);
        if (tid == 0) {
            double m = __ddiv_rn(s1, (double)n);
            double v = __dsub_rn(__ddiv_rn(s2, (double)n), __dmul_rn(m, m));
            mean_sh = __double2float_rn(m);
            var_sh = __double2float_rn(v);
        }
    } else {
        float q1 = select_kth(row, n, n / 4, hist);
        float q2 = select_kth(row, n, n / 2, hist);
        float q3 = select_kth(row, n, n - 1 - n / 4, hist);
        if (tid == 0) {
            double d = __ddiv_rn((double)__fsub_rn(q3, q1), 1.349);
            mean_sh = q2;
            var_sh = __double2float_rn(__dmul_rn(d, d));
        }
    }
    __syncthreads();
    const float mean = mean_sh;
    const long L = (n + BX_THREADS - 1) / BX_THREADS;
    const long a = (long)tid * L, b = a + L < n ? a + L : n;
    float loc = 0.f;
    for (long i = a; i < b; i++) loc = __fadd_rn(loc, __fsub_rn(row[i], mean));
    chunk_off[tid] = (double)loc;
    __syncthreads();
    if (tid < 32) {
        const int per = BX_THREADS / 32;
        double run = 0.;
        for (int q = 0; q < per; q++) run = __dadd_rn(run, chunk_off[tid * per + q]);
        double incl = run;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            double y = __shfl_up_sync(FULL, incl, off);
            if (tid >= off) incl = __dadd_rn(incl, y);
        }
        const double left = __shfl_up_sync(FULL, incl, 1);
        double ex = tid == 0 ? 0. : left;
        for (int q = 0; q < per; q++) {
            const double v = chunk_off[tid * per + q];
            chunk_off[tid * per + q] = ex;
            ex = __dadd_rn(ex, v);
        }
    }
    __syncthreads();
    double *out = scratch + k * (BX_THREADS + 1);
    out[tid] = chunk_off[tid];
    if (tid == 0) {
        float *mv = reinterpret_cast<float *>(out + BX_THREADS);
        mv[0] = mean_sh;
        mv[1] = var_sh;
    }
}

template <bool AVX2, bool TRACK>
__global__ void __launch_bounds__(BX_THREADS)
k_boxcar_seg(const float *__restrict__ tim, long ldt, long n, const int32_t *__restrict__ vwn,
             int nw, float thre, const double *__restrict__ scratch, txg_cand *__restrict__ cand,
             int *__restrict__ ncand, long cap, float *__restrict__ mxS, int32_t *__restrict__ mxwn)
{
    const int avx2_tail = AVX2 ? 1 : 0;
    extern __shared__ __align__(16) float c[];
    __shared__ float temp_w[256];
    __shared__ int4 wpar[256];
    __shared__ int lo_all, hi_all, wlmax_sh, whmax_sh;
    const long k = blockIdx.x;
    const int tid = threadIdx.x;
    const float *row = tim + k * ldt;
    const double *sc = scratch + k * (BX_THREADS + 1);
    const float mean = reinterpret_cast<const float *>(sc + BX_THREADS)[0];
    const float var = reinterpret_cast<const float *>(sc + BX_THREADS)[1];
    const long L = (n + BX_THREADS - 1) / BX_THREADS;
    const long s_lo = (long)blockIdx.y * SEG_CHUNKS * L;
    if (s_lo >= n) return;
    const long s_hi = min(n, s_lo + (long)SEG_CHUNKS * L);

    for (int w = tid; w < nw; w += BX_THREADS) {
        const int wn = vwn[w];
        const int wl = wn / 2 + 1, wh = (wn - 1) / 2;
        temp_w[w] = __double2float_rn(__dsqrt_rn(__ddiv_rn(1., (double)__fmul_rn((float)wn, var))));
        long hi = n - wh;
        if (avx2_tail) {
            long len = n - wh - wl;
            long nv = len >= 0 ? len / 8 : 0;
            hi = nv > 0 ? wl + 8 * nv : wl;
        }
        wpar[w] = make_int4(wl, wh, (int)hi, wn);
    }
    __syncthreads();
    if (tid == 0) {
        int lo = 0, hi = (int)n, wl = 0, wh = 0;
        for (int w = 0; w < nw; w++) {
            lo = max(lo, wpar[w].x);
            hi = min(hi, wpar[w].z);
            wl = max(wl, wpar[w].x);
            wh = max(wh, wpar[w].y);
        }
        lo_all = lo;
        hi_all = hi;
        wlmax_sh = wl;
        whmax_sh = wh;
    }
    __syncthreads();
    /* running sum over the segment and its halo, rebuilt chunk by chunk from the offsets */
    const long h_lo = max(0L, s_lo - wlmax_sh), h_hi = min(n, s_hi + whmax_sh);
    for (long ch = h_lo / L + tid; ch <= (h_hi - 1) / L; ch += BX_THREADS) {
        const long a = ch * L, b = min(a + L, n);
        const double off = sc[ch];
        const float oh = __double2float_rn(off), ol = __double2float_rn(__dsub_rn(off, (double)oh));
        float run = 0.f;
        for (long i = a; i < b; i++) {
            run = __fadd_rn(run, __fsub_rn(row[i], mean));
            if (i >= h_lo && i < h_hi) c[i - h_lo] = __fadd_rn(__fadd_rn(oh, run), ol);
        }
    }
    __syncthreads();

    search_row<AVX2, TRACK>(c, (int)h_lo, (int)s_lo, (int)s_hi, lo_all, hi_all, nw, wpar, temp_w,
                            var > 0.f, thre, k, n, cand, ncand, cap, mxS, mxwn);
}

} // namespace

size_t boxcar_max_samples() { return (BX_SMEM_MAX) / sizeof(float); }

size_t boxcar_scratch_doubles(long ndm) { return (size_t)ndm * (BX_THREADS + 1); }

bool boxcar_supported(long n, int maxwn, int nw)
{
    if (n <= 0 || n >= (1L << 31) || nw > 256) return false;
    if ((size_t)n <= boxcar_max_samples()) return true;
    const long L = (n + BX_THREADS - 1) / BX_THREADS;
    const long seg = (long)SEG_CHUNKS * L;
    return (size_t)(seg + maxwn + 2) * sizeof(float) <= BX_SMEM_MAX && (n + seg - 1) / seg <= 65535;
}

static bool force_segmented()
{
    const char *e = getenv("TXG_BOXCAR_SEGMENTED");
    return e && e[0] == '1';
}

int launch_boxcar(const float *tim, long ldt, long ndm, long n, const int32_t *vwn, int nw,
                  int maxwn, int iqr, int avx2_tail, float thre, txg_cand *cand, int *ncand,
                  long cap, float *mxS, int32_t *mxwn, double *scratch, int *err, cudaStream_t st)
{
    (void)err;
    if (n <= 0 || ndm <= 0) return TXG_OK;
    if (nw > 256 || n >= (1L << 31)) return TXG_ERR_UNSUPPORTED;
    if ((size_t)n <= boxcar_max_samples() && !(force_segmented() && scratch)) {
        size_t smem = (size_t)n * sizeof(float);
#define TXG_BX(A, T)                                                                                  \
    do {                                                                                              \
        cudaFuncSetAttribute(k_boxcar<A, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)BX_SMEM_MAX); \
        k_boxcar<A, T><<<(unsigned)ndm, BX_THREADS, smem, st>>>(tim, ldt, n, vwn, nw, iqr, thre, cand, ncand, \
                                                                 cap, mxS, mxwn);                      \
    } while (0)
        if (avx2_tail)
            TXG_BX(true, true);
        else if (mxS)
            TXG_BX(false, true);
        else
            TXG_BX(false, false);
#undef TXG_BX
        return TXG_OK;
    }
    /* long rows: statistics and chunk offsets per row, then segments of SEG_CHUNKS chunks */
    if (!scratch) return TXG_ERR_UNSUPPORTED;
    const long L = (n + BX_THREADS - 1) / BX_THREADS;
    const long seg = (long)SEG_CHUNKS * L;
    const long nseg = (n + seg - 1) / seg;
    const size_t smem = (size_t)(seg + maxwn + 2) * sizeof(float);
    if (smem > BX_SMEM_MAX || nseg > 65535) return TXG_ERR_UNSUPPORTED;
    k_boxcar_prep<<<(unsigned)ndm, BX_THREADS, 0, st>>>(tim, ldt, n, iqr, scratch);
    dim3 grid((unsigned)ndm, (unsigned)nseg);
#define TXG_BXS(A, T)                                                                                 \
    do {                                                                                              \
        cudaFuncSetAttribute(k_boxcar_seg<A, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
        k_boxcar_seg<A, T><<<grid, BX_THREADS, smem, st>>>(tim, ldt, n, vwn, nw, thre, scratch, cand, ncand, \
                                                            cap, mxS, mxwn);                           \
    } while (0)
    if (avx2_tail)
        TXG_BXS(true, true);
    else if (mxS)
        TXG_BXS(false, true);
    else
        TXG_BXS(false, false);
#undef TXG_BXS
    return TXG_OK;
}

} // namespace txg
