/*
 * txg_pre.cu -- per-block preprocessing kernels of one ddplan row, all on channel-major
 * float blocks x[j*ldx + i]:
 *   unpack + td/fd sum-downsample ............ candidate.cpp:381-427 semantics
 *   equalize (per-channel zero mean, unit var) docs/pipeline/preprocess.rst:15-18
 *   baseline (smoothed zero-DM subtraction) .. docs/pipeline/preprocess.rst:26-29
 *   zap of listed channels ................... singlepulse.cpp:295
 *   kadaneF ................................. candidate.cpp:710-829, singlepulse.cpp:305-308
 *   zdot .................................... candidate.cpp:831-897
 * Every float operation uses an explicit round-to-nearest intrinsic so that no multiply-add
 * is fused: results are bit-identical to a scalar C evaluation of the same expressions in
 * the same order.  Row reductions that need FP64 follow one fixed pattern (lane-strided FP32
 * runs of 32, FP64 lane accumulators, xor butterfly), identical in every implementation.
 */
#include <cstdio>

#include <algorithm>

#include "txg_internal.h"

namespace txg {

namespace {

constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ double warp_sum_d(double v)
{
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) v = __dadd_rn(v, __shfl_xor_sync(FULL, v, off));
    return v;
}

__device__ __forceinline__ long long warp_sum_ll(long long v)
{
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) v += __shfl_xor_sync(FULL, v, off);
    return v;
}

/* r[i] = f(r[i], i) over a row by one warp, 16-byte accesses when the row is aligned, four
 * of them in flight per lane (each element is independent, so the access width does not
 * change any result). */
template <typename F>
__device__ __forceinline__ void row_map(float *__restrict__ r, long n, int lane, F f)
{
    long i0 = 0;
    if ((reinterpret_cast<uintptr_t>(r) & 15) == 0) {
        const long n4 = n / 4;
        float4 *r4 = reinterpret_cast<float4 *>(r);
        long q = lane;
        for (; q + 3 * 32 < n4; q += 4 * 32) {
            float4 v[4];
#pragma unroll
            for (int u = 0; u < 4; u++) v[u] = r4[q + 32 * u];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const long b = 4 * (q + 32 * u);
                v[u].x = f(v[u].x, b);
                v[u].y = f(v[u].y, b + 1);
                v[u].z = f(v[u].z, b + 2);
                v[u].w = f(v[u].w, b + 3);
                r4[q + 32 * u] = v[u];
            }
        }
        for (; q < n4; q += 32) {
            float4 v = r4[q];
            v.x = f(v.x, 4 * q);
            v.y = f(v.y, 4 * q + 1);
            v.z = f(v.z, 4 * q + 2);
            v.w = f(v.w, 4 * q + 3);
            r4[q] = v;
        }
        i0 = 4 * n4;
    }
    for (long i = i0 + lane; i < n; i += 32) r[i] = f(r[i], i);
}

struct Ident {
    __device__ __forceinline__ float operator()(float v) const { return v; }
};

/* v -> (v - m) * inv, the per-channel standardisation of equalize and zdot */
struct Standardise {
    float m, inv;
    __device__ __forceinline__ float operator()(float v) const { return __fmul_rn(__fsub_rn(v, m), inv); }
};

/* Two fixed-pattern reductions of one row by one warp: lane l takes i = l, l+32, l+64, ... in
 * runs of RED_RUN summed in FP32, adds each run total to its FP64 accumulator, and the lanes
 * combine by an xor butterfly.  MODE 1 -> (sum x, sum x*x), MODE 2 -> (sum x, sum x*y),
 * x = f(stored value).  Long runs keep the FP64 work (a small share of this part's arithmetic
 * rate) to two additions per 32 elements of a lane. */
constexpr int RED_RUN = 32;

template <int MODE, typename F = Ident>
__device__ __forceinline__ void red32x2(const float *__restrict__ x, const float *__restrict__ y,
                                        long n, int lane, double &o1, double &o2, F f = F())
{
    double a1 = 0., a2 = 0.;
    long i = lane;
    for (; i + (RED_RUN - 1) * 32 < n; i += RED_RUN * 32) { /* full runs, eight loads at a time */
        float r1 = 0.f, r2 = 0.f;
#pragma unroll
        for (int h = 0; h < RED_RUN / 8; h++) {
            float v[8], q[8];
#pragma unroll
            for (int r = 0; r < 8; r++) {
                v[r] = f(x[i + 32 * (8 * h + r)]);
                q[r] = MODE == 1 ? v[r] : y[i + 32 * (8 * h + r)];
            }
#pragma unroll
            for (int r = 0; r < 8; r++) {
                r1 = __fadd_rn(r1, v[r]);
                r2 = __fadd_rn(r2, __fmul_rn(v[r], q[r]));
            }
        }
        a1 = __dadd_rn(a1, (double)r1);
        a2 = __dadd_rn(a2, (double)r2);
    }
    if (i < n) { /* the last, partial run */
        float r1 = 0.f, r2 = 0.f;
        for (; i < n; i += 32) {
            const float v = f(x[i]);
            r1 = __fadd_rn(r1, v);
            r2 = __fadd_rn(r2, MODE == 1 ? __fmul_rn(v, v) : __fmul_rn(v, y[i]));
        }
        a1 = __dadd_rn(a1, (double)r1);
        a2 = __dadd_rn(a2, (double)r2);
    }
    o1 = warp_sum_d(a1);
    o2 = warp_sum_d(a2);
}

/* ---- skewness/kurtosis channel zap ------------------------------------------------------ */
/* Exact integer sums of (v-128)^p, p = 1..4, per raw channel: threads over channels (4 per
 * thread with 32-bit loads when aligned), time split over blockIdx.y; 64-bit integer atomics
 * make the totals independent of the order. */
constexpr int SK_TCHUNK = 128;

__global__ void __launch_bounds__(256) k_sk_sums(const uint8_t *__restrict__ raw, int C_raw, long n0,
                                                int vec, unsigned long long *__restrict__ sums)
{
    const int per = vec ? 4 : 1;
    const long c0 = ((long)blockIdx.x * blockDim.x + threadIdx.x) * per;
    if (c0 >= C_raw) return;
    const long t0 = (long)blockIdx.y * SK_TCHUNK, t1 = min(t0 + SK_TCHUNK, n0);
    long long a[4][4] = {};
#pragma unroll 8
    for (long t = t0; t < t1; t++) {
        int v[4];
        if (vec) {
            const uchar4 q = *reinterpret_cast<const uchar4 *>(raw + t * C_raw + c0);
            v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
        } else {
            v[0] = raw[t * C_raw + c0];
        }
#pragma unroll
        for (int k = 0; k < 4; k++) {
            if (k < per) {
                const long long d = v[k] - 128, d2 = d * d;
                a[k][0] += d;
                a[k][1] += d2;
                a[k][2] += d2 * d;
                a[k][3] += d2 * d2;
            }
        }
    }
#pragma unroll
    for (int k = 0; k < 4; k++)
        if (k < per)
#pragma unroll
            for (int p = 0; p < 4; p++)
                atomicAdd(&sums[(size_t)p * C_raw + c0 + k], (unsigned long long)a[k][p]);
}

/* Per channel: moments -> skewness and excess kurtosis (double, each operation rounded as
 * written), one thread per channel. */
__global__ void k_sk_stats(const unsigned long long *__restrict__ sums, int C, long n0,
                           double *__restrict__ stats)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= C) return;
    const double n = (double)n0;
    const double a = __ddiv_rn((double)(long long)sums[c], n);
    const double b = __ddiv_rn((double)(long long)sums[(size_t)C + c], n);
    const double cc = __ddiv_rn((double)(long long)sums[(size_t)2 * C + c], n);
    const double d = __ddiv_rn((double)(long long)sums[(size_t)3 * C + c], n);
    const double aa = __dmul_rn(a, a);
    const double m2 = __dsub_rn(b, aa);
    const double m3 = __dadd_rn(__dsub_rn(cc, __dmul_rn(__dmul_rn(3., a), b)), __dmul_rn(__dmul_rn(2., aa), a));
    const double m4 = __dsub_rn(__dadd_rn(__dsub_rn(d, __dmul_rn(__dmul_rn(4., a), cc)),
                                         __dmul_rn(__dmul_rn(6., aa), b)),
                               __dmul_rn(__dmul_rn(3., aa), aa));
    double sk = 0., ku = 0.;
    if (m2 > 0.) {
        sk = __ddiv_rn(m3, __dmul_rn(m2, __dsqrt_rn(m2)));
        ku = __dsub_rn(__ddiv_rn(m4, __dmul_rn(m2, m2)), 3.);
    }
    stats[c] = sk;
    stats[(size_t)C + c] = ku;
}

/* Order-preserving 64-bit key of a double (negative values bit-inverted, positive values with
 * the sign bit set), and its inverse. */
__device__ __forceinline__ unsigned long long dkey(double v)
{
    const unsigned long long u = (unsigned long long)__double_as_longlong(v);
    return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}
__device__ __forceinline__ double dkey_inv(unsigned long long k)
{
    return __longlong_as_double((long long)((k >> 63) ? (k & 0x7fffffffffffffffull) : ~k));
}

/* One CTA: exact quartiles sorted[C/4] and sorted[C-1-C/4] of skewness and kurtosis by a
 * most-significant-digit radix selection on the order-preserving keys (eight 8-bit passes;
 * the four selections share each pass) -> mask of channels outside [Q1 - thr*R, Q3 + thr*R]
 * for either statistic.  Equal values are one value, so the selected quartiles are those of a
 * sort. */
__global__ void __launch_bounds__(1024) k_sk_select(int C, float thr, const double *__restrict__ stats,
                                                   uint8_t *__restrict__ mask)
{
    __shared__ unsigned int hist[4][256];
    __shared__ unsigned long long pref[4];
    __shared__ unsigned int rank[4];
    __shared__ double lo[2], hi[2];
    const int tid = threadIdx.x;
    if (tid < 4) {
        pref[tid] = 0ull;
        rank[tid] = (tid & 1) ? (unsigned)(C - 1 - C / 4) : (unsigned)(C / 4);
    }
    for (int shift = 56; shift >= 0; shift -= 8) {
        for (int e = tid; e < 4 * 256; e += blockDim.x) hist[e >> 8][e & 255] = 0u;
        __syncthreads();
        const unsigned long long hm = shift == 56 ? 0ull : (~0ull << (shift + 8));
        for (int c = tid; c < 2 * C; c += blockDim.x) {
            const int q = c >= C;
            const unsigned long long k = dkey(stats[c]);
            const unsigned d = (unsigned)(k >> shift) & 255u;
            if ((k & hm) == pref[2 * q]) atomicAdd(&hist[2 * q][d], 1u);
            if ((k & hm) == pref[2 * q + 1]) atomicAdd(&hist[2 * q + 1][d], 1u);
        }
        __syncthreads();
        if (tid < 4 * 32) { /* one warp per selection; each lane holds 8 consecutive digits */
            const int sel = tid >> 5, lane = tid & 31;
            unsigned cnt[8], tot = 0;
#pragma unroll
            for (int u = 0; u < 8; u++) {
                cnt[u] = hist[sel][8 * lane + u];
                tot += cnt[u];
            }
            unsigned incl = tot;
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const unsigned y = __shfl_up_sync(FULL, incl, off);
                if (lane >= off) incl += y;
            }
            const unsigned rk = rank[sel], excl = incl - tot;
            __syncwarp();
            if (rk >= excl && rk < incl) {
                unsigned acc = excl;
#pragma unroll
                for (int u = 0; u < 8; u++) {
                    if (rk < acc + cnt[u]) {
                        pref[sel] |= (unsigned long long)(8 * lane + u) << shift;
                        rank[sel] = rk - acc;
                        break;
                    }
                    acc += cnt[u];
                }
            }
        }
        __syncthreads();
    }
    if (tid < 2) {
        const double q1 = dkey_inv(pref[2 * tid]), q3 = dkey_inv(pref[2 * tid + 1]);
        const double R = __dsub_rn(q3, q1);
        lo[tid] = __dsub_rn(q1, __dmul_rn((double)thr, R));
        hi[tid] = __dadd_rn(q3, __dmul_rn((double)thr, R));
    }
    __syncthreads();
    for (int c = threadIdx.x; c < C; c += blockDim.x) {
        const double sk = stats[c], ku = stats[(size_t)C + c];
        mask[c] = (sk < lo[0] || sk > hi[0] || ku < lo[1] || ku > hi[1]) ? 1 : 0;
    }
}

/* ---- unpack + downsample ------------------------------------------------------------- */
constexpr int UP_TJ = 64; /* output channels per CTA */
constexpr int UP_TI = 32; /* output samples per CTA */

/* raw [n0][C_raw] uint8 -> x[j][i] = sum_{k<fd} sum_{t<td} raw[i*td+t][j*fd+k] (k outer). The
 * raw tile is staged in shared memory with 32-bit loads when the row pitch allows. */
__global__ void __launch_bounds__(256) k_unpack(const uint8_t *__restrict__ raw, int C_raw, long n0,
                                               int td, int fd, float *__restrict__ x, long ldx,
                                               int C, long N, const uint8_t *__restrict__ mask)
{
    extern __shared__ uint8_t tile[];
    __shared__ float outt[UP_TJ][UP_TI + 1];
    const int j0 = blockIdx.y * UP_TJ;
    const long i0 = (long)blockIdx.x * UP_TI;
    const int rows = UP_TI * td;           /* raw rows in the tile */
    const int cols = UP_TJ * fd;           /* raw columns in the tile */
    const long r0 = i0 * td;
    const int c0 = j0 * fd;
    const bool vec = (C_raw % 4 == 0) && (cols % 4 == 0) && ((reinterpret_cast<uintptr_t>(raw) & 3) == 0);
    if (vec) {
        const int cq = cols / 4;
        for (int e = threadIdx.x; e < rows * cq; e += blockDim.x) {
            int r = e / cq, q = e % cq;
            long rr = r0 + r;
            int cc = c0 + 4 * q;
            uchar4 v = make_uchar4(0, 0, 0, 0);
            if (rr < n0 && cc + 3 < C_raw)
                v = *reinterpret_cast<const uchar4 *>(raw + rr * C_raw + cc);
            else if (rr < n0) {
                if (cc < C_raw) v.x = raw[rr * C_raw + cc];
                if (cc + 1 < C_raw) v.y = raw[rr * C_raw + cc + 1];
                if (cc + 2 < C_raw) v.z = raw[rr * C_raw + cc + 2];
            }
            *reinterpret_cast<uchar4 *>(tile + r * cols + 4 * q) = v;
        }
    } else {
        for (int e = threadIdx.x; e < rows * cols; e += blockDim.x) {
            int r = e / cols, c = e % cols;
            long rr = r0 + r;
            int cc = c0 + c;
            tile[r * cols + c] = (rr < n0 && cc < C_raw) ? raw[rr * C_raw + cc] : 0;
        }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < UP_TJ * UP_TI; e += blockDim.x) {
        int jj = e / UP_TI, ii = e % UP_TI;
        float acc = 0.f;
        for (int k = 0; k < fd; k++) {
            const int c = c0 + jj * fd + k;
            const bool z = mask && c < C_raw && mask[c];
            for (int t = 0; t < td; t++)
                acc = __fadd_rn(acc, z ? 0.f : (float)tile[(ii * td + t) * cols + jj * fd + k]);
        }
        outt[jj][ii] = acc;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < UP_TJ * UP_TI; e += blockDim.x) {
        int jj = e / UP_TI, ii = e % UP_TI;
        int j = j0 + jj;
        long i = i0 + ii;
        if (j < C && i < N) x[(long)j * ldx + i] = outt[jj][ii];
    }
}

/* Unpack for fd | 16 and 16-byte rows: each thread sums, for one output sample, the td raw
 * rows of one 16-channel group (one 16-byte load per row; 16/fd output channels), and a
 * shared-memory transpose gives channel-major coalesced writes.  The sums are of integers
 * below 2^24, exact in FP32, so they equal k_unpack's in any order.
 * With `part`, the CTA also writes, per output channel, the exact integer sums of its 64
 * values and of their squares (part[(j*gridDim.x + tile)*2 + {0,1}]): equalize's statistics
 * without another pass over the block. */
constexpr int UV_BYTES = 128;  /* raw bytes (channels) per CTA row: 8 groups of 16 */
constexpr int UV_TI = 64;      /* output samples per CTA */

template <int FD>
__global__ void __launch_bounds__(256) k_unpack_vec(const uint8_t *__restrict__ raw, int C_raw,
                                                   long n0, int td, float *__restrict__ x, long ldx,
                                                   int C, long N, const uint8_t *__restrict__ mask,
                                                   unsigned long long *__restrict__ part)
{
    constexpr int TJ = UV_BYTES / FD; /* output channels per CTA */
    constexpr int PER = 16 / FD;      /* output channels per thread */
    __shared__ float outt[TJ][UV_TI + 1];
    const int q = threadIdx.x & 7, srow = threadIdx.x >> 3; /* 16-byte group, sample slot 0..31 */
    const int c0 = blockIdx.y * UV_BYTES + 16 * q;         /* first raw channel of the group */
    const long i0 = (long)blockIdx.x * UV_TI;
    uint4 mk = make_uint4(0u, 0u, 0u, 0u);
    const bool in_c = c0 < C_raw;
    if (mask && in_c) mk = *reinterpret_cast<const uint4 *>(mask + c0);
    const uint32_t mw[4] = {mk.x, mk.y, mk.z, mk.w};
#pragma unroll
    for (int pass = 0; pass < UV_TI / 32; pass++) {
        const int ii = pass * 32 + srow;
        const long i = i0 + ii;
        float acc[PER];
#pragma unroll
        for (int o = 0; o < PER; o++) acc[o] = 0.f;
        if (in_c && i < N) {
            const uint8_t *src = raw + (i * td) * (long)C_raw + c0;
            for (int t = 0; t < td; t++) {
                const uint4 v = *reinterpret_cast<const uint4 *>(src + (long)t * C_raw);
                const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                for (int b = 0; b < 16; b++) {
                    const uint32_t byte = (w[b >> 2] >> (8 * (b & 3))) & 255u;
                    const uint32_t m = (mw[b >> 2] >> (8 * (b & 3))) & 255u;
                    acc[b / FD] = __fadd_rn(acc[b / FD], m ? 0.f : (float)byte);
                }
            }
        }
#pragma unroll
        for (int o = 0; o < PER; o++) outt[q * PER + o][ii] = acc[o];
    }
    __syncthreads();
    const int j0 = blockIdx.y * TJ;
    for (int e = threadIdx.x; e < TJ * UV_TI; e += blockDim.x) {
        const int jj = e / UV_TI, ii = e % UV_TI;
        const int j = j0 + jj;
        const long i = i0 + ii;
        if (j < C && i < N) x[(long)j * ldx + i] = outt[jj][ii];
    }
    if (part) {
        /* samples past N hold 0 and add nothing; values are exact non-negative integers */
        constexpr int TPC = 256 / TJ, SPT = UV_TI / TPC; /* threads per channel, samples each */
        __shared__ unsigned long long ps[TPC > 1 ? TPC - 1 : 1][TJ][2];
        const int jj = threadIdx.x % TJ, pt = threadIdx.x / TJ;
        unsigned long long a1 = 0ull, a2 = 0ull;
#pragma unroll 8
        for (int k = 0; k < SPT; k++) {
            const unsigned v = __float2uint_rz(outt[jj][pt * SPT + k]);
            a1 += v;
            a2 += (unsigned long long)v * v;
        }
        if (pt > 0) {
            ps[pt - 1][jj][0] = a1;
            ps[pt - 1][jj][1] = a2;
        }
        __syncthreads();
        if (pt == 0 && j0 + jj < C) {
#pragma unroll
            for (int p = 0; p < TPC - 1; p++) {
                a1 += ps[p][jj][0];
                a2 += ps[p][jj][1];
            }
            unsigned long long *o = part + ((size_t)(j0 + jj) * gridDim.x + blockIdx.x) * 2;
            o[0] = a1;
            o[1] = a2;
        }
    }
}

/* fallback for large td*fd: one thread per output, no staging */
__global__ void k_unpack_direct(const uint8_t *__restrict__ raw, int C_raw, int td, int fd,
                                float *__restrict__ x, long ldx, int C, long N,
                                const uint8_t *__restrict__ mask)
{
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y;
    if (i >= N || j >= C) return;
    float acc = 0.f;
    for (int k = 0; k < fd; k++) {
        const long c = (long)j * fd + k;
        const bool z = mask && mask[c];
        for (int t = 0; t < td; t++)
            acc = __fadd_rn(acc, z ? 0.f : (float)raw[(i * td + t) * (long)C_raw + c]);
    }
    x[(long)j * ldx + i] = acc;
}

/* ---- float blocks (a caller's DataBuffer<float> after its own preprocessing) ----------- */
/* Transpose + td x fd sum-downsample of a time-major float block [n0][C_raw] into the
 * channel-major buffer: x[j][i] = sum over k < fd (outer) and t < td (inner) of
 * blk[(i*td + t)*C_raw + j*fd + k], added in that order from 0.0f (the order of the 8-bit
 * path and of candidate.cpp:395-407).  A CTA computes FT_J x FT_I outputs: its threads read
 * the raw rows along channels (coalesced), sum in registers, and a shared-memory transpose
 * writes along time. */
constexpr int FT_J = 32, FT_I = 32;

__global__ void __launch_bounds__(FT_J * 8) k_unpack_f32(const float *__restrict__ blk, int C_raw,
                                                        int td, int fd, float *__restrict__ x,
                                                        long ldx, int C, long N)
{
    __shared__ float tile[FT_J][FT_I + 1];
    const int jj = threadIdx.x, iy = threadIdx.y; /* 32 channels x 8 sample rows */
    const int j = blockIdx.y * FT_J + jj;
    const long i0 = (long)blockIdx.x * FT_I;
#pragma unroll
    for (int r = 0; r < FT_I / 8; r++) {
        const int ii = r * 8 + iy;
        const long i = i0 + ii;
        float acc = 0.f;
        if (j < C && i < N) {
            for (int k = 0; k < fd; k++) {
                const float *src = blk + (i * td) * (long)C_raw + (long)j * fd + k;
                for (int t = 0; t < td; t++) acc = __fadd_rn(acc, src[(long)t * C_raw]);
            }
        }
        tile[jj][ii] = acc;
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < FT_J / 8; r++) {
        const int cj = r * 8 + iy;
        const long i = i0 + jj;
        if (blockIdx.y * FT_J + cj < C && i < N)
            x[(long)(blockIdx.y * FT_J + cj) * ldx + i] = tile[cj][jj];
    }
}

/* Equalize statistics of a float block (one warp per channel): the sums of the values and of
 * their squares in the fixed FP64 reduction pattern of red32x2, then the same mean, variance,
 * (mean, 1/sd) pair and live flag as the 8-bit path's exact integer sums give. */
__global__ void __launch_bounds__(256) k_eq_params_f32(const float *__restrict__ x, long ldx, int C,
                                                       long N, float2 *__restrict__ eqp,
                                                       uint8_t *__restrict__ live)
{
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= C) return;
    double s1, s2;
    red32x2<1>(x + (long)w * ldx, nullptr, N, lane, s1, s2);
    if (lane == 0) {
        const double dn = (double)N;
        double mean = __ddiv_rn(s1, dn);
        double var = __dsub_rn(__ddiv_rn(s2, dn), __dmul_rn(mean, mean));
        double sd = var > 0. ? __dsqrt_rn(var) : 1.;
        eqp[w] = make_float2(__double2float_rn(mean), __double2float_rn(__ddiv_rn(1., sd)));
        if (live) live[w] = var > 0. ? 1 : 0;
    }
}

/* ---- equalize: exact integer statistics of the integer-valued downsampled block ---------- */
/* Per channel (one warp): the exact sums of the values and of their squares -- from the
 * unpack's per-tile partial sums when `part` is given, else from the block -- give
 * mean = s1/N, var = s2/N - mean^2, sd = sqrt(var) (1 when var <= 0) and the standardisation
 * (v - (float)mean) * (float)(1/sd), stored as eqp[j]; live[j] = var > 0.  The block itself is
 * standardised later, by whichever pass reads it next. */
__global__ void __launch_bounds__(256) k_eq_params(const unsigned long long *__restrict__ part,
                                                   long ntile, const float *__restrict__ x, long ldx,
                                                   int C, long N, float2 *__restrict__ eqp,
                                                   uint8_t *__restrict__ live)
{
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= C) return;
    long long s1 = 0, s2 = 0; /* exact integer sums: any order */
    if (part) {
        const unsigned long long *p = part + (size_t)w * ntile * 2;
        for (long t = lane; t < ntile; t += 32) {
            s1 += (long long)p[2 * t];
            s2 += (long long)p[2 * t + 1];
        }
    } else {
        const float *r = x + (long)w * ldx;
        long i0 = 0;
        if ((reinterpret_cast<uintptr_t>(r) & 15) == 0) {
            const float4 *r4 = reinterpret_cast<const float4 *>(r);
            const long n4 = N / 4;
            for (long q = lane; q < n4; q += 32) {
                const float4 f = r4[q];
                const long long a = __float2ll_rn(f.x), b = __float2ll_rn(f.y), c = __float2ll_rn(f.z),
                                d = __float2ll_rn(f.w);
                s1 += a + b + c + d;
                s2 += a * a + b * b + c * c + d * d;
            }
            i0 = 4 * n4;
        }
        for (long i = i0 + lane; i < N; i += 32) {
            long long v = __float2ll_rn(r[i]);
            s1 += v;
            s2 += v * v;
        }
    }
    s1 = warp_sum_ll(s1);
    s2 = warp_sum_ll(s2);
    if (lane == 0) {
        const double dn = (double)N;
        double mean = __ddiv_rn((double)s1, dn);
        double var = __dsub_rn(__ddiv_rn((double)s2, dn), __dmul_rn(mean, mean));
        double sd = var > 0. ? __dsqrt_rn(var) : 1.;
        eqp[w] = make_float2(__double2float_rn(mean), __double2float_rn(__ddiv_rn(1., sd)));
        if (live) live[w] = var > 0. ? 1 : 0;
    }
}

/* x[j][i] <- standardise_j(x[j][i]) - b[i] (b null or channel dead: no subtraction): the
 * equalize apply fused with the baseline subtraction, four samples per thread. */
__global__ void k_eq_apply(float *__restrict__ x, long ldx, long N, const float2 *__restrict__ eqp,
                           const float *__restrict__ b, const uint8_t *__restrict__ live)
{
    const long i = 4 * ((long)blockIdx.x * blockDim.x + threadIdx.x);
    const int j = blockIdx.y;
    if (i >= N) return;
    const Standardise f{eqp[j].x, eqp[j].y};
    const float *bb = (b && live[j]) ? b : nullptr;
    float *r = x + (long)j * ldx;
    if (i + 3 < N && ((reinterpret_cast<uintptr_t>(r) | reinterpret_cast<uintptr_t>(b)) & 15) == 0) {
        float4 v = *reinterpret_cast<float4 *>(r + i);
        v.x = f(v.x);
        v.y = f(v.y);
        v.z = f(v.z);
        v.w = f(v.w);
        if (bb) {
            const float4 c = *reinterpret_cast<const float4 *>(bb + i);
            v.x = __fsub_rn(v.x, c.x);
            v.y = __fsub_rn(v.y, c.y);
            v.z = __fsub_rn(v.z, c.z);
            v.w = __fsub_rn(v.w, c.w);
        }
        *reinterpret_cast<float4 *>(r + i) = v;
    } else {
        for (long k = i; k < i + 4 && k < N; k++) r[k] = bb ? __fsub_rn(f(r[k]), bb[k]) : f(r[k]);
    }
}

/* ---- channel mean per sample (zero-DM series), sequential over channels ---------------- */
/* Channel sum per sample, in a fixed order: the channels are cut into CSUM_BLK consecutive
 * blocks of ceil(C/CSUM_BLK); each block is summed sequentially from 0.0f (one warp per block,
 * 32 samples per warp) and the block sums, empty blocks included, are added in block order.
 * Dead channels are exactly 0, so summing all channels equals summing the live ones; the
 * divisor is the live count when `live` is given (BaseLine) and C otherwise (zdot).  With
 * `tp`, each value is first standardised by its channel's (mean, 1/sd) pair: the column mean
 * of the standardised block, which is then not stored.  32 blocks keep 32 independent chains
 * per sample in flight, so short blocks (few CTAs) still cover the GPU. */
constexpr int CSUM_BLK = 32;

template <bool TP>
__global__ void __launch_bounds__(32 * CSUM_BLK) k_colmean(const float *__restrict__ x, long ldx, int C,
                                                         long N, const uint8_t *__restrict__ live,
                                                         const float2 *__restrict__ tp,
                                                         float *__restrict__ out)
{
    __shared__ float part[CSUM_BLK][33];
    __shared__ int nlive_sh;
    const int lane = threadIdx.x, q = threadIdx.y;
    const long i = (long)blockIdx.x * 32 + lane;
    const int cb = (C + CSUM_BLK - 1) / CSUM_BLK;
    const int j0 = q * cb, j1 = min(C, j0 + cb);
    if (q == 0 && lane == 0) nlive_sh = 0;
    auto val = [&](float v, int j) {
        if (!TP) return v;
        const float2 t = tp[j];
        return Standardise{t.x, t.y}(v);
    };
    float acc = 0.f;
    if (i < N) {
        const float *p = x + i;
        int j = j0;
        for (; j + 16 <= j1; j += 16) { /* sixteen loads in flight, added in channel order */
            float v[16];
#pragma unroll
            for (int r = 0; r < 16; r++) v[r] = p[(long)(j + r) * ldx];
#pragma unroll
            for (int r = 0; r < 16; r++) acc = __fadd_rn(acc, val(v[r], j + r));
        }
        for (; j < j1; j++) acc = __fadd_rn(acc, val(p[(long)j * ldx], j));
    }
    part[q][lane] = acc;
    __syncthreads();
    if (live) { /* live channels, counted by the whole CTA */
        int cnt = 0;
        for (int c = q * 32 + lane; c < C; c += 32 * CSUM_BLK) cnt += live[c];
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) cnt += __shfl_xor_sync(FULL, cnt, off);
        if (lane == 0 && cnt) atomicAdd(&nlive_sh, cnt);
        __syncthreads();
    }
    if (q == 0 && i < N) {
        const int nl = live ? nlive_sh : C;
        float t = 0.f;
#pragma unroll 8
        for (int b = 0; b < CSUM_BLK; b++) t = __fadd_rn(t, part[b][lane]);
        out[i] = nl > 0 ? __fdiv_rn(t, (float)nl) : 0.f;
    }
}

__global__ void k_smooth(const float *__restrict__ z, long N, long nw, float *__restrict__ b)
{
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    long h = nw / 2;
    long lo = i - h < 0 ? 0 : i - h;
    long hi = i + h > N - 1 ? N - 1 : i + h;
    float acc = 0.f;
    for (long u = lo; u <= hi; u++) acc = __fadd_rn(acc, z[u]);
    b[i] = __fdiv_rn(acc, (float)(hi - lo + 1));
}

/* x[j][i] -= b[i] on live channels, four samples per thread (16-byte accesses when the row
 * and b are aligned). */
__global__ void k_sub_series(float *__restrict__ x, long ldx, long N, const float *__restrict__ b,
                             const uint8_t *__restrict__ live)
{
    const long i = 4 * ((long)blockIdx.x * blockDim.x + threadIdx.x);
    const int j = blockIdx.y;
    if (i >= N || (live && !live[j])) return;
    float *r = x + (long)j * ldx;
    if (i + 3 < N && ((reinterpret_cast<uintptr_t>(r) | reinterpret_cast<uintptr_t>(b)) & 15) == 0) {
        float4 v = *reinterpret_cast<float4 *>(r + i);
        const float4 c = *reinterpret_cast<const float4 *>(b + i);
        v.x = __fsub_rn(v.x, c.x);
        v.y = __fsub_rn(v.y, c.y);
        v.z = __fsub_rn(v.z, c.z);
        v.w = __fsub_rn(v.w, c.w);
        *reinterpret_cast<float4 *>(r + i) = v;
    } else {
        for (long k = i; k < i + 4 && k < N; k++) r[k] = __fsub_rn(r[k], b[k]);
    }
}

__global__ void k_zero_rows(float *__restrict__ x, long ldx, const int32_t *__restrict__ rows,
                            long N)
{
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    x[(long)rows[blockIdx.y] * ldx + i] = 0.f;
}

/* ---- kadaneF --------------------------------------------------------------------------- */
/* ds[i*Cds + j] = sum_{k<fdk} sum_{t<tdk} x[j*fdk+k][i*tdk+t] (k outer, t inner) */
__global__ void k_kadane_ds(const float *__restrict__ x, long ldx, int Cds, long Nds, int tdk,
                            int fdk, float *__restrict__ ds)
{
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y;
    if (i >= Nds) return;
    float acc = 0.f;
    for (int k = 0; k < fdk; k++) {
        const float *r = x + ((long)j * fdk + k) * ldx + i * tdk;
        for (int t = 0; t < tdk; t++) acc = __fadd_rn(acc, r[t]);
    }
    ds[i * Cds + j] = acc;
}

/* One thread per downsampled channel runs the maximum-sum scan over the positive and the
 * negated series in one pass (strictly larger sum replaces the best window; the running
 * sum restarts after it drops below zero), then applies the S/N test. */
constexpr int KS_T = 96; /* samples per staged tile in the kadaneF scan */
constexpr int KS_NB = 4; /* tile buffers: three in flight while one is scanned */

__device__ __forceinline__ void cp_async4(float *dst, const float *src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)),
                 "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_2() { asm volatile("cp.async.wait_group 2;" ::: "memory"); }

__global__ void __launch_bounds__(32) k_kadane_scan(const float *__restrict__ ds, int Cds, long Nds,
                                                    int tdk, int fdk, float thr, long wnlimit,
                                                    int32_t *__restrict__ ranges)
{
    /* each lane copies (cp.async) and later reads only its own channel's column of the tiles,
     * so no barrier is needed; a buffer is refilled only after the next tile's scan */
    __shared__ float tile[KS_NB][KS_T][32];
    const int lane = threadIdx.x, j = blockIdx.x * 32 + lane;
    float bestp = -INFINITY, bestn = -INFINITY, curp = 0.f, curn = 0.f;
    long csp = 0, csn = 0, sp = 0, ep = -1, sn = 0, en = -1;
    auto step = [&](long i, float v) {
        curp = __fadd_rn(curp, v);
        curn = __fadd_rn(curn, -v);
        if (curp > bestp) { bestp = curp; sp = csp; ep = i; }
        if (curn > bestn) { bestn = curn; sn = csn; en = i; }
        if (curp < 0.f) { curp = 0.f; csp = i + 1; }
        if (curn < 0.f) { curn = 0.f; csn = i + 1; }
    };
    /* the warp's 32 channels are staged KS_T samples at a time (one coalesced 128-byte row per
     * copy instruction), then each lane scans its channel sequentially */
    const long ntl = (Nds + KS_T - 1) / KS_T;
    auto stage = [&](long tl) {
        if (tl < ntl && j < Cds) {
            const long t0 = tl * KS_T;
            const int nt = (int)min((long)KS_T, Nds - t0);
            float(*tb)[32] = tile[tl % KS_NB];
            const float *src = ds + t0 * Cds + j;
            for (int r = 0; r < nt; r++) cp_async4(&tb[r][lane], src + (long)r * Cds);
        }
        cp_async_commit(); /* one group per tile, empty past the end */
    };
    stage(0);
    stage(1);
    stage(2);
    for (long tl = 0; tl < ntl; tl++) {
        cp_async_wait_2(); /* all but the two newest groups done: tile tl has landed */
        if (j < Cds) {
            const long t0 = tl * KS_T;
            const int nt = (int)min((long)KS_T, Nds - t0);
            const float(*tb)[32] = tile[tl % KS_NB];
            for (int r = 0; r < nt; r++) step(t0 + r, tb[r][lane]);
        }
        stage(tl + 3); /* into the buffer of tile tl-1 */
    }
    if (j >= Cds) return;
    const float var = (float)(tdk * fdk);
#pragma unroll
    for (int p = 0; p < 2; p++) {
        float boxsum = p == 0 ? bestp : bestn;
        long s = p == 0 ? sp : sn, e = p == 0 ? ep : en;
        long wn = e - s + 1;
        float snr2 = 0.f;
        if (wn > wnlimit) snr2 = __fdiv_rn(__fmul_rn(boxsum, boxsum), __fmul_rn((float)wn, var));
        bool zap = Nds > 0 && snr2 > thr;
        ranges[4 * j + 2 * p] = zap ? (int32_t)(s * tdk) : -1;
        ranges[4 * j + 2 * p + 1] = zap ? (int32_t)((e + 1) * tdk) : -1;
    }
}

/* One CTA per channel row: zero its downsampled channel's zapped windows (only those
 * samples are touched). */
__global__ void k_kadane_apply(float *__restrict__ x, long ldx, long N, int fdk,
                               const int32_t *__restrict__ ranges)
{
    const int jr = blockIdx.x;
    const int32_t *r = ranges + 4 * (jr / fdk);
    float *row = x + (long)jr * ldx;
#pragma unroll
    for (int p = 0; p < 2; p++) {
        const long a = r[2 * p], b = min((long)r[2 * p + 1], N);
        if (a < 0) continue;
        for (long i = a + threadIdx.x; i < b; i += blockDim.x) row[i] = 0.f;
    }
}

/* ---- kadaneT ---------------------------------------------------------------------------- */
/* One thread per downsampled sample i runs the maximum-sum scan over its band (ds[i*Cds + j],
 * j ascending) for the positive and the negated series, then the S/N test: the band is
 * zapped when it spans more than bwlimit downsampled channels and snr^2 exceeds thr. */
__global__ void k_kadaneT_scan(const float *__restrict__ ds, int Cds, long Nds, int tdk, int fdk,
                               float thr, long bwlimit, int32_t *__restrict__ ranges)
{
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= Nds) return;
    const float *row = ds + i * Cds;
    float bestp = -INFINITY, bestn = -INFINITY, curp = 0.f, curn = 0.f;
    long csp = 0, csn = 0, sp = 0, ep = -1, sn = 0, en = -1;
    auto step = [&](long j, float v) {
        curp = __fadd_rn(curp, v);
        curn = __fadd_rn(curn, -v);
        if (curp > bestp) { bestp = curp; sp = csp; ep = j; }
        if (curn > bestn) { bestn = curn; sn = csn; en = j; }
        if (curp < 0.f) { curp = 0.f; csp = j + 1; }
        if (curn < 0.f) { curn = 0.f; csn = j + 1; }
    };
    long j = 0;
    for (; j + 8 <= Cds; j += 8) {
        float v[8];
#pragma unroll
        for (int r = 0; r < 8; r++) v[r] = row[j + r];
#pragma unroll
        for (int r = 0; r < 8; r++) step(j + r, v[r]);
    }
    for (; j < Cds; j++) step(j, row[j]);
    const float var = (float)(tdk * fdk);
#pragma unroll
    for (int p = 0; p < 2; p++) {
        const float boxsum = p == 0 ? bestp : bestn;
        const long s = p == 0 ? sp : sn, e = p == 0 ? ep : en;
        const long wn = e - s + 1;
        float snr2 = 0.f;
        if (wn > bwlimit) snr2 = __fdiv_rn(__fmul_rn(boxsum, boxsum), __fmul_rn((float)wn, var));
        const bool zap = Cds > 0 && snr2 > thr;
        ranges[4 * i + 2 * p] = zap ? (int32_t)(s * fdk) : -1;
        ranges[4 * i + 2 * p + 1] = zap ? (int32_t)((e + 1) * fdk) : -1;
    }
}

__global__ void k_kadaneT_apply(float *__restrict__ x, long ldx, long N, int tdk, long Nds,
                                const int32_t *__restrict__ ranges)
{
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int c = blockIdx.y;
    if (t >= N || t / tdk >= Nds) return;
    const int32_t *r = ranges + 4 * (t / tdk);
    if ((r[0] >= 0 && c >= r[0] && c < r[1]) || (r[2] >= 0 && c >= r[2] && c < r[3]))
        x[(long)c * ldx + t] = 0.f;
}

/* ---- mask ------------------------------------------------------------------------------- */
/* Exact order statistics of the downsampled block by radix selection on order-preserving
 * 32-bit keys: four 8-bit passes, each a histogram of the keys that still match the selected
 * prefix (two targets at once, Q1 and Q3) and a one-thread pick of the digit holding the
 * remaining rank.  sel: [0,512) histograms, 512.. prefix/rank per target, 516.. results. */
__device__ __forceinline__ uint32_t order_key(float f)
{
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float order_key_inv(uint32_t k)
{
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

__global__ void __launch_bounds__(256) k_mask_hist(const float *__restrict__ ds, long n,
                                                   uint32_t *__restrict__ sel, int shift)
{
    __shared__ uint32_t h[512];
    for (int b = threadIdx.x; b < 512; b += blockDim.x) h[b] = 0;
    __syncthreads();
    const uint32_t p0 = sel[512], p1 = sel[514];
    const int hs = shift + 8;
    for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
        const uint32_t k = order_key(ds[e]);
        const uint32_t d = (k >> shift) & 255u;
        if (hs >= 32 || (k >> hs) == (p0 >> hs)) atomicAdd(&h[d], 1u);
        if (hs >= 32 || (k >> hs) == (p1 >> hs)) atomicAdd(&h[256 + d], 1u);
    }
    __syncthreads();
    for (int b = threadIdx.x; b < 512; b += blockDim.x)
        if (h[b]) atomicAdd(&sel[b], h[b]);
}

__global__ void k_mask_pick(uint32_t *__restrict__ sel, int shift, uint32_t k0, uint32_t k1,
                            float thr)
{
    if (threadIdx.x != 0) return;
    for (int t = 0; t < 2; t++) {
        uint32_t prefix = shift == 24 ? 0u : sel[512 + 2 * t];
        uint32_t rank = shift == 24 ? (t == 0 ? k0 : k1) : sel[513 + 2 * t];
        uint32_t cum = 0, digit = 255;
        for (uint32_t b = 0; b < 256; b++) {
            const uint32_t c = sel[256 * t + b];
            if (rank < cum + c) {
                digit = b;
                break;
            }
            cum += c;
        }
        sel[512 + 2 * t] = prefix | (digit << shift);
        sel[513 + 2 * t] = rank - cum;
    }
    for (int b = 0; b < 512; b++) sel[b] = 0;
    if (shift == 0) {
        const float q1 = order_key_inv(sel[512]), q3 = order_key_inv(sel[514]);
        const float r = __fsub_rn(q3, q1);
        const float lo = __fsub_rn(q1, __fmul_rn(thr, r)), hi = __fadd_rn(q3, __fmul_rn(thr, r));
        sel[516] = __float_as_uint(q1);
        sel[517] = __float_as_uint(q3);
        sel[518] = __float_as_uint(lo);
        sel[519] = __float_as_uint(hi);
    }
}

__global__ void k_mask_apply(float *__restrict__ x, long ldx, long N, int Cds, long Nds, int tdk,
                             int fdk, const float *__restrict__ ds, const uint32_t *__restrict__ sel,
                             int32_t *__restrict__ nzap)
{
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int c = blockIdx.y;
    const long i = t / tdk;
    const int j = c / fdk;
    if (t >= N || i >= Nds || j >= Cds) return;
    const float lo = __uint_as_float(sel[518]), hi = __uint_as_float(sel[519]);
    const float d = ds[i * Cds + j];
    if (d < lo || d > hi) {
        x[(long)c * ldx + t] = 0.f;
        if (c % fdk == 0 && t % tdk == 0) atomicAdd(nzap, 1);
    }
}

/* ---- zdot ------------------------------------------------------------------------------ */
/* Per channel (one warp): mean and standard deviation of the row (fixed-pattern sums) ->
 * zp[j] = ((float)mean, (float)(1/sd)), sd = 1 when the variance is not positive.  The
 * standardised row is never stored: the channel mean and the fit recompute it. */
__global__ void __launch_bounds__(256) k_zdot_norm(const float *__restrict__ x, long ldx, int C, long N,
                                                   float2 *__restrict__ zp)
{
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= C) return;
    const float *r = x + (long)w * ldx;
    double s1, s2;
    red32x2<1>(r, nullptr, N, lane, s1, s2);
    if (lane == 0) {
        const double dn = (double)N;
        double mean = __ddiv_rn(s1, dn);
        double var = __dsub_rn(__ddiv_rn(s2, dn), __dmul_rn(mean, mean));
        double sd = var > 0. ? __dsqrt_rn(var) : 1.;
        zp[w] = make_float2(__double2float_rn(mean), __double2float_rn(__ddiv_rn(1., sd)));
    }
}

/* se and ss of the zero-DM series in the fixed pattern of red32x2: lane l's runs of RED_RUN
 * elements (l + 32*(RED_RUN*rho + r)) are summed in FP32 by all threads at once, then each
 * lane adds its run totals in FP64 in run order and the lanes combine by the xor butterfly. */
constexpr int SST_RUNS = 4096; /* run totals staged per lane set (2 floats each) */

__global__ void __launch_bounds__(1024) k_zdot_sstats(const float *__restrict__ s, long N,
                                                     double *__restrict__ out)
{
    __shared__ float run1[SST_RUNS], run2[SST_RUNS];
    const long nruns = ((N + 31) / 32 + RED_RUN - 1) / RED_RUN; /* runs of the longest lane */
    double a1 = 0., a2 = 0.;
    for (long base = 0; base < nruns; base += SST_RUNS / 32) {
        const long nb = min((long)(SST_RUNS / 32), nruns - base);
        for (long u = threadIdx.x; u < nb * 32; u += blockDim.x) {
            const long rho = base + u / 32, l = u % 32;
            float r1 = 0.f, r2 = 0.f;
#pragma unroll
            for (int r = 0; r < RED_RUN; r++) {
                const long i = l + 32 * (RED_RUN * rho + r);
                if (i < N) {
                    const float v = s[i];
                    r1 = __fadd_rn(r1, v);
                    r2 = __fadd_rn(r2, __fmul_rn(v, v));
                }
            }
            run1[u] = r1;
            run2[u] = r2;
        }
        __syncthreads();
        if (threadIdx.x < 32)
            for (long q = 0; q < nb; q++) { /* an empty run is +0 and leaves the sum unchanged */
                a1 = __dadd_rn(a1, (double)run1[q * 32 + threadIdx.x]);
                a2 = __dadd_rn(a2, (double)run2[q * 32 + threadIdx.x]);
            }
        __syncthreads();
    }
    if (threadIdx.x < 32) {
        a1 = warp_sum_d(a1);
        a2 = warp_sum_d(a2);
        if (threadIdx.x == 0) {
            out[0] = a1;
            out[1] = a2;
        }
    }
}

/* Per channel (one warp), on the standardised row n = (x - m)*inv: least-squares alpha, beta
 * of n on s, then x <- n - (alpha*s + beta). */
__global__ void __launch_bounds__(256) k_zdot_fit(float *__restrict__ x, long ldx, int C, long N,
                                                  const float2 *__restrict__ zp,
                                                  const float *__restrict__ s,
                                                  const double *__restrict__ sst)
{
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= C) return;
    float *r = x + (long)w * ldx;
    const Standardise nf{zp[w].x, zp[w].y};
    double xe, xs;
    red32x2<2>(r, s, N, lane, xe, xs, nf);
    const double se = sst[0], ss = sst[1], dn = (double)N;
    double tmp = __dsub_rn(__dmul_rn(se, se), __dmul_rn(ss, dn));
    double alpha = 0., beta = 0.;
    if (tmp != 0.) {
        alpha = __ddiv_rn(__dsub_rn(__dmul_rn(xe, se), __dmul_rn(xs, dn)), tmp);
        beta = __ddiv_rn(__dsub_rn(__dmul_rn(xs, se), __dmul_rn(xe, ss)), tmp);
    }
    const float af = __double2float_rn(alpha), bf = __double2float_rn(beta);
    row_map(r, N, lane, [=](float v, long i) { return __fsub_rn(nf(v), __fadd_rn(__fmul_rn(af, s[i]), bf)); });
}

inline unsigned nblk(long n, int b) { return (unsigned)((n + b - 1) / b); }

} // namespace

size_t skzap_max_channels() { return 16384; }

void launch_skzap(const uint8_t *raw, int C_raw, long n0, float thr, unsigned long long *sums,
                  double *stats, uint8_t *mask, cudaStream_t st)
{
    cudaMemsetAsync(sums, 0, sizeof(unsigned long long) * 4 * (size_t)C_raw, st);
    const int vec = (C_raw % 4 == 0) && ((reinterpret_cast<uintptr_t>(raw) & 3) == 0);
    const long per_thread = vec ? 4 : 1;
    dim3 g1(nblk((C_raw + per_thread - 1) / per_thread, 256), nblk(n0, SK_TCHUNK));
    k_sk_sums<<<g1, 256, 0, st>>>(raw, C_raw, n0, vec, sums);
    k_sk_stats<<<nblk(C_raw, 256), 256, 0, st>>>(sums, C_raw, n0, stats);
    k_sk_select<<<1, 1024, 0, st>>>(C_raw, thr, stats, mask);
}

long eq_part_tiles(long N) { return (long)nblk(N, UV_TI); }

bool launch_unpack(const uint8_t *raw, int C_raw, long n0, int td, int fd, float *x, long ldx,
                   int C, long N, const uint8_t *mask, unsigned long long *part, cudaStream_t st)
{
    const bool vec = C_raw % 16 == 0 && (reinterpret_cast<uintptr_t>(raw) & 15) == 0 &&
                     (!mask || (reinterpret_cast<uintptr_t>(mask) & 15) == 0) &&
                     (fd == 1 || fd == 2 || fd == 4 || fd == 8 || fd == 16);
    if (vec) {
        dim3 grid(nblk(N, UV_TI), nblk(C_raw, UV_BYTES));
        switch (fd) {
        case 1: k_unpack_vec<1><<<grid, 256, 0, st>>>(raw, C_raw, n0, td, x, ldx, C, N, mask, part); break;
        case 2: k_unpack_vec<2><<<grid, 256, 0, st>>>(raw, C_raw, n0, td, x, ldx, C, N, mask, part); break;
        case 4: k_unpack_vec<4><<<grid, 256, 0, st>>>(raw, C_raw, n0, td, x, ldx, C, N, mask, part); break;
        case 8: k_unpack_vec<8><<<grid, 256, 0, st>>>(raw, C_raw, n0, td, x, ldx, C, N, mask, part); break;
        default: k_unpack_vec<16><<<grid, 256, 0, st>>>(raw, C_raw, n0, td, x, ldx, C, N, mask, part); break;
        }
        return part != nullptr;
    }
    size_t smem = (size_t)UP_TI * td * UP_TJ * fd;
    if (smem <= 96 * 1024) {
        /* per call: the attribute belongs to the current device, and handles may live on
         * different devices of one process */
        if (smem > 48 * 1024)
            cudaFuncSetAttribute(k_unpack, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024);
        dim3 grid(nblk(N, UP_TI), nblk(C, UP_TJ));
        k_unpack<<<grid, 256, smem, st>>>(raw, C_raw, n0, td, fd, x, ldx, C, N, mask);
    } else {
        dim3 grid(nblk(N, 128), C);
        k_unpack_direct<<<grid, 128, 0, st>>>(raw, C_raw, td, fd, x, ldx, C, N, mask);
    }
    return false;
}

void launch_eq_params(const unsigned long long *part, const float *x, long ldx, int C, long N,
                      float2 *eqp, uint8_t *live, cudaStream_t st)
{
    k_eq_params<<<nblk((long)C * 32, 256), 256, 0, st>>>(part, eq_part_tiles(N), x, ldx, C, N, eqp, live);
}

void launch_unpack_f32(const float *blk, int C_raw, long n0, int td, int fd, float *x, long ldx,
                       int C, long N, cudaStream_t st)
{
    (void)n0;
    dim3 grid(nblk(N, FT_I), nblk(C, FT_J));
    k_unpack_f32<<<grid, dim3(FT_J, 8), 0, st>>>(blk, C_raw, td, fd, x, ldx, C, N);
}

void launch_eq_params_f32(const float *x, long ldx, int C, long N, float2 *eqp, uint8_t *live,
                          cudaStream_t st)
{
    k_eq_params_f32<<<nblk((long)C * 32, 256), 256, 0, st>>>(x, ldx, C, N, eqp, live);
}

void launch_eq_apply(float *x, long ldx, int C, long N, const float2 *eqp, const float *b,
                     const uint8_t *live, cudaStream_t st)
{
    dim3 grid(nblk((N + 3) / 4, 256), C);
    k_eq_apply<<<grid, 256, 0, st>>>(x, ldx, N, eqp, b, live);
}

void launch_colmean(const float *x, long ldx, int C, long N, const uint8_t *live, const float2 *tp,
                    float *out, cudaStream_t st)
{
    if (tp)
        k_colmean<true><<<nblk(N, 32), dim3(32, CSUM_BLK), 0, st>>>(x, ldx, C, N, live, tp, out);
    else
        k_colmean<false><<<nblk(N, 32), dim3(32, CSUM_BLK), 0, st>>>(x, ldx, C, N, live, nullptr, out);
}

void launch_smooth(const float *z, long N, long nw, float *b, cudaStream_t st)
{
    k_smooth<<<nblk(N, 128), 128, 0, st>>>(z, N, nw, b);
}

void launch_sub_series(float *x, long ldx, int C, long N, const float *b, const uint8_t *live,
                       cudaStream_t st)
{
    dim3 grid(nblk((N + 3) / 4, 256), C);
    k_sub_series<<<grid, 256, 0, st>>>(x, ldx, N, b, live);
}

void launch_zero_rows(float *x, long ldx, const int32_t *rows, int nrows, long N,
                      cudaStream_t st)
{
    if (nrows <= 0) return;
    dim3 grid(nblk(N, 256), nrows);
    k_zero_rows<<<grid, 256, 0, st>>>(x, ldx, rows, N);
}

void launch_kadane(float *x, long ldx, int C, long N, int tdk, int fdk, float thr,
                   long wnlimit, float *ds, int32_t *ranges, cudaStream_t st)
{
    int Cds = C / fdk;
    long Nds = N / tdk;
    if (Cds <= 0) return;
    if (Nds > 0) {
        dim3 g1(nblk(Nds, 128), Cds);
        k_kadane_ds<<<g1, 128, 0, st>>>(x, ldx, Cds, Nds, tdk, fdk, ds);
    }
    k_kadane_scan<<<nblk(Cds, 32), 32, 0, st>>>(ds, Cds, Nds, tdk, fdk, thr, wnlimit, ranges);
    k_kadane_apply<<<Cds * fdk, 128, 0, st>>>(x, ldx, N, fdk, ranges);
}

void launch_kadaneT(float *x, long ldx, int C, long N, int tdk, int fdk, float thr,
                    long bwlimit, float *ds, int32_t *ranges, cudaStream_t st)
{
    const int Cds = C / fdk;
    const long Nds = N / tdk;
    if (Cds <= 0 || Nds <= 0) return;
    dim3 g1(nblk(Nds, 128), Cds);
    k_kadane_ds<<<g1, 128, 0, st>>>(x, ldx, Cds, Nds, tdk, fdk, ds);
    k_kadaneT_scan<<<nblk(Nds, 64), 64, 0, st>>>(ds, Cds, Nds, tdk, fdk, thr, bwlimit, ranges);
    dim3 g3(nblk(N, 256), Cds * fdk);
    k_kadaneT_apply<<<g3, 256, 0, st>>>(x, ldx, N, tdk, Nds, ranges);
}

void launch_mask(float *x, long ldx, int C, long N, int tdk, int fdk, float thr, float *ds,
                 uint32_t *sel, int32_t *nzap, cudaStream_t st)
{
    const int Cds = C / fdk;
    const long Nds = N / tdk;
    cudaMemsetAsync(nzap, 0, sizeof(int32_t), st);
    if (Cds <= 0 || Nds <= 0) return;
    const long n = (long)Cds * Nds;
    dim3 g1(nblk(Nds, 128), Cds);
    k_kadane_ds<<<g1, 128, 0, st>>>(x, ldx, Cds, Nds, tdk, fdk, ds);
    cudaMemsetAsync(sel, 0, sizeof(uint32_t) * MASK_SEL_WORDS, st);
    /* ranks of the quartiles, as the channel zap takes them: sorted[n/4], sorted[n-1-n/4] */
    const uint32_t k0 = (uint32_t)(n / 4), k1 = (uint32_t)(n - 1 - n / 4);
    const unsigned hb = (unsigned)std::min<long>(nblk(n, 256), 152L * 8);
    for (int shift = 24; shift >= 0; shift -= 8) {
        k_mask_hist<<<hb, 256, 0, st>>>(ds, n, sel, shift);
        k_mask_pick<<<1, 32, 0, st>>>(sel, shift, k0, k1, thr);
    }
    dim3 g3(nblk(N, 256), Cds * fdk);
    k_mask_apply<<<g3, 256, 0, st>>>(x, ldx, N, Cds, Nds, tdk, fdk, ds, sel, nzap);
}

void launch_zdot(float *x, long ldx, int C, long N, float *s, double *sstats, float2 *zp,
                 cudaStream_t st)
{
    k_zdot_norm<<<nblk((long)C * 32, 256), 256, 0, st>>>(x, ldx, C, N, zp);
    k_colmean<true><<<nblk(N, 32), dim3(32, CSUM_BLK), 0, st>>>(x, ldx, C, N, nullptr, zp, s);
    k_zdot_sstats<<<1, 1024, 0, st>>>(s, N, sstats);
    k_zdot_fit<<<nblk((long)C * 32, 256), 256, 0, st>>>(x, ldx, C, N, zp, s, sstats);
}

} // namespace txg
