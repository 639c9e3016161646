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
 * runs of 8, FP64 lane accumulators, xor butterfly), identical in every implementation.
 */
#include <cstdio>

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

/* Fixed-pattern warp reduction of a row: mode 0 -> sum x, 1 -> sum x*x, 2 -> sum x*y. */
template <int MODE>
__device__ __forceinline__ double red32(const float *__restrict__ x, const float *__restrict__ y,
                                        long n, int lane)
{
    double acc = 0.;
    long i = lane;
    while (i < n) {
        float run = 0.f;
        for (int r = 0; r < 8 && i < n; r++, i += 32) {
            float v = x[i];
            if (MODE == 1) v = __fmul_rn(v, v);
            if (MODE == 2) v = __fmul_rn(v, y[i]);
            run = __fadd_rn(run, v);
        }
        acc = __dadd_rn(acc, (double)run);
    }
    return warp_sum_d(acc);
}

/* ---- unpack + downsample ------------------------------------------------------------- */
constexpr int UP_TJ = 64; /* output channels per CTA */
constexpr int UP_TI = 32; /* output samples per CTA */

/* raw [n0][C_raw] uint8 -> x[j][i] = sum_{k<fd} sum_{t<td} raw[i*td+t][j*fd+k] (k outer). The
 * raw tile is staged in shared memory with 32-bit loads when the row pitch allows. */
__global__ void __launch_bounds__(256) k_unpack(const uint8_t *__restrict__ raw, int C_raw, long n0,
                                               int td, int fd, float *__restrict__ x, long ldx,
                                               int C, long N)
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
        for (int k = 0; k < fd; k++)
            for (int t = 0; t < td; t++)
                acc = __fadd_rn(acc, (float)tile[(ii * td + t) * cols + jj * fd + k]);
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

/* fallback for large td*fd: one thread per output, no staging */
__global__ void k_unpack_direct(const uint8_t *__restrict__ raw, int C_raw, int td, int fd,
                                float *__restrict__ x, long ldx, int C, long N)
{
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y;
    if (i >= N || j >= C) return;
    float acc = 0.f;
    for (int k = 0; k < fd; k++)
        for (int t = 0; t < td; t++)
            acc = __fadd_rn(acc, (float)raw[(i * td + t) * (long)C_raw + (long)j * fd + k]);
    x[(long)j * ldx + i] = acc;
}

/* ---- equalize: exact integer statistics of the integer-valued downsampled block ---------- */
__global__ void __launch_bounds__(256) k_equalize(float *__restrict__ x, long ldx, int C, long N)
{
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= C) return;
    float *r = x + (long)w * ldx;
    long long s1 = 0, s2 = 0;
    for (long i = lane; i < N; i += 32) {
        long long v = __float2ll_rn(r[i]);
        s1 += v;
        s2 += v * v;
    }
    s1 = warp_sum_ll(s1);
    s2 = warp_sum_ll(s2);
    const double dn = (double)N;
    double mean = __ddiv_rn((double)s1, dn);
    double var = __dsub_rn(__ddiv_rn((double)s2, dn), __dmul_rn(mean, mean));
    double sd = var > 0. ? __dsqrt_rn(var) : 1.;
    const float mf = __double2float_rn(mean), inv = __double2float_rn(__ddiv_rn(1., sd));
    for (long i = lane; i < N; i += 32) r[i] = __fmul_rn(__fsub_rn(r[i], mf), inv);
}

/* ---- channel mean per sample (zero-DM series), sequential over channels ---------------- */
__global__ void k_colmean(const float *__restrict__ x, long ldx, int C, long N,
                          float *__restrict__ out)
{
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    float acc = 0.f;
    const float *p = x + i;
    int j = 0;
    for (; j + 4 <= C; j += 4) {
        float a = p[(long)j * ldx], b = p[(long)(j + 1) * ldx], c = p[(long)(j + 2) * ldx],
              d = p[(long)(j + 3) * ldx];
        acc = __fadd_rn(acc, a);
        acc = __fadd_rn(acc, b);
        acc = __fadd_rn(acc, c);
        acc = __fadd_rn(acc, d);
    }
    for (; j < C; j++) acc = __fadd_rn(acc, p[(long)j * ldx]);
    out[i] = __fdiv_rn(acc, (float)C);
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

__global__ void k_sub_series(float *__restrict__ x, long ldx, long N, const float *__restrict__ b)
{
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y;
    if (i >= N) return;
    x[(long)j * ldx + i] = __fsub_rn(x[(long)j * ldx + i], b[i]);
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
__global__ void k_kadane_scan(const float *__restrict__ ds, int Cds, long Nds, int tdk, int fdk,
                              float thr, long wnlimit, int32_t *__restrict__ ranges)
{
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= Cds) return;
    float bestp = -INFINITY, bestn = -INFINITY, curp = 0.f, curn = 0.f;
    long csp = 0, csn = 0, sp = 0, ep = -1, sn = 0, en = -1;
    for (long i = 0; i < Nds; i++) {
        float v = ds[i * Cds + j];
        curp = __fadd_rn(curp, v);
        curn = __fadd_rn(curn, -v);
        if (curp > bestp) { bestp = curp; sp = csp; ep = i; }
        if (curn > bestn) { bestn = curn; sn = csn; en = i; }
        if (curp < 0.f) { curp = 0.f; csp = i + 1; }
        if (curn < 0.f) { curn = 0.f; csn = i + 1; }
    }
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

__global__ void k_kadane_apply(float *__restrict__ x, long ldx, long N, int fdk,
                               const int32_t *__restrict__ ranges)
{
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    int jr = blockIdx.y;
    if (i >= N) return;
    const int32_t *r = ranges + 4 * (jr / fdk);
    if ((r[0] >= 0 && i >= r[0] && i < r[1]) || (r[2] >= 0 && i >= r[2] && i < r[3]))
        x[(long)jr * ldx + i] = 0.f;
}

/* ---- zdot ------------------------------------------------------------------------------ */
__global__ void __launch_bounds__(256) k_zdot_norm(float *__restrict__ x, long ldx, int C, long N)
{
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= C) return;
    float *r = x + (long)w * ldx;
    double s1 = red32<0>(r, nullptr, N, lane);
    double s2 = red32<1>(r, nullptr, N, lane);
    const double dn = (double)N;
    double mean = __ddiv_rn(s1, dn);
    double var = __dsub_rn(__ddiv_rn(s2, dn), __dmul_rn(mean, mean));
    double sd = var > 0. ? __dsqrt_rn(var) : 1.;
    const float mf = __double2float_rn(mean), inv = __double2float_rn(__ddiv_rn(1., sd));
    for (long i = lane; i < N; i += 32) r[i] = __fmul_rn(__fsub_rn(r[i], mf), inv);
}

__global__ void k_zdot_sstats(const float *__restrict__ s, long N, double *__restrict__ out)
{
    const int lane = threadIdx.x & 31;
    if (threadIdx.x >= 32) return;
    double se = red32<0>(s, nullptr, N, lane);
    double ss = red32<1>(s, nullptr, N, lane);
    if (lane == 0) {
        out[0] = se;
        out[1] = ss;
    }
}

__global__ void __launch_bounds__(256) k_zdot_fit(float *__restrict__ x, long ldx, int C, long N,
                                                  const float *__restrict__ s,
                                                  const double *__restrict__ sst)
{
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= C) return;
    float *r = x + (long)w * ldx;
    double xe = red32<0>(r, nullptr, N, lane);
    double xs = red32<2>(r, s, N, lane);
    const double se = sst[0], ss = sst[1], dn = (double)N;
    double tmp = __dsub_rn(__dmul_rn(se, se), __dmul_rn(ss, dn));
    double alpha = 0., beta = 0.;
    if (tmp != 0.) {
        alpha = __ddiv_rn(__dsub_rn(__dmul_rn(xe, se), __dmul_rn(xs, dn)), tmp);
        beta = __ddiv_rn(__dsub_rn(__dmul_rn(xs, se), __dmul_rn(xe, ss)), tmp);
    }
    const float af = __double2float_rn(alpha), bf = __double2float_rn(beta);
    for (long i = lane; i < N; i += 32)
        r[i] = __fsub_rn(r[i], __fadd_rn(__fmul_rn(af, s[i]), bf));
}

inline unsigned nblk(long n, int b) { return (unsigned)((n + b - 1) / b); }

} // namespace

void launch_unpack(const uint8_t *raw, int C_raw, long n0, int td, int fd, float *x, long ldx,
                   int C, long N, cudaStream_t st)
{
    size_t smem = (size_t)UP_TI * td * UP_TJ * fd;
    if (smem <= 96 * 1024) {
        static bool attr = false;
        if (!attr) {
            cudaFuncSetAttribute(k_unpack, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024);
            attr = true;
        }
        dim3 grid(nblk(N, UP_TI), nblk(C, UP_TJ));
        k_unpack<<<grid, 256, smem, st>>>(raw, C_raw, n0, td, fd, x, ldx, C, N);
    } else {
        dim3 grid(nblk(N, 128), C);
        k_unpack_direct<<<grid, 128, 0, st>>>(raw, C_raw, td, fd, x, ldx, C, N);
    }
}

void launch_equalize(float *x, long ldx, int C, long N, cudaStream_t st)
{
    k_equalize<<<nblk((long)C * 32, 256), 256, 0, st>>>(x, ldx, C, N);
}

void launch_colmean(const float *x, long ldx, int C, long N, float *out, cudaStream_t st)
{
    k_colmean<<<nblk(N, 128), 128, 0, st>>>(x, ldx, C, N, out);
}

void launch_smooth(const float *z, long N, long nw, float *b, cudaStream_t st)
{
    k_smooth<<<nblk(N, 128), 128, 0, st>>>(z, N, nw, b);
}

void launch_sub_series(float *x, long ldx, int C, long N, const float *b, cudaStream_t st)
{
    dim3 grid(nblk(N, 256), C);
    k_sub_series<<<grid, 256, 0, st>>>(x, ldx, N, b);
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
    k_kadane_scan<<<nblk(Cds, 64), 64, 0, st>>>(ds, Cds, Nds, tdk, fdk, thr, wnlimit, ranges);
    dim3 g3(nblk(N, 256), Cds * fdk);
    k_kadane_apply<<<g3, 256, 0, st>>>(x, ldx, N, fdk, ranges);
}

void launch_zdot(float *x, long ldx, int C, long N, float *s, double *sstats, cudaStream_t st)
{
    k_zdot_norm<<<nblk((long)C * 32, 256), 256, 0, st>>>(x, ldx, C, N);
    k_colmean<<<nblk(N, 128), 128, 0, st>>>(x, ldx, C, N, s);
    k_zdot_sstats<<<1, 32, 0, st>>>(s, N, sstats);
    k_zdot_fit<<<nblk((long)C * 32, 256), 256, 0, st>>>(x, ldx, C, N, s, sstats);
}

} // namespace txg
