/*
 * txg_dedisp.cu -- two-stage subband dedispersion (the RealTime::SubbandDedispersion role,
 * call sites singlepulse.cpp:230-238,328,338 and boxcar.cpp:183).
 *
 * Stage 1: for subband s, coarse-DM group g and new output time t
 *     sub[g][s][t] = sum_{j in s, ascending} x_j[t + d1[g][j]]
 * written into a per-(g,s) ring of modulus R (time index t mod R), stored as T
 * (float, bf16 or half; accumulation is always FP32).
 * Stage 2: for fine DM k of group g and output sample i of the gated block
 *     tim[k][i] = sum_{s ascending} sub[g][s][t0 + i + d2[k][s]].
 *
 * Both kernels stage their input windows in shared memory with the Blackwell bulk-copy
 * engine (cp.async.bulk global->shared, completion tracked by an mbarrier with a bounded
 * wait): one window per channel row (stage 1) or per subband ring segment (stage 2), so each
 * input element crosses HBM/L2 once per CTA tile.  A wait that runs out sets *err and the
 * CTA returns without touching its outputs.
 */
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "txg_internal.h"

namespace txg {

namespace {

/* ---- storage conversions -------------------------------------------------------------- */
template <typename T> __device__ __forceinline__ T to_store(float v);
template <> __device__ __forceinline__ float to_store<float>(float v) { return v; }
template <> __device__ __forceinline__ __nv_bfloat16 to_store<__nv_bfloat16>(float v) { return __float2bfloat16_rn(v); }
template <> __device__ __forceinline__ __half to_store<__half>(float v) { return __float2half_rn(v); }
__device__ __forceinline__ float to_f(float v) { return v; }
__device__ __forceinline__ float to_f(__nv_bfloat16 v) { return __bfloat162float(v); }
__device__ __forceinline__ float to_f(__half v) { return __half2float(v); }

/* ---- bulk copy + mbarrier helpers (PTX) ------------------------------------------------ */
__device__ __forceinline__ uint32_t smem_addr(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count));
}

__device__ __forceinline__ void fence_mbar_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.shared::cta.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

/* Orders earlier generic-proxy accesses of shared memory before later bulk copies into it. */
__device__ __forceinline__ void fence_proxy_async()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

/* Bounded wait on phase `parity`; returns false if it gave up. */
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity)
{
    uint32_t done = 0;
    for (long it = 0; it < (1L << 24); it++) {
        asm volatile(
            "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
            : "=r"(done)
            : "r"(smem_addr(bar)), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

/* ---- stage 1 ---------------------------------------------------------------------------- */
constexpr int S1_THREADS = 128;
constexpr int S1_U = 2;                       /* samples per thread */
constexpr int S1_TT = S1_THREADS * S1_U;      /* samples per CTA */
constexpr int S1_GPC = 16;                    /* coarse-DM groups per CTA */

/* grid: x = time tiles, y = subband, z = group chunks.  xh points at buffer column 0; output
 * sample u of channel j reads column u + col0 + d1[g][j].  Shared memory: channel windows
 * [cj][wmax] floats followed by the chunk's d1 [cj][S1_GPC]. */
template <typename T>
__global__ void __launch_bounds__(S1_THREADS)
k_stage1(const float *__restrict__ xh, long ldh, long col0, int C, long N, int nsub, int ng,
         const int32_t *__restrict__ sub_start, const int32_t *__restrict__ d1, int cj,
         long wmax, T *__restrict__ ring, long R, long tbase_mod, int *err)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ __align__(8) uint64_t bar;
    __shared__ int span_sh;
    float *win = reinterpret_cast<float *>(smraw);
    const int s = blockIdx.y;
    const long u0 = (long)blockIdx.x * S1_TT;
    const int g0 = blockIdx.z * S1_GPC;
    const int gn = min(S1_GPC, ng - g0);
    const int j0 = sub_start[s], j1 = sub_start[s + 1];
    int32_t *dsm = reinterpret_cast<int32_t *>(win + (size_t)cj * wmax);
    const int tid = threadIdx.x;
    /* copies start on a 16-byte boundary; al = elements skipped in front */
    const long cstart = (u0 + col0) & ~3L;
    const int al = (int)(u0 + col0 - cstart);

    if (tid == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    __syncthreads();

    float acc[S1_GPC][S1_U];
#pragma unroll
    for (int g = 0; g < S1_GPC; g++)
#pragma unroll
        for (int q = 0; q < S1_U; q++) acc[g][q] = 0.f;

    uint32_t phase = 0;
    for (int jc = j0; jc < j1; jc += cj) {
        const int jn = min(cj, j1 - jc);
        /* window span: the largest delay of the chunk's channels in the last group */
        if (tid == 0) span_sh = 0;
        __syncthreads();
        for (int jj = tid; jj < jn; jj += S1_THREADS)
            atomicMax(&span_sh, d1[(size_t)(g0 + gn - 1) * C + jc + jj]);
        for (int e = tid; e < jn * S1_GPC; e += S1_THREADS) {
            int jj = e / S1_GPC, g = e % S1_GPC;
            dsm[e] = g < gn ? d1[(size_t)(g0 + g) * C + jc + jj] : 0;
        }
        __syncthreads();
        const long W = ((long)S1_TT + span_sh + al + 3) / 4 * 4; /* <= wmax */
        if (tid == 0) {
            const uint32_t bytes = (uint32_t)(W * sizeof(float));
            fence_proxy_async();
            mbar_expect_tx(&bar, bytes * (uint32_t)jn);
            for (int jj = 0; jj < jn; jj++)
                bulk_g2s(win + (size_t)jj * W, xh + (long)(jc + jj) * ldh + cstart, bytes, &bar);
        }
        bool ok = mbar_wait(&bar, phase);
        phase ^= 1;
        if (!__syncthreads_and(ok)) {
            if (tid == 0) atomicExch(err, 1);
            mbar_wait(&bar, phase ^ 1); /* let copies still in flight land (bounded) */
            return;
        }
        for (int jj = 0; jj < jn; jj++) {
            const float *wr = win + (size_t)jj * W + al + tid;
            const int4 *dv = reinterpret_cast<const int4 *>(dsm + jj * S1_GPC);
#pragma unroll
            for (int gq = 0; gq < S1_GPC / 4; gq++) {
                const int4 d = dv[gq];
                const int dd[4] = {d.x, d.y, d.z, d.w};
#pragma unroll
                for (int r = 0; r < 4; r++)
#pragma unroll
                    for (int q = 0; q < S1_U; q++)
                        acc[gq * 4 + r][q] =
                            __fadd_rn(acc[gq * 4 + r][q], wr[dd[r] + q * S1_THREADS]);
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int g = 0; g < S1_GPC; g++) {
        if (g < gn) {
            T *out = ring + ((size_t)(g0 + g) * nsub + s) * R;
#pragma unroll
            for (int q = 0; q < S1_U; q++) {
                long u = u0 + tid + q * S1_THREADS;
                if (u < N) {
                    long t = tbase_mod + u;
                    t = t >= R ? t - R : t;
                    out[t] = to_store<T>(acc[g][q]);
                }
            }
        }
    }
}

/* Stage 1 with the subband's whole channel window resident in shared memory: one CTA per
 * (512-sample tile, subband) loads every channel row of the subband once (so each input
 * element crosses HBM once per tile) and then walks all coarse-DM groups, 16 at a time.  Each
 * output adds its channels in ascending order from 0.0f. */
constexpr int S1R_THREADS = 256;
constexpr int S1R_U = 2;
constexpr int S1R_TT = S1R_THREADS * S1R_U;

template <typename T>
__global__ void __launch_bounds__(S1R_THREADS)
k_stage1r(const float *__restrict__ xh, long ldh, long col0, int C, long N, int nsub, int ng,
          const int32_t *__restrict__ sub_start, const int32_t *__restrict__ d1, long wmax,
          int maxch, T *__restrict__ ring, long R, long tbase_mod, int *err)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ __align__(8) uint64_t bar;
    __shared__ int span_sh;
    float *win = reinterpret_cast<float *>(smraw);
    int32_t *dsm = reinterpret_cast<int32_t *>(win + (size_t)maxch * wmax);
    const int s = blockIdx.y;
    const long u0 = (long)blockIdx.x * S1R_TT;
    const int j0 = sub_start[s], j1 = sub_start[s + 1], jn = j1 - j0;
    const int tid = threadIdx.x;
    const long cstart = (u0 + col0) & ~3L;
    const int al = (int)(u0 + col0 - cstart);

    if (tid == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
        span_sh = 0;
    }
    __syncthreads();
    for (int jj = tid; jj < jn; jj += S1R_THREADS)
        atomicMax(&span_sh, d1[(size_t)(ng - 1) * C + j0 + jj]);
    __syncthreads();
    const long W = ((long)S1R_TT + span_sh + al + 3) / 4 * 4; /* <= wmax */
    if (tid == 0) {
        const uint32_t bytes = (uint32_t)(W * sizeof(float));
        mbar_expect_tx(&bar, bytes * (uint32_t)jn);
        for (int jj = 0; jj < jn; jj++)
            bulk_g2s(win + (size_t)jj * W, xh + (long)(j0 + jj) * ldh + cstart, bytes, &bar);
    }
    const bool ok = mbar_wait(&bar, 0);
    if (!__syncthreads_and(ok)) {
        if (tid == 0) atomicExch(err, 1);
        mbar_wait(&bar, 0);
        return;
    }
    for (int g0 = 0; g0 < ng; g0 += S1_GPC) {
        const int gn = min(S1_GPC, ng - g0);
        /* delays of the chunk; groups past the end repeat the last one (no reload) */
        for (int e = tid; e < jn * S1_GPC; e += S1R_THREADS) {
            const int jj = e / S1_GPC, g = e % S1_GPC;
            dsm[e] = d1[(size_t)(g0 + (g < gn ? g : gn - 1)) * C + j0 + jj];
        }
        __syncthreads();
        float acc[S1_GPC][S1R_U];
#pragma unroll
        for (int g = 0; g < S1_GPC; g++)
#pragma unroll
            for (int q = 0; q < S1R_U; q++) acc[g][q] = 0.f;
        for (int jj = 0; jj < jn; jj++) {
            const float *wr = win + (size_t)jj * W + al + tid;
            const int4 *dv = reinterpret_cast<const int4 *>(dsm + jj * S1_GPC);
            int dd[S1_GPC];
#pragma unroll
            for (int gq = 0; gq < S1_GPC / 4; gq++) {
                const int4 d = dv[gq];
                dd[4 * gq] = d.x;
                dd[4 * gq + 1] = d.y;
                dd[4 * gq + 2] = d.z;
                dd[4 * gq + 3] = d.w;
            }
            float v[S1R_U];
#pragma unroll
            for (int q = 0; q < S1R_U; q++) v[q] = wr[dd[0] + q * S1R_THREADS];
#pragma unroll
            for (int g = 0; g < S1_GPC; g++) {
                if (g > 0) {
#pragma unroll
                    for (int q = 0; q < S1R_U; q++) v[q] = wr[dd[g] + q * S1R_THREADS];
                }
#pragma unroll
                for (int q = 0; q < S1R_U; q++) acc[g][q] = __fadd_rn(acc[g][q], v[q]);
            }
        }
#pragma unroll
        for (int g = 0; g < S1_GPC; g++) {
            if (g < gn) {
                T *out = ring + ((size_t)(g0 + g) * nsub + s) * R;
#pragma unroll
                for (int q = 0; q < S1R_U; q++) {
                    const long u = u0 + tid + q * S1R_THREADS;
                    if (u < N) {
                        long t = tbase_mod + u;
                        t = t >= R ? t - R : t;
                        out[t] = to_store<T>(acc[g][q]);
                    }
                }
            }
        }
        __syncthreads();
    }
}

/* ---- stage 2 ---------------------------------------------------------------------------- */
constexpr int S2_THREADS = 128;
constexpr int S2_U = 2;                  /* samples per thread */
constexpr int S2_TT = S2_THREADS * S2_U;

/* grid: x = time tiles, y = (group, DM chunk of KPC).  Shared memory: for a chunk of `sc`
 * subbands their ring windows (each S2_TT + d2[klast][s] - d2[kfirst][s] plus alignment),
 * then the d2 offsets [sc][KPC] and the window bookkeeping.  Each output adds its subbands
 * in ascending order from 0.0f. */
template <typename T, int KPC>
__global__ void __launch_bounds__(S2_THREADS)
k_stage2(const T *__restrict__ ring, long R, int nsub, int G, long ndm, long nout,
         const int32_t *__restrict__ d2, long t0_mod, int sc, long wtot_max,
         float *__restrict__ tim, long ldt, int *err)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ __align__(8) uint64_t bar;
    T *win = reinterpret_cast<T *>(smraw);
    int32_t *doff = reinterpret_cast<int32_t *>(smraw + ((wtot_max * sizeof(T) + 15) / 16) * 16);
    int32_t *wbeg = doff + sc * KPC;
    int32_t *wts = wbeg + sc, *wal = wts + sc, *wlen = wal + sc, *wpos = wlen + sc;
    const int tid = threadIdx.x;
    const int nkc = (G + KPC - 1) / KPC;
    const int g = blockIdx.y / nkc, kc = blockIdx.y % nkc;
    const long k0 = (long)g * G + (long)kc * KPC;
    const long kend = min((long)(g + 1) * G, ndm);
    const int kn = (int)min((long)KPC, kend - k0);
    if (kn <= 0) return;
    const long u0 = (long)blockIdx.x * S2_TT;

    if (tid == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    __syncthreads();

    float acc[KPC][S2_U];
#pragma unroll
    for (int k = 0; k < KPC; k++)
#pragma unroll
        for (int q = 0; q < S2_U; q++) acc[k][q] = 0.f;

    uint32_t phase = 0;
    constexpr int EPC = 16 / (int)sizeof(T); /* elements per 16 bytes */
    for (int s0 = 0; s0 < nsub; s0 += sc) {
        const int sn = min(sc, nsub - s0);
        for (int e = tid; e < sn * KPC; e += S2_THREADS) {
            const int ss = e / KPC, k = e % KPC;
            const int lo = d2[(size_t)k0 * nsub + s0 + ss];
            doff[e] = d2[(size_t)(k0 + (k < kn ? k : kn - 1)) * nsub + s0 + ss] - lo;
        }
        /* window of each subband: ring start rounded down to 16 bytes, length, offset */
        for (int ss = tid; ss < sn; ss += S2_THREADS) {
            const int s = s0 + ss;
            const long lo = d2[(size_t)k0 * nsub + s];
            const long hi = d2[(size_t)(k0 + kn - 1) * nsub + s];
            long tstart = (t0_mod + u0 + lo) % R;
            const long al = tstart % EPC;
            tstart -= al;
            wts[ss] = (int32_t)tstart;
            wal[ss] = (int32_t)al;
            wlen[ss] = (int32_t)(((long)S2_TT + (hi - lo) + al + EPC - 1) / EPC * EPC);
        }
        __syncthreads();
        if (tid < 32) { /* exclusive prefix of the lengths (one warp) */
            int carry = 0;
            for (int base = 0; base < sn; base += 32) {
                const int ss = base + tid;
                const int v = ss < sn ? wlen[ss] : 0;
                int incl = v;
#pragma unroll
                for (int off = 1; off < 32; off <<= 1) {
                    const int y = __shfl_up_sync(0xffffffffu, incl, off);
                    if (tid >= off) incl += y;
                }
                if (ss < sn) wpos[ss] = carry + incl - v;
                carry += __shfl_sync(0xffffffffu, incl, 31);
            }
            if (tid == 0) {
                fence_proxy_async();
                mbar_expect_tx(&bar, (uint32_t)(carry * (int)sizeof(T)));
            }
        }
        __syncthreads();
        for (int ss = tid; ss < sn; ss += S2_THREADS) {
            const T *row = ring + ((size_t)g * nsub + s0 + ss) * R;
            const long pos = wpos[ss], len = wlen[ss], tstart = wts[ss];
            wbeg[ss] = (int32_t)(pos + wal[ss]);
            /* split at the ring end; R is a multiple of 32 elements and exceeds len, so both
             * parts are whole 16-byte units inside the row */
            const long first = min(len, R - tstart);
            fence_proxy_async();
            bulk_g2s(win + pos, row + tstart, (uint32_t)(first * sizeof(T)), &bar);
            if (first < len)
                bulk_g2s(win + pos + first, row, (uint32_t)((len - first) * sizeof(T)), &bar);
        }
        __syncthreads();
        bool ok = mbar_wait(&bar, phase);
        phase ^= 1;
        if (!__syncthreads_and(ok)) {
            if (tid == 0) atomicExch(err, 2);
            mbar_wait(&bar, phase ^ 1);
            return;
        }
        for (int ss = 0; ss < sn; ss++) {
            const T *wr = win + wbeg[ss] + tid;
            const int4 *dv = reinterpret_cast<const int4 *>(doff + ss * KPC);
            int dd[KPC];
#pragma unroll
            for (int kq = 0; kq < KPC / 4; kq++) {
                const int4 d = dv[kq];
                dd[4 * kq] = d.x;
                dd[4 * kq + 1] = d.y;
                dd[4 * kq + 2] = d.z;
                dd[4 * kq + 3] = d.w;
            }
            /* DMs past the end of a partial group repeat the last offset; their sums are
             * discarded, and no per-DM branch keeps all loads free to issue together */
#pragma unroll
            for (int k = 0; k < KPC; k++)
#pragma unroll
                for (int q = 0; q < S2_U; q++)
                    acc[k][q] = __fadd_rn(acc[k][q], to_f(wr[dd[k] + q * S2_THREADS]));
        }
        __syncthreads();
    }
#pragma unroll
    for (int k = 0; k < KPC; k++) {
        if (k < kn) {
#pragma unroll
            for (int q = 0; q < S2_U; q++) {
                const long u = u0 + tid + q * S2_THREADS;
                if (u < nout) tim[(k0 + k) * ldt + u] = acc[k][q];
            }
        }
    }
}

inline unsigned nblk(long n, int b) { return (unsigned)((n + b - 1) / b); }

constexpr size_t SMEM_BUDGET = 100 * 1024;     /* two CTAs per SM overlap copies and math */
constexpr size_t RESIDENT_BUDGET = 200 * 1024; /* whole-subband stage-1 windows */

} // namespace

/* Largest window any stage-1 CTA needs: tile + maxd1 + alignment (delays grow with the
 * group index).  xh points at column 0 of the channel buffer; col0 = H - maxd1.  When the
 * widest subband's full window fits in shared memory the resident kernel reads every channel
 * row once; otherwise the chunked kernel (channel chunks, 16 groups per CTA) is used. */
void launch_stage1(const float *xh, long ldh, long col0, int C, long N, int nsub, int ng,
                   const int32_t *sub_start, const int32_t *d1, long maxd1, int maxch, void *ring,
                   long R, long tbase_mod, int prec, int *err, cudaStream_t st)
{
    const long wr = ((long)S1R_TT + maxd1 + 3 + 3) / 4 * 4;
    const size_t smem_r = (size_t)maxch * wr * sizeof(float) + (size_t)maxch * S1_GPC * sizeof(int32_t);
    if (smem_r <= RESIDENT_BUDGET) {
        dim3 grid(nblk(N, S1R_TT), nsub);
#define TXG_S1R(TY)                                                                                \
    cudaFuncSetAttribute(k_stage1r<TY>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_r);  \
    k_stage1r<TY><<<grid, S1R_THREADS, smem_r, st>>>(xh, ldh, col0, C, N, nsub, ng, sub_start, d1, \
                                                     wr, maxch, (TY *)ring, R, tbase_mod, err)
        if (prec == TXG_PREC_BF16) {
            TXG_S1R(__nv_bfloat16);
        } else if (prec == TXG_PREC_FP16) {
            TXG_S1R(__half);
        } else {
            TXG_S1R(float);
        }
#undef TXG_S1R
        return;
    }
    long wmax = ((long)S1_TT + maxd1 + 3 + 3) / 4 * 4;
    size_t per = wmax * sizeof(float) + S1_GPC * sizeof(int32_t);
    int cj = (int)((SMEM_BUDGET - 64) / per);
    if (cj > maxch) cj = maxch;
    if (cj < 1) cj = 1;
    size_t smem = (size_t)cj * wmax * sizeof(float) + (size_t)cj * S1_GPC * sizeof(int32_t);
    dim3 grid(nblk(N, S1_TT), nsub, nblk(ng, S1_GPC));
    if (prec == TXG_PREC_BF16) {
        cudaFuncSetAttribute(k_stage1<__nv_bfloat16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_stage1<__nv_bfloat16><<<grid, S1_THREADS, smem, st>>>(
            xh, ldh, col0, C, N, nsub, ng, sub_start, d1, cj, wmax, (__nv_bfloat16 *)ring, R, tbase_mod, err);
    } else if (prec == TXG_PREC_FP16) {
        cudaFuncSetAttribute(k_stage1<__half>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_stage1<__half><<<grid, S1_THREADS, smem, st>>>(
            xh, ldh, col0, C, N, nsub, ng, sub_start, d1, cj, wmax, (__half *)ring, R, tbase_mod, err);
    } else {
        cudaFuncSetAttribute(k_stage1<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_stage1<float><<<grid, S1_THREADS, smem, st>>>(
            xh, ldh, col0, C, N, nsub, ng, sub_start, d1, cj, wmax, (float *)ring, R, tbase_mod, err);
    }
}

/* DMs per stage-2 CTA for a group of G fine DMs (one chunk per group when G <= 32). */
static int stage2_kpc(int G) { return G <= 8 ? 8 : G <= 16 ? 16 : G <= 24 ? 24 : 32; }

/* Largest d2 spread inside one stage-2 DM chunk, over all chunks and subbands. */
long stage2_span(const int32_t *d2h, int nsub, int G, long ndm)
{
    const long kpc = stage2_kpc(G);
    long span = 0;
    for (long g0 = 0; g0 < ndm; g0 += G)
        for (long k0 = g0; k0 < min(g0 + (long)G, ndm); k0 += kpc) {
            long k1 = min(min(k0 + kpc, g0 + (long)G), ndm) - 1;
            for (int s = 0; s < nsub; s++) {
                long d = (long)d2h[k1 * nsub + s] - d2h[k0 * nsub + s];
                span = d > span ? d : span;
            }
        }
    return span;
}

/* Ring length a stage-2 window may need (the ring must be longer, so a window wraps once). */
long stage2_window(long span) { return (long)S2_TT + span + 16; }

template <typename T, int KPC>
static void stage2_impl(const void *ring, long R, int nsub, int G, long ndm, long nout,
                        const int32_t *d2, long span, long t0_mod, float *tim, long ldt, int *err,
                        cudaStream_t st)
{
    const long epc = 16 / (long)sizeof(T);
    const long wlen = ((long)S2_TT + span + 2 * epc) / epc * epc;
    const size_t per = wlen * sizeof(T) + KPC * sizeof(int32_t) + 5 * sizeof(int32_t);
    int sc = (int)((SMEM_BUDGET - 64) / per);
    if (sc > nsub) sc = nsub;
    if (sc < 1) sc = 1;
    const long wtot = (long)sc * wlen;
    const size_t smem = ((wtot * sizeof(T) + 15) / 16) * 16 + (size_t)sc * KPC * 4 + (size_t)sc * 5 * 4;
    const int nkc = (G + KPC - 1) / KPC;
    const long ng = (ndm + G - 1) / G;
    dim3 grid(nblk(nout, S2_TT), (unsigned)(ng * nkc));
    cudaFuncSetAttribute(k_stage2<T, KPC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_stage2<T, KPC><<<grid, S2_THREADS, smem, st>>>((const T *)ring, R, nsub, G, ndm, nout, d2,
                                                     t0_mod, sc, wtot, tim, ldt, err);
}

template <typename T>
static void stage2_dispatch(const void *ring, long R, int nsub, int G, long ndm, long nout,
                            const int32_t *d2, long span, long t0_mod, float *tim, long ldt,
                            int *err, cudaStream_t st)
{
    switch (stage2_kpc(G)) {
    case 8: stage2_impl<T, 8>(ring, R, nsub, G, ndm, nout, d2, span, t0_mod, tim, ldt, err, st); break;
    case 16: stage2_impl<T, 16>(ring, R, nsub, G, ndm, nout, d2, span, t0_mod, tim, ldt, err, st); break;
    case 24: stage2_impl<T, 24>(ring, R, nsub, G, ndm, nout, d2, span, t0_mod, tim, ldt, err, st); break;
    default: stage2_impl<T, 32>(ring, R, nsub, G, ndm, nout, d2, span, t0_mod, tim, ldt, err, st); break;
    }
}

void launch_stage2(const void *ring, long R, int nsub, int G, long ndm, long nout,
                   const int32_t *d2, long span, long t0_mod, int prec, float *tim, long ldt,
                   int *err, cudaStream_t st)
{
    if (prec == TXG_PREC_BF16)
        stage2_dispatch<__nv_bfloat16>(ring, R, nsub, G, ndm, nout, d2, span, t0_mod, tim, ldt, err, st);
    else if (prec == TXG_PREC_FP16)
        stage2_dispatch<__half>(ring, R, nsub, G, ndm, nout, d2, span, t0_mod, tim, ldt, err, st);
    else
        stage2_dispatch<float>(ring, R, nsub, G, ndm, nout, d2, span, t0_mod, tim, ldt, err, st);
}

} // namespace txg
