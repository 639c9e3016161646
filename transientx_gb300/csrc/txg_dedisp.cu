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
#include <algorithm>
#include <type_traits>

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

/* 4-byte asynchronous global->shared copies (completion per thread by group). */
__device__ __forceinline__ void cp_async4(void *dst, const void *src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

/* Nanosecond clock of the GPU. */
__device__ __forceinline__ uint64_t gtimer()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

/* A window copy lands in microseconds; a wait that has not seen its phase complete after this
 * long gives up (the kernel then reports an error instead of hanging). */
constexpr uint64_t MBAR_LIMIT_NS = 2000000000ull;

/* Bounded wait on phase `parity`: gives up (returns false) after limit_ns of the GPU clock,
 * or after 2^30 polls should that clock not advance. */
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, uint64_t limit_ns = MBAR_LIMIT_NS)
{
    const uint64_t t0 = gtimer();
    uint32_t done = 0;
    for (long it = 0; it < (1L << 30); it++) {
        asm volatile(
            "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
            : "=r"(done)
            : "r"(smem_addr(bar)), "r"(parity)
            : "memory");
        if (done) return true;
        if (gtimer() - t0 > limit_ns) return false;
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
 * (TH*U-sample tile, subband) loads every channel row of the subband once (so each input
 * element crosses HBM once per tile) and then walks all coarse-DM groups, GS*GPT at a time:
 * the CTA's GS thread sets share the window and take GPT groups each.  Each output adds its
 * channels in ascending order from 0.0f. */
template <typename T, int TH, int U, int GS, int GPT>
__global__ void __launch_bounds__(TH * GS)
k_stage1r(const float *__restrict__ xh, long ldh, long col0, int C, long N, int nsub, int ng,
          const int32_t *__restrict__ sub_start, const int32_t *__restrict__ d1, long wmax,
          int maxch, T *__restrict__ ring, long R, long tbase_mod, int *err)
{
    constexpr int NT = TH * GS, TT = TH * U, GPC = GS * GPT;
    static_assert(GPT % 4 == 0, "delays are read four at a time");
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ __align__(8) uint64_t bar;
    __shared__ int span_sh;
    float *win = reinterpret_cast<float *>(smraw);
    int32_t *dsm = reinterpret_cast<int32_t *>(win + (size_t)maxch * wmax); /* 2 x [maxch][GPC] */
    const int s = blockIdx.y;
    const long u0 = (long)blockIdx.x * TT;
    const int j0 = sub_start[s], j1 = sub_start[s + 1], jn = j1 - j0;
    const int tid = threadIdx.x, lt = tid % TH, gs = tid / TH;
    const long cstart = (u0 + col0) & ~3L;
    const int al = (int)(u0 + col0 - cstart);
    const int nch = (ng + GPC - 1) / GPC;
    /* delays of chunk c (groups past the end repeat the last one) into table buffer c & 1 */
    auto fetch = [&](int c) {
        if (c < nch) {
            const int g0 = c * GPC, gn = min(GPC, ng - g0);
            int32_t *dt = dsm + (size_t)(c & 1) * maxch * GPC;
#pragma unroll 1
            for (int e = tid; e < jn * GPC; e += NT) {
                const int jj = e / GPC, g = e % GPC;
                cp_async4(&dt[e], &d1[(size_t)(g0 + (g < gn ? g : gn - 1)) * C + j0 + jj]);
            }
        }
        cp_async_commit();
    };

    if (tid == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
        span_sh = 0;
    }
    fetch(0);
    __syncthreads();
    for (int jj = tid; jj < jn; jj += NT) atomicMax(&span_sh, d1[(size_t)(ng - 1) * C + j0 + jj]);
    __syncthreads();
    const long W = ((long)TT + span_sh + al + 3) / 4 * 4; /* <= wmax */
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
        cp_async_wait_all();
        return;
    }
    for (int c = 0; c < nch; c++) {
        const int g0 = c * GPC, gn = min(GPC, ng - g0);
        cp_async_wait_all(); /* this thread's copies of chunk c */
        __syncthreads();     /* everyone's; and buffer (c+1)&1 is no longer read */
        fetch(c + 1);        /* overlaps this chunk's sums */
        const int32_t *dtab = dsm + (size_t)(c & 1) * maxch * GPC;
        /* the thread's samples in pairs (q, q + 1): one packed FP32 add (add.rn.f32x2, each
         * half rounded as __fadd_rn) serves two samples of a group */
        constexpr int UH = (U + 1) / 2;
        float2 acc[GPT][UH];
#pragma unroll
        for (int g = 0; g < GPT; g++)
#pragma unroll
            for (int q = 0; q < UH; q++) acc[g][q] = make_float2(0.f, 0.f);
        for (int jj = 0; jj < jn; jj++) {
            const float *wr = win + (size_t)jj * W + al + lt;
            const int4 *dv = reinterpret_cast<const int4 *>(dtab + jj * GPC + gs * GPT);
            int dd[GPT];
#pragma unroll
            for (int gq = 0; gq < GPT / 4; gq++) {
                const int4 d = dv[gq];
                dd[4 * gq] = d.x;
                dd[4 * gq + 1] = d.y;
                dd[4 * gq + 2] = d.z;
                dd[4 * gq + 3] = d.w;
            }
            /* neighbouring coarse-DM groups often share a channel's delay (it moves by a
             * third of a sample per group on average): the window values are loaded again only
             * where the delay changes (a branch uniform over the thread set) */
            float2 v[UH];
#pragma unroll
            for (int g = 0; g < GPT; g++) {
                if (g == 0 || dd[g] != dd[g - 1]) {
#pragma unroll
                    for (int q = 0; q < UH; q++) {
                        v[q].x = wr[dd[g] + 2 * q * TH];
                        v[q].y = 2 * q + 1 < U ? wr[dd[g] + (2 * q + 1) * TH] : 0.f;
                    }
                }
#pragma unroll
                for (int q = 0; q < UH; q++) {
                    if (2 * q + 1 < U)
                        acc[g][q] = __fadd2_rn(acc[g][q], v[q]);
                    else
                        acc[g][q].x = __fadd_rn(acc[g][q].x, v[q].x);
                }
            }
        }
#pragma unroll
        for (int g = 0; g < GPT; g++) {
            const int gc = gs * GPT + g;
            if (gc < gn) {
                T *out = ring + ((size_t)(g0 + gc) * nsub + s) * R;
#pragma unroll
                for (int q = 0; q < U; q++) {
                    const long u = u0 + lt + q * TH;
                    if (u < N) {
                        long t = tbase_mod + u;
                        t = t >= R ? t - R : t;
                        out[t] = to_store<T>((q & 1) ? acc[g][q / 2].y : acc[g][q / 2].x);
                    }
                }
            }
        }
    }
}

/* ---- 16-bit pairs ---------------------------------------------------------------------- */
/* FP32 += one 16-bit value (exact conversion, one rounding), PTX mixed-precision add. */
__device__ __forceinline__ void addp(float &lo_acc, float &hi_acc, uint32_t v, __half)
{
    asm("{ .reg .b16 l, h; mov.b32 {l, h}, %2; add.rn.f32.f16 %0, l, %0; add.rn.f32.f16 %1, h, %1; }"
        : "+f"(lo_acc), "+f"(hi_acc)
        : "r"(v));
}
__device__ __forceinline__ void addp(float &lo_acc, float &hi_acc, uint32_t v, __nv_bfloat16)
{
    asm("{ .reg .b16 l, h; mov.b32 {l, h}, %2; add.rn.f32.bf16 %0, l, %0; add.rn.f32.bf16 %1, h, %1; }"
        : "+f"(lo_acc), "+f"(hi_acc)
        : "r"(v));
}

/* Odd-aligned pair copy of a 16-bit window: o[k] = (e[2k+1], e[2k+2]) as one word. */
__device__ __forceinline__ void build_odd(const uint32_t *e, uint32_t *o, long nwords, int tid, int nth)
{
    for (long k = tid; k < nwords; k += nth) o[k] = __byte_perm(e[k], e[k + 1], 0x5432);
}

/* ---- stage 2 ---------------------------------------------------------------------------- */
constexpr int S2_THREADS = 128;
constexpr int S2_U = 2;                  /* samples per thread */
constexpr int S2_TT = S2_THREADS * S2_U;

/* grid: x = time tiles, y = (group, DM chunk of KPC); TH threads take U samples each of the
 * S2_TT-sample tile.  Shared memory: for a chunk of `sc`
 * subbands their ring windows (each S2_TT + d2[klast][s] - d2[kfirst][s] plus alignment),
 * then the d2 offsets [sc][KPC] and the window bookkeeping.  Each output adds its subbands
 * in ascending order from 0.0f. */
template <typename T, int KPC, int TH, int U>
__global__ void __launch_bounds__(TH)
k_stage2(const T *__restrict__ ring, long R, int nsub, int G, long ndm, long nout,
         const int32_t *__restrict__ d2, long t0_mod, int sc, long wtot_max,
         float *__restrict__ tim, long ldt, int *err)
{
    static_assert(TH * U == S2_TT && TH >= 32, "the tile is S2_TT samples");
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

    float acc[KPC][U];
#pragma unroll
    for (int k = 0; k < KPC; k++)
#pragma unroll
        for (int q = 0; q < U; q++) acc[k][q] = 0.f;

    uint32_t phase = 0;
    constexpr int EPC = 16 / (int)sizeof(T); /* elements per 16 bytes */
    for (int s0 = 0; s0 < nsub; s0 += sc) {
        const int sn = min(sc, nsub - s0);
        for (int e = tid; e < sn * KPC; e += TH) {
            const int ss = e / KPC, k = e % KPC;
            const int lo = d2[(size_t)k0 * nsub + s0 + ss];
            doff[e] = d2[(size_t)(k0 + (k < kn ? k : kn - 1)) * nsub + s0 + ss] - lo;
        }
        /* window of each subband: ring start rounded down to 16 bytes, length, offset */
        for (int ss = tid; ss < sn; ss += TH) {
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
        for (int ss = tid; ss < sn; ss += TH) {
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
                for (int q = 0; q < U; q++)
                    acc[k][q] = __fadd_rn(acc[k][q], to_f(wr[dd[k] + q * TH]));
        }
        __syncthreads();
    }
#pragma unroll
    for (int k = 0; k < KPC; k++) {
        if (k < kn) {
#pragma unroll
            for (int q = 0; q < U; q++) {
                const long u = u0 + tid + q * TH;
                if (u < nout) tim[(k0 + k) * ldt + u] = acc[k][q];
            }
        }
    }
}

/* Stage 2 on a 16-bit ring, two consecutive samples per 32-bit shared-memory load: the
 * subband windows are held as even-aligned pairs (bulk copies) and odd-aligned pairs (built
 * in shared memory).  Same order of additions as k_stage2. */
template <typename T, int KPC, int TH, int UP>
__global__ void __launch_bounds__(TH)
k_stage2p(const T *__restrict__ ring, long R, int nsub, int G, long ndm, long nout,
          const int32_t *__restrict__ d2, long t0_mod, int sc, long wtot_max,
          float *__restrict__ tim, long ldt, int *err)
{
    constexpr int TT = 2 * TH * UP;
    static_assert(TT == S2_TT && TH >= 32, "the tile is S2_TT samples");
    constexpr int EPC = 8; /* 16-bit elements per 16 bytes */
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ __align__(8) uint64_t bar;
    uint32_t *words = reinterpret_cast<uint32_t *>(smraw);
    T *win = reinterpret_cast<T *>(smraw);
    /* even pairs: wtot_max halves + one pad word; odd pairs: wtot_max/2 words */
    const long ewords = wtot_max / 2 + 4;
    uint32_t *ow = words + ewords;
    int32_t *doff = reinterpret_cast<int32_t *>(ow + wtot_max / 2);
    int32_t *wts = doff + sc * KPC, *wal = wts + sc, *wlen = wal + sc, *wpos = wlen + sc;
    const int tid = threadIdx.x;
    const int nkc = (G + KPC - 1) / KPC;
    const int g = blockIdx.y / nkc, kc = blockIdx.y % nkc;
    const long k0 = (long)g * G + (long)kc * KPC;
    const long kend = min((long)(g + 1) * G, ndm);
    const int kn = (int)min((long)KPC, kend - k0);
    if (kn <= 0) return;
    const long u0 = (long)blockIdx.x * TT;

    if (tid == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    __syncthreads();

    float acc[KPC][2 * UP];
#pragma unroll
    for (int k = 0; k < KPC; k++)
#pragma unroll
        for (int q = 0; q < 2 * UP; q++) acc[k][q] = 0.f;

    uint32_t phase = 0;
    for (int s0 = 0; s0 < nsub; s0 += sc) {
        const int sn = min(sc, nsub - s0);
        /* windows: ring start rounded down to 16 bytes, length covering the last pair */
        for (int ss = tid; ss < sn; ss += TH) {
            const int s = s0 + ss;
            const long lo = d2[(size_t)k0 * nsub + s];
            const long hi = d2[(size_t)(k0 + kn - 1) * nsub + s];
            long tstart = (t0_mod + u0 + lo) % R;
            const long al = tstart % EPC;
            tstart -= al;
            wts[ss] = (int32_t)tstart;
            wal[ss] = (int32_t)al;
            wlen[ss] = (int32_t)(((long)TT + (hi - lo) + al + 2 + EPC - 1) / EPC * EPC);
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
        /* word offsets of each (subband, DM): even or odd copy by the parity */
        for (int e = tid; e < sn * KPC; e += TH) {
            const int ss = e / KPC, k = e % KPC;
            const int lo = d2[(size_t)k0 * nsub + s0 + ss];
            const int h = wpos[ss] + wal[ss] + d2[(size_t)(k0 + (k < kn ? k : kn - 1)) * nsub + s0 + ss] - lo;
            doff[e] = (h & 1) ? (int)(ewords + (h - 1) / 2) : h / 2;
        }
        for (int ss = tid; ss < sn; ss += TH) {
            const T *row = ring + ((size_t)g * nsub + s0 + ss) * R;
            const long pos = wpos[ss], len = wlen[ss], tstart = wts[ss];
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
        {
            const long nw = (wpos[sn - 1] + wlen[sn - 1]) / 2;
            build_odd(words, ow, nw, tid, TH);
        }
        __syncthreads();
        const uint32_t *wr = words + tid;
        for (int ss = 0; ss < sn; ss++) {
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
#pragma unroll
            for (int k = 0; k < KPC; k++)
#pragma unroll
                for (int q = 0; q < UP; q++) addp(acc[k][2 * q], acc[k][2 * q + 1], wr[dd[k] + q * TH], T());
        }
        __syncthreads();
    }
#pragma unroll
    for (int k = 0; k < KPC; k++) {
        if (k < kn) {
#pragma unroll
            for (int q = 0; q < 2 * UP; q++) {
                const long u = u0 + 2 * (tid + (q >> 1) * TH) + (q & 1);
                if (u < nout) tim[(k0 + k) * ldt + u] = acc[k][q];
            }
        }
    }
}

inline unsigned nblk(long n, int b) { return (unsigned)((n + b - 1) / b); }

constexpr size_t SMEM_BUDGET = 100 * 1024;     /* chunked stage 1: two CTAs per SM */
constexpr size_t RESIDENT_BUDGET = 200 * 1024; /* whole-subband stage-1 windows */

} // namespace

/* Largest window any stage-1 CTA needs: tile + maxd1 + alignment (delays grow with the
 * group index).  xh points at column 0 of the channel buffer; col0 = H - maxd1.  When the
 * widest subband's full window fits in shared memory the resident kernel reads every channel
 * row once; otherwise the chunked kernel (channel chunks, 16 groups per CTA) is used.  Every
 * precision sums the FP32 block; only the ring's element type differs. */
template <typename T, int TH, int U, int GS, int GPT>
static bool stage1r_try(const float *xh, long ldh, long col0, int C, long N, int nsub, int ng,
                        const int32_t *sub_start, const int32_t *d1, long maxd1, int maxch, T *ring,
                        long R, long tbase_mod, int *err, cudaStream_t st)
{
    const long tt = (long)TH * U;
    const long wr = (tt + maxd1 + 3 + 3) / 4 * 4;
    const size_t smem = (size_t)maxch * wr * sizeof(float) + 2 * (size_t)maxch * GS * GPT * sizeof(int32_t);
    if (smem > RESIDENT_BUDGET) return false;
    auto kern = k_stage1r<T, TH, U, GS, GPT>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    kern<<<dim3(nblk(N, (int)tt), nsub), TH * GS, smem, st>>>(xh, ldh, col0, C, N, nsub, ng, sub_start,
                                                              d1, wr, maxch, ring, R, tbase_mod, err);
    return true;
}

template <typename T>
static void stage1_chunked(const float *xh, long ldh, long col0, int C, long N, int nsub, int ng,
                           const int32_t *sub_start, const int32_t *d1, long maxd1, int maxch,
                           T *ring, long R, long tbase_mod, int *err, cudaStream_t st)
{
    long wmax = ((long)S1_TT + maxd1 + 3 + 3) / 4 * 4;
    size_t per = wmax * sizeof(float) + S1_GPC * sizeof(int32_t);
    int cj = (int)((SMEM_BUDGET - 64) / per);
    if (cj > maxch) cj = maxch;
    if (cj < 1) cj = 1;
    size_t smem = (size_t)cj * wmax * sizeof(float) + (size_t)cj * S1_GPC * sizeof(int32_t);
    dim3 grid(nblk(N, S1_TT), nsub, nblk(ng, S1_GPC));
    cudaFuncSetAttribute(k_stage1<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_stage1<T><<<grid, S1_THREADS, smem, st>>>(xh, ldh, col0, C, N, nsub, ng, sub_start, d1, cj,
                                                wmax, ring, R, tbase_mod, err);
}

/* Resident launch shapes (threads per set x samples per thread, thread sets x groups each),
 * the same for every ring precision:
 *   0 = 32x16 16x4 (default), 1 = 256x2 1x16, 2 = 512x1 1x16, 3 = 256x2 2x8, 4 = 256x2 2x16,
 *   5 = 256x1 2x8, 6 = 256x2 4x4, 7 = 128x4 4x8, 8 = 256x4 2x8, 9 = 128x4 2x8, 10 = 128x4 8x4,
 *   11 = 64x8 8x4, 12 = 64x8 4x4, 13 = 64x8 16x4, 14 = 64x8 8x8, 15 = 64x16 8x4,
 *   16 = 256x2 4x8, 17 = 32x8 16x8
 * Every channel step loads the thread's delays (broadcast 16-byte loads, two shared-memory
 * wavefronts each) and then one window element per sample for each distinct delay among its
 * groups: many samples per thread and one warp per set keep the delay loads a small share of
 * the shared-memory traffic (measured on the 4096-channel workload: 32x16 16x4 took stage 1
 * from 185 to 159 ms per 20 blocks against 256x2 4x8; loading only where the delay changes,
 * 159 to 114 ms; a sweep of all shapes on the GB300 kept 32x16 16x4, the 1024-thread 64x8
 * 16x4 at 60 registers being 3 % slower).  A shape whose windows do not fit falls back to
 * 256x2 1x16, then to the chunked kernel (any negative variant selects the chunked kernel
 * directly). */
template <typename T>
static void stage1_dispatch(const float *xh, long ldh, long col0, int C, long N,
                            int nsub, int ng, const int32_t *sub_start, const int32_t *d1, long maxd1,
                            int maxch, T *ring, long R, long tbase_mod, int var, int *err,
                            cudaStream_t st)
{
    if (var < 0) { /* the chunked kernel, whatever fits */
        stage1_chunked<T>(xh, ldh, col0, C, N, nsub, ng, sub_start, d1, maxd1, maxch, ring, R, tbase_mod, err, st);
        return;
    }
    bool done = false;
#define TXG_ARGS xh, ldh, col0, C, N, nsub, ng, sub_start, d1, maxd1, maxch, ring, R, tbase_mod, err, st
    switch (var) {
    case 1: break;
    case 2: done = stage1r_try<T, 512, 1, 1, 16>(TXG_ARGS); break;
    case 3: done = stage1r_try<T, 256, 2, 2, 8>(TXG_ARGS); break;
    case 4: done = stage1r_try<T, 256, 2, 2, 16>(TXG_ARGS); break;
    case 5: done = stage1r_try<T, 256, 1, 2, 8>(TXG_ARGS); break;
    case 6: done = stage1r_try<T, 256, 2, 4, 4>(TXG_ARGS); break;
    case 7: done = stage1r_try<T, 128, 4, 4, 8>(TXG_ARGS); break;
    case 8: done = stage1r_try<T, 256, 4, 2, 8>(TXG_ARGS); break;
    case 9: done = stage1r_try<T, 128, 4, 2, 8>(TXG_ARGS); break;
    case 10: done = stage1r_try<T, 128, 4, 8, 4>(TXG_ARGS); break;
    case 11: done = stage1r_try<T, 64, 8, 8, 4>(TXG_ARGS); break;
    case 12: done = stage1r_try<T, 64, 8, 4, 4>(TXG_ARGS); break;
    case 13: done = stage1r_try<T, 64, 8, 16, 4>(TXG_ARGS); break;
    case 14: done = stage1r_try<T, 64, 8, 8, 8>(TXG_ARGS); break;
    case 15: done = stage1r_try<T, 64, 16, 8, 4>(TXG_ARGS); break;
    case 16: done = stage1r_try<T, 256, 2, 4, 8>(TXG_ARGS); break;
    case 17: done = stage1r_try<T, 32, 8, 16, 8>(TXG_ARGS); break;
    default: done = stage1r_try<T, 32, 16, 16, 4>(TXG_ARGS); break;
    }
    if (!done) done = stage1r_try<T, 256, 2, 1, 16>(TXG_ARGS);
#undef TXG_ARGS
    if (!done) stage1_chunked<T>(xh, ldh, col0, C, N, nsub, ng, sub_start, d1, maxd1, maxch, ring, R, tbase_mod, err, st);
}

void launch_stage1(const float *xh, long ldh, long col0, int C, long N, int nsub,
                   int ng, const int32_t *sub_start, const int32_t *d1, long maxd1, int maxch, void *ring,
                   long R, long tbase_mod, int prec, int var, int *err, cudaStream_t st)
{
    if (prec == TXG_PREC_BF16)
        stage1_dispatch<__nv_bfloat16>(xh, ldh, col0, C, N, nsub, ng, sub_start, d1, maxd1, maxch,
                                       (__nv_bfloat16 *)ring, R, tbase_mod, var, err, st);
    else if (prec == TXG_PREC_FP16)
        stage1_dispatch<__half>(xh, ldh, col0, C, N, nsub, ng, sub_start, d1, maxd1, maxch,
                                (__half *)ring, R, tbase_mod, var, err, st);
    else
        stage1_dispatch<float>(xh, ldh, col0, C, N, nsub, ng, sub_start, d1, maxd1, maxch,
                               (float *)ring, R, tbase_mod, var, err, st);
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

/* ---- subband series of one DM (get_subdata) and candidate bands ------------------------ */
template <typename T>
__global__ void k_subdata(const T *__restrict__ ring, long R, int nsub, int G, const int32_t *__restrict__ d2,
                          long k, long t0_mod, long nout, float *__restrict__ out)
{
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int s = blockIdx.y;
    if (i >= nout) return;
    const long g = k / G;
    const long t = (t0_mod + i + d2[(size_t)k * nsub + s]) % R;
    out[(size_t)s * nout + i] = to_f(ring[((size_t)g * nsub + s) * R + t]);
}

/* One CTA per candidate: per subband, the sum over samples (isamp-wn, isamp+wn) of the
 * subband sample divided by its channel count, ascending from 0.0f. */
template <typename T>
__global__ void k_cand_vpf(const T *__restrict__ ring, long R, int nsub, int G,
                           const int32_t *__restrict__ d2, const int32_t *__restrict__ sub_start,
                           long t0_mod, long nout, const txg_cand *__restrict__ c,
                           float *__restrict__ vpf)
{
    const txg_cand cd = c[blockIdx.x];
    const long k = cd.idm, g = k / G;
    const long lo = max(0L, (long)cd.isamp - cd.wn + 1), hi = min(nout, (long)cd.isamp + cd.wn);
    for (int s = threadIdx.x; s < nsub; s += blockDim.x) {
        const float cnt = (float)(sub_start[s + 1] - sub_start[s]);
        const T *row = ring + ((size_t)g * nsub + s) * R;
        const long d = d2[(size_t)k * nsub + s];
        float acc = 0.f;
        for (long i = lo; i < hi; i++) acc = __fadd_rn(acc, __fdiv_rn(to_f(row[(t0_mod + i + d) % R]), cnt));
        vpf[(size_t)blockIdx.x * nsub + s] = acc;
    }
}

template <typename T>
static void subdata_impl(const void *ring, long R, int nsub, int G, const int32_t *d2, long k,
                         long t0_mod, long nout, float *out, cudaStream_t st)
{
    dim3 grid(nblk(nout, 256), nsub);
    k_subdata<T><<<grid, 256, 0, st>>>((const T *)ring, R, nsub, G, d2, k, t0_mod, nout, out);
}

void launch_subdata(const void *ring, long R, int nsub, int G, const int32_t *d2, long k,
                    long t0_mod, long nout, int prec, float *out, cudaStream_t st)
{
    if (prec == TXG_PREC_BF16)
        subdata_impl<__nv_bfloat16>(ring, R, nsub, G, d2, k, t0_mod, nout, out, st);
    else if (prec == TXG_PREC_FP16)
        subdata_impl<__half>(ring, R, nsub, G, d2, k, t0_mod, nout, out, st);
    else
        subdata_impl<float>(ring, R, nsub, G, d2, k, t0_mod, nout, out, st);
}

void launch_cand_vpf(const void *ring, long R, int nsub, int G, const int32_t *d2,
                     const int32_t *sub_start, long t0_mod, long nout, const txg_cand *c, long n,
                     int prec, float *vpf, cudaStream_t st)
{
    if (n <= 0) return;
    if (prec == TXG_PREC_BF16)
        k_cand_vpf<__nv_bfloat16><<<(unsigned)n, 128, 0, st>>>((const __nv_bfloat16 *)ring, R, nsub, G, d2,
                                                               sub_start, t0_mod, nout, c, vpf);
    else if (prec == TXG_PREC_FP16)
        k_cand_vpf<__half><<<(unsigned)n, 128, 0, st>>>((const __half *)ring, R, nsub, G, d2, sub_start,
                                                        t0_mod, nout, c, vpf);
    else
        k_cand_vpf<float><<<(unsigned)n, 128, 0, st>>>((const float *)ring, R, nsub, G, d2, sub_start,
                                                       t0_mod, nout, c, vpf);
}

/* Ring length a stage-2 window may need (the ring must be longer, so a window wraps once). */
long stage2_window(long span) { return (long)S2_TT + span + 16; }

template <typename T, int KPC, int TH>
static void stage2_impl(const void *ring, long R, int nsub, int G, long ndm, long nout,
                        const int32_t *d2, long span, long t0_mod, float *tim, long ldt, size_t budget,
                        int *err, cudaStream_t st)
{
    const long epc = 16 / (long)sizeof(T);
    const long wlen = ((long)S2_TT + span + 2 * epc) / epc * epc;
    const size_t per = wlen * sizeof(T) + KPC * sizeof(int32_t) + 5 * sizeof(int32_t);
    int sc = (int)((budget - 64) / per);
    if (sc > nsub) sc = nsub;
    if (sc < 1) sc = 1;
    const long wtot = (long)sc * wlen;
    const size_t smem = ((wtot * sizeof(T) + 15) / 16) * 16 + (size_t)sc * KPC * 4 + (size_t)sc * 5 * 4;
    const int nkc = (G + KPC - 1) / KPC;
    const long ng = (ndm + G - 1) / G;
    dim3 grid(nblk(nout, S2_TT), (unsigned)(ng * nkc));
    auto kern = k_stage2<T, KPC, TH, S2_TT / TH>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    kern<<<grid, TH, smem, st>>>((const T *)ring, R, nsub, G, ndm, nout, d2, t0_mod, sc, wtot, tim, ldt,
                                 err);
}

/* 16-bit ring: pair kernel, TH threads of UP pairs over the S2_TT-sample tile, windows doubled
 * by the odd copy. */
template <typename T, int KPC, int TH>
static void stage2p_impl(const void *ring, long R, int nsub, int G, long ndm, long nout,
                         const int32_t *d2, long span, long t0_mod, float *tim, long ldt, size_t budget,
                         int *err, cudaStream_t st)
{
    constexpr int UP = S2_TT / 2 / TH;
    const long wlen = ((long)S2_TT + span + 2 + 7 + 7) / 8 * 8; /* halves */
    const size_t per = wlen * 4 + KPC * sizeof(int32_t) + 4 * sizeof(int32_t);
    int sc = (int)((budget - 80) / per);
    if (sc > nsub) sc = nsub;
    if (sc < 1) sc = 1;
    const long wtot = (long)sc * wlen;
    const size_t smem = (size_t)(wtot / 2 + 4) * 4 + (size_t)(wtot / 2) * 4 + (size_t)sc * KPC * 4 +
                        (size_t)sc * 4 * 4;
    const int nkc = (G + KPC - 1) / KPC;
    const long ng = (ndm + G - 1) / G;
    dim3 grid(nblk(nout, S2_TT), (unsigned)(ng * nkc));
    auto kern = k_stage2p<T, KPC, TH, UP>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    kern<<<grid, TH, smem, st>>>((const T *)ring, R, nsub, G, ndm, nout, d2, t0_mod, sc, wtot, tim, ldt,
                                 err);
}

/* FP32 threads per CTA by variant: 0 = 32 (8 samples each; DM chunks wider than 16 take 64),
 * 1 = 64 (4), 2 = 128 (2).  Fewer threads with more samples each load the per-subband delays
 * (broadcast 16-byte loads) for more additions: on the 4096-channel workload variant 0 with
 * 18 KB per CTA took stage 2 from 91 to 81 ms per 20 blocks against 128 threads with 36 KB. */
template <typename T, int K>
static void stage2_var(int var, const void *ring, long R, int nsub, int G, long ndm, long nout,
                       const int32_t *d2, long span, long t0_mod, float *tim, long ldt, size_t budget,
                       int *err, cudaStream_t st)
{
    if constexpr (K <= 16) {
        if (var == 0) {
            stage2_impl<T, K, 32>(ring, R, nsub, G, ndm, nout, d2, span, t0_mod, tim, ldt, budget, err, st);
            return;
        }
    }
    if (var == 2)
        stage2_impl<T, K, 128>(ring, R, nsub, G, ndm, nout, d2, span, t0_mod, tim, ldt, budget, err, st);
    else
        stage2_impl<T, K, 64>(ring, R, nsub, G, ndm, nout, d2, span, t0_mod, tim, ldt, budget, err, st);
}

/* 16-bit pair kernel by variant: 0 = 32 threads of 4 pairs (DM chunks wider than 16: 64 of
 * 2), 1 = 64 of 2, 2 = 128 of 1 (variant 0 with 18 KB per CTA: 71 -> 65 ms per 20 blocks of
 * the 4096-channel workload against variant 2 with 36 KB). */
template <typename T, int K>
static void stage2p_var(int var, const void *ring, long R, int nsub, int G, long ndm, long nout,
                        const int32_t *d2, long span, long t0_mod, float *tim, long ldt, size_t budget,
                        int *err, cudaStream_t st)
{
    if constexpr (K <= 16) {
        if (var == 0) {
            stage2p_impl<T, K, 32>(ring, R, nsub, G, ndm, nout, d2, span, t0_mod, tim, ldt, budget, err, st);
            return;
        }
    }
    if (var == 2)
        stage2p_impl<T, K, 128>(ring, R, nsub, G, ndm, nout, d2, span, t0_mod, tim, ldt, budget, err, st);
    else
        stage2p_impl<T, K, 64>(ring, R, nsub, G, ndm, nout, d2, span, t0_mod, tim, ldt, budget, err, st);
}

template <typename T, bool PAIRS>
static void stage2_dispatch(int var, const void *ring, long R, int nsub, int G, long ndm, long nout,
                            const int32_t *d2, long span, long t0_mod, float *tim, long ldt,
                            size_t budget, int *err, cudaStream_t st)
{
    /* variants 3-5: the thread shapes of 0-2 with half the DMs of a group per CTA (8 for
     * groups up to 24, 16 for 32): half the accumulators, so more CTAs per SM, each subband
     * window loaded by twice as many CTAs; every DM's sum is the same */
    const int kfull = stage2_kpc(G);
    const int kuse = var >= 3 ? (kfull == 32 ? 16 : 8) : kfull;
    const int v = var >= 3 ? var - 3 : var;
#define TXG_S2(K)                                                                                   \
    if constexpr (PAIRS)                                                                            \
        stage2p_var<T, K>(v, ring, R, nsub, G, ndm, nout, d2, span, t0_mod, tim, ldt, budget, err, st); \
    else                                                                                            \
        stage2_var<T, K>(v, ring, R, nsub, G, ndm, nout, d2, span, t0_mod, tim, ldt, budget, err, st)
    switch (kuse) {
    case 8: TXG_S2(8); break;
    case 16: TXG_S2(16); break;
    case 24: TXG_S2(24); break;
    default: TXG_S2(32); break;
    }
#undef TXG_S2
}

/* One CTA waits, with the bounded wait of the window copies, for a 256-byte bulk copy whose
 * barrier expects 256 + extra bytes: with extra > 0 the phase never completes (the copy lands,
 * nothing else comes), the wait runs out after limit_ns and the CTA reports it in status[0]. */
__global__ void k_wait_selftest(const uint8_t *__restrict__ src, int extra, uint64_t limit_ns,
                                int *__restrict__ status)
{
    __shared__ __align__(16) unsigned char buf[256];
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        mbar_expect_tx(&bar, 256u + (uint32_t)extra);
        bulk_g2s(buf, src, 256u, &bar);
    }
    const bool ok = mbar_wait(&bar, 0, limit_ns);
    if (!__syncthreads_and(ok)) {
        if (threadIdx.x == 0) status[0] = 1;
        return;
    }
    if (threadIdx.x == 0) status[0] = buf[0] == src[0] && buf[255] == src[255] ? 0 : 2;
}

void launch_wait_selftest(const uint8_t *src, int extra, long limit_ms, int *status, cudaStream_t st)
{
    k_wait_selftest<<<1, 32, 0, st>>>(src, extra, (uint64_t)limit_ms * 1000000ull, status);
}

void launch_stage2(const void *ring, long R, int nsub, int G, long ndm, long nout,
                   const int32_t *d2, long span, long t0_mod, int prec, int s2_var, int s2_kb,
                   float *tim, long ldt, int *err, cudaStream_t st)
{
    /* s2_kb 0: 18 KB per CTA (one-warp CTAs, about twelve per SM) */
    const size_t budget = (size_t)(s2_kb >= 8 ? s2_kb : 18) * 1024;
    if (prec == TXG_PREC_BF16)
        stage2_dispatch<__nv_bfloat16, true>(s2_var, ring, R, nsub, G, ndm, nout, d2, span, t0_mod, tim, ldt,
                                             budget, err, st);
    else if (prec == TXG_PREC_FP16)
        stage2_dispatch<__half, true>(s2_var, ring, R, nsub, G, ndm, nout, d2, span, t0_mod, tim, ldt, budget,
                                      err, st);
    else
        stage2_dispatch<float, false>(s2_var, ring, R, nsub, G, ndm, nout, d2, span, t0_mod, tim, ldt, budget,
                                      err, st);
}

} // namespace txg
