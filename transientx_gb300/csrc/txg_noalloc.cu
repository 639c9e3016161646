/*
 * txg_noalloc.cu -- kadaneF on a block that already lives in device memory, with no
 * allocation of any kind.
 *
 * Some callers cannot call cudaMalloc while they process data: real-time beam-former back
 * ends that reserve all device memory once at start-up and must not stall their capture
 * stream (cudaMalloc and cudaFree can synchronise the device, and a stall drops incoming
 * samples), and host frameworks that own the GPU memory through their own pool and hand a
 * plug-in nothing but pointers.  txg_kadaneF_noalloc serves them: the caller passes the block
 * and the output, and the one scratch buffer the filter needs (the td x fd downsampled copy
 * of the block that the maximum-sum scan reads) is the file-scope array below, reserved by
 * the loader on every GPU that loads the library and held until the process exits.
 *
 * Limits: (nsamples/td) * (nchans/fd) <= TXG_KADANE_NOALLOC_MAX floats (8 MiB), nchans/fd
 * between 1 and 65535 (one grid row per downsampled channel) and nsamples <= 2^31 - 1 (the
 * zapped windows are int32 sample indices); anything else is rejected with TXG_ERR_ARG
 * before any kernel is queued, so x and ranges stay untouched.  All calls share the array and each call overwrites every
 * element it reads before reading it, so nothing has to start at zero; calls whose work
 * overlaps on the GPU (for example on two streams at once) race on it.  The first call on a
 * device looks up the array's device address (cudaGetSymbolAddress) with that device
 * current; make that first call before any stream capture on the device.  The address is
 * kept for the life of the process: a caller that destroys the device's primary context
 * (cudaDeviceReset) must not call this entry point on that device afterwards.
 */
#include <mutex>

#include "txg_internal.h"

#define TXG_KADANE_NOALLOC_MAX (1 << 21)

static __device__ __align__(256) float g_kadane_scratch[TXG_KADANE_NOALLOC_MAX];

namespace {
constexpr int MAX_DEVICES = 64;
std::mutex g_mu;
float *g_scratch[MAX_DEVICES] = {};
} // namespace

extern "C" int txg_kadaneF_noalloc(float *x, int64_t ldx, int32_t nchans, int64_t nsamples,
                                   int32_t td, int32_t fd, float thr2, int64_t wnlimit,
                                   int32_t *ranges, void *stream)
{
    if (!x || !ranges || nchans < 1 || nsamples < 1 || td < 1 || fd < 1 || ldx < nsamples)
        return txg::set_arg_error("txg_kadaneF_noalloc: need x, ranges, nchans >= 1, "
                                  "nsamples >= 1, td, fd >= 1, ldx >= nsamples");
    if (nchans < fd || nchans / fd > 65535)
        return txg::set_arg_error("txg_kadaneF_noalloc: nchans/fd must be between 1 and 65535");
    if (nsamples > 0x7fffffffLL)
        return txg::set_arg_error("txg_kadaneF_noalloc: nsamples must fit the int32 zap ranges");
    const long long need = (long long)(nsamples / td) * (long long)(nchans / fd);
    if (need > TXG_KADANE_NOALLOC_MAX)
        return txg::set_arg_error("txg_kadaneF_noalloc: (nsamples/td)*(nchans/fd) = " +
                                  std::to_string(need) + " exceeds the fixed scratch of " +
                                  std::to_string(TXG_KADANE_NOALLOC_MAX) + " floats");
    int dev = 0;
    TXG_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= MAX_DEVICES) return txg::set_arg_error("txg_kadaneF_noalloc: device index too large");
    float *scratch = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_mu);
        if (!g_scratch[dev]) {
            float *p = nullptr;
            TXG_CUDA_TRY(cudaGetSymbolAddress((void **)&p, g_kadane_scratch));
            g_scratch[dev] = p;
        }
        scratch = g_scratch[dev];
    }
    txg::launch_kadane(x, (long)ldx, nchans, (long)nsamples, td, fd, thr2, (long)wnlimit, scratch,
                       ranges, (cudaStream_t)stream);
    TXG_CUDA_TRY(cudaGetLastError());
    return TXG_OK;
}
