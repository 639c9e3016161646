/*
 * txg_api.cu -- the extern "C" boundary (include/transientx_gb300.h): plan, device state,
 * per-block launch sequence and candidate harvesting.
 *
 * Per pushed block and ddplan row, on the handle's stream (SinglePulse::run order,
 * src/singlepulse/singlepulse.cpp:287-341):
 *   history copy -> unpack+downsample -> equalize -> baseline -> zap -> rfilist ops ->
 *   stage 1 (ring) -> [gate, boxcar.cpp:161] stage 2 -> boxcar+threshold -> async D2H.
 * Candidate buffers rotate over NSLOT slots per (beam,row) so the device runs ahead of the
 * host; a slot is harvested before it is reused and at txg_sync.  Each block's candidates
 * are copied into pinned memory (two buffers per slot) on a copy stream; sorting them
 * into Cluster::run order (cluster.cpp:91-112) and clustering run on worker threads, so the
 * launching thread only waits for the device.  Raw blocks from host memory are copied on a
 * second stream, overlapping the previous block's kernels.
 */
#include <algorithm>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <array>
#include <cstring>
#include <deque>
#include <functional>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "txg_internal.h"

namespace txg {

static thread_local std::string g_err;

int set_cuda_error(cudaError_t e, const char *expr, const char *file, int line)
{
    char buf[512];
    snprintf(buf, sizeof(buf), "%s failed: %s (%s:%d)", expr, cudaGetErrorString(e), file, line);
    g_err = buf;
    if (e == cudaErrorMemoryAllocation) return TXG_ERR_NOMEM;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return TXG_ERR_NODEVICE;
    return TXG_ERR_CUDA;
}

const char *last_error_text() { return g_err.c_str(); }

static int fail(int code, const std::string &msg)
{
    g_err = msg;
    return code;
}

int set_arg_error(const std::string &msg) { return fail(TXG_ERR_ARG, msg); }

static constexpr int NSLOT = 3;
static constexpr long HCAP_MAX = 1 << 18; /* candidates read back into pinned memory per block */
static constexpr int NCLASS = 5;

struct Result;

struct Slot {
    txg_cand *dcand = nullptr;              /* device [cap] */
    int *dcount = nullptr;                  /* device [2]: count, error code */
    txg_cand *hbuf[2] = {nullptr, nullptr}; /* pinned [hcap] */
    long nread = 0;                         /* candidates copied into hbuf[buf] */
    cudaEvent_t boxed = nullptr;            /* the block's candidate list is complete */
    std::shared_ptr<Result> reader[2];      /* result whose sort may still read hbuf[i] */
    int buf = 0;                            /* buffer of the pending block */
    long uses = 0;
    int *hcount = nullptr;                  /* pinned [2] */
    cudaEvent_t done = nullptr;
    cudaEvent_t ev[NCLASS + 1] = {};
    bool pending = false;
    bool gated = false;
    long counter = 0;
};

struct Result {
    long counter = 0;
    int gated = 0;
    long count = 0;                /* points above threshold (may exceed the capacity) */
    const txg_cand *src = nullptr; /* pinned read-back of the first nsrc points */
    long nsrc = 0;
    std::vector<txg_cand> tail;    /* points beyond the pinned read-back */
    std::vector<txg_cand> cands;   /* (idm, isamp) order */
    std::vector<txg_cand> clusters;
    bool failed = false;
    bool released = false; /* the pinned read-back is read no more (guarded by Workers::m) */
    bool ready = false;    /* guarded by Workers::m */
};
using ResultP = std::shared_ptr<Result>;

/* Worker threads for the host side of harvested blocks. */
struct Workers {
    std::mutex m;
    std::condition_variable more, done;
    std::deque<std::function<void()>> q;
    std::vector<std::thread> th;
    long inflight = 0;
    bool stop = false;

    void start(int n)
    {
        try {
            for (int i = 0; i < n; i++) th.emplace_back([this] { loop(); });
        } catch (...) { /* fewer threads; with none, jobs run on the caller */
        }
    }
    void loop()
    {
        for (;;) {
            std::function<void()> f;
            {
                std::unique_lock<std::mutex> lk(m);
                more.wait(lk, [&] { return stop || !q.empty(); });
                if (q.empty()) return;
                f = std::move(q.front());
                q.pop_front();
            }
            f();
        }
    }
    void submit(std::function<void()> f)
    {
        {
            std::lock_guard<std::mutex> lk(m);
            inflight++;
            if (!th.empty()) q.push_back(std::move(f));
        }
        if (th.empty()) f();
        else more.notify_one();
    }
    void finish(Result &r)
    {
        {
            std::lock_guard<std::mutex> lk(m);
            r.ready = true;
            inflight--;
        }
        done.notify_all();
    }
    void complete(Result &r) /* a result with nothing to do on a worker */
    {
        std::lock_guard<std::mutex> lk(m);
        r.released = r.ready = true;
    }
    void release(Result &r) /* the job has copied its points out of the pinned read-back */
    {
        {
            std::lock_guard<std::mutex> lk(m);
            r.released = true;
        }
        done.notify_all();
    }
    void wait_released(const Result &r)
    {
        std::unique_lock<std::mutex> lk(m);
        done.wait(lk, [&] { return r.released || r.ready; });
    }
    void wait(const Result &r)
    {
        std::unique_lock<std::mutex> lk(m);
        done.wait(lk, [&] { return r.ready; });
    }
    bool is_ready(const Result &r)
    {
        std::lock_guard<std::mutex> lk(m);
        return r.ready;
    }
    void drain()
    {
        std::unique_lock<std::mutex> lk(m);
        done.wait(lk, [&] { return inflight == 0; });
    }
    void shutdown()
    {
        {
            std::lock_guard<std::mutex> lk(m);
            stop = true;
        }
        more.notify_all();
        for (auto &t : th) t.join();
        th.clear();
    }
};

struct BeamRow {
    float *xh[2] = {nullptr, nullptr};
    int cur = 0;
    float *ds = nullptr;
    int32_t *ranges[8] = {nullptr};
    uint32_t *sel = nullptr; /* mask: quartile selection state */
    float *z = nullptr, *b = nullptr, *s = nullptr;
    double *sst = nullptr;
    uint8_t *live = nullptr;
    unsigned long long *eqpart = nullptr; /* equalize: per-(channel, 64-sample tile) sums */
    float2 *eqp = nullptr, *zp = nullptr; /* (mean, 1/sd) per channel: equalize, zdot */
    void *ring = nullptr;
    float *tim = nullptr;
    double *bx_scratch = nullptr; /* boxcar statistics and chunk offsets of long rows */
    float *mxS = nullptr;
    int32_t *mxwn = nullptr;
    Slot slot[NSLOT];
    long nblocks = 0;      /* blocks pushed */
    long pushed = 0;       /* counter as of the last pushed block */
    /* state of the most recently harvested block */
    long counter = 0;
    int gated = 0;
    ResultP last;
    long last_count = 0;
    bool overflow = false;
    int dev_error = 0;
    std::deque<ResultP> fifo; /* harvested blocks not yet popped */
    long guess = 4096;        /* candidates to read back with the next gated block */
};

static constexpr size_t FIFO_MAX = 256;

struct RowDev {
    int32_t *sub_start = nullptr, *d1 = nullptr, *d2 = nullptr, *vwn = nullptr, *zap = nullptr;
};

/* Per-beam scratch of the skewness/kurtosis channel zap. */
struct BeamPrep {
    unsigned long long *sums = nullptr; /* [4][nchans] */
    double *stats = nullptr;            /* [2][nchans] */
    uint8_t *mask = nullptr;            /* [nchans] */
};

} // namespace txg

using namespace txg;

struct txg_handle {
    int device = 0; /* the CUDA device current at txg_create */
    txg_plan plan;
    std::vector<double> freqs;
    std::vector<txg_row> rows;
    std::vector<RowPlan> rp;
    std::vector<RowDev> rd;
    std::vector<std::vector<BeamRow>> br; /* [beam][row] */
    std::vector<BeamPrep> prep;           /* [beam] */
    cudaStream_t st = nullptr;
    cudaStream_t cst = nullptr; /* host-to-device copies of raw blocks */
    cudaStream_t dst = nullptr; /* device-to-host copies of candidates */
    /* one stream per ddplan row: the rows of a block run concurrently (the single-CTA and
     * latency-bound kernels and the last waves of one row leave SMs to the others); each
     * forks from the handle stream after the block's shared steps (raw copy, channel zap),
     * and the handle stream waits only for every row's unpack before the next block's shared
     * steps, so consecutive blocks overlap too; readers of results join all rows first */
    std::vector<cudaStream_t> rst;
    std::vector<cudaEvent_t> row_done;     /* join of everything queued on a row stream */
    std::vector<cudaEvent_t> row_unpacked; /* a row's unpack (the last reader of the raw block
                                            * and of the channel-zap mask) is done */
    cudaEvent_t fork = nullptr;
    uint8_t *raw[2] = {nullptr, nullptr};
    uint8_t *stage[2] = {nullptr, nullptr}; /* pinned staging for pageable host input */
    /* float blocks (txg_push_block_f32): device double buffer, pinned staging and their
     * events, allocated by the first such push */
    float *rawf[2] = {nullptr, nullptr};
    float *stagef[2] = {nullptr, nullptr};
    cudaEvent_t rawf_free[2] = {nullptr, nullptr};
    cudaEvent_t rawf_loaded[2] = {nullptr, nullptr};
    int rawf_cur = 0;
    bool rawf_ready = false;
    cudaEvent_t raw_free[2] = {nullptr, nullptr};   /* kernels done with raw[i] */
    cudaEvent_t raw_loaded[2] = {nullptr, nullptr}; /* raw[i] copied in */
    int raw_cur = 0;
    long cap = 0, hcap = 0;
    std::unique_ptr<Workers> pool;
    int prec = 0, flags = 0;
    double class_ms[NCLASS] = {0};
    long class_n[NCLASS] = {0};
    std::vector<std::array<double, NCLASS>> row_ms; /* the same per ddplan row */
    std::vector<std::array<long, NCLASS>> row_n;
    std::vector<void *> allocs;
};

/* Makes the handle's device current for the duration of an entry point and restores the
 * caller's current device on return, so that handles on different devices can be driven from
 * one thread. */
struct DeviceScope {
    int prev = -1;
    explicit DeviceScope(const txg_handle *h)
    {
        int cur = -1;
        if (h && cudaGetDevice(&cur) == cudaSuccess && cur != h->device &&
            cudaSetDevice(h->device) == cudaSuccess)
            prev = cur;
    }
    ~DeviceScope()
    {
        if (prev >= 0) cudaSetDevice(prev);
    }
    DeviceScope(const DeviceScope &) = delete;
    DeviceScope &operator=(const DeviceScope &) = delete;
};

namespace {

const char *status_text(int s)
{
    switch (s) {
    case TXG_OK: return "ok";
    case TXG_ERR_ARG: return "invalid argument";
    case TXG_ERR_NOMEM: return "out of memory";
    case TXG_ERR_CUDA: return "CUDA error";
    case TXG_ERR_OVERFLOW: return "candidate buffer overflow";
    case TXG_ERR_TIMEOUT: return "device wait timed out";
    case TXG_ERR_STATE: return "invalid state";
    case TXG_ERR_NODEVICE: return "no usable CUDA device";
    case TXG_ERR_UNSUPPORTED: return "unsupported option";
    default: return "unknown status";
    }
}

template <typename T> int dalloc(txg_handle *h, T **p, size_t count)
{
    void *q = nullptr;
    size_t bytes = count * sizeof(T);
    if (bytes == 0) bytes = 16;
    TXG_CUDA_TRY(cudaMalloc(&q, bytes));
    h->allocs.push_back(q);
    TXG_CUDA_TRY(cudaMemsetAsync(q, 0, bytes, h->st));
    *p = (T *)q;
    return TXG_OK;
}

template <typename T> int upload(txg_handle *h, T **p, const std::vector<T> &v)
{
    int rc = dalloc(h, p, v.size());
    if (rc) return rc;
    if (!v.empty())
        TXG_CUDA_TRY(cudaMemcpyAsync(*p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, h->st));
    return TXG_OK;
}

size_t ring_elem(int prec) { return prec == TXG_PREC_FP32 ? 4 : 2; }

void free_all(txg_handle *h)
{
    for (cudaStream_t s : h->rst)
        if (s) cudaStreamSynchronize(s);
    if (h->st) cudaStreamSynchronize(h->st);
    if (h->cst) cudaStreamSynchronize(h->cst);
    if (h->dst) cudaStreamSynchronize(h->dst);
    if (h->pool) h->pool->shutdown();
    for (auto &beam : h->br)
        for (auto &b : beam)
            for (auto &sl : b.slot) {
                for (int i = 0; i < 2; i++)
                    if (sl.hbuf[i]) cudaFreeHost(sl.hbuf[i]);
                if (sl.hcount) cudaFreeHost(sl.hcount);
                if (sl.done) cudaEventDestroy(sl.done);
                if (sl.boxed) cudaEventDestroy(sl.boxed);
                for (auto &e : sl.ev)
                    if (e) cudaEventDestroy(e);
            }
    for (void *p : h->allocs) cudaFree(p);
    h->allocs.clear();
    for (int i = 0; i < 2; i++) {
        if (h->stage[i]) cudaFreeHost(h->stage[i]);
        if (h->raw_free[i]) cudaEventDestroy(h->raw_free[i]);
        if (h->raw_loaded[i]) cudaEventDestroy(h->raw_loaded[i]);
        if (h->stagef[i]) cudaFreeHost(h->stagef[i]);
        if (h->rawf_free[i]) cudaEventDestroy(h->rawf_free[i]);
        if (h->rawf_loaded[i]) cudaEventDestroy(h->rawf_loaded[i]);
        h->stagef[i] = nullptr;
        h->rawf_free[i] = h->rawf_loaded[i] = nullptr;
    }
    for (cudaStream_t s : h->rst)
        if (s) cudaStreamDestroy(s);
    for (cudaEvent_t e : h->row_done)
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : h->row_unpacked)
        if (e) cudaEventDestroy(e);
    h->rst.clear();
    h->row_done.clear();
    h->row_unpacked.clear();
    if (h->fork) cudaEventDestroy(h->fork);
    h->fork = nullptr;
    if (h->st) cudaStreamDestroy(h->st);
    if (h->cst) cudaStreamDestroy(h->cst);
    if (h->dst) cudaStreamDestroy(h->dst);
    h->dst = nullptr;
    h->st = nullptr;
    h->cst = nullptr;
}

/* Candidates into (idm, isamp) order, the order of Cluster::run's threshold scan
 * (cluster.cpp:91-112): stable counting passes by isamp, then by idm. */
void sort_points(const txg_cand *a, long na, const txg_cand *b, long nb, long ndm, long nout,
                 std::vector<txg_cand> &out)
{
    const long n = na + nb;
    out.resize(n);
    auto at = [&](long i) -> const txg_cand & { return i < na ? a[i] : b[i - na]; };
    bool inrange = true;
    for (long i = 0; i < n && inrange; i++) {
        const txg_cand &c = at(i);
        inrange = c.idm >= 0 && c.idm < ndm && c.isamp >= 0 && c.isamp < nout;
    }
    if (!inrange) {
        for (long i = 0; i < n; i++) out[i] = at(i);
        std::stable_sort(out.begin(), out.end(), [](const txg_cand &x, const txg_cand &y) {
            return x.idm != y.idm ? x.idm < y.idm : x.isamp < y.isamp;
        });
        return;
    }
    std::vector<txg_cand> tmp(n);
    std::vector<long> pos(std::max(ndm, nout) + 1);
    std::fill(pos.begin(), pos.begin() + nout + 1, 0);
    for (long i = 0; i < n; i++) pos[at(i).isamp + 1]++;
    for (long k = 0; k < nout; k++) pos[k + 1] += pos[k];
    for (long i = 0; i < n; i++) tmp[pos[at(i).isamp]++] = at(i);
    std::fill(pos.begin(), pos.begin() + ndm + 1, 0);
    for (long i = 0; i < n; i++) pos[tmp[i].idm + 1]++;
    for (long k = 0; k < ndm; k++) pos[k + 1] += pos[k];
    for (long i = 0; i < n; i++) out[pos[tmp[i].idm]++] = tmp[i];
}

/* Host side of one harvested block (on a worker thread): sort its points, cluster them. */
void post_process(const txg_handle *h, const RowPlan &P, Result &r, Workers *pool)
{
    try {
        sort_points(r.src, r.nsrc, r.tail.data(), (long)r.tail.size(), P.cfg.ndm, P.nout, r.cands);
        r.src = nullptr;
        pool->release(r); /* the slot's pinned buffer may take the next block now */
        std::vector<txg_cand>().swap(r.tail);
        if ((h->flags & TXG_FLAG_CLUSTER) && r.gated && !r.cands.empty()) {
            const txg_row &c = P.cfg;
            r.clusters.resize(std::max(1, c.maxncand));
            long m = cluster_run(r.cands.data(), (long)r.cands.size(), c.dms, c.ddm, P.fmax, P.fmin,
                                 P.tsamp, c.radius_smearing, c.maxncand, c.minpts, c.drop, P.maxwn,
                                 r.clusters.data(), (long)r.clusters.size());
            r.clusters.resize(std::min<long>(m, (long)r.clusters.size()));
        }
    } catch (...) {
        r.failed = true;
        r.cands.clear();
        r.clusters.clear();
        pool->release(r);
    }
}

int result_status(const txg_handle *h, const Result &r)
{
    if (r.failed) return fail(TXG_ERR_NOMEM, "host memory exhausted while sorting candidates");
    if (r.count > h->cap) return TXG_ERR_OVERFLOW;
    return TXG_OK;
}

/* Collect one slot: wait for its block, take its candidates and hand them to a worker; the
 * result becomes the row's last block and joins its queue. */
int harvest(txg_handle *h, BeamRow &b, Slot &sl, const RowPlan &P)
{
    if (!sl.pending) return TXG_OK;
    TXG_CUDA_TRY(cudaEventSynchronize(sl.done));
    sl.pending = false;
    if (h->flags & TXG_FLAG_TIMING) {
        for (int c = 0; c < NCLASS; c++) {
            if ((c == 3 || c == 4) && !sl.gated) continue;
            float ms = 0.f;
            TXG_CUDA_TRY(cudaEventElapsedTime(&ms, sl.ev[c], sl.ev[c + 1]));
            h->class_ms[c] += ms;
            h->class_n[c] += 1;
            const size_t r = (size_t)(&P - h->rp.data());
            h->row_ms[r][c] += ms;
            h->row_n[r][c] += 1;
        }
    }
    b.counter = sl.counter;
    b.gated = sl.gated;
    auto r = std::make_shared<Result>();
    r->counter = sl.counter;
    r->gated = sl.gated;
    b.last = r;
    b.last_count = 0;
    if (sl.hcount[1] != 0) {
        b.dev_error = sl.hcount[1];
        h->pool->complete(*r);
        return fail(TXG_ERR_TIMEOUT, "a bounded device wait gave up (kernel code " +
                                         std::to_string(sl.hcount[1]) + ")");
    }
    int rc = TXG_OK;
    if (sl.gated) {
        const long cnt = sl.hcount[0];
        r->count = cnt;
        b.last_count = cnt;
        const long keep = std::min(cnt, h->cap);
        const long pre = std::min(keep, sl.nread);
        /* next read-back of this row: this count with a margin */
        b.guess = std::min(h->hcap, std::max(4096L, cnt + cnt / 4 + 1024));
        r->src = sl.hbuf[sl.buf];
        r->nsrc = pre;
        sl.reader[sl.buf] = r;
        if (keep > pre) {
            r->tail.resize(keep - pre);
            TXG_CUDA_TRY(cudaMemcpy(r->tail.data(), sl.dcand + pre, (keep - pre) * sizeof(txg_cand),
                                    cudaMemcpyDeviceToHost));
        }
        if (cnt > h->cap) {
            b.overflow = true;
            rc = fail(TXG_ERR_OVERFLOW, "candidate buffer overflow: " + std::to_string(cnt) +
                                            " points above threshold, capacity " + std::to_string(h->cap));
        }
    }
    if (b.fifo.size() >= FIFO_MAX) b.fifo.pop_front();
    b.fifo.push_back(r);
    Workers *pool = h->pool.get();
    const RowPlan *pp = &P;
    if (r->nsrc > 0 || !r->tail.empty())
        pool->submit([h, pool, pp, r] {
            post_process(h, *pp, *r, pool);
            pool->finish(*r);
        });
    else
        pool->complete(*r);
    return rc;
}

long pmod(long a, long m)
{
    long r = a % m;
    return r < 0 ? r + m : r;
}

/* The handle stream waits for everything queued so far on the row streams (and so does
 * whatever is queued on it next). */
int join_rows(txg_handle *h)
{
    for (size_t r = 0; r < h->rst.size(); r++) {
        TXG_CUDA_TRY(cudaEventRecord(h->row_done[r], h->rst[r]));
        TXG_CUDA_TRY(cudaStreamWaitEvent(h->st, h->row_done[r], 0));
    }
    return TXG_OK;
}

/* Queue every ddplan row of one block whose raw samples are at `raw` on the device. */
int run_block(txg_handle *h, int beam, const uint8_t *raw, const float *rawf = nullptr)
{
    const long n0 = h->plan.ndump;
    const int Craw = h->plan.nchans;
    const bool timing = h->flags & TXG_FLAG_TIMING;
    int status = TXG_OK;
    const uint8_t *mask = nullptr;
    if (!rawf && h->plan.zapthre > 0.f) {
        BeamPrep &bp = h->prep[beam];
        launch_skzap(raw, Craw, n0, h->plan.zapthre, bp.sums, bp.stats, bp.mask, h->st);
        TXG_CUDA_TRY(cudaGetLastError());
        mask = bp.mask;
    }
    TXG_CUDA_TRY(cudaEventRecord(h->fork, h->st));
    for (size_t r = 0; r < h->rp.size(); r++) {
        const RowPlan &P = h->rp[r];
        RowDev &D = h->rd[r];
        BeamRow &b = h->br[beam][r];
        Slot &sl = b.slot[b.nblocks % NSLOT];
        /* with per-kernel-class timing the rows run one after another on the handle stream,
         * so that each class's event span holds its own kernels only */
        const cudaStream_t rs = timing ? h->st : h->rst[r];
        int rc = harvest(h, b, sl, P);
        if (rc && rc != TXG_ERR_OVERFLOW) return rc;
        if (rc) status = rc;
        TXG_CUDA_TRY(cudaStreamWaitEvent(rs, h->fork, 0));
        if (timing) TXG_CUDA_TRY(cudaEventRecord(sl.ev[0], rs));

        /* history: the last H columns of the previous block go in front of this one */
        /* one buffer when the history is shorter than a block (the previous block's last H
         * columns [N, N+H) move to [0, H), stream-ordered after its stage 1); two otherwise */
        float *xprev = b.xh[1] ? b.xh[b.cur ^ 1] : b.xh[0], *xcur = b.xh[1] ? b.xh[b.cur] : b.xh[0];
        if (P.H > 0)
            TXG_CUDA_TRY(cudaMemcpy2DAsync(xcur, P.ldh * sizeof(float), xprev + P.N,
                                           P.ldh * sizeof(float), P.H * sizeof(float), P.C,
                                           cudaMemcpyDeviceToDevice, rs));
        float *x = xcur + P.H;
        bool part = false;
        if (rawf)
            launch_unpack_f32(rawf, Craw, n0, P.cfg.td, P.cfg.fd, x, P.ldh, P.C, P.N, rs);
        else
            part = launch_unpack(raw, Craw, n0, P.cfg.td, P.cfg.fd, x, P.ldh, P.C, P.N, mask,
                                 b.eqpart, rs);
        TXG_CUDA_TRY(cudaEventRecord(h->row_unpacked[r], rs));
        TXG_CUDA_TRY(cudaStreamWaitEvent(h->st, h->row_unpacked[r], 0));
        if (timing) TXG_CUDA_TRY(cudaEventRecord(sl.ev[1], rs));

        /* equalize from the unpack's integer sums (float blocks: FP64 sums of the block); its
         * apply rides on the baseline pass */
        if (rawf)
            launch_eq_params_f32(x, P.ldh, P.C, P.N, b.eqp, b.live, rs);
        else
            launch_eq_params(part ? b.eqpart : nullptr, x, P.ldh, P.C, P.N, b.eqp, b.live, rs);
        if (P.bl_nw > 0) {
            launch_colmean(x, P.ldh, P.C, P.N, b.live, b.eqp, b.z, rs);
            launch_smooth(b.z, P.N, P.bl_nw, b.b, rs);
            launch_eq_apply(x, P.ldh, P.C, P.N, b.eqp, b.b, b.live, rs);
        } else {
            launch_eq_apply(x, P.ldh, P.C, P.N, b.eqp, nullptr, b.live, rs);
        }
        if (!P.zap_chan.empty())
            launch_zero_rows(x, P.ldh, D.zap, (int)P.zap_chan.size(), P.N, rs);
        for (int q = 0; q < P.cfg.nrfi; q++) {
            if (P.cfg.rfi_kind[q] == TXG_RFI_KADANEF)
                launch_kadane(x, P.ldh, P.C, P.N, P.cfg.rfi_td[q], P.cfg.rfi_fd[q], P.kad_thr,
                              P.kad_wnlimit[q], b.ds, b.ranges[q], rs);
            else if (P.cfg.rfi_kind[q] == TXG_RFI_ZDOT)
                launch_zdot(x, P.ldh, P.C, P.N, b.s, b.sst, b.zp, rs);
            else if (P.cfg.rfi_kind[q] == TXG_RFI_KADANET)
                launch_kadaneT(x, P.ldh, P.C, P.N, P.cfg.rfi_td[q], P.cfg.rfi_fd[q], P.kadT_thr,
                               P.kad_wnlimit[q], b.ds, b.ranges[q], rs);
            else if (P.cfg.rfi_kind[q] == TXG_RFI_MASK)
                launch_mask(x, P.ldh, P.C, P.N, P.cfg.rfi_td[q], P.cfg.rfi_fd[q], P.mask_thr, b.ds,
                            b.sel, b.ranges[q], rs);
            else if (P.cfg.rfi_kind[q] == TXG_RFI_ZERO) {
                /* zero-DM filter: the live-channel mean series off every live channel */
                launch_colmean(x, P.ldh, P.C, P.N, b.live, nullptr, b.z, rs);
                launch_sub_series(x, P.ldh, P.C, P.N, b.z, b.live, rs);
            }
        }
        if (timing) TXG_CUDA_TRY(cudaEventRecord(sl.ev[2], rs));

        /* stage 1: new subband samples t in [counter-N-maxd1, counter-maxd1) */
        const long counter = b.pushed + P.N;
        const long tbase = counter - P.N - P.maxd1;
        TXG_CUDA_TRY(cudaMemsetAsync(sl.dcount, 0, 2 * sizeof(int), rs));
        launch_stage1(xcur, P.ldh, P.H - P.maxd1, P.C, P.N, P.nsub, P.ng, D.sub_start, D.d1,
                      P.maxd1, P.maxch, b.ring, P.R, pmod(tbase, P.R), h->prec, P.s1_var,
                      sl.dcount + 1, rs);
        TXG_CUDA_TRY(cudaGetLastError());
        if (timing) TXG_CUDA_TRY(cudaEventRecord(sl.ev[3], rs));

        const bool gated = counter >= P.offset - P.noverlap + P.N;
        if (gated) {
            const long t0 = counter - P.N - P.offset;
            launch_stage2(b.ring, P.R, P.nsub, P.G, P.cfg.ndm, P.nout, D.d2, P.s2_span,
                          pmod(t0, P.R), h->prec, P.s2_var, P.s2_kb, b.tim, P.nout, sl.dcount + 1, rs);
            TXG_CUDA_TRY(cudaGetLastError());
            if (timing) TXG_CUDA_TRY(cudaEventRecord(sl.ev[4], rs));
            rc = launch_boxcar(b.tim, P.nout, P.cfg.ndm, P.nout, D.vwn, (int)P.vwn.size(), P.maxwn,
                               P.cfg.iqr, (h->flags & TXG_FLAG_AVX2_TAIL) ? 1 : 0, P.cfg.thre,
                               sl.dcand, sl.dcount, h->cap, b.mxS, b.mxwn, b.bx_scratch,
                               sl.dcount + 1, rs);
            if (rc) return rc;
            TXG_CUDA_TRY(cudaGetLastError());
            if (timing) TXG_CUDA_TRY(cudaEventRecord(sl.ev[5], rs));
            /* read-back on the copy stream, overlapping the next kernels: the row's expected
             * count of candidates (the rest, if any, is fetched at harvest) and the count.
             * The buffer's previous reader (two uses of this slot ago) must be done. */
            sl.buf = (int)(sl.uses++ & 1);
            if (sl.reader[sl.buf]) { /* its previous block's sort must have read it */
                h->pool->wait_released(*sl.reader[sl.buf]);
                sl.reader[sl.buf].reset();
            }
            sl.nread = std::min(b.guess, h->hcap);
            TXG_CUDA_TRY(cudaEventRecord(sl.boxed, rs));
            TXG_CUDA_TRY(cudaStreamWaitEvent(h->dst, sl.boxed, 0));
            TXG_CUDA_TRY(cudaMemcpyAsync(sl.hbuf[sl.buf], sl.dcand, sl.nread * sizeof(txg_cand),
                                         cudaMemcpyDeviceToHost, h->dst));
            TXG_CUDA_TRY(cudaMemcpyAsync(sl.hcount, sl.dcount, 2 * sizeof(int), cudaMemcpyDeviceToHost, h->dst));
            TXG_CUDA_TRY(cudaEventRecord(sl.done, h->dst));
        } else {
            if (timing) {
                TXG_CUDA_TRY(cudaEventRecord(sl.ev[4], rs));
                TXG_CUDA_TRY(cudaEventRecord(sl.ev[5], rs));
            }
            TXG_CUDA_TRY(cudaMemcpyAsync(sl.hcount, sl.dcount, 2 * sizeof(int), cudaMemcpyDeviceToHost, rs));
            TXG_CUDA_TRY(cudaEventRecord(sl.done, rs));
        }
        sl.pending = true;
        sl.gated = gated;
        sl.counter = counter;
        b.pushed = counter;
        b.nblocks++;
        if (b.xh[1]) b.cur ^= 1;
    }
    return status;
}

/* Device-layout decisions on top of plan_row: stage-2 window span, ring length, buffer
 * pitch, and the limits of the kernels. */
int finish_plan(RowPlan &P, int r)
{
    P.s2_span = stage2_span(P.d2.data(), P.nsub, P.G, P.cfg.ndm);
    const long need = stage2_window(P.s2_span) + 64;
    if (P.R < need) P.R = (need + 31) / 32 * 32;
    P.maxch = 0;
    for (int s = 0; s < P.nsub; s++) P.maxch = std::max(P.maxch, P.sub_start[s + 1] - P.sub_start[s]);
    /* a stage-1 tile copy starts at most 7 columns before its tile and spans the tile (at
     * most 1024 samples) plus the largest within-subband delay plus alignment and one pair
     * element, so it may read up to H + N + 1040 columns: pad the pitch past that */
    P.ldh = ((P.H + P.N + 1056) + 31) / 32 * 32;
    /* launch shapes; TXG_DEDISP_SHAPE="s1=<variant>,s2=<variant>,s2kb=<KB>" overrides them */
    if (const char *e = getenv("TXG_DEDISP_SHAPE")) {
        int v = 0;
        if (const char *q = strstr(e, "s1=")) P.s1_var = (sscanf(q + 3, "%d", &v) == 1) ? v : P.s1_var;
        if (const char *q = strstr(e, "s2kb=")) P.s2_kb = (sscanf(q + 5, "%d", &v) == 1 && v >= 8 && v <= 200) ? v : P.s2_kb;
        if (const char *q = strstr(e, "s2=")) P.s2_var = (sscanf(q + 3, "%d", &v) == 1) ? v : P.s2_var;
    }
    if (P.vwn.size() > 256) return fail(TXG_ERR_UNSUPPORTED, "more than 256 boxcar widths");
    if (!boxcar_supported(P.nout, P.maxwn, (int)P.vwn.size()))
        return fail(TXG_ERR_UNSUPPORTED, "row " + std::to_string(r) +
                                             ": ndump+noverlap or the widest boxcar exceeds the "
                                             "boxcar kernels' limits");
    return TXG_OK;
}

void fill_info(const RowPlan &P, txg_row_info *out)
{
    memset(out, 0, sizeof(*out));
    out->nchans = P.C;
    out->nsub = P.nsub;
    out->dm_group = P.G;
    out->ngroup = P.ng;
    out->nwidths = (int32_t)P.vwn.size();
    out->maxwn = P.maxwn;
    out->ndm = P.cfg.ndm;
    out->ndump = P.N;
    out->noverlap = P.noverlap;
    out->offset = P.offset;
    out->nsamples = P.nout;
    out->maxd1 = P.maxd1;
    out->maxd2 = P.maxd2;
    out->tsamp = P.tsamp;
    out->dms = P.cfg.dms;
    out->ddm = P.cfg.ddm;
    out->fmin = P.fmin;
    out->fmax = P.fmax;
}

void copy_tables(const RowPlan &P, int32_t *d1, int32_t *d2, int32_t *sub_start, int32_t *vwn)
{
    if (d1) memcpy(d1, P.d1.data(), P.d1.size() * sizeof(int32_t));
    if (d2) memcpy(d2, P.d2.data(), P.d2.size() * sizeof(int32_t));
    if (sub_start) memcpy(sub_start, P.sub_start.data(), P.sub_start.size() * sizeof(int32_t));
    if (vwn) memcpy(vwn, P.vwn.data(), P.vwn.size() * sizeof(int32_t));
}

int check_beam_row(txg_handle *h, int beam, int row)
{
    if (!h) return fail(TXG_ERR_ARG, "null handle");
    if (beam < 0 || beam >= (int)h->br.size() || row < 0 || row >= (int)h->rp.size())
        return fail(TXG_ERR_ARG, "beam or row out of range");
    return TXG_OK;
}

/* Timing-based choice of a row's launch shapes (TXG_FLAG_AUTOTUNE).  Every candidate adds the
 * same values in the same order, so the results do not depend on the choice: the fastest
 * stage-1 shape (time tile x coarse-DM groups per CTA) and stage-2 variant (threads per CTA x
 * shared-memory window budget) are kept, each timed over three launches on the row's own
 * buffers (beam 0) after one untimed launch.  A TXG_DEDISP_SHAPE override wins over it. */
int autotune_row(txg_handle *h, int r)
{
    RowPlan &P = h->rp[r];
    RowDev &D = h->rd[r];
    BeamRow &b = h->br[0][r];
    int *err = b.slot[0].dcount;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        if (e0) cudaEventDestroy(e0);
        return fail(TXG_ERR_CUDA, "event creation failed");
    }
    auto time_of = [&](auto &&launch, float &ms) -> int {
        launch();
        TXG_CUDA_TRY(cudaEventRecord(e0, h->st));
        for (int k = 0; k < 3; k++) launch();
        TXG_CUDA_TRY(cudaEventRecord(e1, h->st));
        TXG_CUDA_TRY(cudaEventSynchronize(e1));
        TXG_CUDA_TRY(cudaGetLastError());
        TXG_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
        return TXG_OK;
    };
    int rc = TXG_OK;
    const char *env = getenv("TXG_DEDISP_SHAPE");
    TXG_CUDA_TRY(cudaMemsetAsync(err, 0, 2 * sizeof(int), h->st));
    if (!(env && strstr(env, "s1="))) {
        static const int cand1[] = {0, 13, 17, 14, 16, 10, 1};
        float best = -1.f;
        for (int v : cand1) {
            float ms = 0.f;
            rc = time_of([&] {
                launch_stage1(b.xh[0], P.ldh, P.H - P.maxd1, P.C, P.N, P.nsub, P.ng, D.sub_start,
                              D.d1, P.maxd1, P.maxch, b.ring, P.R, 0, h->prec, v, err + 1, h->st);
            }, ms);
            if (rc) break;
            if (best < 0.f || ms < best) {
                best = ms;
                P.s1_var = v;
            }
        }
    }
    if (!rc && !(env && (strstr(env, "s2=") || strstr(env, "s2kb=")))) {
        static const int cand2[][2] = {{0, 0}, {1, 0}, {2, 0}, {0, 36}, {2, 36}, {1, 24},
                                       {3, 0}, {4, 0}, {5, 0}};
        float best = -1.f;
        for (auto &c : cand2) {
            float ms = 0.f;
            rc = time_of([&] {
                launch_stage2(b.ring, P.R, P.nsub, P.G, P.cfg.ndm, P.nout, D.d2, P.s2_span, 0,
                              h->prec, c[0], c[1], b.tim, P.nout, err + 1, h->st);
            }, ms);
            if (rc) break;
            if (best < 0.f || ms < best) {
                best = ms;
                P.s2_var = c[0];
                P.s2_kb = c[1];
            }
        }
    }
    int hostc[2] = {0, 0};
    if (!rc && cudaMemcpy(hostc, err, sizeof(hostc), cudaMemcpyDeviceToHost) != cudaSuccess)
        rc = fail(TXG_ERR_CUDA, "autotune read-back failed");
    if (!rc && hostc[1] != 0) rc = fail(TXG_ERR_TIMEOUT, "a bounded device wait gave up while autotuning");
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (!rc) TXG_CUDA_TRY(cudaMemsetAsync(err, 0, 2 * sizeof(int), h->st));
    return rc;
}

} // namespace

extern "C" {

int32_t txg_version(void) { return TXG_ABI_VERSION; }

const char *txg_strerror(int32_t status)
{
    static thread_local std::string s;
    s = status_text(status);
    if (status != TXG_OK && !g_err.empty()) s += ": " + g_err;
    return s.c_str();
}

int txg_selftest_wait(int32_t never_complete, int32_t limit_ms)
{
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return fail(TXG_ERR_NODEVICE, "no CUDA device");
    if (limit_ms < 1 || limit_ms > 10000) return fail(TXG_ERR_ARG, "limit_ms must lie in [1, 10000]");
    uint8_t *src = nullptr;
    int *dstatus = nullptr;
    cudaStream_t st = nullptr;
    int hstatus = -1;
    cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&src, 256);
    if (e == cudaSuccess) e = cudaMalloc(&dstatus, sizeof(int));
    if (e == cudaSuccess) e = cudaMemsetAsync(src, 0x5a, 256, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(dstatus, 0xff, sizeof(int), st);
    if (e == cudaSuccess) {
        launch_wait_selftest(src, never_complete ? 256 : 0, limit_ms, dstatus, st);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hstatus, dstatus, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (src) cudaFree(src);
    if (dstatus) cudaFree(dstatus);
    if (st) cudaStreamDestroy(st);
    if (e != cudaSuccess) return set_cuda_error(e, "txg_selftest_wait", __FILE__, __LINE__);
    if (hstatus == 1) return fail(TXG_ERR_TIMEOUT, "a bounded device wait gave up (self-test)");
    if (hstatus != 0) return fail(TXG_ERR_CUDA, "self-test copy arrived wrong");
    return TXG_OK;
}

int txg_width_ladder(float minw, float maxw, float snrloss, double tsamp, int32_t *vwn, int32_t cap)
{
    if (!vwn || cap <= 0) return 0;
    return width_ladder(minw, maxw, snrloss, tsamp, vwn, cap);
}

int txg_create(const txg_plan *plan, txg_handle **out)
{
    if (!plan || !out) return fail(TXG_ERR_ARG, "null plan or output");
    *out = nullptr;
    if (plan->nchans < 1 || plan->ndump < 1 || plan->nrows < 1 || plan->nbeams < 1 ||
        !plan->frequencies || !plan->rows || plan->tsamp <= 0.)
        return fail(TXG_ERR_ARG, "plan needs nchans, ndump, nrows, nbeams >= 1, tsamp > 0");
    if (plan->precision < TXG_PREC_FP32 || plan->precision > TXG_PREC_FP16)
        return fail(TXG_ERR_ARG, "unknown precision");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1)
        return fail(TXG_ERR_NODEVICE, "no CUDA device");
    txg_handle *h = new txg_handle();
    if (cudaGetDevice(&h->device) != cudaSuccess) h->device = 0;
    h->plan = *plan;
    h->freqs.assign(plan->frequencies, plan->frequencies + plan->nchans);
    h->rows.assign(plan->rows, plan->rows + plan->nrows);
    h->plan.frequencies = h->freqs.data();
    h->plan.rows = h->rows.data();
    if (plan->zapthre > 0.f && (size_t)plan->nchans > skzap_max_channels()) {
        delete h;
        return fail(TXG_ERR_UNSUPPORTED, "the channel zap handles at most " +
                                             std::to_string(skzap_max_channels()) + " channels");
    }
    h->prec = plan->precision;
    h->flags = plan->flags;
    h->cap = plan->cand_capacity > 0 ? plan->cand_capacity : (1L << 20);
    h->hcap = std::min(h->cap, HCAP_MAX);
    int rc = TXG_OK;
    h->rp.resize(plan->nrows);
    h->row_ms.assign(plan->nrows, {});
    h->row_n.assign(plan->nrows, {});
    for (int r = 0; r < plan->nrows && !rc; r++) {
        std::string err;
        rc = plan_row(h->rows[r], plan->nchans, h->freqs.data(), plan->tsamp, plan->ndump, h->rp[r], err);
        if (rc) {
            fail(rc, "row " + std::to_string(r) + ": " + err);
            break;
        }
        rc = finish_plan(h->rp[r], r);
    }
    if (rc) {
        delete h;
        return rc;
    }
    if (cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking) != cudaSuccess) {
        delete h;
        return fail(TXG_ERR_CUDA, "cudaStreamCreate failed");
    }
    if (cudaStreamCreateWithFlags(&h->cst, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&h->dst, cudaStreamNonBlocking) != cudaSuccess) {
        if (h->cst) cudaStreamDestroy(h->cst);
        cudaStreamDestroy(h->st);
        delete h;
        return fail(TXG_ERR_CUDA, "cudaStreamCreate failed");
    }
    h->pool.reset(new Workers());
    {
        const unsigned hw = std::thread::hardware_concurrency();
        h->pool->start((int)std::max(1u, std::min(4u, hw / 2)));
    }
    auto bail = [&](int code) {
        free_all(h);
        delete h;
        return code;
    };
    const size_t raw_bytes = (size_t)plan->ndump * plan->nchans;
    for (int i = 0; i < 2; i++) {
        if ((rc = dalloc(h, &h->raw[i], raw_bytes))) return bail(rc);
        if (cudaHostAlloc((void **)&h->stage[i], raw_bytes, cudaHostAllocDefault) != cudaSuccess)
            return bail(fail(TXG_ERR_NOMEM, "pinned staging allocation failed"));
        if (cudaEventCreateWithFlags(&h->raw_free[i], cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&h->raw_loaded[i], cudaEventDisableTiming) != cudaSuccess)
            return bail(fail(TXG_ERR_CUDA, "event creation failed"));
    }
    h->rst.assign(plan->nrows, nullptr);
    h->row_done.assign(plan->nrows, nullptr);
    h->row_unpacked.assign(plan->nrows, nullptr);
    if (cudaEventCreateWithFlags(&h->fork, cudaEventDisableTiming) != cudaSuccess)
        return bail(fail(TXG_ERR_CUDA, "event creation failed"));
    for (int r = 0; r < plan->nrows; r++)
        if (cudaStreamCreateWithFlags(&h->rst[r], cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&h->row_done[r], cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&h->row_unpacked[r], cudaEventDisableTiming) != cudaSuccess)
            return bail(fail(TXG_ERR_CUDA, "row stream creation failed"));
    h->rd.resize(plan->nrows);
    for (int r = 0; r < plan->nrows; r++) {
        RowPlan &P = h->rp[r];
        RowDev &D = h->rd[r];
        if ((rc = upload(h, &D.sub_start, P.sub_start)) || (rc = upload(h, &D.d1, P.d1)) ||
            (rc = upload(h, &D.d2, P.d2)) || (rc = upload(h, &D.vwn, P.vwn)) ||
            (rc = upload(h, &D.zap, P.zap_chan)))
            return bail(rc);
    }
    h->br.resize(plan->nbeams);
    h->prep.resize(plan->nbeams);
    for (int beam = 0; beam < plan->nbeams; beam++) {
        BeamPrep &bp = h->prep[beam];
        if ((rc = dalloc(h, &bp.sums, (size_t)4 * plan->nchans)) ||
            (rc = dalloc(h, &bp.stats, (size_t)2 * plan->nchans)) ||
            (rc = dalloc(h, &bp.mask, (size_t)plan->nchans)))
            return bail(rc);
        h->br[beam].resize(plan->nrows);
        for (int r = 0; r < plan->nrows; r++) {
            RowPlan &P = h->rp[r];
            BeamRow &b = h->br[beam][r];
            for (int i = 0; i < (P.N >= P.H ? 1 : 2); i++)
                if ((rc = dalloc(h, &b.xh[i], (size_t)P.C * P.ldh))) return bail(rc);
            long kmax = 1;
            for (int q = 0; q < P.cfg.nrfi; q++) {
                const int kind = P.cfg.rfi_kind[q];
                if (kind != TXG_RFI_KADANEF && kind != TXG_RFI_KADANET && kind != TXG_RFI_MASK) continue;
                long nds = P.N / P.cfg.rfi_td[q], cds = P.C / P.cfg.rfi_fd[q];
                kmax = std::max(kmax, nds * cds);
                /* kadaneF: 4 per downsampled channel; kadaneT: 4 per downsampled sample;
                 * mask: the zapped-pixel count */
                const long nr = kind == TXG_RFI_KADANEF ? cds + 1 : kind == TXG_RFI_KADANET ? nds + 1 : 1;
                if ((rc = dalloc(h, &b.ranges[q], (size_t)4 * nr))) return bail(rc);
                if (kind == TXG_RFI_MASK && !b.sel && (rc = dalloc(h, &b.sel, (size_t)MASK_SEL_WORDS)))
                    return bail(rc);
            }
            if ((rc = dalloc(h, &b.ds, (size_t)kmax)) || (rc = dalloc(h, &b.z, (size_t)P.N)) ||
                (rc = dalloc(h, &b.live, (size_t)P.C)) ||
                (rc = dalloc(h, &b.b, (size_t)P.N)) || (rc = dalloc(h, &b.s, (size_t)P.N)) ||
                (rc = dalloc(h, &b.sst, (size_t)2)) ||
                (rc = dalloc(h, &b.eqpart, (size_t)2 * P.C * eq_part_tiles(P.N))) ||
                (rc = dalloc(h, &b.eqp, (size_t)P.C)) || (rc = dalloc(h, &b.zp, (size_t)P.C)))
                return bail(rc);
            unsigned char *ring = nullptr;
            if ((rc = dalloc(h, &ring, (size_t)P.ng * P.nsub * P.R * ring_elem(h->prec)))) return bail(rc);
            b.ring = ring;
            if ((rc = dalloc(h, &b.tim, (size_t)P.cfg.ndm * P.nout))) return bail(rc);
            if ((rc = dalloc(h, &b.bx_scratch, boxcar_scratch_doubles(P.cfg.ndm)))) return bail(rc);
            if (h->flags & TXG_FLAG_DENSE) {
                if ((rc = dalloc(h, &b.mxS, (size_t)P.cfg.ndm * P.nout)) ||
                    (rc = dalloc(h, &b.mxwn, (size_t)P.cfg.ndm * P.nout)))
                    return bail(rc);
            }
            for (auto &sl : b.slot) {
                if ((rc = dalloc(h, &sl.dcand, (size_t)h->cap)) || (rc = dalloc(h, &sl.dcount, (size_t)2)))
                    return bail(rc);
                for (int i = 0; i < 2; i++)
                    if (cudaHostAlloc((void **)&sl.hbuf[i], sizeof(txg_cand) * h->hcap, cudaHostAllocDefault) !=
                        cudaSuccess)
                        return bail(fail(TXG_ERR_NOMEM, "pinned candidate buffer allocation failed"));
                if (cudaHostAlloc((void **)&sl.hcount, 2 * sizeof(int), cudaHostAllocDefault) != cudaSuccess)
                    return bail(fail(TXG_ERR_NOMEM, "pinned count allocation failed"));
                sl.hcount[0] = sl.hcount[1] = 0;
                if (cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming) != cudaSuccess ||
                    cudaEventCreateWithFlags(&sl.boxed, cudaEventDisableTiming) != cudaSuccess)
                    return bail(fail(TXG_ERR_CUDA, "event creation failed"));
                if (h->flags & TXG_FLAG_TIMING)
                    for (auto &e : sl.ev)
                        if (cudaEventCreate(&e) != cudaSuccess)
                            return bail(fail(TXG_ERR_CUDA, "event creation failed"));
            }
        }
    }
    if (cudaStreamSynchronize(h->st) != cudaSuccess) return bail(fail(TXG_ERR_CUDA, "initialisation failed"));
    if (h->flags & TXG_FLAG_AUTOTUNE)
        for (int r = 0; r < plan->nrows; r++)
            if ((rc = autotune_row(h, r))) return bail(rc);
    *out = h;
    return TXG_OK;
}

void txg_destroy(txg_handle *h)
{
    DeviceScope device_scope(h);
    if (!h) return;
    free_all(h);
    delete h;
}

int txg_push_block_device(txg_handle *h, int32_t beam, const uint8_t *dev, int64_t nsamp)
{
    DeviceScope device_scope(h);
    if (!h || !dev) return fail(TXG_ERR_ARG, "null handle or buffer");
    if (beam < 0 || beam >= (int)h->br.size()) return fail(TXG_ERR_ARG, "beam out of range");
    if (nsamp != h->plan.ndump) return fail(TXG_ERR_ARG, "nsamp must equal the plan's ndump");
    return run_block(h, beam, dev);
}

int txg_push_block(txg_handle *h, int32_t beam, const uint8_t *host, int64_t nsamp)
{
    DeviceScope device_scope(h);
    if (!h || !host) return fail(TXG_ERR_ARG, "null handle or buffer");
    if (beam < 0 || beam >= (int)h->br.size()) return fail(TXG_ERR_ARG, "beam out of range");
    if (nsamp != h->plan.ndump) return fail(TXG_ERR_ARG, "nsamp must equal the plan's ndump");
    const size_t bytes = (size_t)nsamp * h->plan.nchans;
    const int i = h->raw_cur;
    h->raw_cur ^= 1;
    cudaPointerAttributes attr;
    const bool pinned = cudaPointerGetAttributes(&attr, host) == cudaSuccess &&
                        (attr.type == cudaMemoryTypeHost || attr.type == cudaMemoryTypeManaged);
    const uint8_t *src = host;
    if (!pinned) {
        /* the staging buffer's previous copy (two blocks ago) must be done */
        TXG_CUDA_TRY(cudaEventSynchronize(h->raw_loaded[i]));
        memcpy(h->stage[i], host, bytes);
        src = h->stage[i];
    }
    /* copy stream: wait until the kernels of two blocks ago are done with raw[i]; the kernel
     * stream waits for the copy, so the copy overlaps the previous block's kernels */
    TXG_CUDA_TRY(cudaStreamWaitEvent(h->cst, h->raw_free[i], 0));
    TXG_CUDA_TRY(cudaMemcpyAsync(h->raw[i], src, bytes, cudaMemcpyHostToDevice, h->cst));
    TXG_CUDA_TRY(cudaEventRecord(h->raw_loaded[i], h->cst));
    TXG_CUDA_TRY(cudaStreamWaitEvent(h->st, h->raw_loaded[i], 0));
    int rc = run_block(h, beam, h->raw[i]);
    TXG_CUDA_TRY(cudaEventRecord(h->raw_free[i], h->st));
    return rc;
}

int txg_push_block_f32(txg_handle *h, int32_t beam, const float *host, int64_t nsamp)
{
    DeviceScope device_scope(h);
    if (!h || !host) return fail(TXG_ERR_ARG, "null handle or buffer");
    if (beam < 0 || beam >= (int)h->br.size()) return fail(TXG_ERR_ARG, "beam out of range");
    if (nsamp != h->plan.ndump) return fail(TXG_ERR_ARG, "nsamp must equal the plan's ndump");
    const size_t count = (size_t)nsamp * h->plan.nchans;
    if (!h->rawf_ready) { /* the first float block: its buffers (a failed attempt is retried) */
        for (int k = 0; k < 2; k++) {
            if (!h->rawf[k]) {
                int rc = dalloc(h, &h->rawf[k], count);
                if (rc) return rc;
            }
            if (!h->stagef[k] && cudaHostAlloc((void **)&h->stagef[k], count * sizeof(float),
                                               cudaHostAllocDefault) != cudaSuccess) {
                h->stagef[k] = nullptr;
                return fail(TXG_ERR_NOMEM, "pinned staging allocation failed");
            }
            if ((!h->rawf_free[k] &&
                 cudaEventCreateWithFlags(&h->rawf_free[k], cudaEventDisableTiming) != cudaSuccess) ||
                (!h->rawf_loaded[k] &&
                 cudaEventCreateWithFlags(&h->rawf_loaded[k], cudaEventDisableTiming) != cudaSuccess))
                return fail(TXG_ERR_CUDA, "event creation failed");
        }
        h->rawf_ready = true;
    }
    const int i = h->rawf_cur;
    h->rawf_cur ^= 1;
    cudaPointerAttributes attr;
    const bool pinned = cudaPointerGetAttributes(&attr, host) == cudaSuccess &&
                        (attr.type == cudaMemoryTypeHost || attr.type == cudaMemoryTypeManaged);
    const float *src = host;
    if (!pinned) {
        TXG_CUDA_TRY(cudaEventSynchronize(h->rawf_loaded[i]));
        memcpy(h->stagef[i], host, count * sizeof(float));
        src = h->stagef[i];
    }
    TXG_CUDA_TRY(cudaStreamWaitEvent(h->cst, h->rawf_free[i], 0));
    TXG_CUDA_TRY(cudaMemcpyAsync(h->rawf[i], src, count * sizeof(float), cudaMemcpyHostToDevice, h->cst));
    TXG_CUDA_TRY(cudaEventRecord(h->rawf_loaded[i], h->cst));
    TXG_CUDA_TRY(cudaStreamWaitEvent(h->st, h->rawf_loaded[i], 0));
    int rc = run_block(h, beam, nullptr, h->rawf[i]);
    TXG_CUDA_TRY(cudaEventRecord(h->rawf_free[i], h->st));
    return rc;
}

int txg_sync(txg_handle *h)
{
    DeviceScope device_scope(h);
    if (!h) return fail(TXG_ERR_ARG, "null handle");
    if (int jr = join_rows(h)) return jr; /* results of the row streams */
    TXG_CUDA_TRY(cudaStreamSynchronize(h->st));
    int status = TXG_OK;
    for (auto &beam : h->br)
        for (size_t r = 0; r < beam.size(); r++) {
            BeamRow &b = beam[r];
            /* harvest in push order so `last` ends as the newest block */
            for (long k = b.nblocks - NSLOT; k < b.nblocks; k++) {
                if (k < 0) continue;
                int rc = harvest(h, b, b.slot[k % NSLOT], h->rp[r]);
                if (rc && (status == TXG_OK || status == TXG_ERR_OVERFLOW)) status = rc;
            }
        }
    h->pool->drain();
    return status;
}

int txg_reset_beam(txg_handle *h, int32_t beam)
{
    DeviceScope device_scope(h);
    if (!h) return fail(TXG_ERR_ARG, "null handle");
    if (beam < 0 || beam >= (int)h->br.size()) return fail(TXG_ERR_ARG, "beam out of range");
    const bool timing = h->flags & TXG_FLAG_TIMING;
    /* history columns and subband rings back to their state at txg_create (zeros), ordered on
     * each row's stream after the beam's queued blocks and before its next one; nothing waits
     * on the host.  The slots keep rotating, so blocks queued before the reset are harvested
     * and popped in push order as usual. */
    for (size_t r = 0; r < h->br[beam].size(); r++) {
        const RowPlan &P = h->rp[r];
        BeamRow &b = h->br[beam][r];
        const cudaStream_t rs = timing ? h->st : h->rst[r];
        for (int i = 0; i < 2; i++)
            if (b.xh[i]) TXG_CUDA_TRY(cudaMemsetAsync(b.xh[i], 0, sizeof(float) * P.C * P.ldh, rs));
        TXG_CUDA_TRY(cudaMemsetAsync(b.ring, 0, (size_t)P.ng * P.nsub * P.R * ring_elem(h->prec), rs));
        b.pushed = 0;
    }
    return TXG_OK;
}

int txg_get_row_info(txg_handle *h, int32_t beam, int32_t row, txg_row_info *out)
{
    int rc = check_beam_row(h, beam, row);
    if (rc) return rc;
    if (!out) return fail(TXG_ERR_ARG, "null output");
    const BeamRow &b = h->br[beam][row];
    fill_info(h->rp[row], out);
    out->counter = b.counter;
    out->gated = b.gated;
    return TXG_OK;
}

int txg_get_candidates(txg_handle *h, int32_t beam, int32_t row, txg_cand *out, int64_t cap, int64_t *n)
{
    DeviceScope device_scope(h);
    int rc = check_beam_row(h, beam, row);
    if (rc) return rc;
    const BeamRow &b = h->br[beam][row];
    if (n) *n = b.last_count;
    if (!b.last) return TXG_OK;
    h->pool->wait(*b.last);
    if (out && cap > 0) {
        long m = std::min<long>(cap, (long)b.last->cands.size());
        if (m > 0) memcpy(out, b.last->cands.data(), m * sizeof(txg_cand));
    }
    return result_status(h, *b.last);
}

int txg_pop_result(txg_handle *h, int32_t beam, int32_t row, txg_result *res, txg_cand *points,
                   int64_t pcap, txg_cand *clusters, int64_t ccap)
{
    DeviceScope device_scope(h);
    int rc = check_beam_row(h, beam, row);
    if (rc) return rc;
    BeamRow &b = h->br[beam][row];
    if (b.fifo.empty()) return fail(TXG_ERR_STATE, "no block result waiting");
    ResultP rp = b.fifo.front();
    b.fifo.pop_front();
    h->pool->wait(*rp);
    const Result &r = *rp;
    const bool over = r.count > h->cap;
    if (res) {
        res->counter = r.counter;
        res->gated = r.gated;
        res->overflow = over ? 1 : 0;
        res->npoints = r.count;
        res->nclusters = (int64_t)r.clusters.size();
    }
    if (points && pcap > 0) {
        const long m = std::min<long>(pcap, (long)r.cands.size());
        if (m > 0) memcpy(points, r.cands.data(), m * sizeof(txg_cand));
    }
    if (clusters && ccap > 0) {
        const long m = std::min<long>(ccap, (long)r.clusters.size());
        if (m > 0) memcpy(clusters, r.clusters.data(), m * sizeof(txg_cand));
    }
    return result_status(h, r);
}

int txg_result_ready(txg_handle *h, int32_t beam, int32_t row, int32_t *ready)
{
    int rc = check_beam_row(h, beam, row);
    if (rc) return rc;
    if (!ready) return fail(TXG_ERR_ARG, "null output");
    BeamRow &b = h->br[beam][row];
    *ready = 0;
    if (b.fifo.empty()) return fail(TXG_ERR_STATE, "no block result waiting");
    *ready = h->pool->is_ready(*b.fifo.front()) ? 1 : 0;
    return TXG_OK;
}

int txg_get_dense(txg_handle *h, int32_t beam, int32_t row, float *mxS, int32_t *mxwn)
{
    DeviceScope device_scope(h);
    int rc = check_beam_row(h, beam, row);
    if (rc) return rc;
    if (!(h->flags & TXG_FLAG_DENSE)) return fail(TXG_ERR_STATE, "plan was created without TXG_FLAG_DENSE");
    const RowPlan &P = h->rp[row];
    const BeamRow &b = h->br[beam][row];
    if (int jr = join_rows(h)) return jr; /* results of the row streams */
    TXG_CUDA_TRY(cudaStreamSynchronize(h->st));
    size_t cnt = (size_t)P.cfg.ndm * P.nout;
    if (mxS) TXG_CUDA_TRY(cudaMemcpy(mxS, b.mxS, cnt * sizeof(float), cudaMemcpyDeviceToHost));
    if (mxwn) TXG_CUDA_TRY(cudaMemcpy(mxwn, b.mxwn, cnt * sizeof(int32_t), cudaMemcpyDeviceToHost));
    return TXG_OK;
}

int txg_get_timdata(txg_handle *h, int32_t beam, int32_t row, int64_t idm0, int64_t count, float *out)
{
    DeviceScope device_scope(h);
    int rc = check_beam_row(h, beam, row);
    if (rc) return rc;
    const RowPlan &P = h->rp[row];
    if (!out || idm0 < 0 || count < 0 || idm0 + count > P.cfg.ndm) return fail(TXG_ERR_ARG, "DM range");
    if (int jr = join_rows(h)) return jr; /* results of the row streams */
    TXG_CUDA_TRY(cudaStreamSynchronize(h->st));
    TXG_CUDA_TRY(cudaMemcpy(out, h->br[beam][row].tim + idm0 * P.nout, count * P.nout * sizeof(float),
                            cudaMemcpyDeviceToHost));
    return TXG_OK;
}

/* Dedispersed series of DMs [idm0, idm0+count) of the last block, each standardised by its own
 * mean and standard deviation over the first nsamp samples (double, lane-strided), then
 * scaled to out = z*ostd + omean: nbits 32 -> float, 16/8 -> round-to-even, clamped to the
 * unsigned range. */
__global__ void k_tim_quant(const float *__restrict__ tim, long ldt, long nsamp, int nbits,
                            float omean, float ostd, void *__restrict__ out)
{
    const long k = blockIdx.x;
    const float *r = tim + k * ldt;
    __shared__ double red[2][32];
    double s1 = 0., s2 = 0.;
    for (long i = threadIdx.x; i < nsamp; i += blockDim.x) {
        const double v = r[i];
        s1 = __dadd_rn(s1, v);
        s2 = __dadd_rn(s2, __dmul_rn(v, v));
    }
    for (int off = 16; off >= 1; off >>= 1) {
        s1 = __dadd_rn(s1, __shfl_xor_sync(0xffffffffu, s1, off));
        s2 = __dadd_rn(s2, __shfl_xor_sync(0xffffffffu, s2, off));
    }
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    if (lane == 0) {
        red[0][w] = s1;
        red[1][w] = s2;
    }
    __syncthreads();
    double a = 0., b = 0.;
    for (int q = 0; q < nw; q++) {
        a = __dadd_rn(a, red[0][q]);
        b = __dadd_rn(b, red[1][q]);
    }
    const double mean = __ddiv_rn(a, (double)nsamp);
    const double var = __dsub_rn(__ddiv_rn(b, (double)nsamp), __dmul_rn(mean, mean));
    const double sd = var > 0. ? __dsqrt_rn(var) : 1.;
    for (long i = threadIdx.x; i < nsamp; i += blockDim.x) {
        const double z = __ddiv_rn(__dsub_rn((double)r[i], mean), sd);
        const float q = __double2float_rn(__dadd_rn(__dmul_rn(z, (double)ostd), (double)omean));
        if (nbits == 32) {
            reinterpret_cast<float *>(out)[k * nsamp + i] = q;
        } else {
            const float hi = nbits == 16 ? 65535.f : 255.f;
            const float c = fminf(fmaxf(rintf(q), 0.f), hi);
            if (nbits == 16) reinterpret_cast<uint16_t *>(out)[k * nsamp + i] = (uint16_t)c;
            else reinterpret_cast<uint8_t *>(out)[k * nsamp + i] = (uint8_t)c;
        }
    }
}

int txg_get_timdata_q(txg_handle *h, int32_t beam, int32_t row, int64_t idm0, int64_t count,
                      int64_t nsamp, int32_t nbits, float mean, float std, void *out)
{
    DeviceScope device_scope(h);
    int rc = check_beam_row(h, beam, row);
    if (rc) return rc;
    const RowPlan &P = h->rp[row];
    if (!out || idm0 < 0 || count < 1 || idm0 + count > P.cfg.ndm) return fail(TXG_ERR_ARG, "DM range");
    if (nsamp < 1 || nsamp > P.nout) return fail(TXG_ERR_ARG, "nsamp must be 1..nsamples");
    if (nbits != 8 && nbits != 16 && nbits != 32) return fail(TXG_ERR_ARG, "nbits must be 8, 16 or 32");
    const size_t bytes = (size_t)count * nsamp * (nbits / 8);
    if (int jr = join_rows(h)) return jr; /* results of the row streams */
    void *d = nullptr;
    TXG_CUDA_TRY(cudaStreamSynchronize(h->st));
    TXG_CUDA_TRY(cudaMalloc(&d, bytes));
    k_tim_quant<<<(unsigned)count, 256, 0, h->st>>>(h->br[beam][row].tim + idm0 * P.nout, P.nout, nsamp,
                                                    nbits, mean, std, d);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
    if (e == cudaSuccess) e = cudaMemcpy(out, d, bytes, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return set_cuda_error(e, "txg_get_timdata_q", __FILE__, __LINE__);
    return TXG_OK;
}

int txg_get_block(txg_handle *h, int32_t beam, int32_t row, float *out)
{
    DeviceScope device_scope(h);
    int rc = check_beam_row(h, beam, row);
    if (rc) return rc;
    if (!out) return fail(TXG_ERR_ARG, "null output");
    const RowPlan &P = h->rp[row];
    const BeamRow &b = h->br[beam][row];
    if (b.nblocks == 0) return fail(TXG_ERR_STATE, "no block pushed");
    if (int jr = join_rows(h)) return jr; /* results of the row streams */
    TXG_CUDA_TRY(cudaStreamSynchronize(h->st));
    const float *x = (b.xh[1] ? b.xh[b.cur ^ 1] : b.xh[0]) + P.H; /* buffer of the newest block */
    TXG_CUDA_TRY(cudaMemcpy2D(out, P.N * sizeof(float), x, P.ldh * sizeof(float), P.N * sizeof(float), P.C,
                              cudaMemcpyDeviceToHost));
    return TXG_OK;
}

int txg_get_zap_ranges(txg_handle *h, int32_t beam, int32_t row, int32_t irfi, int32_t *out, int64_t cap)
{
    DeviceScope device_scope(h);
    int rc = check_beam_row(h, beam, row);
    if (rc) return rc;
    const RowPlan &P = h->rp[row];
    if (irfi < 0 || irfi >= P.cfg.nrfi)
        return fail(TXG_ERR_ARG, "rfilist entry out of range");
    const int kind = P.cfg.rfi_kind[irfi];
    if (kind != TXG_RFI_KADANEF && kind != TXG_RFI_KADANET && kind != TXG_RFI_MASK)
        return fail(TXG_ERR_ARG, "rfilist entry is not a kadaneF, kadaneT or mask");
    if (int jr = join_rows(h)) return jr; /* results of the row streams */
    if (kind == TXG_RFI_MASK) {
        if (!out || cap < 4) return fail(TXG_ERR_ARG, "output too small");
        TXG_CUDA_TRY(cudaStreamSynchronize(h->st));
        TXG_CUDA_TRY(cudaMemcpy(out, h->br[beam][row].ranges[irfi], sizeof(int32_t), cudaMemcpyDeviceToHost));
        out[1] = out[2] = out[3] = 0;
        return TXG_OK;
    }
    const long rows = kind == TXG_RFI_KADANEF ? P.C / P.cfg.rfi_fd[irfi] : P.N / P.cfg.rfi_td[irfi];
    if (!out || cap < 4 * rows) return fail(TXG_ERR_ARG, "output too small");
    TXG_CUDA_TRY(cudaStreamSynchronize(h->st));
    TXG_CUDA_TRY(cudaMemcpy(out, h->br[beam][row].ranges[irfi], 4 * rows * sizeof(int32_t),
                            cudaMemcpyDeviceToHost));
    return TXG_OK;
}

/* The subband ring holds the last block's output window only while that block is the row's
 * newest: every pushed block harvested (txg_sync) and the block gated. */
static int last_block_window(txg_handle *h, int32_t beam, int32_t row, long *t0_mod)
{
    int rc = check_beam_row(h, beam, row);
    if (rc) return rc;
    const RowPlan &P = h->rp[row];
    const BeamRow &b = h->br[beam][row];
    for (const Slot &sl : b.slot)
        if (sl.pending) return fail(TXG_ERR_STATE, "call txg_sync first");
    if (!b.gated) return fail(TXG_ERR_STATE, "the row's last block produced no output");
    *t0_mod = pmod(b.counter - P.N - P.offset, P.R);
    return TXG_OK;
}

int txg_get_subdata(txg_handle *h, int32_t beam, int32_t row, int64_t idm, float *out)
{
    DeviceScope device_scope(h);
    long t0_mod = 0;
    int rc = last_block_window(h, beam, row, &t0_mod);
    if (rc) return rc;
    const RowPlan &P = h->rp[row];
    if (!out || idm < 0 || idm >= P.cfg.ndm) return fail(TXG_ERR_ARG, "DM index or output");
    if (int jr = join_rows(h)) return jr; /* results of the row streams */
    const size_t cnt = (size_t)P.nsub * P.nout;
    float *d = nullptr;
    TXG_CUDA_TRY(cudaMalloc(&d, cnt * sizeof(float)));
    launch_subdata(h->br[beam][row].ring, P.R, P.nsub, P.G, h->rd[row].d2, idm, t0_mod, P.nout,
                   h->prec, d, h->st);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
    if (e == cudaSuccess) e = cudaMemcpy(out, d, cnt * sizeof(float), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return set_cuda_error(e, "txg_get_subdata", __FILE__, __LINE__);
    return TXG_OK;
}

int txg_cand_band(txg_handle *h, int32_t beam, int32_t row, const txg_cand *c, int64_t n,
                  float *fl, float *fh)
{
    DeviceScope device_scope(h);
    long t0_mod = 0;
    int rc = last_block_window(h, beam, row, &t0_mod);
    if (rc) return rc;
    if (n <= 0) return TXG_OK;
    if (!c || !fl || !fh) return fail(TXG_ERR_ARG, "null argument");
    const RowPlan &P = h->rp[row];
    for (long k = 0; k < n; k++)
        if (c[k].idm < 0 || c[k].idm >= P.cfg.ndm || c[k].wn < 1)
            return fail(TXG_ERR_ARG, "candidate outside the row");
    if (int jr = join_rows(h)) return jr; /* results of the row streams */
    std::vector<float> vpf((size_t)n * P.nsub);
    txg_cand *dc = nullptr;
    float *dv = nullptr;
    cudaError_t e = cudaMalloc(&dc, n * sizeof(txg_cand));
    if (e == cudaSuccess) e = cudaMalloc(&dv, vpf.size() * sizeof(float));
    if (e == cudaSuccess) e = cudaMemcpyAsync(dc, c, n * sizeof(txg_cand), cudaMemcpyHostToDevice, h->st);
    if (e == cudaSuccess) {
        launch_cand_vpf(h->br[beam][row].ring, P.R, P.nsub, P.G, h->rd[row].d2, h->rd[row].sub_start,
                        t0_mod, P.nout, dc, n, h->prec, dv, h->st);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
    if (e == cudaSuccess) e = cudaMemcpy(vpf.data(), dv, vpf.size() * sizeof(float), cudaMemcpyDeviceToHost);
    cudaFree(dc);
    cudaFree(dv);
    if (e != cudaSuccess) return set_cuda_error(e, "txg_cand_band", __FILE__, __LINE__);
    /* the maximum-sum run of subbands (strictly larger sum wins, restart below zero) and its
     * ends on the linear frequency axis of candplot.cpp:151 */
    const double den = P.nsub > 1 ? P.nsub - 1. : 1.;
    const double f0 = P.fsub.front(), f1 = P.fsub.back();
    for (long k = 0; k < n; k++) {
        const float *v = vpf.data() + (size_t)k * P.nsub;
        float best = -INFINITY, cur = 0.f;
        long cs = 0, fs = 0, fe = 0;
        for (long j = 0; j < P.nsub; j++) {
            cur = cur + v[j];
            if (cur > best) {
                best = cur;
                fs = cs;
                fe = j;
            }
            if (cur < 0.f) {
                cur = 0.f;
                cs = j + 1;
            }
        }
        fl[k] = (float)(f0 + fs / den * (f1 - f0));
        fh[k] = (float)(f0 + fe / den * (f1 - f0));
    }
    return TXG_OK;
}

int txg_get_mask(txg_handle *h, int32_t beam, uint8_t *mask)
{
    DeviceScope device_scope(h);
    if (!h || !mask) return fail(TXG_ERR_ARG, "null argument");
    if (beam < 0 || beam >= (int)h->prep.size()) return fail(TXG_ERR_ARG, "beam out of range");
    if (int jr = join_rows(h)) return jr; /* results of the row streams */
    TXG_CUDA_TRY(cudaStreamSynchronize(h->st));
    TXG_CUDA_TRY(cudaMemcpy(mask, h->prep[beam].mask, h->plan.nchans, cudaMemcpyDeviceToHost));
    return TXG_OK;
}

int txg_get_tables(txg_handle *h, int32_t row, int32_t *d1, int32_t *d2, int32_t *sub_start, int32_t *vwn)
{
    DeviceScope device_scope(h);
    if (!h || row < 0 || row >= (int)h->rp.size()) return fail(TXG_ERR_ARG, "row out of range");
    copy_tables(h->rp[row], d1, d2, sub_start, vwn);
    return TXG_OK;
}

int txg_describe_row(const txg_plan *plan, int32_t row, txg_row_info *info, int32_t *d1, int32_t *d2,
                     int32_t *sub_start, int32_t *vwn)
{
    if (!plan || !plan->rows || !plan->frequencies || row < 0 || row >= plan->nrows)
        return fail(TXG_ERR_ARG, "bad plan or row");
    RowPlan P;
    std::string err;
    int rc = plan_row(plan->rows[row], plan->nchans, plan->frequencies, plan->tsamp, plan->ndump, P, err);
    if (rc) return fail(rc, err);
    if ((rc = finish_plan(P, row))) return rc;
    if (info) fill_info(P, info);
    copy_tables(P, d1, d2, sub_start, vwn);
    return TXG_OK;
}

int txg_get_row_timing(txg_handle *h, int32_t row, double *ms, int64_t *launches, int32_t n)
{
    DeviceScope device_scope(h);
    if (!h) return fail(TXG_ERR_ARG, "null handle");
    if (row < 0 || row >= (int)h->rp.size()) return fail(TXG_ERR_ARG, "row out of range");
    for (int c = 0; c < NCLASS && c < n; c++) {
        if (ms) ms[c] = h->row_ms[row][c];
        if (launches) launches[c] = h->row_n[row][c];
        h->row_ms[row][c] = 0.;
        h->row_n[row][c] = 0;
    }
    return NCLASS;
}

int txg_get_launch_shape(txg_handle *h, int32_t row, int32_t *stage1, int32_t *stage2,
                         int32_t *stage2_kb)
{
    if (!h) return fail(TXG_ERR_ARG, "null handle");
    if (row < 0 || row >= (int)h->rp.size()) return fail(TXG_ERR_ARG, "row out of range");
    const RowPlan &P = h->rp[row];
    if (stage1) *stage1 = P.s1_var;
    if (stage2) *stage2 = P.s2_var;
    if (stage2_kb) *stage2_kb = P.s2_kb;
    return TXG_OK;
}

int txg_get_timing(txg_handle *h, double *ms, int64_t *launches, int32_t n)
{
    DeviceScope device_scope(h);
    if (!h) return fail(TXG_ERR_ARG, "null handle");
    for (int c = 0; c < NCLASS && c < n; c++) {
        if (ms) ms[c] = h->class_ms[c];
        if (launches) launches[c] = h->class_n[c];
        h->class_ms[c] = 0.;
        h->class_n[c] = 0;
    }
    return NCLASS;
}

int txg_get_stream(txg_handle *h, void **stream)
{
    if (!h || !stream) return fail(TXG_ERR_ARG, "null argument");
    *stream = (void *)h->st;
    return TXG_OK;
}

int txg_boxcar(const float *tim, int64_t ndm, int64_t nsamples, const int32_t *vwn, int32_t nw,
               int32_t iqr, int32_t flags, float thre, float *mxS, int32_t *mxwn, txg_cand *cands,
               int64_t cap, int64_t *ncand)
{
    if (!tim || !vwn || ndm < 1 || nsamples < 1 || nw < 1 || nw > 256)
        return fail(TXG_ERR_ARG, "need tim, vwn, ndm >= 1, nsamples >= 1, 1 <= nw <= 256");
    int maxwn = 0;
    for (int w = 0; w < nw; w++) maxwn = std::max(maxwn, (int)vwn[w]);
    if (!boxcar_supported(nsamples, maxwn, nw))
        return fail(TXG_ERR_UNSUPPORTED, "nsamples or the widest boxcar exceeds the boxcar kernels' limits");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return fail(TXG_ERR_NODEVICE, "no CUDA device");
    cudaStream_t st;
    TXG_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    float *dtim = nullptr, *dS = nullptr;
    int32_t *dwn = nullptr, *dvwn = nullptr;
    txg_cand *dc = nullptr;
    int *dcount = nullptr;
    double *dscr = nullptr;
    const size_t cnt = (size_t)ndm * nsamples;
    const long ccap = cands ? (cap > 0 ? cap : 0) : 0;
    int rc = TXG_OK;
    auto cleanup = [&]() {
        cudaStreamSynchronize(st);
        cudaFree(dtim);
        cudaFree(dS);
        cudaFree(dwn);
        cudaFree(dvwn);
        cudaFree(dc);
        cudaFree(dcount);
        cudaFree(dscr);
        cudaStreamDestroy(st);
    };
    do {
        cudaError_t e;
        if ((e = cudaMalloc(&dtim, cnt * sizeof(float))) != cudaSuccess ||
            (e = cudaMalloc(&dvwn, nw * sizeof(int32_t))) != cudaSuccess ||
            (e = cudaMalloc(&dcount, 2 * sizeof(int))) != cudaSuccess ||
            (e = cudaMalloc(&dscr, boxcar_scratch_doubles(ndm) * sizeof(double))) != cudaSuccess ||
            (e = cudaMalloc(&dc, (ccap > 0 ? ccap : 1) * sizeof(txg_cand))) != cudaSuccess ||
            (mxS && (e = cudaMalloc(&dS, cnt * sizeof(float))) != cudaSuccess) ||
            (mxS && (e = cudaMalloc(&dwn, cnt * sizeof(int32_t))) != cudaSuccess)) {
            rc = set_cuda_error(e, "cudaMalloc", __FILE__, __LINE__);
            break;
        }
        if ((e = cudaMemcpyAsync(dtim, tim, cnt * sizeof(float), cudaMemcpyHostToDevice, st)) != cudaSuccess ||
            (e = cudaMemcpyAsync(dvwn, vwn, nw * sizeof(int32_t), cudaMemcpyHostToDevice, st)) != cudaSuccess ||
            (e = cudaMemsetAsync(dcount, 0, 2 * sizeof(int), st)) != cudaSuccess) {
            rc = set_cuda_error(e, "copy-in", __FILE__, __LINE__);
            break;
        }
        rc = launch_boxcar(dtim, nsamples, ndm, nsamples, dvwn, nw, maxwn, iqr,
                           (flags & TXG_FLAG_AVX2_TAIL) ? 1 : 0, thre, dc, dcount, ccap, dS, dwn,
                           dscr, dcount + 1, st);
        if (rc) break;
        if ((e = cudaGetLastError()) != cudaSuccess) {
            rc = set_cuda_error(e, "boxcar launch", __FILE__, __LINE__);
            break;
        }
        int hc[2] = {0, 0};
        if ((e = cudaMemcpyAsync(hc, dcount, 2 * sizeof(int), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
            (e = cudaStreamSynchronize(st)) != cudaSuccess) {
            rc = set_cuda_error(e, "boxcar", __FILE__, __LINE__);
            break;
        }
        if (mxS) {
            if ((e = cudaMemcpy(mxS, dS, cnt * sizeof(float), cudaMemcpyDeviceToHost)) != cudaSuccess ||
                (mxwn && (e = cudaMemcpy(mxwn, dwn, cnt * sizeof(int32_t), cudaMemcpyDeviceToHost)) != cudaSuccess)) {
                rc = set_cuda_error(e, "copy-out", __FILE__, __LINE__);
                break;
            }
        }
        if (ncand) *ncand = hc[0];
        if (cands && ccap > 0) {
            long keep = std::min<long>(hc[0], ccap);
            if (keep > 0 &&
                (e = cudaMemcpy(cands, dc, keep * sizeof(txg_cand), cudaMemcpyDeviceToHost)) != cudaSuccess) {
                rc = set_cuda_error(e, "copy-out", __FILE__, __LINE__);
                break;
            }
            std::sort(cands, cands + keep, [](const txg_cand &x, const txg_cand &y) {
                return x.idm != y.idm ? x.idm < y.idm : x.isamp < y.isamp;
            });
            if (hc[0] > ccap) rc = fail(TXG_ERR_OVERFLOW, "candidate buffer overflow");
        }
    } while (0);
    cleanup();
    return rc;
}

int txg_cluster(const txg_cand *cands, int64_t n, double dms, double ddm, double fmax, double fmin,
                double tsamp, double radius_smearing, int32_t maxncand, int32_t minpts, int32_t drop,
                int32_t maxwn, txg_cand *out, int64_t cap, int64_t *nout)
{
    if ((n > 0 && !cands) || n < 0 || tsamp <= 0.) return fail(TXG_ERR_ARG, "bad arguments");
    long m = cluster_run(cands, n, dms, ddm, fmax, fmin, tsamp, radius_smearing, maxncand, minpts, drop,
                         maxwn, out, out ? cap : 0);
    if (nout) *nout = m;
    return (out && m > cap) ? fail(TXG_ERR_OVERFLOW, "output too small") : TXG_OK;
}

} /* extern "C" */
