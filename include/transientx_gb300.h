/*
 * transientx_gb300.h -- C ABI of the GB300 (sm_103a) implementation of TransientX's per-block
 * single-pulse search: unpack -> downsample -> equalize -> baseline -> RFI (zap, kadaneF,
 * zdot) -> two-stage subband dedispersion -> boxcar matched filter -> S/N threshold.
 *
 * Plain C types only; every function returns a txg_status (0 = success, < 0 = error) unless
 * noted.  One handle owns its device memory and CUDA streams; calls on one handle must be
 * serialised by the caller, different handles are independent.  A handle lives on the CUDA
 * device current at txg_create; each call on it makes that device current for the call and
 * restores the caller's.  No exceptions cross this boundary.  Paths below are relative to
 * the TransientX source tree.
 */
#ifndef TRANSIENTX_GB300_H
#define TRANSIENTX_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TXG_ABI_VERSION 1

typedef enum {
    TXG_OK = 0,
    TXG_ERR_ARG = -1,          /* invalid argument or plan */
    TXG_ERR_NOMEM = -2,        /* device or pinned-host allocation failed */
    TXG_ERR_CUDA = -3,         /* CUDA runtime error (context still usable) */
    TXG_ERR_OVERFLOW = -4,     /* candidate buffer overflowed; raise cand_capacity */
    TXG_ERR_TIMEOUT = -5,      /* a bounded device wait gave up */
    TXG_ERR_STATE = -6,        /* call not valid in the handle's current state */
    TXG_ERR_NODEVICE = -7,     /* no CUDA device / extension unusable */
    TXG_ERR_UNSUPPORTED = -8   /* option not implemented for these sizes */
} txg_status;

/* rfilist entries (singlepulse.cpp:298-325): kadaneF td fd, zdot, mask td fd, kadaneT td fd,
 * zero */
typedef enum {
    TXG_RFI_KADANEF = 1,
    TXG_RFI_ZDOT = 2,
    TXG_RFI_MASK = 3,
    TXG_RFI_KADANET = 4,
    TXG_RFI_ZERO = 5
} txg_rfi_kind;

typedef enum {
    TXG_PREC_FP32 = 0,         /* subband series and prefix sums in FP32 (reference arithmetic) */
    TXG_PREC_BF16 = 1,         /* subband series stored as BF16, FP32 accumulation */
    TXG_PREC_FP16 = 2          /* subband series stored as FP16, FP32 accumulation */
} txg_precision;

typedef enum {
    TXG_FLAG_AVX2_TAIL = 1,    /* reproduce the -mavx2 build's per-width range of boxcar.cpp:264-279 */
    TXG_FLAG_DENSE = 2,        /* keep dense mxS/mxwn (Boxcar::mxS/mxwn, include/boxcar.h:40-41) */
    TXG_FLAG_KEEP_SERIES = 4,  /* keep preprocessed block and dedispersed series for inspection */
    TXG_FLAG_TIMING = 8,       /* bracket each kernel class with CUDA events (txg_get_timing) */
    TXG_FLAG_CLUSTER = 16,     /* run Cluster::run on every gated block while harvesting it */
    TXG_FLAG_AUTOTUNE = 32     /* time the dedispersion launch shapes at txg_create and keep
                                * the fastest per row (txg_get_launch_shape) */
} txg_flags;

/* One ddplan row: the fields of SinglePulse that SinglePulse::prepare/run read
 * (include/singlepulse.h:95-133, src/singlepulse/singlepulse.cpp:206-341). */
typedef struct {
    int32_t td, fd;            /* Downsample (singlepulse.cpp:208-209) */
    float bswidth;             /* BaseLine width in s, <= 0 disables (singlepulse.cpp:218) */
    int32_t nrfi;              /* rfilist entries, run in order (singlepulse.cpp:298-325) */
    int32_t rfi_kind[8];       /* txg_rfi_kind */
    int32_t rfi_td[8], rfi_fd[8];
    int32_t nzap;              /* zaplist (singlepulse.cpp:295) */
    double zap[16][2];         /* [fl, fh] in MHz */
    float threKadaneF;         /* S/N threshold of kadaneF (squared before use, :307) */
    double widthlimit;         /* kadaneF minimum window in s (:307) */
    double dms, ddm;           /* SubbandDedispersion dms/ddm/ndm/overlap (:230-233) */
    int64_t ndm;
    double overlap;
    float minw, maxw, snrloss; /* boxcar width ladder (singlepulse.cpp:242-254) */
    int32_t iqr;               /* Boxcar::run iqr argument (boxcar.cpp:204-227) */
    float thre;                /* S/N threshold (cluster.cpp:95) */
    int32_t nsub;              /* subbands; 0 = automatic */
    int32_t dm_group;          /* fine DMs per coarse DM; 0 = automatic */
    double radius_smearing;    /* Cluster::run arguments (singlepulse.cpp:332): radius in s */
    int32_t maxncand, minpts;
    int32_t drop;              /* remove_cand_with_maxwidth */
    float threMask;            /* mask outlier threshold in IQR units (singlepulse.cpp:302) */
    float threKadaneT;         /* S/N threshold of kadaneT (squared before use, :312) */
    int32_t pad;
    double bandlimitKT;        /* kadaneT minimum band in MHz (:312) */
} txg_row;

typedef struct {
    int32_t nchans;            /* raw channels */
    double tsamp;              /* raw sampling time (s) */
    const double *frequencies; /* nchans channel centre frequencies (MHz) */
    int64_t ndump;             /* raw samples per block (dedisperse_fil.cpp:244) */
    int32_t nrows;
    const txg_row *rows;
    int32_t nbeams;            /* independent beams sharing the plan */
    int32_t precision;         /* txg_precision */
    int32_t flags;             /* txg_flags */
    int64_t cand_capacity;     /* candidates kept per (beam,row,block); 0 = default */
    float zapthre;             /* skewness/kurtosis channel zap of each raw block, IQR units
                                * (PreprocessLite, dedisperse_fil.cpp:264-276,329); <= 0 off */
} txg_plan;

/* One point above threshold, in the order Cluster::run scans mxS (cluster.cpp:91-112). */
typedef struct {
    int32_t idm;
    int32_t isamp;
    int32_t wn;
    float S;
} txg_cand;

/* Geometry of one row: the public members of SubbandDedispersion and Boxcar that the
 * reference reads (boxcar.cpp:142-161, cluster.cpp:65-117, candplot.cpp:47). */
typedef struct {
    int32_t nchans, nsub, dm_group, ngroup, nwidths, maxwn;
    int64_t ndm, ndump, noverlap, offset, nsamples, counter, maxd1, maxd2;
    double tsamp, dms, ddm, fmin, fmax;
    int32_t gated;             /* 1 if the last block produced boxcar output */
    int32_t pad;
} txg_row_info;

typedef struct txg_handle txg_handle;

/* Plan all ddplan rows and allocate device state: SinglePulse::prepare for every row
 * (singlepulse.cpp:206-254) plus Boxcar::prepare (boxcar.cpp:142-156). */
int txg_create(const txg_plan *plan, txg_handle **out);
void txg_destroy(txg_handle *h);

/* Feed one block of raw uint8 time-major samples [nsamp][nchans] for one beam and run every
 * ddplan row on it: the body of the transientx_fil block loop (dedisperse_fil.cpp:324-337)
 * calling SinglePulse::run (singlepulse.cpp:287-341).  nsamp must equal the plan's ndump.
 * The call returns once the block is queued.  A pageable host buffer is first copied into a
 * pinned staging buffer and may be reused on return; a page-locked host buffer is copied to
 * the device asynchronously and must stay unchanged until the next txg_sync. */
int txg_push_block(txg_handle *h, int32_t beam, const uint8_t *host, int64_t nsamp);
int txg_push_block_device(txg_handle *h, int32_t beam, const uint8_t *dev, int64_t nsamp);

/* The same for a float block [nsamp][nchans] (time-major) that the caller has already
 * unpacked and preprocessed, the DataBuffer<float> that SinglePulse::run receives
 * (singlepulse.cpp:287, after PreprocessLite::run, dedisperse_fil.cpp:329): each row's
 * td x fd downsample sums the floats in the 8-bit path's order, and equalize takes its mean
 * and variance from FP64 sums in a fixed order instead of exact integer sums; the plan's
 * channel zap (zapthre) does not apply to float blocks (PreprocessLite has done it).  The
 * first call allocates the handle's float staging buffers; buffer rules as txg_push_block. */
int txg_push_block_f32(txg_handle *h, int32_t beam, const float *host, int64_t nsamp);

/* Start a new observation on a beam: the next block pushed to it is the first block of a new
 * file, its history, sample counter and subband rings as at txg_create.  Blocks queued
 * before the call are searched as part of the previous observation and their results are
 * popped in push order as usual (txg_pop_result; row info and the inspection calls describe
 * the newest harvested block).  Nothing waits on the host: the beam's buffers are cleared on
 * the device after its queued blocks.  The reference prepares a fresh SinglePulse for every
 * observation it searches (dedisperse_fil.cpp:292-311, SinglePulse::prepare,
 * singlepulse.cpp:206-254); a handle reused for file after file calls this instead of
 * txg_destroy + txg_create.  Cost: one device memset of the beam's rings. */
int txg_reset_beam(txg_handle *h, int32_t beam);

/* Wait for queued work and collect candidates; returns TXG_ERR_OVERFLOW if any buffer
 * overflowed since the last call. */
int txg_sync(txg_handle *h);

int txg_get_row_info(txg_handle *h, int32_t beam, int32_t row, txg_row_info *out);

/* Points with S > thre of the last block of (beam,row), sorted by (idm, isamp): the input
 * Cluster::run builds from mxS (cluster.cpp:84-112).  *n receives the full count. */
int txg_get_candidates(txg_handle *h, int32_t beam, int32_t row, txg_cand *out, int64_t cap,
                       int64_t *n);

/* Outcome of one block of one (beam,row). */
typedef struct {
    int64_t counter;           /* the row's sample counter after the block (boxcar.cpp:160) */
    int32_t gated;             /* the block produced boxcar output */
    int32_t overflow;          /* more points than cand_capacity (points list truncated) */
    int64_t npoints;           /* S > thre points (Cluster::run input, cluster.cpp:91-112) */
    int64_t nclusters;         /* reported candidates (Cluster::run candlist), with
                                * TXG_FLAG_CLUSTER */
} txg_result;

/* Per-block results in push order: pops the oldest harvested block of (beam,row) not yet
 * popped (up to 256 are kept; older ones are dropped).  Points are sorted as in
 * txg_get_candidates and written up to pcap; clusters in Cluster::run's order up to ccap.
 * Returns TXG_ERR_STATE when no block is waiting. */
int txg_pop_result(txg_handle *h, int32_t beam, int32_t row, txg_result *res, txg_cand *points,
                   int64_t pcap, txg_cand *clusters, int64_t ccap);

/* Whether txg_pop_result would return at once: *ready = 1 when the oldest waiting block of
 * (beam,row) has its points sorted and clustered, 0 while a worker thread is still on it.
 * Returns TXG_ERR_STATE when no block is waiting.  No reference counterpart: a streaming
 * caller polls with it so that the thread pushing blocks never waits on host clustering. */
int txg_result_ready(txg_handle *h, int32_t beam, int32_t row, int32_t *ready);

/* Dense Boxcar::mxS / mxwn of the last block (plan flag TXG_FLAG_DENSE): [ndm][nsamples]. */
int txg_get_dense(txg_handle *h, int32_t beam, int32_t row, float *mxS, int32_t *mxwn);

/* SubbandDedispersion::get_timdata(tim, idm, true) for idm0..idm0+count-1 of the last block
 * (boxcar.cpp:183; plan flag TXG_FLAG_KEEP_SERIES): [count][nsamples]. */
int txg_get_timdata(txg_handle *h, int32_t beam, int32_t row, int64_t idm0, int64_t count,
                    float *out);

/* The dedispersed series of DMs idm0..idm0+count-1 of the last block quantised for dumping
 * (the --savetim/--mean/--std/--nbits output of SubbandDedispersion::rundump,
 * singlepulse.cpp:237-238,339-340, dedisperse_fil.cpp:95-99): each series standardised by its
 * own mean and standard deviation over its first nsamp samples, then z*std + mean as float
 * (nbits 32) or rounded to even and clamped to 0..255 / 0..65535 (nbits 8 / 16).  out:
 * [count][nsamp] of that type.  Pass nsamp = ndump to dump consecutive blocks without the
 * overlap. */
int txg_get_timdata_q(txg_handle *h, int32_t beam, int32_t row, int64_t idm0, int64_t count,
                      int64_t nsamp, int32_t nbits, float mean, float std, void *out);

/* The row's preprocessed block after the rfilist ([nchans][ndump], TXG_FLAG_KEEP_SERIES),
 * and the zapped windows of rfilist entry irfi: kadaneF [nchans/fd][4] (start,end of the
 * positive and negative window in block samples, -1 if not zapped); kadaneT [ndump/td][4]
 * (start,end of the positive and negative band in channels per downsampled sample); mask
 * [1][4] (number of zapped pixels, 0, 0, 0). */
int txg_get_block(txg_handle *h, int32_t beam, int32_t row, float *out);
int txg_get_zap_ranges(txg_handle *h, int32_t beam, int32_t row, int32_t irfi, int32_t *out,
                       int64_t cap);

/* SubbandDedispersion::get_subdata(sub, idm, true) (candplot.cpp:123) of the row's last
 * block: the nsub subband series of fine DM idm aligned at that DM, [nsub][nsamples], each the
 * sum of its subband's channels (txg_get_tables' sub_start gives the counts).  Valid after
 * txg_sync when that block was gated; TXG_ERR_STATE otherwise. */
int txg_get_subdata(txg_handle *h, int32_t beam, int32_t row, int64_t idm, float *out);

/* The frequency band of each candidate, the fl and fh columns of the .cands line
 * (candplot.cpp:143-231,423-433): per subband the sum over samples (isamp-wn, isamp+wn) of its
 * channel mean, the maximum-sum run of subbands, and fl/fh = the run's ends on the linear
 * axis from the first to the last subband's mean frequency.  Same validity as
 * txg_get_subdata. */
int txg_cand_band(txg_handle *h, int32_t beam, int32_t row, const txg_cand *c, int64_t n,
                  float *fl, float *fh);

/* Channels zapped by the skewness/kurtosis filter in the last block of a beam: mask[c] = 1
 * (nchans raw channels). */
int txg_get_mask(txg_handle *h, int32_t beam, uint8_t *mask);

/* Integer tables of a row: within-subband delays d1 [ngroup][nchans], subband delays
 * d2 [ndm][nsub], first channel of each subband [nsub+1], width ladder [nwidths]. */
int txg_get_tables(txg_handle *h, int32_t row, int32_t *d1, int32_t *d2, int32_t *sub_start,
                   int32_t *vwn);

/* Plan one row without a device (host only): fills info (counter 0) and, when non-NULL, the
 * tables of txg_get_tables.  Lets a caller size buffers before txg_create. */
int txg_describe_row(const txg_plan *plan, int32_t row, txg_row_info *info, int32_t *d1,
                     int32_t *d2, int32_t *sub_start, int32_t *vwn);

/* Self-test of the failure path of every kernel that waits for its shared-memory copies: one
 * CTA waits, with the same bounded wait, for a 256-byte bulk copy.  never_complete = 0: the copy
 * completes (TXG_OK).  never_complete != 0: its barrier expects more bytes than the copy brings,
 * the wait runs out after limit_ms (1..10000) of GPU clock and the kernel reports it:
 * TXG_ERR_TIMEOUT, the CUDA context stays usable.  (The kernels' own waits give up after 2 s.)
 * No reference counterpart. */
int txg_selftest_wait(int32_t never_complete, int32_t limit_ms);

/* Boxcar width ladder of SinglePulse::prepare (singlepulse.cpp:242-254); returns the count. */
int txg_width_ladder(float minw, float maxw, float snrloss, double tsamp, int32_t *vwn,
                     int32_t cap);

/* Boxcar::run over series supplied by the caller (boxcar.cpp:158-296): tim [ndm][nsamples]
 * host memory; writes dense mxS/mxwn when non-NULL and the S > thre points (sorted) when
 * cands is non-NULL.  flags: TXG_FLAG_AVX2_TAIL. */
int txg_boxcar(const float *tim, int64_t ndm, int64_t nsamples, const int32_t *vwn, int32_t nw,
               int32_t iqr, int32_t flags, float thre, float *mxS, int32_t *mxwn,
               txg_cand *cands, int64_t cap, int64_t *ncand);

/* Cluster<double>::run (cluster.cpp:63-161, clustering.h:26-100) on a sorted candidate list;
 * out receives the reported candidates (idm, isamp, wn, S) in the reference's order. */
int txg_cluster(const txg_cand *cands, int64_t n, double dms, double ddm, double fmax,
                double fmin, double tsamp, double radius_smearing, int32_t maxncand,
                int32_t minpts, int32_t drop, int32_t maxwn, txg_cand *out, int64_t cap,
                int64_t *nout);

/* kadaneF (one rfilist entry) on a block already in device memory, allocating nothing.  It
 * has no counterpart in the reference; it exists for callers that cannot call cudaMalloc
 * while they run (real-time back ends with all memory reserved at start-up, frameworks that
 * own GPU memory through their own pool).  x: device block [nchans][ldx], zapped windows set
 * to 0 in place; ranges: device output [nchans/fd][4] as in txg_get_zap_ranges; thr2: squared
 * S/N threshold; wnlimit: minimum window in downsampled samples; stream: cudaStream_t or
 * NULL.  Its scratch is a fixed device array of 2^21 floats (8 MiB) that every GPU loading the
 * library holds until exit: (nsamples/td)*(nchans/fd) above that returns TXG_ERR_ARG, and so
 * do nchans/fd outside 1..65535 and nsamples above 2^31-1, before anything is queued.  Calls
 * share that array, so calls overlapping on the GPU race.  The first call on a device looks up
 * the array's address; make it before any stream capture on that device, and make no call on
 * a device after cudaDeviceReset there (the address kept from the first call is stale). */
int txg_kadaneF_noalloc(float *x, int64_t ldx, int32_t nchans, int64_t nsamples, int32_t td,
                        int32_t fd, float thr2, int64_t wnlimit, int32_t *ranges, void *stream);

/* ---- replot: the per-candidate chain of replot_fil (replot_fil.cpp:409-457) -------------- */
/* Options of replot_fil that the chain reads (replot_fil.cpp:49-88 defaults in brackets). */
typedef struct {
    int32_t zdot;          /* --zdot: zero-DM matched filter first [0] */
    int32_t kadane[3];     /* --kadane td fd threshold; kadane[0] = 0 disables [off] */
    int32_t clip[3];       /* --clip td fd threshold; clip[0] = 0 disables [off] */
    float zapthre;         /* --zapthre: skewness/kurtosis/autocorrelation IQR cut [3] */
    int32_t nzap;
    double zap[16][2];     /* --zap fl fh: channels with fl <= f <= fh set to 0 */
    int32_t fd;            /* --fd: channel downsample before the search [1] */
    float snrloss;         /* --snrloss: boxcar width ladder [0.1] */
    int32_t nwidth;        /* --nw: the data are cut to 2*nw*width [20] */
    int32_t pow2bin;       /* --pow2bin */
    int32_t nopt;          /* --nopt: peak search at the candidate DM instead of the DM-time map */
    int32_t upto;          /* stop after step 1..12 of the chain (0 = all; for checks) */
} txg_replot_opts;

/* One candidate: its filterbank cut as Candidate::data holds it (one polarisation, channel-major
 * [nchan][nbin], host memory), sampling time, channel frequencies, the DM and the width (s) of
 * its .cands line. */
typedef struct {
    const float *data;
    int32_t nchan;
    int64_t nbin;
    double tbin;
    const double *frequencies;
    double dm;
    float width;
} txg_replot_cand;

typedef struct {
    float snr;             /* Candidate::snr after matched_filter / peak_search */
    float width;           /* Candidate::width (s) */
    double dm_maxsnr;      /* Candidate::dm_maxsnr */
    int64_t maxtid;        /* peak sample: mjd = mjd_start + maxtid*tbin/86400 */
    int64_t nbin;          /* samples after shrink_to_fit */
    int32_t nchan;         /* channels after the fd downsample */
    int32_t ndm;           /* rows of the S/N map (the DM-time map; 1 with nopt) */
    double dms, ddm;       /* DM axis of the map */
} txg_replot_result;

/* Runs the chain on n candidates at once on the GPU: [zdot] get_stats, dedisperse (incoherent),
 * shrink_to_fit(2*nw), azap, zap, get_stats, normalize, [clip], [kadaneF], downsample(1, fd),
 * then optimize (DM-time Hough transform, hough_transform.h) + matched_filter, or
 * peak_search (candidate.cpp:56-1200).  snrmap (optional) receives each candidate's S/N map
 * [ndm][nbin] one after the other; data_out (optional) the data after the last step run. */
int txg_replot(const txg_replot_opts *opts, const txg_replot_cand *cands, int64_t n,
               txg_replot_result *out, float *snrmap, int64_t snrmap_cap, float *data_out,
               int64_t data_cap);

/* Device time per kernel class accumulated since the last call (plan flag TXG_FLAG_TIMING),
 * measured with CUDA events on the handle's stream: ms[c] total milliseconds and launches[c]
 * number of launches of class c; classes 0 unpack, 1 preprocess+RFI, 2 stage 1,
 * 3 stage 2, 4 boxcar.  Returns the number of classes. */
int txg_get_timing(txg_handle *h, double *ms, int64_t *launches, int32_t n);

/* txg_get_timing for one ddplan row (its own accumulators, reset by this call). */
int txg_get_row_timing(txg_handle *h, int32_t row, double *ms, int64_t *launches, int32_t n);

/* The dedispersion launch shapes a row runs with: stage1 = resident stage-1 shape (time tile
 * x coarse-DM groups per CTA), stage2 = stage-2 threads-per-CTA variant, stage2_kb = its
 * shared-memory budget in KB (0 = default); see txg_dedisp.cu.  With TXG_FLAG_AUTOTUNE they
 * are the fastest of a few candidates timed at txg_create (all candidates give bit-identical
 * results; the subband count and DM group stay as planned, since they change the sums).  No
 * reference counterpart. */
int txg_get_launch_shape(txg_handle *h, int32_t row, int32_t *stage1, int32_t *stage2,
                         int32_t *stage2_kb);

/* The handle's CUDA stream (cudaStream_t) so callers can order or time work against it.  The
 * rows of a block run on streams of their own that fork from this one; their work joins it at
 * txg_sync and before every call that reads results (txg_get_*), so work queued on it after
 * txg_sync follows everything pushed before. */
int txg_get_stream(txg_handle *h, void **stream);

const char *txg_strerror(int32_t status);
int32_t txg_version(void);

#ifdef __cplusplus
}
#endif

#endif /* TRANSIENTX_GB300_H */
