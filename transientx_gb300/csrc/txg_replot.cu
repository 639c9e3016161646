/*
 * txg_replot.cu -- the per-candidate chain of replot_fil (src/singlepulse/replot_fil.cpp:409-457)
 * on the GPU, batched over candidates: Candidate::zdot, get_stats, dedisperse (incoherent),
 * shrink_to_fit, azap, zap, normalize, clip, kadaneF, downsample, optimize (the DM-time Hough
 * transform of include/hough_transform.h), matched_filter and peak_search
 * (src/singlepulse/candidate.cpp:56-1200).
 *
 * Every kernel restates one Candidate method for one polarisation with the reference's own
 * mixture of float and double arithmetic (each expression rounded as the C++ evaluates it;
 * this file is compiled without multiply-add contraction), so results equal the reference's.
 * Candidates of a batch share the launches: blockIdx.y is the candidate, and each candidate's
 * rows keep their original pitch while its nbin and nchan shrink.  The small per-candidate
 * decisions the reference makes on the host (delays, the chop length, the azap quantiles, the
 * Hough shift plan) are made on the host here too.
 */
#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <vector>

#include "txg_internal.h"

namespace txg {

namespace {

/* device view of one candidate */
struct RpMeta {
    long off;   /* first float of its rows in the data buffers */
    long pitch; /* row pitch (its original nbin) */
    long nbin;  /* current samples */
    int nchan;  /* current channels */
    int pad;
    long coff;  /* first entry of its per-channel arrays (original nchan of them) */
    long hoff;  /* first float of its DM-time rows (nchans x nbin) */
    int nchans; /* rows of the Hough transform: nchan rounded up to a power of two */
    int levels; /* log2(nchans) */
    long soff;  /* first entry of its shift plan (levels x nchans) */
    long roff;  /* first entry of its row order hrange (nchans) */
};

inline unsigned nblk(long n, int b) { return (unsigned)((n + b - 1) / b); }

/* Candidate::zdot, first loop (candidate.cpp:837-859): per channel, double mean and (float
 * square) power, then x = (x - mean) / std in double, stored as float. */
__global__ void k_rp_zdot_norm(float *__restrict__ buf, const RpMeta *__restrict__ m)
{
    const RpMeta c = m[blockIdx.y];
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= c.nchan) return;
    float *r = buf + c.off + (long)j * c.pitch;
    double tmpmean = 0., tmpstd = 0.;
    for (long i = 0; i < c.nbin; i++) {
        tmpmean += r[i];
        tmpstd += r[i] * r[i];
    }
    tmpmean /= c.nbin;
    tmpstd /= c.nbin;
    tmpstd -= tmpmean * tmpmean;
    tmpstd = sqrt(tmpstd);
    if (tmpstd == 0.) tmpstd = 1.;
    for (long i = 0; i < c.nbin; i++) {
        r[i] = (float)(r[i] - tmpmean);
        r[i] = (float)(r[i] / tmpstd);
    }
}

/* zdot's zero-DM series: s[i] = sum over channels in order (double), / nchan (:857-864) */
__global__ void k_rp_zdot_s(const float *__restrict__ buf, const RpMeta *__restrict__ m,
                            double *__restrict__ s, long soff_stride)
{
    const RpMeta c = m[blockIdx.y];
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.nbin) return;
    double acc = 0.;
    for (int j = 0; j < c.nchan; j++) acc += buf[c.off + (long)j * c.pitch + i];
    acc /= c.nchan;
    s[blockIdx.y * soff_stride + i] = acc;
}

/* zdot's least-squares fit and subtraction (:866-895) */
__global__ void k_rp_zdot_fit(float *__restrict__ buf, const RpMeta *__restrict__ m,
                              const double *__restrict__ s_all, long soff_stride)
{
    const RpMeta c = m[blockIdx.y];
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= c.nchan) return;
    float *r = buf + c.off + (long)j * c.pitch;
    const double *s = s_all + blockIdx.y * soff_stride;
    double xe = 0., xs = 0., se = 0., ss = 0., alpha = 0., beta = 0.;
    for (long i = 0; i < c.nbin; i++) {
        xe += r[i];
        xs += r[i] * s[i];
        se += s[i];
        ss += s[i] * s[i];
    }
    const double tmp = se * se - ss * c.nbin;
    if (tmp != 0) {
        alpha = (xe * se - xs * c.nbin) / tmp;
        beta = (xs * se - xe * ss) / tmp;
    }
    for (long i = 0; i < c.nbin; i++) r[i] = (float)(r[i] - (alpha * s[i] + beta));
}

/* Candidate::get_stats (:429-534) for one polarisation: the half-length window of least sum
 * (circular), mean/var of the data over it in double, and skewness, kurtosis and lag-1
 * autocorrelation in float. */
__global__ void k_rp_stats(const float *__restrict__ buf, const RpMeta *__restrict__ m,
                           double *__restrict__ mean, double *__restrict__ var, float *__restrict__ skew,
                           float *__restrict__ kurt, float *__restrict__ ac)
{
    const RpMeta c = m[blockIdx.y];
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= c.nchan) return;
    const float *r = buf + c.off + (long)j * c.pitch;
    const long nbin = c.nbin, h = nbin / 2;
    auto sumif = [&](long i) { return 0.f + r[i]; }; /* data_sumif starts at 0 and adds the data */
    float boxsum = 0.;
    for (long i = 0; i < h; i++) boxsum += sumif(i);
    float mn = boxsum;
    long istart = 0, iend = h;
    for (long i = 0; i < nbin; i++) {
        boxsum -= sumif(i);
        boxsum += sumif((i + h) % nbin);
        if (boxsum < mn) {
            mn = boxsum;
            istart = i + 1;
            iend = h + i + 1;
        }
    }
    double mu = 0., v = 0.;
    for (long i = istart; i < iend; i++) {
        mu += r[i % nbin];
        v += r[i % nbin] * r[i % nbin];
    }
    mu /= h;
    v /= h;
    v -= mu * mu;
    const float tmp_mean = mn / h;
    float tmp_var = 0., sk = 0., ku = 0., a1 = 0., last = 0;
    for (long i = istart; i < iend; i++) {
        const float t = sumif(i % nbin) - tmp_mean;
        const float t2 = t * t, t3 = t2 * t, t4 = t3 * t;
        tmp_var += t2;
        sk += t3;
        ku += t4;
        a1 += t * last;
        last = t;
    }
    tmp_var /= h;
    if (tmp_var <= 0) {
        sk = 0.;
        ku = 0.;
        a1 = 0.;
    }
    sk /= h;
    sk /= tmp_var * sqrtf(tmp_var);
    ku /= h;
    ku /= tmp_var * tmp_var;
    ku -= 3.;
    a1 /= h - 1;
    a1 /= tmp_var;
    const long q = c.coff + j;
    mean[q] = mu;
    var[q] = v;
    skew[q] = sk;
    kurt[q] = ku;
    ac[q] = a1;
}

/* Candidate::dedisperse, incoherent branch (:106-140): row j rotated left by its delay */
__global__ void k_rp_dedisp(const float *__restrict__ src, float *__restrict__ dst,
                            const RpMeta *__restrict__ m, const int *__restrict__ delay)
{
    const RpMeta c = m[blockIdx.y];
    const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long)c.nchan * c.nbin) return;
    const int j = (int)(e / c.nbin);
    const long i = e - (long)j * c.nbin;
    const long d = delay[c.coff + j];
    const long k = i + d < c.nbin ? i + d : i + d - c.nbin;
    dst[c.off + (long)j * c.pitch + i] = src[c.off + (long)j * c.pitch + k];
}

/* data *= weights[j] (azap :610-621, zap :641-653) */
__global__ void k_rp_scale(float *__restrict__ buf, const RpMeta *__restrict__ m,
                           const float *__restrict__ w)
{
    const RpMeta c = m[blockIdx.y];
    const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long)c.nchan * c.nbin) return;
    const int j = (int)(e / c.nbin);
    float *p = buf + c.off + (long)j * c.pitch + (e - (long)j * c.nbin);
    *p *= w[c.coff + j];
}

/* Candidate::normalize (:536-567) */
__global__ void k_rp_normalize(float *__restrict__ buf, const RpMeta *__restrict__ m,
                               const double *__restrict__ mean, const double *__restrict__ var)
{
    const RpMeta c = m[blockIdx.y];
    const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long)c.nchan * c.nbin) return;
    const int j = (int)(e / c.nbin);
    float *p = buf + c.off + (long)j * c.pitch + (e - (long)j * c.nbin);
    const double mu = mean[c.coff + j], v = var[c.coff + j];
    if (v <= 0.) {
        *p = (float)(*p - mu);
    } else {
        const float sd = (float)sqrt(v);
        *p = (float)(*p - mu);
        *p = *p / sd;
    }
}

/* Candidate::clip (:656-708): td x fd sums (fd outer, td inner) above thre zero their cells */
__global__ void k_rp_clip(float *__restrict__ buf, const RpMeta *__restrict__ m, int td, int fd,
                          float thre)
{
    const RpMeta c = m[blockIdx.y];
    const long nsds = c.nbin / td, ncds = c.nchan / fd;
    const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ncds * nsds) return;
    const long j = e / nsds, i = e - j * nsds;
    float acc = 0.;
    for (int k = 0; k < fd; k++)
        for (int n = 0; n < td; n++) acc += buf[c.off + (j * fd + k) * c.pitch + i * td + n];
    if (acc > thre)
        for (int k = 0; k < fd; k++)
            for (int n = 0; n < td; n++) buf[c.off + (j * fd + k) * c.pitch + i * td + n] = 0.;
}

/* kadane<float> of the XLibs helpers as the reference tree's callers use it: a new maximum
 * needs a strictly larger sum, the running sum restarts after it drops below zero */
__device__ float rp_kadane(const float *a, long n, long *start, long *end)
{
    float best = -INFINITY, cur = 0;
    long cs = 0;
    *start = 0;
    *end = -1;
    for (long i = 0; i < n; i++) {
        cur = cur + a[i];
        if (cur > best) {
            best = cur;
            *start = cs;
            *end = i;
        }
        if (cur < 0) {
            cur = 0;
            cs = i + 1;
        }
    }
    return best;
}

/* Candidate::kadaneF (:710-829), one thread per downsampled channel; ds: scratch of
 * stride `dstride` floats per (candidate, channel) */
__global__ void k_rp_kadane(float *__restrict__ buf, const RpMeta *__restrict__ m, int td, int fd,
                            float threshold, int nwidth, const float *__restrict__ width,
                            const double *__restrict__ tbin, float *__restrict__ ds, long dstride)
{
    const RpMeta c = m[blockIdx.y];
    const long nsds = c.nbin / td, ncds = c.nchan / fd;
    const long j = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= ncds) return;
    float *ch = ds + (c.coff + j) * dstride;
    for (long i = 0; i < nsds; i++) ch[i] = 0.;
    for (int k = 0; k < fd; k++)
        for (int n = 0; n < td; n++)
            for (long i = 0; i < nsds; i++) ch[i] += buf[c.off + (j * fd + k) * c.pitch + i * td + n];
    const int wnlimit = (int)(nwidth * width[blockIdx.y] / tbin[blockIdx.y] / td);
    const float var = (float)(td * fd);
    for (int p = 0; p < 2; p++) {
        if (p == 1)
            for (long i = 0; i < nsds; i++) ch[i] = -ch[i];
        long start, end;
        const float boxsum = rp_kadane(ch, nsds, &start, &end);
        const long wn = end - start + 1;
        float snr2 = 0.;
        if (wn > wnlimit) snr2 = boxsum * boxsum / (wn * var);
        start *= td;
        end += 1;
        end *= td;
        if (snr2 > threshold * threshold)
            for (int k = 0; k < fd; k++)
                for (long i = start; i < end; i++) buf[c.off + (j * fd + k) * c.pitch + i] = 0.;
    }
}

/* Candidate::downsample(1, fd) (:381-427): channel sums in order, out of place */
__global__ void k_rp_fsum(const float *__restrict__ src, float *__restrict__ dst,
                          const RpMeta *__restrict__ m, int fd)
{
    const RpMeta c = m[blockIdx.y]; /* geometry before the downsample */
    const long nc = c.nchan / fd;
    const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nc * c.nbin) return;
    const long j = e / c.nbin, i = e - j * c.nbin;
    float acc = 0.;
    for (int jj = 0; jj < fd; jj++) acc += src[c.off + (j * fd + jj) * c.pitch + i];
    dst[c.off + j * c.pitch + i] = acc;
}

/* Candidate::optimize (:899-966): the Hough input rows, frequency-descending, zero padded to
 * nchans rows */
__global__ void k_rp_hough_fill(const float *__restrict__ buf, float *__restrict__ h,
                                const RpMeta *__restrict__ m, const int *__restrict__ flip)
{
    const RpMeta c = m[blockIdx.y];
    const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long)c.nchans * c.nbin) return;
    const long j = e / c.nbin, i = e - j * c.nbin;
    float v = 0.;
    if (j < c.nchan) {
        const long src = flip[blockIdx.y] ? c.nchan - 1 - j : j;
        v = 0.f + buf[c.off + src * c.pitch + i];
    }
    h[c.hoff + e] = v;
}

/* One level of the transform of hough_transform.h:29-55 (depth = levels-1-t): for block irow of
 * 2*nrowsub rows, row k of the first half becomes x0 + rot(y, d0) and row k of the second half
 * x0 + rot(y, d1), y being the old second-half row and rot(y, d)[i] = y[(i+d) mod ncol]. */
__global__ void k_rp_hough_level(const float *__restrict__ hin, float *__restrict__ hout,
                                 const RpMeta *__restrict__ m, const int *__restrict__ shift, int t)
{
    const RpMeta c = m[blockIdx.y];
    const long ncol = c.nbin;
    const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long)c.nchans * ncol) return;
    const long r = e / ncol, i = e - r * ncol;
    const int depth = c.levels - 1 - t;
    if (depth < 0) {
        hout[c.hoff + e] = hin[c.hoff + e];
        return;
    }
    const long nrowsub = (long)c.nchans >> (depth + 1);
    const long blk = r / (2 * nrowsub), k = r - blk * 2 * nrowsub;
    const int *sh = shift + c.soff + (long)(c.levels - 1 - depth) * c.nchans;
    const long d = sh[blk * 2 * nrowsub + k];
    const long x0 = k < nrowsub ? r : r - nrowsub, y = x0 + nrowsub;
    const long iy = i + d < ncol ? i + d : i + d - ncol;
    hout[c.hoff + e] = hin[c.hoff + x0 * ncol + i] + hin[c.hoff + y * ncol + iy];
}

/* the transform's last step: output row hrange[j] = row j */
__global__ void k_rp_hough_perm(const float *__restrict__ hin, float *__restrict__ hout,
                                const RpMeta *__restrict__ m, const int *__restrict__ hrange)
{
    const RpMeta c = m[blockIdx.y];
    const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long)c.nchans * c.nbin) return;
    const long j = e / c.nbin, i = e - j * c.nbin;
    hout[c.hoff + (long)hrange[c.roff + j] * c.nbin + i] = hin[c.hoff + e];
}

/* peak_search's profile (:1115-1129): sum of the channels in order, from 0 */
__global__ void k_rp_profile(const float *__restrict__ buf, float *__restrict__ h,
                             const RpMeta *__restrict__ m)
{
    const RpMeta c = m[blockIdx.y];
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.nbin) return;
    float acc = 0.;
    for (int j = 0; j < c.nchan; j++) acc += buf[c.off + (long)j * c.pitch + i];
    h[c.hoff + i] = acc;
}

/* matched_filter / peak_search boxcar of one row (:1000-1063, :1131-1180): double mean and
 * variance (get_mean_var), float circular running sum of (x - mean) in double, widths of the
 * float ladder, S >= best keeps the later width.  csum: scratch of 2*nbin floats per row. */
__global__ void k_rp_boxcar(const float *__restrict__ h, const RpMeta *__restrict__ m,
                            const int *__restrict__ rows, const float *__restrict__ vwn,
                            const int *__restrict__ nbox, long wstride, float *__restrict__ snr,
                            int *__restrict__ wid, float *__restrict__ csump)
{
    const RpMeta c = m[blockIdx.y];
    const long j = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= rows[blockIdx.y]) return;
    const long nbin = c.nbin;
    const float *tim = h + c.hoff + j * nbin;
    float *cs = csump + (c.hoff + j * nbin) * 2;
    float *vS = snr + c.hoff + j * nbin;
    int *vw = wid + c.hoff + j * nbin;
    double s1 = 0., s2 = 0.;
    for (long i = 0; i < nbin; i++) {
        const double v = tim[i];
        s1 += v;
        s2 += v * v;
    }
    const double mean = s1 / nbin, var = s2 / nbin - mean * mean;
    float csum = 0.;
    for (long i = 0; i < nbin; i++) {
        csum += tim[i] - mean;
        cs[i] = csum;
    }
    for (long i = nbin; i < 2 * nbin; i++) {
        csum += tim[i - nbin] - mean;
        cs[i] = csum;
    }
    for (long i = 0; i < nbin; i++) {
        vS[i] = 0.;
        vw[i] = 0;
    }
    if (var > 0) {
        const float *lad = vwn + blockIdx.y * wstride;
        for (int k = 0; k < nbox[blockIdx.y]; k++) {
            const int wn = (int)lad[k];
            const int wl = wn / 2 + 1, wh = (wn - 1) / 2;
            const float temp = (float)sqrt(1. / (wn * var));
            for (long i = wl; i < nbin; i++) {
                const float S = (cs[i + wh] - cs[i - wl]) * temp;
                if (S >= vS[i]) {
                    vS[i] = S;
                    vw[i] = wn;
                }
            }
            for (long i = nbin; i < nbin + wl; i++) {
                const float S = (cs[i + wh] - cs[i - wl]) * temp;
                if (S >= vS[i - nbin]) {
                    vS[i - nbin] = S;
                    vw[i - nbin] = wn;
                }
            }
        }
    }
}

/* the first largest S of each candidate's map in row-major order (the scan of :1065-1078) */
__global__ void __launch_bounds__(256) k_rp_argmax(const float *__restrict__ snr, const RpMeta *__restrict__ m,
                                                   const int *__restrict__ rows, long *__restrict__ best)
{
    const RpMeta c = m[blockIdx.x];
    const long n = (long)rows[blockIdx.x] * c.nbin;
    const float *v = snr + c.hoff;
    __shared__ float bv[256];
    __shared__ long bi[256];
    float b = -INFINITY;
    long idx = -1;
    for (long e = threadIdx.x; e < n; e += blockDim.x)
        if (idx < 0 ? !(v[e] != v[e]) && v[e] >= b : v[e] > b) { /* NaN never wins */
            b = v[e];
            idx = e;
        }
    bv[threadIdx.x] = b;
    bi[threadIdx.x] = idx;
    __syncthreads();
    if (threadIdx.x == 0) {
        float B = -INFINITY;
        long I = -1;
        for (int t = 0; t < (int)blockDim.x; t++) {
            if (bi[t] < 0) continue;
            if (I < 0 || bv[t] > B || (bv[t] == B && bi[t] < I)) {
                B = bv[t];
                I = bi[t];
            }
        }
        /* the reference starts from element 0: a NaN there, or no number at all, keeps it */
        if (n > 0 && (v[0] != v[0] || I < 0 || !(B > v[0]))) I = 0;
        best[blockIdx.x] = I;
    }
}

} // namespace

} // namespace txg

using namespace txg;

namespace {

/* host mirror of one candidate through the chain */
struct RpHost {
    long off, pitch, nbin, coff;
    int nchan;
    double tbin, dm;
    float width;
    std::vector<double> f;
    /* Hough geometry (step 12) */
    int nchans = 1, levels = 0;
    long hoff = 0, soff = 0, roff = 0, rows = 1;
    double dms = 0., ddm = 0.;
};

double rp_dmdelay(double dm, double fh, double fl) { return 4.148741601e3 * dm * (1. / (fl * fl) - 1. / (fh * fh)); }

/* get_shiftplan of hough_transform.h:57-101, as written */
void rp_shiftplan(std::vector<std::vector<int>> &shiftplan, std::vector<int> &hrange, int nrow, int ncol,
                  const std::function<int(int, int, int)> &get_shift)
{
    int nrow_tmp = nrow;
    int nrowsub_tmp = nrow / nrow_tmp;
    hrange.assign(nrow, 0);
    for (long k = 0; k < nrowsub_tmp; k++) hrange[k] = k * nrow_tmp;
    std::vector<int> xrange_tmp(nrow, 0);
    for (long j = 0; j < nrow; j++) xrange_tmp[j] = j;
    int n = (int)std::log2(nrow);
    for (long l = 0; l < n; l++) {
        std::vector<int> shift_tmp(nrow_tmp * nrowsub_tmp);
        for (long j = 0; j < nrow_tmp / 2; j++) {
            for (long k = 0; k < nrowsub_tmp; k++) {
                hrange[k] = hrange[k];
                hrange[k + nrowsub_tmp] = hrange[k] + nrow_tmp / 2;
            }
            for (long k = 0; k < nrowsub_tmp * 2; k++) {
                int s = get_shift(xrange_tmp[j * 2], xrange_tmp[j * 2 + 1], hrange[k]) % ncol;
                if (s < 0) s += ncol;
                shift_tmp[j * (nrowsub_tmp * 2) + k] = s;
            }
            xrange_tmp[j] = xrange_tmp[j * 2];
        }
        shiftplan.push_back(shift_tmp);
        nrowsub_tmp <<= 1;
        nrow_tmp >>= 1;
    }
}

/* azap's IQR cut of one statistic (candidate.cpp:573-597): q1 the n/4-th smallest, q3 the
 * n/4-th largest, by nth_element as the reference takes them */
void rp_quartiles(const float *v, int n, float &q1, float &q3)
{
    std::vector<float> s(v, v + n);
    std::nth_element(s.begin(), s.begin() + s.size() / 4, s.end(), std::less<float>());
    q1 = s[s.size() / 4];
    std::nth_element(s.begin(), s.begin() + s.size() / 4, s.end(), std::greater<float>());
    q3 = s[s.size() / 4];
}

struct DevBuf {
    std::vector<void *> p;
    ~DevBuf()
    {
        for (void *q : p) cudaFree(q);
    }
    template <typename T> cudaError_t alloc(T **out, size_t count)
    {
        void *q = nullptr;
        cudaError_t e = cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(T));
        if (e == cudaSuccess) {
            p.push_back(q);
            *out = (T *)q;
        }
        return e;
    }
};

} // namespace

extern "C" int txg_replot(const txg_replot_opts *o, const txg_replot_cand *cands, int64_t n,
                          txg_replot_result *out, float *snrmap, int64_t snrmap_cap, float *data_out,
                          int64_t data_cap)
{
    if (!o || !cands || !out || n <= 0) return set_arg_error("null options, candidates or results");
    const bool kad = o->kadane[0] > 0, clp = o->clip[0] > 0;
    if ((kad && (o->kadane[1] < 1)) || (clp && (o->clip[1] < 1)) || o->fd < 1 || o->nwidth < 1 ||
        o->nzap < 0 || o->nzap > 16)
        return set_arg_error("kadane/clip td and fd, fd and nw must be positive; at most 16 zap ranges");
    const int upto = o->upto > 0 ? o->upto : 12;
    std::vector<RpHost> H(n);
    long total = 0, tchan = 0, maxnbin = 0;
    for (long b = 0; b < n; b++) {
        const txg_replot_cand &c = cands[b];
        if (!c.data || !c.frequencies || c.nchan < 2 || c.nbin < 4 || !(c.tbin > 0.) || !(c.width > 0.f))
            return set_arg_error("candidate " + std::to_string(b) + ": need data, frequencies, nchan >= 2, nbin >= 4, tbin > 0, width > 0");
        if (c.nchan / o->fd < 2) return set_arg_error("fd leaves fewer than 2 channels");
        RpHost &h = H[b];
        h.off = total;
        h.pitch = h.nbin = c.nbin;
        h.nchan = c.nchan;
        h.coff = tchan;
        h.tbin = c.tbin;
        h.dm = c.dm;
        h.width = c.width;
        h.f.assign(c.frequencies, c.frequencies + c.nchan);
        total += (long)c.nchan * c.nbin;
        tchan += c.nchan;
        maxnbin = std::max(maxnbin, (long)c.nbin);
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return set_cuda_error(cudaErrorNoDevice, "txg_replot", __FILE__, __LINE__);

    DevBuf mem;
    float *buf[2] = {nullptr, nullptr}, *skew, *kurt, *ac, *w, *ds;
    double *mean, *var, *zs;
    int *delay;
    RpMeta *dmeta;
    cudaStream_t st = nullptr;
    cudaError_t e = cudaSuccess;
#define RP_TRY(x)                                                                  \
    do {                                                                           \
        e = (x);                                                                   \
        if (e != cudaSuccess) {                                                    \
            if (st) cudaStreamDestroy(st);                                         \
            return set_cuda_error(e, #x, __FILE__, __LINE__);                      \
        }                                                                          \
    } while (0)
    RP_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    RP_TRY(mem.alloc(&buf[0], total));
    RP_TRY(mem.alloc(&buf[1], total));
    RP_TRY(mem.alloc(&mean, tchan));
    RP_TRY(mem.alloc(&var, tchan));
    RP_TRY(mem.alloc(&skew, tchan));
    RP_TRY(mem.alloc(&kurt, tchan));
    RP_TRY(mem.alloc(&ac, tchan));
    RP_TRY(mem.alloc(&w, tchan));
    RP_TRY(mem.alloc(&delay, tchan));
    RP_TRY(mem.alloc(&dmeta, n));
    RP_TRY(mem.alloc(&zs, (size_t)n * maxnbin));
    RP_TRY(mem.alloc(&ds, (size_t)tchan * maxnbin));
    for (long b = 0; b < n; b++)
        RP_TRY(cudaMemcpyAsync(buf[0] + H[b].off, cands[b].data, sizeof(float) * H[b].nchan * H[b].nbin,
                               cudaMemcpyHostToDevice, st));
    int cur = 0;
    std::vector<RpMeta> meta(n);
    auto push_meta = [&]() -> cudaError_t {
        for (long b = 0; b < n; b++) {
            const RpHost &h = H[b];
            RpMeta &m = meta[b];
            m.off = h.off;
            m.pitch = h.pitch;
            m.nbin = h.nbin;
            m.nchan = h.nchan;
            m.pad = 0;
            m.coff = h.coff;
            m.hoff = h.hoff;
            m.nchans = h.nchans;
            m.levels = h.levels;
            m.soff = h.soff;
            m.roff = h.roff;
        }
        return cudaMemcpyAsync(dmeta, meta.data(), sizeof(RpMeta) * n, cudaMemcpyHostToDevice, st);
    };
    auto maxchan = [&]() {
        int mc = 0;
        for (auto &h : H) mc = std::max(mc, h.nchan);
        return mc;
    };
    auto maxelem = [&]() {
        long me = 0;
        for (auto &h : H) me = std::max(me, (long)h.nchan * h.nbin);
        return me;
    };
    const unsigned NB = (unsigned)n;
    RP_TRY(push_meta());
    std::vector<float> w_h(tchan, 1.f);

    /* 1: zdot */
    if (o->zdot) {
        k_rp_zdot_norm<<<dim3(nblk(maxchan(), 128), NB), 128, 0, st>>>(buf[cur], dmeta);
        k_rp_zdot_s<<<dim3(nblk(maxnbin, 128), NB), 128, 0, st>>>(buf[cur], dmeta, zs, maxnbin);
        k_rp_zdot_fit<<<dim3(nblk(maxchan(), 128), NB), 128, 0, st>>>(buf[cur], dmeta, zs, maxnbin);
        RP_TRY(cudaGetLastError());
    }
    /* 2: get_stats (their skewness, kurtosis, autocorrelation drive azap) */
    std::vector<float> sk_h(tchan), ku_h(tchan), ac_h(tchan);
    if (upto >= 2) {
        k_rp_stats<<<dim3(nblk(maxchan(), 128), NB), 128, 0, st>>>(buf[cur], dmeta, mean, var, skew, kurt, ac);
        RP_TRY(cudaGetLastError());
        RP_TRY(cudaMemcpyAsync(sk_h.data(), skew, sizeof(float) * tchan, cudaMemcpyDeviceToHost, st));
        RP_TRY(cudaMemcpyAsync(ku_h.data(), kurt, sizeof(float) * tchan, cudaMemcpyDeviceToHost, st));
        RP_TRY(cudaMemcpyAsync(ac_h.data(), ac, sizeof(float) * tchan, cudaMemcpyDeviceToHost, st));
    }
    /* 3: dedisperse at the candidate DM (incoherent) */
    if (upto >= 3) {
        std::vector<int> dl(tchan);
        for (long b = 0; b < n; b++) {
            const RpHost &h = H[b];
            const double fmax = *std::max_element(h.f.begin(), h.f.end());
            for (int j = 0; j < h.nchan; j++) {
                int d = (int)std::round(rp_dmdelay(h.dm, fmax, h.f[j]) / h.tbin);
                d %= h.nbin;
                if (d < 0) d += h.nbin;
                dl[h.coff + j] = d;
            }
        }
        RP_TRY(cudaMemcpyAsync(delay, dl.data(), sizeof(int) * tchan, cudaMemcpyHostToDevice, st));
        k_rp_dedisp<<<dim3(nblk(maxelem(), 256), NB), 256, 0, st>>>(buf[cur], buf[cur ^ 1], dmeta, delay);
        RP_TRY(cudaGetLastError());
        RP_TRY(cudaStreamSynchronize(st)); /* dl goes out of scope */
        cur ^= 1;
    }
    /* 4: shrink_to_fit(2*nw, pow2bin, kadane td) (:234-264) */
    if (upto >= 4) {
        const int nw2 = 2 * o->nwidth, factor = kad ? o->kadane[0] : 1;
        for (auto &h : H) {
            long nbin_new = (long)(nw2 * h.width / h.tbin);
            if (o->pow2bin) nbin_new = (long)std::pow(2, std::ceil(std::log2(nbin_new)));
            nbin_new = (long)(std::ceil(nbin_new / factor) * factor);
            if (nbin_new < h.nbin) h.nbin = nbin_new;
        }
        for (auto &h : H)
            if (h.nbin < 4) {
                cudaStreamDestroy(st);
                return set_arg_error("the chop to 2*nw*width leaves fewer than 4 samples");
            }
        RP_TRY(push_meta());
    }
    /* 5: azap(zapthre) with the statistics of step 2 */
    if (upto >= 5) {
        RP_TRY(cudaStreamSynchronize(st));
        const float t = o->zapthre;
        for (auto &h : H) {
            float k1, k3, s1, s3, a1, a3;
            rp_quartiles(ku_h.data() + h.coff, h.nchan, k1, k3);
            rp_quartiles(sk_h.data() + h.coff, h.nchan, s1, s3);
            rp_quartiles(ac_h.data() + h.coff, h.nchan, a1, a3);
            const float kR = k3 - k1, sR = s3 - s1, aR = a3 - a1;
            for (int j = 0; j < h.nchan; j++) {
                const float ku = ku_h[h.coff + j], sk = sk_h[h.coff + j], a = ac_h[h.coff + j];
                if ((ku < k1 - t * kR) || (ku > k3 + t * kR) || (sk < s1 - t * sR) || (sk > s3 + t * sR) ||
                    (a < a1 - t * aR) || (a > a3 + t * aR))
                    w_h[h.coff + j] = 0.;
            }
        }
        RP_TRY(cudaMemcpyAsync(w, w_h.data(), sizeof(float) * tchan, cudaMemcpyHostToDevice, st));
        k_rp_scale<<<dim3(nblk(maxelem(), 256), NB), 256, 0, st>>>(buf[cur], dmeta, w);
        RP_TRY(cudaGetLastError());
    }
    /* 6: zap(zaplist): weights keep azap's zeros */
    if (upto >= 6 && o->nzap > 0) {
        RP_TRY(cudaStreamSynchronize(st));
        for (auto &h : H)
            for (int j = 0; j < h.nchan; j++)
                for (int z = 0; z < o->nzap; z++)
                    if (h.f[j] >= o->zap[z][0] && h.f[j] <= o->zap[z][1]) w_h[h.coff + j] = 0;
        RP_TRY(cudaMemcpyAsync(w, w_h.data(), sizeof(float) * tchan, cudaMemcpyHostToDevice, st));
        k_rp_scale<<<dim3(nblk(maxelem(), 256), NB), 256, 0, st>>>(buf[cur], dmeta, w);
        RP_TRY(cudaGetLastError());
    }
    /* 7, 8: get_stats, normalize */
    if (upto >= 7)
        k_rp_stats<<<dim3(nblk(maxchan(), 128), NB), 128, 0, st>>>(buf[cur], dmeta, mean, var, skew, kurt, ac);
    if (upto >= 8)
        k_rp_normalize<<<dim3(nblk(maxelem(), 256), NB), 256, 0, st>>>(buf[cur], dmeta, mean, var);
    RP_TRY(cudaGetLastError());
    /* 9: clip */
    if (upto >= 9 && clp) {
        const int td = o->clip[0], fd = o->clip[1];
        const float thre = (float)((float)o->clip[2] * std::sqrt(td * fd));
        k_rp_clip<<<dim3(nblk(maxelem(), 256), NB), 256, 0, st>>>(buf[cur], dmeta, td, fd, thre);
        RP_TRY(cudaGetLastError());
    }
    /* 10: kadaneF (nwidth 0, as replot_fil calls it) */
    if (upto >= 10 && kad) {
        std::vector<float> wid_h(n);
        std::vector<double> tb_h(n);
        for (long b = 0; b < n; b++) {
            wid_h[b] = H[b].width;
            tb_h[b] = H[b].tbin;
        }
        float *dwid;
        double *dtb;
        RP_TRY(mem.alloc(&dwid, n));
        RP_TRY(mem.alloc(&dtb, n));
        RP_TRY(cudaMemcpyAsync(dwid, wid_h.data(), sizeof(float) * n, cudaMemcpyHostToDevice, st));
        RP_TRY(cudaMemcpyAsync(dtb, tb_h.data(), sizeof(double) * n, cudaMemcpyHostToDevice, st));
        k_rp_kadane<<<dim3(nblk(maxchan(), 64), NB), 64, 0, st>>>(buf[cur], dmeta, o->kadane[0], o->kadane[1],
                                                                 (float)o->kadane[2], 0, dwid, dtb, ds, maxnbin);
        RP_TRY(cudaGetLastError());
        RP_TRY(cudaStreamSynchronize(st));
    }
    /* 11: downsample(1, fd) */
    if (upto >= 11 && o->fd > 1) {
        k_rp_fsum<<<dim3(nblk(maxelem(), 256), NB), 256, 0, st>>>(buf[cur], buf[cur ^ 1], dmeta, o->fd);
        RP_TRY(cudaGetLastError());
        cur ^= 1;
        for (auto &h : H) {
            const int nc = h.nchan / o->fd;
            std::vector<double> fn(nc, 0.);
            for (int j = 0; j < nc; j++) {
                for (int jj = 0; jj < o->fd; jj++) fn[j] += h.f[j * o->fd + jj];
                fn[j] /= o->fd;
            }
            h.f.swap(fn);
            h.nchan = nc;
        }
        RP_TRY(push_meta());
    }
    /* 12: optimize + matched_filter, or peak_search */
    std::vector<long> best(n, 0);
    long hsize = 0;
    std::vector<int> rows_h(n, 1);
    float *hb[2] = {nullptr, nullptr}, *dsnr = nullptr, *csump = nullptr, *dvwn = nullptr;
    int *dwidm = nullptr, *drows = nullptr, *dnbox = nullptr;
    if (upto >= 12) {
        std::vector<int> shifts, hranges, flip(n, 0);
        for (long b = 0; b < n; b++) {
            RpHost &h = H[b];
            h.hoff = hsize;
            if (!o->nopt) {
                const double fmx = *std::max_element(h.f.begin(), h.f.end());
                const double fmn = *std::min_element(h.f.begin(), h.f.end());
                const double tmp = rp_dmdelay(1., fmx, fmn);
                const double dmrange = (h.nbin * h.tbin) / tmp;
                h.dms = std::max(0., h.dm - dmrange / 2.);
                const double dme = h.dm + dmrange / 2.;
                h.nchans = (int)std::pow(2, std::ceil(std::log2(h.nchan)));
                h.levels = (int)std::log2(h.nchans);
                h.ddm = (dme - h.dms) / h.nchans;
                std::vector<double> fP(h.nchans, 0.);
                const double foff = h.f[1] - h.f[0];
                if (foff < 0.) {
                    for (int j = 0; j < h.nchan; j++) fP[j] = h.f[j];
                    for (int j = h.nchan; j < h.nchans; j++) fP[j] = h.f[0] + j * foff;
                } else {
                    flip[b] = 1;
                    for (int j = 0; j < h.nchan; j++) fP[j] = h.f[h.nchan - 1 - j];
                    for (int j = h.nchan; j < h.nchans; j++) fP[j] = h.f[0] + (h.nchan - 1 - j) * foff;
                }
                const double dms = h.dms, ddm = h.ddm, dm = h.dm, tbin = h.tbin;
                std::function<int(int, int, int)> gs = [&](int x0, int x1, int p) {
                    return (int)std::round(rp_dmdelay(dms + p * ddm - dm, fP[x0], fP[x1]) / tbin);
                };
                std::vector<std::vector<int>> plan;
                std::vector<int> hr;
                rp_shiftplan(plan, hr, h.nchans, (int)h.nbin, gs);
                h.soff = (long)shifts.size();
                for (auto &lv : plan) shifts.insert(shifts.end(), lv.begin(), lv.end());
                h.roff = (long)hranges.size();
                hranges.insert(hranges.end(), hr.begin(), hr.end());
                h.rows = h.nchans;
            } else {
                h.nchans = 1;
                h.levels = 0;
                h.rows = 1;
                h.dms = h.dm;
                h.ddm = 0.;
            }
            rows_h[b] = (int)h.rows;
            hsize += h.rows * h.nbin;
        }
        int *dshift, *dhr, *dflip;
        RP_TRY(mem.alloc(&hb[0], hsize));
        RP_TRY(mem.alloc(&hb[1], hsize));
        RP_TRY(mem.alloc(&dsnr, hsize));
        RP_TRY(mem.alloc(&dwidm, hsize));
        RP_TRY(mem.alloc(&csump, 2 * hsize));
        RP_TRY(mem.alloc(&dshift, shifts.size()));
        RP_TRY(mem.alloc(&dhr, hranges.size()));
        RP_TRY(mem.alloc(&dflip, n));
        RP_TRY(mem.alloc(&drows, n));
        RP_TRY(push_meta());
        if (!shifts.empty())
            RP_TRY(cudaMemcpyAsync(dshift, shifts.data(), sizeof(int) * shifts.size(), cudaMemcpyHostToDevice, st));
        if (!hranges.empty())
            RP_TRY(cudaMemcpyAsync(dhr, hranges.data(), sizeof(int) * hranges.size(), cudaMemcpyHostToDevice, st));
        RP_TRY(cudaMemcpyAsync(dflip, flip.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st));
        RP_TRY(cudaMemcpyAsync(drows, rows_h.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st));
        int hc = 0; /* which of hb holds the rows the boxcar reads */
        long maxrows_elem = 0;
        int maxlevels = 0;
        for (auto &h : H) {
            maxrows_elem = std::max(maxrows_elem, h.rows * h.nbin);
            maxlevels = std::max(maxlevels, h.levels);
        }
        if (!o->nopt) {
            k_rp_hough_fill<<<dim3(nblk(maxrows_elem, 256), NB), 256, 0, st>>>(buf[cur], hb[0], dmeta, dflip);
            for (int t = 0; t < maxlevels; t++) {
                k_rp_hough_level<<<dim3(nblk(maxrows_elem, 256), NB), 256, 0, st>>>(hb[hc], hb[hc ^ 1], dmeta, dshift, t);
                hc ^= 1;
            }
            k_rp_hough_perm<<<dim3(nblk(maxrows_elem, 256), NB), 256, 0, st>>>(hb[hc], hb[hc ^ 1], dmeta, dhr);
            hc ^= 1;
        } else {
            k_rp_profile<<<dim3(nblk(maxnbin, 128), NB), 128, 0, st>>>(buf[cur], hb[0], dmeta);
        }
        RP_TRY(cudaGetLastError());
        /* boxcar width ladder of matched_filter / peak_search (:979-993), a float vector */
        const float wfactor = (float)(1. / ((1. - o->snrloss) * (1. - o->snrloss)));
        long wstride = 1;
        std::vector<std::vector<float>> lads(n);
        for (long b = 0; b < n; b++) {
            std::vector<float> &v = lads[b];
            v.push_back(1);
            while (true) {
                int w1 = (int)v.back();
                int w2 = (int)(w1 * wfactor);
                w2 = w2 < w1 + 1 ? w1 + 1 : w2;
                if (w2 > H[b].nbin / 2) break;
                v.push_back((float)w2);
            }
            wstride = std::max(wstride, (long)v.size());
        }
        std::vector<float> lad_h((size_t)n * wstride, 0.f);
        std::vector<int> nbox_h(n);
        for (long b = 0; b < n; b++) {
            std::copy(lads[b].begin(), lads[b].end(), lad_h.begin() + b * wstride);
            nbox_h[b] = (int)lads[b].size();
        }
        RP_TRY(mem.alloc(&dvwn, lad_h.size()));
        RP_TRY(mem.alloc(&dnbox, n));
        RP_TRY(cudaMemcpyAsync(dvwn, lad_h.data(), sizeof(float) * lad_h.size(), cudaMemcpyHostToDevice, st));
        RP_TRY(cudaMemcpyAsync(dnbox, nbox_h.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st));
        int maxrows = *std::max_element(rows_h.begin(), rows_h.end());
        k_rp_boxcar<<<dim3(nblk(maxrows, 64), NB), 64, 0, st>>>(hb[hc], dmeta, drows, dvwn, dnbox, wstride,
                                                                dsnr, dwidm, csump);
        long *dbest;
        RP_TRY(mem.alloc(&dbest, n));
        k_rp_argmax<<<NB, 256, 0, st>>>(dsnr, dmeta, drows, dbest);
        RP_TRY(cudaGetLastError());
        RP_TRY(cudaMemcpyAsync(best.data(), dbest, sizeof(long) * n, cudaMemcpyDeviceToHost, st));
        RP_TRY(cudaStreamSynchronize(st));
        for (long b = 0; b < n; b++) {
            const RpHost &h = H[b];
            float S = 0.f;
            int wn = 0;
            RP_TRY(cudaMemcpy(&S, dsnr + h.hoff + best[b], sizeof(float), cudaMemcpyDeviceToHost));
            RP_TRY(cudaMemcpy(&wn, dwidm + h.hoff + best[b], sizeof(int), cudaMemcpyDeviceToHost));
            const long maxdmid = best[b] / h.nbin, maxtid = best[b] % h.nbin;
            out[b].snr = S;
            out[b].width = (float)(wn * h.tbin);
            out[b].dm_maxsnr = o->nopt ? h.dm : h.dms + maxdmid * h.ddm;
            out[b].maxtid = maxtid;
            out[b].ndm = (int)h.rows;
            out[b].dms = h.dms;
            out[b].ddm = h.ddm;
        }
        if (snrmap) {
            long pos = 0;
            for (long b = 0; b < n && pos < snrmap_cap; b++) {
                const long cnt = std::min(H[b].rows * H[b].nbin, (long)snrmap_cap - pos);
                RP_TRY(cudaMemcpy(snrmap + pos, dsnr + H[b].hoff, sizeof(float) * cnt, cudaMemcpyDeviceToHost));
                pos += cnt;
            }
        }
    }
    for (long b = 0; b < n; b++) {
        out[b].nbin = H[b].nbin;
        out[b].nchan = H[b].nchan;
        if (upto < 12) {
            out[b].snr = 0.f;
            out[b].width = 0.f;
            out[b].dm_maxsnr = 0.;
            out[b].maxtid = 0;
            out[b].ndm = 0;
            out[b].dms = out[b].ddm = 0.;
        }
    }
    if (data_out) {
        RP_TRY(cudaStreamSynchronize(st));
        long pos = 0;
        for (long b = 0; b < n && pos < data_cap; b++) {
            const RpHost &h = H[b];
            const long cnt = std::min((long)h.nchan * h.nbin, (long)data_cap - pos);
            RP_TRY(cudaMemcpy2D(data_out + pos, sizeof(float) * h.nbin, buf[cur] + h.off, sizeof(float) * h.pitch,
                                sizeof(float) * h.nbin, (size_t)(cnt / h.nbin), cudaMemcpyDeviceToHost));
            pos += cnt;
        }
    }
    RP_TRY(cudaStreamSynchronize(st));
    cudaStreamDestroy(st);
#undef RP_TRY
    return TXG_OK;
}
