/*
 * txg_plan.cpp -- host planning of one ddplan row: downsampled geometry, subband
 * dedispersion tables, the boxcar width ladder and RFI parameters.  Compiled with
 * -ffp-contract=off so that every double expression rounds as written (the integer delay
 * tables must be bit-exact).
 */
#include <cmath>
#include <cstdio>

#include "txg_internal.h"

namespace txg {

/* include/candidate.h:116-119 */
double dmdelay(double dm, double fh, double fl)
{
    return 4.148741601e3 * dm * (1. / (fl * fl) - 1. / (fh * fh));
}

/* src/singlepulse/singlepulse.cpp:242-254, including its int*float truncation. */
int width_ladder(float minw, float maxw, float snrloss, double tsamp, int32_t *vwn, int cap)
{
    if (cap <= 0 || tsamp <= 0.) return 0;
    float mw = (double)minw < tsamp ? (float)tsamp : minw;
    float wfactor = (float)(1. / ((1. - (double)snrloss) * (1. - (double)snrloss)));
    int n = 0;
    vwn[n++] = (int32_t)std::round((double)mw / tsamp);
    while (n < cap) {
        int w1 = vwn[n - 1];
        int w2 = (int)((float)w1 * wfactor);
        w2 = w2 < w1 + 1 ? w1 + 1 : w2;
        if ((double)w2 * tsamp > (double)maxw) break;
        vwn[n++] = w2;
    }
    return n;
}

static void subbands(int C, int nsub, const std::vector<double> &f, std::vector<int32_t> &start,
                     std::vector<double> &fref, std::vector<double> &flow)
{
    start.resize(nsub + 1);
    for (int s = 0; s <= nsub; s++) start[s] = (int32_t)(((long)s * C + nsub - 1) / nsub);
    fref.assign(nsub, 0.);
    flow.assign(nsub, 0.);
    for (int s = 0; s < nsub; s++) {
        double hi = f[start[s]], lo = f[start[s]];
        for (int j = start[s]; j < start[s + 1]; j++) {
            hi = f[j] > hi ? f[j] : hi;
            lo = f[j] < lo ? f[j] : lo;
        }
        fref[s] = hi;
        flow[s] = lo;
    }
}

/* Largest DM group whose within-subband smearing stays within one sample,
 * group*ddm/2 * max_s dmdelay(1, fref_s, flow_s) <= tsamp, rounded down to a multiple of 8
 * when it is at least 8 (the stage-2 kernel handles 8, 16, 24 or 32 DMs of one group per CTA). */
int auto_group(int C, int nsub, const std::vector<double> &freqs, double tsamp, double ddm,
               long ndm)
{
    std::vector<int32_t> st;
    std::vector<double> fref, flow;
    subbands(C, nsub, freqs, st, fref, flow);
    double kmax = 0.;
    for (int s = 0; s < nsub; s++) {
        double k = dmdelay(1., fref[s], flow[s]);
        kmax = k > kmax ? k : kmax;
    }
    if (!(ddm * kmax > 0.)) return (int)(ndm < 1 ? 1 : (ndm > 1 << 30 ? 1 << 30 : ndm));
    double g = std::floor(2. * tsamp / (ddm * kmax));
    if (g >= 8.) g = std::floor(g / 8.) * 8.;
    if (g < 1.) g = 1.;
    if (g > (double)ndm) g = (double)ndm;
    return (int)g;
}

/* Subband count (a power of two <= C) minimising the adds per output sample,
 * C*ceil(ndm/group) + nsub*ndm; ties go to the smaller count. */
int auto_nsub(int C, const std::vector<double> &freqs, double tsamp, double ddm, long ndm)
{
    int best = 1;
    double bestcost = -1.;
    for (int p = 1; p <= C; p *= 2) {
        int g = auto_group(C, p, freqs, tsamp, ddm, ndm);
        double ngroup = (double)((ndm + g - 1) / g);
        double cost = (double)C * ngroup + (double)p * (double)ndm;
        if (bestcost < 0. || cost < bestcost) {
            bestcost = cost;
            best = p;
        }
    }
    return best;
}

static long roundup(long a, long m) { return (a + m - 1) / m * m; }

int plan_row(const txg_row &cfg, int nchans_raw, const double *freqs_raw, double tsamp_raw,
             long ndump_raw, RowPlan &P, std::string &err)
{
    char buf[256];
    if (cfg.td < 1 || cfg.fd < 1 || nchans_raw < 1 || ndump_raw < 1 || tsamp_raw <= 0.) {
        err = "td, fd, nchans, ndump and tsamp must be positive";
        return TXG_ERR_ARG;
    }
    if (ndump_raw % cfg.td != 0) {
        snprintf(buf, sizeof(buf), "ndump %ld is not a multiple of td %d", ndump_raw, cfg.td);
        err = buf;
        return TXG_ERR_ARG;
    }
    if (nchans_raw / cfg.fd < 1 || cfg.ndm < 1 || cfg.dms < 0. || cfg.ddm < 0.) {
        err = "need nchans/fd >= 1, ndm >= 1, dms >= 0, ddm >= 0";
        return TXG_ERR_ARG;
    }
    if (cfg.nrfi < 0 || cfg.nrfi > 8 || cfg.nzap < 0 || cfg.nzap > 16) {
        err = "at most 8 rfilist and 16 zaplist entries";
        return TXG_ERR_ARG;
    }
    P.cfg = cfg;
    P.C = nchans_raw / cfg.fd;
    P.N = ndump_raw / cfg.td;
    P.tsamp = tsamp_raw * cfg.td;
    P.freqs.assign(P.C, 0.);
    for (int j = 0; j < P.C; j++) {
        double s = 0.;
        for (int k = 0; k < cfg.fd; k++) s += freqs_raw[j * cfg.fd + k];
        P.freqs[j] = s / cfg.fd;
    }
    P.fmax = P.freqs[0];
    P.fmin = P.freqs[0];
    for (int j = 0; j < P.C; j++) {
        P.fmax = P.freqs[j] > P.fmax ? P.freqs[j] : P.fmax;
        P.fmin = P.freqs[j] < P.fmin ? P.freqs[j] : P.fmin;
    }
    if (!(P.fmin > 0.)) {
        err = "channel frequencies must be positive";
        return TXG_ERR_ARG;
    }
    long ndm = cfg.ndm;
    P.nsub = cfg.nsub > 0 ? (cfg.nsub < P.C ? cfg.nsub : P.C)
                          : auto_nsub(P.C, P.freqs, P.tsamp, cfg.ddm, ndm);
    P.G = cfg.dm_group > 0 ? (int)(cfg.dm_group < ndm ? cfg.dm_group : ndm)
                           : auto_group(P.C, P.nsub, P.freqs, P.tsamp, cfg.ddm, ndm);
    P.ng = (int)((ndm + P.G - 1) / P.G);
    std::vector<double> flow;
    subbands(P.C, P.nsub, P.freqs, P.sub_start, P.fref, flow);
    P.fsub.assign(P.nsub, 0.);
    for (int s = 0; s < P.nsub; s++) {
        double acc = 0.;
        for (int j = P.sub_start[s]; j < P.sub_start[s + 1]; j++) acc += P.freqs[j];
        P.fsub[s] = acc / (double)(P.sub_start[s + 1] - P.sub_start[s]);
    }
    P.d1.assign((size_t)P.ng * P.C, 0);
    P.d2.assign((size_t)ndm * P.nsub, 0);
    P.maxd1 = 0;
    P.maxd2 = 0;
    for (int g = 0; g < P.ng; g++) {
        long first = (long)g * P.G;
        long last = first + P.G < ndm ? first + P.G - 1 : ndm - 1;
        double dmc = cfg.dms + cfg.ddm * 0.5 * (double)(first + last);
        for (int s = 0; s < P.nsub; s++)
            for (int j = P.sub_start[s]; j < P.sub_start[s + 1]; j++) {
                double d = std::round(dmdelay(dmc, P.fref[s], P.freqs[j]) / P.tsamp);
                if (!(d >= 0. && d < 1e9)) {
                    err = "within-subband delay out of range";
                    return TXG_ERR_ARG;
                }
                P.d1[(size_t)g * P.C + j] = (int32_t)d;
                P.maxd1 = (long)d > P.maxd1 ? (long)d : P.maxd1;
            }
    }
    for (long k = 0; k < ndm; k++) {
        double dm = cfg.dms + (double)k * cfg.ddm;
        for (int s = 0; s < P.nsub; s++) {
            double d = std::round(dmdelay(dm, P.fmax, P.fref[s]) / P.tsamp);
            if (!(d >= 0. && d < 1e9)) {
                err = "subband delay out of range";
                return TXG_ERR_ARG;
            }
            P.d2[(size_t)k * P.nsub + s] = (int32_t)d;
            P.maxd2 = (long)d > P.maxd2 ? (long)d : P.maxd2;
        }
    }
    P.noverlap = (long)(cfg.overlap * (double)P.N);
    if (P.noverlap < 0) P.noverlap = 0;
    P.offset = (P.maxd1 + P.maxd2 + P.noverlap + P.N - 1) / P.N * P.N;
    P.nout = P.N + P.noverlap;
    P.R = roundup(P.offset + P.N, 32);
    P.H = roundup(P.maxd1, 4);
    P.ldh = roundup(P.H + P.N + 8, 32);
    P.vwn.assign(256, 0);
    int nw = width_ladder(cfg.minw, cfg.maxw, cfg.snrloss, P.tsamp, P.vwn.data(), 256);
    P.vwn.resize(nw);
    P.maxwn = nw > 0 ? P.vwn[nw - 1] : 0;
    P.bl_nw = cfg.bswidth > 0.f ? (long)std::round((double)cfg.bswidth / P.tsamp) : 0;
    P.zap_chan.clear();
    for (int j = 0; j < P.C; j++) {
        bool hit = false;
        for (int z = 0; z < cfg.nzap; z++) {
            double lo = cfg.zap[z][0] < cfg.zap[z][1] ? cfg.zap[z][0] : cfg.zap[z][1];
            double hi = cfg.zap[z][0] < cfg.zap[z][1] ? cfg.zap[z][1] : cfg.zap[z][0];
            if (P.freqs[j] >= lo && P.freqs[j] <= hi) hit = true;
        }
        if (hit) P.zap_chan.push_back(j);
    }
    P.kad_thr = cfg.threKadaneF * cfg.threKadaneF;
    P.kadT_thr = cfg.threKadaneT * cfg.threKadaneT;
    P.mask_thr = cfg.threMask;
    /* channel width of the row, for the kadaneT band limit */
    const double chbw = P.C > 1 ? std::fabs(P.freqs[1] - P.freqs[0]) : 0.;
    for (int r = 0; r < cfg.nrfi; r++) {
        const int kind = cfg.rfi_kind[r];
        if (kind == TXG_RFI_KADANEF || kind == TXG_RFI_KADANET || kind == TXG_RFI_MASK) {
            if (cfg.rfi_td[r] < 1 || cfg.rfi_fd[r] < 1) {
                err = "kadaneF/kadaneT/mask td and fd must be positive";
                return TXG_ERR_ARG;
            }
            if (kind == TXG_RFI_KADANEF)
                P.kad_wnlimit[r] = (long)(cfg.widthlimit / (P.tsamp * cfg.rfi_td[r]));
            else if (kind == TXG_RFI_KADANET) /* minimum band in downsampled channels */
                P.kad_wnlimit[r] = chbw > 0. ? (long)(cfg.bandlimitKT / (chbw * cfg.rfi_fd[r])) : 0;
        } else if (kind != TXG_RFI_ZDOT && kind != TXG_RFI_ZERO) {
            err = "unsupported rfilist entry";
            return TXG_ERR_UNSUPPORTED;
        }
    }
    return TXG_OK;
}

} // namespace txg
