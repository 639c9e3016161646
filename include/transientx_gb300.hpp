/*
 * transientx_gb300.hpp -- header-only C++ layer over the C ABI (transientx_gb300.h) with the
 * host-side shapes of the reference's classes for the single-pulse path:
 *   txgpu::SinglePulse  - the per-ddplan-row configuration members of SinglePulse
 *                         (include/singlepulse.h:95-133, defaults singlepulse.cpp:18-65)
 *   txgpu::parse_ddplan - ddplan rows "td fd dms ddm ndm snrloss maxw [rfi opts]"
 *                         (singlepulse.cpp:407-456)
 *   txgpu::Search       - prepare (SinglePulse::prepare, singlepulse.cpp:206-254) for all rows,
 *                         run(block) (the block-loop body, dedisperse_fil.cpp:324-337) on 8-bit
 *                         or preprocessed float blocks, reset(beam) between observations
 *   txgpu::Search::cluster - Cluster<double>::run's candlist (cluster.cpp:63-161) as
 *                         (idm, isamp, wn, S) tuples, the order CandPlot::plot consumes
 *   txgpu::Boxcar       - the public members of Boxcar (include/boxcar.h:31-43) for one row
 *                         after its last block (Search::boxcar), with dump2txt
 * Errors from the C ABI become txgpu::Error exceptions on the C++ side only.
 */
#ifndef TRANSIENTX_GB300_HPP
#define TRANSIENTX_GB300_HPP

#include <algorithm>
#include <cctype>
#include <cstdio>
#include <sstream>
#include <stdexcept>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include "transientx_gb300.h"

namespace txgpu {

struct Error : std::runtime_error {
    int status;
    Error(int s, const std::string &what) : std::runtime_error(what), status(s) {}
};

inline void check(int rc, const char *what)
{
    if (rc != TXG_OK) throw Error(rc, std::string(what) + ": " + txg_strerror(rc));
}

struct SinglePulse {
    int td = 1, fd = 1;
    float bswidth = 0.1f;
    std::vector<std::pair<double, double>> zaplist;
    std::vector<std::vector<std::string>> rfilist;
    double widthlimit = 50e-3;
    float threKadaneF = 7.f;
    float threMask = 10.f, threKadaneT = 7.f; /* CLI defaults, dedisperse_fil.cpp:79-83 */
    double bandlimitKT = 10.;
    double dms = 0., ddm = 1.;
    long ndm = 200;
    double overlap = 0.;
    float minw = 1e-4f, maxw = 0.02f, snrloss = 0.1f;
    bool iqr = false;
    float thre = 7.f;
    double radius_smearing = 1e-3;
    int kvalue = 2, maxncand = 100, minpts = 5;
    bool remove_cand_with_maxwidth = false;
    int nsub = 0, dm_group = 0;
    int id = 1;

    txg_row to_c() const
    {
        txg_row r{};
        r.td = td;
        r.fd = fd;
        r.bswidth = bswidth;
        if (rfilist.size() > 8 || zaplist.size() > 16) throw Error(TXG_ERR_ARG, "too many rfi entries");
        r.nrfi = (int32_t)rfilist.size();
        for (size_t i = 0; i < rfilist.size(); i++) {
            const auto &op = rfilist[i];
            if (op[0] == "kadaneF" && op.size() >= 3) {
                r.rfi_kind[i] = TXG_RFI_KADANEF;
                r.rfi_td[i] = std::stoi(op[1]);
                r.rfi_fd[i] = std::stoi(op[2]);
            } else if (op[0] == "zdot") {
                r.rfi_kind[i] = TXG_RFI_ZDOT;
                r.rfi_td[i] = r.rfi_fd[i] = 1;
            } else if ((op[0] == "mask" || op[0] == "kadaneT") && op.size() >= 3) {
                r.rfi_kind[i] = op[0] == "mask" ? TXG_RFI_MASK : TXG_RFI_KADANET;
                r.rfi_td[i] = std::stoi(op[1]);
                r.rfi_fd[i] = std::stoi(op[2]);
            } else if (op[0] == "zero") {
                r.rfi_kind[i] = TXG_RFI_ZERO;
                r.rfi_td[i] = r.rfi_fd[i] = 1;
            } else {
                throw Error(TXG_ERR_UNSUPPORTED, "rfilist entry " + op[0] + " is not implemented");
            }
        }
        r.nzap = (int32_t)zaplist.size();
        for (size_t i = 0; i < zaplist.size(); i++) {
            r.zap[i][0] = zaplist[i].first;
            r.zap[i][1] = zaplist[i].second;
        }
        r.threKadaneF = threKadaneF;
        r.widthlimit = widthlimit;
        r.threMask = threMask;
        r.threKadaneT = threKadaneT;
        r.bandlimitKT = bandlimitKT;
        r.dms = dms;
        r.ddm = ddm;
        r.ndm = ndm;
        r.overlap = overlap;
        r.minw = minw;
        r.maxw = maxw;
        r.snrloss = snrloss;
        r.iqr = iqr ? 1 : 0;
        r.thre = thre;
        r.nsub = nsub;
        r.dm_group = dm_group;
        r.radius_smearing = radius_smearing;
        r.maxncand = maxncand;
        r.minpts = minpts;
        r.drop = remove_cand_with_maxwidth ? 1 : 0;
        return r;
    }
};

/* rfi options of one ddplan line or of the -z command-line option */
inline void parse_rfi(const std::vector<std::string> &t, size_t i, SinglePulse &sp)
{
    while (i < t.size()) {
        if ((t[i] == "mask" || t[i] == "kadaneF" || t[i] == "kadaneT") && i + 2 < t.size()) {
            sp.rfilist.push_back({t[i], t[i + 1], t[i + 2]});
            i += 3;
        } else if (t[i] == "zap" && i + 2 < t.size()) {
            sp.zaplist.emplace_back(std::stod(t[i + 1]), std::stod(t[i + 2]));
            i += 3;
        } else if (t[i] == "zero" || t[i] == "zdot") {
            sp.rfilist.push_back({t[i]});
            i += 1;
        } else {
            i += 1;
        }
    }
}

inline std::vector<SinglePulse> parse_ddplan(const std::string &text, SinglePulse sp = SinglePulse())
{
    std::vector<SinglePulse> rows;
    std::istringstream in(text);
    std::string line;
    int id = 0;
    while (std::getline(in, line)) {
        size_t a = line.find_first_not_of(" \t\r");
        if (a == std::string::npos || !std::isdigit((unsigned char)line[a])) continue;
        std::istringstream ls(line.substr(a));
        std::vector<std::string> t;
        for (std::string w; ls >> w;) t.push_back(w);
        if (t.size() < 7) continue;
        sp.td = std::stoi(t[0]);
        sp.fd = std::stoi(t[1]);
        sp.dms = std::stod(t[2]);
        sp.ddm = std::stod(t[3]);
        sp.ndm = std::stol(t[4]);
        sp.snrloss = std::stof(t[5]);
        sp.maxw = std::stof(t[6]);
        parse_rfi(t, 7, sp);
        sp.id = ++id;
        rows.push_back(sp);
    }
    return rows;
}

/* The .cands lines of CandPlot::plot (candplot.cpp:32-433): one per reported candidate of a
 * block, descending S/N (stable), columns beam, running number, MJD, DM, width (ms), S/N,
 * fl, fh, plot name, row id, input file name.  The plot is not produced. */
class CandsWriter {
public:
    CandsWriter(std::string rootname, double tstart, std::string beam = "0", std::string fname = "")
        : root_(std::move(rootname)), beam_(std::move(beam)), fname_(std::move(fname)), tstart_(tstart)
    {
    }
    /* <rootname>_<tstart, 10 decimals>_<beam>.cands (candplot.cpp:420) */
    std::string filename() const { return root_ + "_" + fixed(tstart_, 10) + "_" + beam_ + ".cands"; }

    std::vector<std::string> format_block(const std::vector<txg_cand> &c, long counter, long offset,
                                          long ndump, double tsamp, double dms, double ddm,
                                          const std::vector<float> &fl, const std::vector<float> &fh,
                                          int row_id)
    {
        std::vector<size_t> idx(c.size());
        for (size_t k = 0; k < idx.size(); k++) idx[k] = k;
        std::stable_sort(idx.begin(), idx.end(), [&](size_t a, size_t b) { return c[a].S > c[b].S; });
        char sid[16];
        snprintf(sid, sizeof(sid), "%02d", row_id);
        const double bmjd = tstart_ + (-offset + counter - ndump) * tsamp / 86400.;
        std::vector<std::string> lines;
        for (size_t i = 0; i < idx.size(); i++) {
            const txg_cand &x = c[idx[i]];
            const double mjd = tstart_ + (-offset + counter - ndump + (long)x.isamp) * tsamp / 86400.;
            char sk[16];
            snprintf(sk, sizeof(sk), "%02d", (int)(i + 1));
            const std::string base = root_ + "_" + fixed(bmjd, 10) + "_" + beam_ + "_" + sk + "_" + sid;
            std::ostringstream o;
            o << beam_ << "\t" << ++num_cand_ << "\t" << fixed(mjd, 15) << "\t"
              << fixed(dms + (long)x.idm * ddm, 2) << "\t" << fixed(x.wn * tsamp * 1000, 2) << "\t"
              << fixed(x.S, 1) << "\t" << fixed(fl[idx[i]], 0) << "\t" << fixed(fh[idx[i]], 0) << "\t"
              << base << ".png\t" << sid << "\t" << fname_ << "\n";
            lines.push_back(o.str());
        }
        return lines;
    }
    long count() const { return num_cand_; }

private:
    static std::string fixed(double v, int prec)
    {
        char b[64];
        snprintf(b, sizeof(b), "%.*f", prec, v);
        return b;
    }
    std::string root_, beam_, fname_;
    double tstart_;
    long num_cand_ = 0;
};

/* The public members of the reference's Boxcar (include/boxcar.h:31-43) for one (row, beam)
 * after its last block, as Search::boxcar fills them.  mxS / mxwn are the dense
 * [ndm][nsamples] planes when the plan has TXG_FLAG_DENSE and stay empty otherwise (the GPU
 * path feeds clustering from the compacted points instead); gated is what Boxcar::run
 * returned (boxcar.cpp:160-161).  finterval and match2D (marked "not work",
 * boxcar.cpp:298) are not carried. */
struct Boxcar {
    long counter = 0;
    double tsamp = 0.;
    long nsamples = 0;
    double dms = 0., ddm = 0.;
    long ndm = 0;
    int maxwn = 0;
    double fmin = 0., fmax = 0.;
    std::vector<float> mxS;
    std::vector<int> mxwn;
    bool gated = false;

    /* mxS as text, one line per DM trial, each value printed "%f " (boxcar.cpp:473-489) */
    void dump2txt(const std::string &fname) const
    {
        if (mxS.size() != (size_t)ndm * (size_t)nsamples)
            throw Error(TXG_ERR_STATE, "dump2txt: no dense mxS (plan without TXG_FLAG_DENSE)");
        FILE *f = std::fopen(fname.c_str(), "w");
        if (!f) throw Error(TXG_ERR_ARG, "dump2txt: cannot open " + fname);
        const float *p = mxS.data();
        for (long j = 0; j < ndm; j++) {
            for (long i = 0; i < nsamples; i++) std::fprintf(f, "%f ", *p++);
            std::fprintf(f, "\n");
        }
        std::fclose(f);
    }
};

class Search {
public:
    Search(const std::vector<SinglePulse> &rows, int nchans, double tsamp,
           const std::vector<double> &freqs, long ndump, int nbeams = 1, int precision = TXG_PREC_FP32,
           int flags = 0, float zapthre = 4.f)
        : rows_(rows)
    {
        std::vector<txg_row> c;
        for (const auto &r : rows) c.push_back(r.to_c());
        txg_plan p{};
        p.nchans = nchans;
        p.tsamp = tsamp;
        p.frequencies = freqs.data();
        p.ndump = ndump;
        p.nrows = (int32_t)c.size();
        p.rows = c.data();
        p.nbeams = nbeams;
        p.precision = precision;
        p.flags = flags;
        p.zapthre = zapthre;
        check(txg_create(&p, &h_), "txg_create");
        ndump_ = ndump;
        flags_ = flags;
    }
    ~Search() { txg_destroy(h_); }
    Search(const Search &) = delete;
    Search &operator=(const Search &) = delete;

    /* one block of raw 8-bit samples [ndump][nchans] */
    void run(const uint8_t *block, int beam = 0) { push(txg_push_block(h_, beam, block, ndump_)); }
    void run_device(const uint8_t *dev_block, int beam = 0)
    {
        push(txg_push_block_device(h_, beam, dev_block, ndump_));
    }
    /* one preprocessed float block [ndump][nchans] (txg_push_block_f32) */
    void run_f32(const float *block, int beam = 0) { push(txg_push_block_f32(h_, beam, block, ndump_)); }
    /* the next block pushed to `beam` starts a new observation (txg_reset_beam) */
    void reset(int beam = 0) { check(txg_reset_beam(h_, beam), "txg_reset_beam"); }
    /* {stage-1 shape, stage-2 variant, stage-2 KB} of a row (txg_get_launch_shape) */
    std::tuple<int, int, int> launch_shape(int row) const
    {
        int32_t a = 0, b = 0, c = 0;
        check(txg_get_launch_shape(h_, row, &a, &b, &c), "txg_get_launch_shape");
        return std::make_tuple(a, b, c);
    }
    void sync() { push(txg_sync(h_)); }

    txg_row_info info(int row, int beam = 0) const
    {
        txg_row_info i;
        check(txg_get_row_info(h_, beam, row, &i), "txg_get_row_info");
        return i;
    }

    std::vector<txg_cand> candidates(int row, int beam = 0) const
    {
        int64_t n = 0;
        txg_get_candidates(h_, beam, row, nullptr, 0, &n);
        std::vector<txg_cand> out((size_t)n);
        int rc = txg_get_candidates(h_, beam, row, out.data(), n, &n);
        if (rc != TXG_OK && rc != TXG_ERR_OVERFLOW) check(rc, "txg_get_candidates");
        out.resize(std::min<size_t>(out.size(), (size_t)n));
        return out;
    }

    /* Cluster<double>::run candlist of the row's last block */
    std::vector<std::tuple<long, long, int, float>> cluster(int row, int beam = 0) const
    {
        const txg_row_info i = info(row, beam);
        const SinglePulse &sp = rows_[row];
        std::vector<txg_cand> c = candidates(row, beam);
        std::vector<txg_cand> out(std::max(1, sp.maxncand));
        int64_t n = 0;
        check(txg_cluster(c.data(), (int64_t)c.size(), i.dms, i.ddm, i.fmax, i.fmin, i.tsamp,
                          sp.radius_smearing, sp.maxncand, sp.minpts,
                          sp.remove_cand_with_maxwidth ? 1 : 0, i.maxwn, out.data(),
                          (int64_t)out.size(), &n),
              "txg_cluster");
        std::vector<std::tuple<long, long, int, float>> list;
        for (int64_t k = 0; k < n; k++) list.emplace_back(out[k].idm, out[k].isamp, out[k].wn, out[k].S);
        return list;
    }

    /* Boxcar's members for the row's last block; the dense planes with TXG_FLAG_DENSE */
    Boxcar boxcar(int row, int beam = 0) const
    {
        const txg_row_info i = info(row, beam);
        Boxcar b;
        b.counter = (long)i.counter;
        b.tsamp = i.tsamp;
        b.nsamples = (long)i.nsamples;
        b.dms = i.dms;
        b.ddm = i.ddm;
        b.ndm = (long)i.ndm;
        b.maxwn = i.maxwn;
        b.fmin = i.fmin;
        b.fmax = i.fmax;
        b.gated = i.gated != 0;
        if (flags_ & TXG_FLAG_DENSE) {
            b.mxS.resize((size_t)i.ndm * (size_t)i.nsamples);
            b.mxwn.resize(b.mxS.size());
            check(txg_get_dense(h_, beam, row, b.mxS.data(), b.mxwn.data()), "txg_get_dense");
        }
        return b;
    }

    /* fl, fh of each candidate of the row's last block (for CandsWriter) */
    void band(int row, const std::vector<txg_cand> &c, std::vector<float> &fl, std::vector<float> &fh,
              int beam = 0) const
    {
        fl.assign(c.size(), 0.f);
        fh.assign(c.size(), 0.f);
        check(txg_cand_band(h_, beam, row, c.data(), (int64_t)c.size(), fl.data(), fh.data()),
              "txg_cand_band");
    }

    txg_handle *handle() const { return h_; }

private:
    void push(int rc)
    {
        if (rc != TXG_OK && rc != TXG_ERR_OVERFLOW) check(rc, "txg_push_block");
    }
    std::vector<SinglePulse> rows_;
    txg_handle *h_ = nullptr;
    long ndump_ = 0;
    int flags_ = 0;
};

} // namespace txgpu

#endif /* TRANSIENTX_GB300_HPP */
