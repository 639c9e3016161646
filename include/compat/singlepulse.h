/*
 * singlepulse.h -- class SinglePulse with the public interface of the reference's
 * include/singlepulse.h:29-117 (members, defaults of singlepulse.cpp:18-68), backed by the GPU
 * search of transientx_gb300.h: one SinglePulse is one ddplan row and owns one GPU handle.
 *
 *   prepare(DataBuffer<float>&)  plans the row for blocks of databuffer's shape
 *                                (SinglePulse::prepare, singlepulse.cpp:206-284): the GPU
 *                                handle, the width ladder vwn and nbox, Boxcar::prepare
 *   run(DataBuffer<float>&)      one block (singlepulse.cpp:287-341): downsample, equalize,
 *                                baseline, zaplist, rfilist, dedispersion and the boxcar on the
 *                                GPU (txg_push_block_f32), then Boxcar::run, Cluster::run and
 *                                CandPlot::plot as the reference chains them
 *   parse / parse_json           the reference's option and JSON parsers, over any
 *                                variables-map type with operator[](key).as<T>() and count(key)
 *                                (boost::program_options::variables_map) and any JSON type with
 *                                operator[], iteration and conversion (nlohmann::json)
 *
 * The components the reference runs on the CPU (Downsample, Equalize, BaseLine, RFI) are
 * empty stand-ins here: their work happens inside the GPU handle.  Errors log and exit(-1)
 * as the reference does.  savetim (the series dump) is not served by this layer: use
 * txg_get_timdata_q, or transientx_gb300.timdump from Python.
 */
#ifndef TXG_COMPAT_SINGLEPULSE_H
#define TXG_COMPAT_SINGLEPULSE_H

#include <cctype>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <utility>
#include <vector>

#include "boxcar.h"
#include "candplot.h"
#include "cluster.h"
#include "compat_common.h"
#include "databuffer.h"
#include "subdedispersion.h"

/* stand-ins for the XLibs stages that run inside the GPU handle */
struct Downsample { int td = 1, fd = 1; };
struct Equalize {};
struct BaseLine { float width = 0.f; };
struct RFI { std::string filltype = "mean"; };
struct Filterbank {};

class SinglePulse {
public:
    SinglePulse() = default;
    SinglePulse(const SinglePulse &) = default;
    SinglePulse &operator=(const SinglePulse &) = default;
    ~SinglePulse() = default;

    void prepare(DataBuffer<float> &databuffer)
    {
        txg_row row = to_row();
        txg_plan plan{};
        plan.nchans = databuffer.nchans;
        plan.tsamp = databuffer.tsamp;
        plan.frequencies = databuffer.frequencies.data();
        plan.ndump = databuffer.nsamples;
        plan.nrows = 1;
        plan.rows = &row;
        plan.nbeams = 1;
        plan.precision = compat_precision;
        plan.flags = TXG_FLAG_KEEP_SERIES | (compat_dense ? TXG_FLAG_DENSE : 0) |
                     (compat_avx2_tail ? TXG_FLAG_AVX2_TAIL : 0);
        plan.zapthre = 0.f; /* a float block arrives after PreprocessLite's channel zap */
        txg_handle *h = nullptr;
        txg_compat::check(txg_create(&plan, &h), "SinglePulse::prepare");
        gpu_.reset(h, txg_destroy);

        downsample.td = td;
        downsample.fd = fd;
        baseline.width = bswidth;
        rfi.filltype = filltype;
        dedisp.dms = dms;
        dedisp.ddm = ddm;
        dedisp.ndm = ndm;
        dedisp.overlap = overlap;
        dedisp.rootname = rootname;
        dedisp.prepare(databuffer);
        dedisp.gpu.h = h;
        dedisp.gpu.dense = compat_dense;
        dedisp.refresh();
        fill_sub_frequencies(databuffer);
        boxcar.prepare(dedisp);

        /* the width ladder (singlepulse.cpp:242-254) */
        minw = minw < boxcar.tsamp ? (float)boxcar.tsamp : minw;
        vwn.assign(256, 0);
        const int n = txg_width_ladder(minw, maxw, snrloss, boxcar.tsamp, vwn.data(), 256);
        vwn.resize(n > 0 ? (size_t)n : 0);
        nbox = (int)vwn.size();
        if (obsinfo.find("Beam") == obsinfo.end()) {
            char b[32];
            std::snprintf(b, sizeof(b), "%s%05d", incoherent ? "ifbf" : "cfbf", ibeam);
            obsinfo["Beam"] = b;
        }
        obsinfo["Source_name"] = source_name;
        obsinfo["Telescope"] = telescope;
    }

    void run(DataBuffer<float> &databuffer)
    {
        txg_handle *h = gpu_.get();
        if (!h) {
            std::fprintf(stderr, "[error] SinglePulse::run before prepare\n");
            std::exit(-1);
        }
        txg_compat::check(txg_push_block_f32(h, 0, databuffer.buffer.data(), databuffer.nsamples),
                          "SinglePulse::run");
        txg_compat::check(txg_sync(h), "SinglePulse::run");
        dedisp.run(databuffer, databuffer.nsamples);
        if (boxcar.run(dedisp, vwn, iqr)) {
            if (cluster.run(boxcar, thre, radius_smearing, kvalue, maxncand, minpts,
                            remove_cand_with_maxwidth))
                candplot.plot(cluster, boxcar, dedisp, (double)tstart, thre, rootname, id, fileid,
                              fname, obsinfo, saveimage, white);
        }
        dedisp.cache();
        if (savetim) {
            std::fprintf(stderr, "[error] SinglePulse::run: savetim is not served by this layer\n");
            std::exit(-1);
        }
    }

public:
    /* components */
    Downsample downsample;
    Equalize equalize;
    BaseLine baseline;
    RFI rfi;
    RealTime::SubbandDedispersion dedisp;
    Boxcar boxcar;
    Cluster<double> cluster;
    CandPlot candplot;

    /* downsample */
    int td = 1;
    int fd = 1;
    /* baseline */
    float bswidth = 0.f;
    /* rfi */
    std::vector<std::pair<double, double>> zaplist;
    std::vector<std::vector<std::string>> rfilist;
    double bandlimit = 10.;
    double bandlimitKT = 10.;
    double widthlimit = 10e-3;
    float threKadaneT = 7.f;
    float threKadaneF = 7.f;
    float threMask = 7.f;
    std::string filltype = "mean";
    /* dedisperse */
    double dms = 0.;
    double ddm = 1.;
    long int ndm = 1000;
    double overlap = 0.;
    /* boxcar */
    float minw = 1e-4f;
    float maxw = 2e-2f;
    float snrloss = 0.1f;
    int nbox = 0;
    bool iqr = false;
    std::vector<int> vwn;
    /* cluster */
    float thre = 7.f;
    double radius_smearing = 0.003;
    int kvalue = 2;
    int maxncand = 100;
    int minpts = 0;
    bool remove_cand_with_maxwidth = false;
    /* candplot */
    long double tstart = 0;
    int ibeam = 1;
    double src_raj = 0.;
    double src_dej = 0.;
    std::string source_name;
    std::string rootname;
    int id = 1;
    std::string telescope;
    bool saveimage = false;
    bool white = false;

    int fileid = 1;
    std::string fname;
    bool incoherent = false;

    bool verbose = false;

    float outmean = 0.f;
    float outstd = 0.f;
    int outnbits = 0;
    bool savetim = false;
    std::string format;

    Filterbank fildedisp;

    std::map<std::string, std::string> obsinfo;

    /* GPU-side choices with no reference counterpart: subband storage (TXG_PREC_*), keeping
     * the dense mxS / mxwn planes for Boxcar's readers, the -mavx2 build's boxcar tail
     * (boxcar.cpp:264-279), and the subband count and DM group (0 = automatic) */
    int compat_precision = TXG_PREC_FP32;
    bool compat_dense = false;
    bool compat_avx2_tail = false;
    int compat_nsub = 0;
    int compat_dm_group = 0;

private:
    txg_row to_row() const
    {
        txg_row r{};
        r.td = td;
        r.fd = fd;
        r.bswidth = bswidth;
        if (rfilist.size() > 8 || zaplist.size() > 16) {
            std::fprintf(stderr, "[error] SinglePulse: at most 8 rfilist and 16 zaplist entries\n");
            std::exit(-1);
        }
        r.nrfi = (int32_t)rfilist.size();
        for (size_t i = 0; i < rfilist.size(); i++) {
            const auto &op = rfilist[i];
            const bool three = op.size() >= 3;
            if (op[0] == "kadaneF" && three) r.rfi_kind[i] = TXG_RFI_KADANEF;
            else if (op[0] == "kadaneT" && three) r.rfi_kind[i] = TXG_RFI_KADANET;
            else if (op[0] == "mask" && three) r.rfi_kind[i] = TXG_RFI_MASK;
            else if (op[0] == "zdot") r.rfi_kind[i] = TXG_RFI_ZDOT;
            else if (op[0] == "zero") r.rfi_kind[i] = TXG_RFI_ZERO;
            else {
                std::fprintf(stderr, "[error] SinglePulse: rfilist entry %s\n", op[0].c_str());
                std::exit(-1);
            }
            r.rfi_td[i] = three ? std::stoi(op[1]) : 1;
            r.rfi_fd[i] = three ? std::stoi(op[2]) : 1;
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
        r.nsub = compat_nsub;
        r.dm_group = compat_dm_group;
        r.radius_smearing = radius_smearing;
        r.maxncand = maxncand;
        r.minpts = minpts;
        r.drop = remove_cand_with_maxwidth ? 1 : 0;
        return r;
    }
    /* dedisp.sub.frequencies: each subband's mean channel frequency */
    void fill_sub_frequencies(const DataBuffer<float> &db)
    {
        txg_row_info i;
        txg_compat::check(txg_get_row_info(gpu_.get(), 0, 0, &i), "SinglePulse::prepare");
        std::vector<int32_t> d1((size_t)i.ngroup * i.nchans), d2((size_t)i.ndm * i.nsub),
            ss((size_t)i.nsub + 1), w(256);
        txg_compat::check(txg_get_tables(gpu_.get(), 0, d1.data(), d2.data(), ss.data(), w.data()),
                          "SinglePulse::prepare");
        dedisp.sub.frequencies.assign((size_t)i.nsub, 0.);
        for (int s = 0; s < i.nsub; s++) {
            double acc = 0.;
            for (int j = ss[s]; j < ss[s + 1]; j++) {
                double f = 0.;
                for (int k = 0; k < fd; k++) f += db.frequencies[(size_t)j * fd + k];
                acc += f / fd;
            }
            dedisp.sub.frequencies[s] = ss[s + 1] > ss[s] ? acc / (ss[s + 1] - ss[s]) : 0.;
        }
    }
    std::shared_ptr<txg_handle> gpu_;
};

/* rfi option words of a ddplan line or of the rfi option (singlepulse.cpp:350-372,432-451);
 * an rfilist entry of the JSON configuration takes no zap (singlepulse.cpp:525-540) */
inline void txg_compat_rfi_words(const std::vector<std::string> &w, size_t i, SinglePulse &sp,
                                 bool zap = true)
{
    for (; i < w.size(); i++) {
        if ((w[i] == "mask" || w[i] == "kadaneF" || w[i] == "kadaneT") && i + 2 < w.size()) {
            sp.rfilist.push_back({w[i], w[i + 1], w[i + 2]});
            i += 2;
        } else if (zap && w[i] == "zap" && i + 2 < w.size()) {
            sp.zaplist.emplace_back(std::stod(w[i + 1]), std::stod(w[i + 2]));
            i += 2;
        } else if (w[i] == "zero" || w[i] == "zdot") {
            sp.rfilist.push_back({w[i]});
        }
    }
}

/* parse(vm, search) of singlepulse.cpp:343-459: the command-line options into one row, or
 * with --ddplan one row per ddplan line ("td fd dms ddm ndm snrloss maxw [rfi words]").  As in
 * the reference one SinglePulse is carried down the lines, so a line's zap and rfi words stay
 * in the zaplist and rfilist of every later row. */
template <class VariablesMap>
void parse(VariablesMap &vm, std::vector<SinglePulse> &search)
{
    SinglePulse sp;
    sp.bswidth = vm["baseline"].template as<std::vector<float>>().back();
    if (vm.count("rfi"))
        txg_compat_rfi_words(vm["rfi"].template as<std::vector<std::string>>(), 0, sp);
    sp.filltype = vm["fill"].template as<std::string>();
    sp.bandlimit = vm["bandlimit"].template as<double>();
    sp.bandlimitKT = vm["bandlimitKT"].template as<double>();
    sp.widthlimit = vm["widthlimit"].template as<double>();
    sp.threMask = vm["threMask"].template as<float>();
    sp.threKadaneF = vm["threKadaneF"].template as<float>();
    sp.threKadaneT = vm["threKadaneT"].template as<float>();
    sp.dms = vm["dms"].template as<double>();
    sp.ddm = vm["ddm"].template as<double>();
    sp.ndm = vm["ndm"].template as<int>();
    sp.overlap = vm["overlap"].template as<double>();
    sp.minw = vm["minw"].template as<float>();
    sp.snrloss = vm["snrloss"].template as<float>();
    sp.maxw = vm["maxw"].template as<float>();
    sp.iqr = vm.count("iqr");
    sp.thre = vm["thre"].template as<float>();
    sp.radius_smearing = vm["radius"].template as<double>() / 1000.;
    sp.kvalue = (int)vm["neighbors"].template as<unsigned int>();
    sp.maxncand = vm["maxncand"].template as<int>();
    sp.minpts = vm["minpts"].template as<int>();
    sp.remove_cand_with_maxwidth = vm.count("drop");
    sp.incoherent = vm.count("incoherent");
    sp.outmean = vm["mean"].template as<float>();
    sp.outstd = vm["std"].template as<float>();
    sp.outnbits = vm["nbits"].template as<int>();
    sp.savetim = vm.count("savetim");
    sp.format = vm["format"].template as<std::string>();
    if (!vm.count("ddplan")) {
        sp.id = 1;
        search.push_back(sp);
        return;
    }
    const std::string filename = vm["ddplan"].template as<std::string>();
    std::ifstream ddplan(filename);
    if (ddplan.fail()) {
        std::fprintf(stderr, "[error] %s not exist\n", filename.c_str());
        std::exit(-1);
    }
    int id = 0;
    std::string line;
    while (std::getline(ddplan, line)) {
        const size_t a = line.find_first_not_of(" \t\r");
        if (a == std::string::npos || !std::isdigit((unsigned char)line[a])) continue;
        std::istringstream ls(line.substr(a));
        std::vector<std::string> p;
        for (std::string w; ls >> w;) p.push_back(w);
        if (p.size() < 7) continue;
        sp.td = std::stoi(p[0]);
        sp.fd = std::stoi(p[1]);
        sp.dms = std::stod(p[2]);
        sp.ddm = std::stod(p[3]);
        sp.ndm = std::stol(p[4]);
        sp.snrloss = std::stof(p[5]);
        sp.maxw = std::stof(p[6]);
        txg_compat_rfi_words(p, 7, sp);
        sp.id = ++id;
        search.push_back(sp);
    }
}

/* parse_json(vm, config, search) of singlepulse.cpp:461-545: one row per entry of
 * config["ddplan"]; as in the reference one SinglePulse is carried down the entries, so an
 * entry's zaplist and rfilist stay in every later row's */
template <class VariablesMap, class Json>
void parse_json(VariablesMap &vm, Json &config, std::vector<SinglePulse> &search)
{
    SinglePulse sp;
    sp.incoherent = vm.count("incoherent");
    sp.outmean = vm["mean"].template as<float>();
    sp.outstd = vm["std"].template as<float>();
    sp.outnbits = vm["nbits"].template as<int>();
    sp.savetim = vm.count("savetim");
    sp.format = vm["format"].template as<std::string>();
    int id = 0;
    auto rows = config["ddplan"];
    for (auto c = rows.begin(); c != rows.end(); ++c) {
        auto ds = (*c)["downsample"], bl = (*c)["baseline"], rf = (*c)["rfi"];
        auto dd = (*c)["subdedispersion"], bx = (*c)["boxcar"], cl = (*c)["clustering"];
        sp.td = ds["td"];
        sp.fd = ds["fd"];
        sp.bswidth = bl["width"];
        sp.dms = dd["dms"];
        sp.ddm = dd["ddm"];
        sp.ndm = dd["ndm"];
        sp.overlap = dd["overlap"];
        sp.bandlimit = rf["bandlimit"];
        sp.bandlimitKT = rf["bandlimitKT"];
        sp.widthlimit = rf["widthlimit"];
        sp.threMask = rf["threMask"];
        sp.threKadaneF = rf["threKadaneF"];
        sp.threKadaneT = rf["threKadaneT"];
        sp.minw = bx["minw"];
        sp.snrloss = bx["snrloss"];
        sp.maxw = bx["maxw"];
        sp.iqr = bx["iqr"];
        sp.thre = cl["thre"];
        sp.radius_smearing = (double)(cl["radius"]) / 1000.;
        sp.kvalue = cl["neighbors"];
        sp.maxncand = cl["maxncand"];
        sp.minpts = cl["minpts"];
        sp.remove_cand_with_maxwidth = cl["drop"];
        auto zl = rf["zaplist"];
        for (auto z = zl.begin(); z != zl.end(); ++z)
            sp.zaplist.emplace_back((double)z->front(), (double)z->back());
        auto rl = rf["rfilist"];
        for (auto e = rl.begin(); e != rl.end(); ++e) {
            std::vector<std::string> w;
            for (auto item = e->begin(); item != e->end(); ++item) w.push_back(*item);
            txg_compat_rfi_words(w, 0, sp, false);
        }
        sp.id = ++id;
        search.push_back(sp);
    }
}

#endif
