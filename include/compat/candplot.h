/*
 * candplot.h -- CandPlot with the public interface of the reference's include/candplot.h:
 * plot() appends one line per reported candidate to <rootname>_<tstart>_<beam>.cands in the
 * reference's format and order (candplot.cpp:32-433: descending S/N, stable; beam, running
 * number, MJD, DM, width in ms, S/N, fl, fh, plot name, row id, file name).  fl and fh come
 * from the GPU row's subband data (txg_cand_band).  No image is drawn: the line names the
 * PNG the reference would have written.
 */
#ifndef TXG_COMPAT_CANDPLOT_H
#define TXG_COMPAT_CANDPLOT_H

#include <algorithm>
#include <fstream>
#include <iomanip>
#include <map>
#include <numeric>
#include <sstream>
#include <string>
#include <tuple>
#include <vector>

#include "boxcar.h"
#include "cluster.h"
#include "compat_common.h"
#include "subdedispersion.h"

class CandPlot {
public:
    CandPlot() = default;
    ~CandPlot() = default;

    void plot(const Cluster<double> &cluster, const Boxcar &boxcar,
              const RealTime::SubbandDedispersion &dedisp, double tstart, float threS,
              const std::string &rootname, int id, int fileid, std::string &fname,
              std::map<std::string, std::string> &obsinfo, bool saveimage = false,
              bool white = false)
    {
        (void)threS;
        (void)fileid;
        (void)saveimage;
        (void)white;
        const auto &cl = cluster.candlist;
        const long int ncand = (long int)cl.size();
        if (ncand == 0) return;
        std::vector<size_t> idx(cl.size());
        std::iota(idx.begin(), idx.end(), 0);
        std::stable_sort(idx.begin(), idx.end(), [&cl](size_t a, size_t b) {
            return std::get<3>(cl[a]) > std::get<3>(cl[b]);
        });
        std::vector<txg_cand> c(cl.size());
        for (size_t k = 0; k < cl.size(); k++)
            c[k] = {(int32_t)std::get<0>(cl[k]), (int32_t)std::get<1>(cl[k]), std::get<2>(cl[k]),
                    std::get<3>(cl[k])};
        std::vector<float> fl(c.size()), fh(c.size());
        const txg_compat::Binding &g = boxcar.gpu();
        txg_compat::check(txg_cand_band(g.h, g.beam, g.row, c.data(), (int64_t)c.size(),
                                        fl.data(), fh.data()),
                          "CandPlot::plot");
        const std::string s_ibeam = obsinfo["Beam"];
        const std::string s_date = fixed(tstart, 10);
        std::ostringstream sid;
        sid << std::setw(2) << std::setfill('0') << id;
        std::ofstream out(rootname + "_" + s_date + "_" + s_ibeam + ".cands", std::ios_base::app);
        const double bmjd =
            tstart + (-dedisp.offset + boxcar.counter - dedisp.ndump) * boxcar.tsamp / 86400.;
        for (long int i = 0; i < ncand; i++) {
            const size_t k = idx[(size_t)i];
            const long int idm = std::get<0>(cl[k]), isamp = std::get<1>(cl[k]);
            const int wn = std::get<2>(cl[k]);
            const float snr = std::get<3>(cl[k]);
            const double mjd =
                tstart + (-dedisp.offset + boxcar.counter - dedisp.ndump + isamp) * boxcar.tsamp / 86400.;
            std::ostringstream sk;
            sk << std::setw(2) << std::setfill('0') << i + 1;
            const std::string basename =
                rootname + "_" + fixed(bmjd, 10) + "_" + s_ibeam + "_" + sk.str() + "_" + sid.str();
            out << s_ibeam << "\t" << ++num_cand << "\t" << fixed(mjd, 15) << "\t"
                << fixed(boxcar.dms + idm * boxcar.ddm, 2) << "\t" << fixed(wn * boxcar.tsamp * 1000, 2)
                << "\t" << fixed(snr, 1) << "\t" << fixed(fl[k], 0) << "\t" << fixed(fh[k], 0) << "\t"
                << basename + ".png" << "\t" << sid.str() << "\t" << fname << std::endl;
        }
    }

public:
    static long int num_cand;

private:
    static std::string fixed(double v, int prec)
    {
        std::ostringstream o;
        o << std::setprecision(prec) << std::fixed << v;
        return o.str();
    }
};

/* the running candidate number of the .cands lines (candplot.cpp:26) */
inline long int CandPlot::num_cand = 0;

#endif
