/* The C++ replacement of transientx_fil's block loop (dedisperse_fil.cpp:319-338) from the
 * integration guide (section 1), with the reference-side names it uses declared around it: the
 * command-line map, the reader, the .cands writer and its output stream. */
#include <fstream>
#include <string>
#include "transientx_gb300.hpp"

struct OptionValue { float v; template <class T> T as() const { return (T)v; } };
struct OptionMap { OptionValue operator[](const char *) const { return {4.f}; } };
static bool read_raw_block(uint8_t *, long) { return false; }

int run(const std::string &ddplan_text, const txgpu::SinglePulse &base_row, int nchans,
        double tsamp, const std::vector<double> &frequencies, long ndump, const OptionMap &vm,
        txgpu::CandsWriter &writer, std::ofstream &cands_file)
{
    std::vector<txgpu::SinglePulse> rows = txgpu::parse_ddplan(ddplan_text, base_row);
    txgpu::Search gpu(rows, nchans, tsamp, frequencies, ndump, /*nbeams=*/1,
                      TXG_PREC_FP32, /*flags=*/0, /*zapthre=*/vm["zapthre"].as<float>());
    std::vector<uint8_t> raw(ndump * nchans);          // 8-bit samples, time-major
    while (read_raw_block(raw.data(), ndump)) {        // the reader's bytes before float unpacking
        gpu.run(raw.data());                           // every ddplan row on this block
        gpu.sync();
        for (int r = 0; r < (int)rows.size(); r++) {
            txg_row_info info = gpu.info(r);
            if (!info.gated) continue;                 // Boxcar::run returned false (boxcar.cpp:161)
            auto candlist = gpu.cluster(r);            // Cluster<double>::candlist (cluster.cpp:145-158)
            std::vector<txg_cand> c;                   // the .cands lines of CandPlot::plot
            for (auto &t : candlist) c.push_back({(int32_t)std::get<0>(t), (int32_t)std::get<1>(t),
                                                  std::get<2>(t), std::get<3>(t)});
            std::vector<float> fl, fh;
            gpu.band(r, c, fl, fh);                    // fl/fh columns (candplot.cpp:218-231)
            for (auto &line : writer.format_block(c, info.counter, info.offset, info.ndump, info.tsamp,
                                                  info.dms, info.ddm, fl, fh, rows[r].id))
                cands_file << line;                    // writer: txgpu::CandsWriter(rootname, tstart, beam)
        }
    }
    return 0;
}
