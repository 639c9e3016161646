/*
 * archivewriter_tx.h -- stand-in for the PSRFITS archive writer used by Candidate::save2ar,
 * so that the reference's candidate.cpp compiles in place; it writes nothing.
 * Test infrastructure only.
 */
#ifndef TXREF_ARCHIVEWRITER_H
#define TXREF_ARCHIVEWRITER_H
#include <string>
#include <vector>
struct MJD {
    MJD() {}
    template <class T> MJD(T) {}
};
namespace Integration {
enum Mode { FOLD, SEARCH };
}
namespace TransientX {
struct ArchiveWriter {
    int npol = 0, nchan = 0, nbin = 0, ibeam = 0;
    Integration::Mode mode = Integration::FOLD;
    std::string template_file, rootname, src_name, ra, dec;
    MJD start_mjd;
    double dm = 0.;
    std::vector<double> frequencies;
    void prepare() {}
    template <class... A> void run(A &&...) {}
    void close() {}
};
} // namespace TransientX
#endif
