/*
 * boxcar.h -- class Boxcar with the public interface of the reference's include/boxcar.h:17-43,
 * over the GPU search of transientx_gb300.h.
 *
 * run() reports the block the bound GPU row last searched: whether it produced boxcar output
 * (the gate of boxcar.cpp:160-161) and the members Cluster::run and CandPlot::plot read.  The
 * GPU feeds clustering from its compacted S > thre points, so the dense mxS / mxwn planes
 * are only filled when the row keeps them (SinglePulse::compat_dense); otherwise they stay
 * null.  match() scores one DM trial of the last block on the GPU (txg_boxcar) into those
 * planes.  match2D, marked "not work" in the reference (boxcar.cpp:298), scores like match.
 */
#ifndef TXG_COMPAT_BOXCAR_H
#define TXG_COMPAT_BOXCAR_H

#include <algorithm>
#include <cstdio>
#include <string>
#include <utility>
#include <vector>

#include "compat_common.h"
#include "dedisperse.h"
#include "subdedispersion.h"

using std::string;
using std::vector;

class Boxcar {
public:
    Boxcar() = default;
    Boxcar(const Boxcar &b) { *this = b; }
    Boxcar &operator=(const Boxcar &b)
    {
        if (this == &b) return *this;
        counter = b.counter;
        tsamp = b.tsamp;
        nsamples = b.nsamples;
        dms = b.dms;
        ddm = b.ddm;
        ndm = b.ndm;
        maxwn = b.maxwn;
        fmin = b.fmin;
        fmax = b.fmax;
        finterval = b.finterval;
        gpu_ = b.gpu_;
        release();
        if (b.mxS) {
            resize(b.nsamples, b.ndm);
            std::copy(b.mxS, b.mxS + (size_t)ndm * nsamples, mxS);
            std::copy(b.mxwn, b.mxwn + (size_t)ndm * nsamples, mxwn);
        }
        return *this;
    }
    ~Boxcar() { release(); }

    /* sizes from the dedispersion (boxcar.cpp:142-156) */
    void prepare(RealTime::SubbandDedispersion &dedisp)
    {
        gpu_ = dedisp.gpu;
        dedisp.refresh();
        txg_row_info i;
        txg_compat::check(txg_get_row_info(gpu_.h, gpu_.beam, gpu_.row, &i), "Boxcar::prepare");
        counter = 0;
        tsamp = i.tsamp;
        nsamples = (long int)i.nsamples;
        dms = i.dms;
        ddm = i.ddm;
        ndm = (long int)i.ndm;
        maxwn = i.maxwn;
        fmin = i.fmin;
        fmax = i.fmax;
        if (gpu_.dense) resize(nsamples, ndm);
    }
    void resize(long int nt, long int nd)
    {
        release();
        mxS = new float[(size_t)nt * (size_t)nd]();
        mxwn = new int[(size_t)nt * (size_t)nd]();
    }
    /* the last block of the bound row: true when it produced boxcar output */
    bool run(RealTime::SubbandDedispersion &dedisp, vector<int> &vwn, bool iqr = false)
    {
        (void)vwn;
        (void)iqr; /* both were fixed when the row was planned */
        gpu_ = dedisp.gpu;
        dedisp.refresh();
        txg_row_info i;
        txg_compat::check(txg_get_row_info(gpu_.h, gpu_.beam, gpu_.row, &i), "Boxcar::run");
        counter = (long int)i.counter;
        if (!i.gated) return false;
        if (gpu_.dense && mxS)
            txg_compat::check(txg_get_dense(gpu_.h, gpu_.beam, gpu_.row, mxS, mxwn), "Boxcar::run");
        return true;
    }
    /* Boxcar::match of one DM trial of the last block (boxcar.cpp:166-296) into row idm of
     * mxS / mxwn */
    void match(int idm, vector<int> &vwn, RealTime::SubbandDedispersion &dedisp, bool iqr)
    {
        vector<float> tim;
        dedisp.get_timdata(tim, idm, true);
        if (!mxS) resize(nsamples, ndm);
        int64_t n = 0;
        txg_compat::check(txg_boxcar(tim.data(), 1, (int64_t)tim.size(), vwn.data(),
                                     (int32_t)vwn.size(), iqr ? 1 : 0, 0, 0.f,
                                     mxS + (size_t)idm * nsamples, mxwn + (size_t)idm * nsamples,
                                     nullptr, 0, &n),
                          "Boxcar::match");
    }
    void match2D(int idm, vector<int> &vwn, RealTime::SubbandDedispersion &dedisp)
    {
        match(idm, vwn, dedisp, false);
    }
    /* mxS as text, one line per DM trial, each value "%f " (boxcar.cpp:473-489) */
    void dump2txt(const string fname) const
    {
        if (!mxS) {
            std::fprintf(stderr, "[error] Boxcar::dump2txt: no dense mxS\n");
            std::exit(-1);
        }
        FILE *f = std::fopen(fname.c_str(), "w");
        if (!f) {
            std::fprintf(stderr, "[error] Boxcar::dump2txt: cannot open %s\n", fname.c_str());
            std::exit(-1);
        }
        const float *p = mxS;
        for (long int j = 0; j < ndm; j++) {
            for (long int i = 0; i < nsamples; i++) std::fprintf(f, "%f ", *p++);
            std::fprintf(f, "\n");
        }
        std::fclose(f);
    }

    /* the GPU row behind this object (for Cluster::run) */
    const txg_compat::Binding &gpu() const { return gpu_; }

public:
    long int counter = 0;
    double tsamp = 0.;
    long int nsamples = 0;
    double dms = 0.;
    double ddm = 0.;
    long int ndm = 0;
    int maxwn = 0;
    double fmin = 0.;
    double fmax = 0.;
    float *mxS = nullptr;
    int *mxwn = nullptr;
    vector<vector<std::pair<int, int>>> finterval;

private:
    void release()
    {
        delete[] mxS;
        delete[] mxwn;
        mxS = nullptr;
        mxwn = nullptr;
    }
    txg_compat::Binding gpu_;
};

#endif
