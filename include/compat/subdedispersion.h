/*
 * subdedispersion.h -- RealTime::SubbandDedispersion with the members and methods the
 * reference's single-pulse code uses (singlepulse.cpp:230-238,328,338; boxcar.cpp:144-183;
 * candplot.cpp:47,122-123,143-153; cluster.cpp:102).  The dedispersion itself runs on the GPU
 * inside the handle that SinglePulse::prepare creates: this object describes that row
 * (geometry after prepare, counter after each block) and reads its series back.
 */
#ifndef TXG_COMPAT_SUBDEDISPERSION_H
#define TXG_COMPAT_SUBDEDISPERSION_H

#include <string>
#include <vector>

#include "compat_common.h"
#include "databuffer.h"

namespace RealTime {

class SubbandDedispersion {
public:
    struct Sub {
        int nchans = 0;
        double tsamp = 0.;
        std::vector<double> frequencies;
    };

    /* the channel axis of the blocks that will arrive */
    void prepare(DataBuffer<float> &databuffer)
    {
        nchans = databuffer.nchans;
        tsamp = databuffer.tsamp;
        frequencies = databuffer.frequencies;
    }
    /* the block reaches the GPU through SinglePulse::run; only the geometry is refreshed */
    void run(DataBuffer<float> &databuffer, long int ns)
    {
        (void)databuffer;
        (void)ns;
        refresh();
    }
    void cache() {}

    /* get_timdata(tim, idm, true): the series of DM idm of the last block, nsamples long
     * (boxcar.cpp:183) */
    void get_timdata(std::vector<float> &tim, long int idm, bool = true) const
    {
        tim.assign((size_t)nsamples, 0.f);
        txg_compat::check(txg_get_timdata(gpu.h, gpu.beam, gpu.row, idm, 1, tim.data()),
                          "SubbandDedispersion::get_timdata");
    }
    /* get_subdata(sub, idm, true): the subband series of DM idm, [nsub][nsamples]
     * (candplot.cpp:123) */
    void get_subdata(std::vector<float> &subdata, long int idm, bool = true) const
    {
        subdata.assign((size_t)sub.nchans * (size_t)nsamples, 0.f);
        txg_compat::check(txg_get_subdata(gpu.h, gpu.beam, gpu.row, idm, subdata.data()),
                          "SubbandDedispersion::get_subdata");
    }

    /* the dispersion delay (s) between frequencies fh and fl (MHz), constant of
     * candidate.h:116-119 */
    static double dmdelay(double dm, double fh, double fl)
    {
        return 4.148741601e3 * dm * (1. / (fl * fl) - 1. / (fh * fh));
    }

    /* geometry and counter of the bound row (after prepare and after every block) */
    void refresh()
    {
        if (!gpu.h) return;
        txg_row_info i;
        txg_compat::check(txg_get_row_info(gpu.h, gpu.beam, gpu.row, &i), "SubbandDedispersion");
        counter = (long int)i.counter;
        offset = (long int)i.offset;
        noverlap = (long int)i.noverlap;
        ndump = (long int)i.ndump;
        nsamples = (long int)i.nsamples;
        tsamp = i.tsamp;
        sub.nchans = i.nsub;
        sub.tsamp = i.tsamp;
    }

public:
    /* configuration (singlepulse.cpp:230-235) */
    double dms = 0.;
    double ddm = 1.;
    long int ndm = 0;
    double overlap = 0.;
    long int ndump = 0;
    std::string rootname;
    /* geometry */
    long int counter = 0;
    long int offset = 0;
    long int noverlap = 0;
    long int nsamples = 0;
    double tsamp = 0.;
    int nchans = 0;
    std::vector<double> frequencies;
    Sub sub;
    /* the GPU row serving this object */
    txg_compat::Binding gpu;
};

} // namespace RealTime

#endif
