/*
 * databuffer.h -- the members of XLibs' DataBuffer<T> that the single-pulse path reads: a
 * time-major block buffer[nsamples][nchans] (replot_fil.cpp:359, ringbuffer.h:33-38 of the
 * reference), its sample counter, sampling time and channel frequencies.  XLibs itself is
 * not part of the reference tree; this stand-in carries the data between a reader and
 * SinglePulse::run.
 */
#ifndef TXG_COMPAT_DATABUFFER_H
#define TXG_COMPAT_DATABUFFER_H

#include <vector>

template <typename T>
class DataBuffer {
public:
    DataBuffer() = default;
    DataBuffer(long int ns, int nc) { resize(ns, nc); }
    virtual ~DataBuffer() = default;

    void resize(long int ns, int nc)
    {
        nsamples = ns;
        nchans = nc;
        buffer.assign((size_t)ns * (size_t)nc, T());
        if ((int)frequencies.size() != nc) frequencies.assign((size_t)nc, 0.);
    }
    /* takes the shape and axes of another buffer (the role of the XLibs prepare calls) */
    void prepare(DataBuffer<T> &db)
    {
        tsamp = db.tsamp;
        frequencies = db.frequencies;
        resize(db.nsamples, db.nchans);
    }

public:
    long int counter = 0;
    double tsamp = 0.;
    long int nsamples = 0;
    int nchans = 0;
    std::vector<double> frequencies;
    std::vector<T> buffer;
    bool isbusy = false;
    bool closable = false;
};

#endif
