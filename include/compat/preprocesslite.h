/*
 * preprocesslite.h -- a pass-through PreprocessLite with the calls transientx_fil makes
 * (dedisperse_fil.cpp:264-276,329: prepare, run, isbusy).  The reference's PreprocessLite
 * (XLibs, not in its tree) downsamples by --td/--fd, zaps channels by skewness and kurtosis and
 * normalises; this stand-in hands the reader's block on unchanged.  A caller with XLibs keeps
 * the real one: SinglePulse::run takes whatever DataBuffer<float> it produces.
 */
#ifndef TXG_COMPAT_PREPROCESSLITE_H
#define TXG_COMPAT_PREPROCESSLITE_H

#include <string>

#include "databuffer.h"

class PreprocessLite : public DataBuffer<float> {
public:
    void prepare(DataBuffer<float> &db) { DataBuffer<float>::prepare(db); }
    DataBuffer<float> *run(DataBuffer<float> &db)
    {
        counter = db.counter;
        buffer = db.buffer;
        return this;
    }
    int td = 1, fd = 1;
    float thresig = 3.f;
    std::string filltype = "mean";
};

#endif
