/* transientx_fil's block loop (dedisperse_fil.cpp:319-338) over the class-compatible headers
 * of include/compat/: the ddplan is parsed by parse(vm, search1), every row is prepared on the
 * first block's shape, and each block read from a raw 8-bit filterbank (time-major
 * [nsamples][nchans], no header) goes through PreprocessLite and every row's
 * SinglePulse::run, which searches it on the GPU and appends the row's candidates to the
 * .cands file.  Patch (its fill defaults to none, a no-op) is left out.
 *
 *   fil_loop <raw file> <nchans> <tsamp> <fch1> <foff> <ndump> <ddplan file> <rootname>
 *
 * prints each searched block's candidate list: "cand <row id> <counter> <idm> <isamp> <wn> <S>" */
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "compat/preprocesslite.h"
#include "compat/singlepulse.h"

unsigned int dbscan_radius = 4;
unsigned int dbscan_k = 2;
unsigned int num_threads = 1;
bool repeater = false;
bool dumptim = false;

/* a variables map of string values with the interface parse() reads */
struct OptionValue {
    std::string s;
    template <class T> T as() const
    {
        std::istringstream in(s);
        T v{};
        in >> v;
        return v;
    }
};
template <> std::string OptionValue::as<std::string>() const { return s; }
template <> std::vector<float> OptionValue::as<std::vector<float>>() const
{
    std::istringstream in(s);
    std::vector<float> v;
    for (float x; in >> x;) v.push_back(x);
    return v;
}
template <> std::vector<std::string> OptionValue::as<std::vector<std::string>>() const
{
    std::istringstream in(s);
    std::vector<std::string> v;
    for (std::string x; in >> x;) v.push_back(x);
    return v;
}
struct VariablesMap {
    std::map<std::string, std::string> m;
    OptionValue operator[](const char *k) const
    {
        auto it = m.find(k);
        return {it == m.end() ? std::string() : it->second};
    }
    size_t count(const char *k) const { return m.count(k); }
};

/* the reader: 8-bit samples unpacked to float, as the filterbank reader fills databuf */
struct RawReader {
    FILE *f = nullptr;
    int nchans = 0;
    bool is_end = false;
    std::vector<uint8_t> tmp;
    long int read_data(DataBuffer<float> &db, long int ndump)
    {
        tmp.resize((size_t)ndump * nchans);
        const size_t got = std::fread(tmp.data(), (size_t)nchans, (size_t)ndump, f);
        if (got < (size_t)ndump) is_end = true;
        for (size_t i = 0; i < got * (size_t)nchans; i++) db.buffer[i] = (float)tmp[i];
        return (long int)got;
    }
};

int main(int argc, char **argv)
{
    if (argc < 9) {
        std::fprintf(stderr, "usage: fil_loop raw nchans tsamp fch1 foff ndump ddplan rootname\n");
        return 2;
    }
    RawReader reader;
    reader.f = std::fopen(argv[1], "rb");
    if (!reader.f) return 2;
    reader.nchans = std::atoi(argv[2]);
    const double tsamp = std::atof(argv[3]), fch1 = std::atof(argv[4]), foff = std::atof(argv[5]);
    const long int ndump = std::atol(argv[6]);

    VariablesMap vm;
    vm.m = {{"baseline", "0 0.1"}, {"fill", "mean"}, {"bandlimit", "10"}, {"bandlimitKT", "10"},
            {"widthlimit", "0.01"}, {"threMask", "10"}, {"threKadaneF", "7"},
            {"threKadaneT", "7"}, {"dms", "0"}, {"ddm", "1"}, {"ndm", "1000"}, {"overlap", "0"},
            {"minw", "0.0001"}, {"snrloss", "0.1"}, {"maxw", "0.02"}, {"thre", "7"},
            {"radius", "1"}, {"neighbors", "2"}, {"maxncand", "100"}, {"minpts", "5"},
            {"mean", "0"}, {"std", "0"}, {"nbits", "8"}, {"format", "sigproc"},
            {"ddplan", argv[7]}};
    std::vector<SinglePulse> search1;
    parse(vm, search1);
    std::string fname = argv[1];

    DataBuffer<float> databuf(ndump, reader.nchans);
    databuf.tsamp = tsamp;
    for (int j = 0; j < reader.nchans; j++) databuf.frequencies[j] = fch1 + j * foff;
    PreprocessLite prep;
    prep.prepare(databuf);
    for (auto sp = search1.begin(); sp != search1.end(); ++sp) {
        (*sp).rootname = argv[8];
        (*sp).compat_nsub = 16;
        (*sp).prepare(prep);
    }

    while (!reader.is_end) {
        if (reader.read_data(databuf, ndump) != ndump) break;
        databuf.counter += ndump;
        prep.run(databuf);
        for (auto sp = search1.begin(); sp != search1.end(); ++sp) {
            prep.isbusy = true;
            (*sp).fileid = 1;
            (*sp).fname = fname;
            (*sp).verbose = false;
            (*sp).run(prep);
            if ((*sp).cluster.counter == (*sp).boxcar.counter && (*sp).boxcar.counter > 0)
                for (auto &c : (*sp).cluster.candlist)
                    std::printf("cand %d %ld %ld %ld %d %.7g\n", (*sp).id, (*sp).boxcar.counter,
                                std::get<0>(c), std::get<1>(c), std::get<2>(c), (double)std::get<3>(c));
        }
    }
    std::fclose(reader.f);
    return 0;
}
