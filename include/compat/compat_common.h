/*
 * compat_common.h -- shared by the class-compatible headers of include/compat/: the C ABI,
 * and the reference's error behaviour (log the error, then exit(-1), as
 * singlepulse.cpp:414-415 does) for every failing call.
 */
#ifndef TXG_COMPAT_COMMON_H
#define TXG_COMPAT_COMMON_H

#include <cstdio>
#include <cstdlib>
#include <string>

#include "../transientx_gb300.h"

namespace txg_compat {

/* A failing call logs "[error] <what>: <reason>" to stderr and ends the process with -1.
 * TXG_ERR_OVERFLOW (points beyond the candidate capacity) only logs a warning: the block's
 * first cand_capacity points were kept. */
inline void check(int rc, const char *what)
{
    if (rc == TXG_OK) return;
    if (rc == TXG_ERR_OVERFLOW) {
        std::fprintf(stderr, "[warning] %s: %s\n", what, txg_strerror(rc));
        return;
    }
    std::fprintf(stderr, "[error] %s: %s\n", what, txg_strerror(rc));
    std::exit(-1);
}

/* The GPU row a dedispersion object is bound to by SinglePulse::prepare. */
struct Binding {
    txg_handle *h = nullptr;
    int beam = 0, row = 0;
    bool dense = false;
};

} // namespace txg_compat

#endif
