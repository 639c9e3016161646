/*
 * logging.h -- stand-in for the reference's Boost.Log macro: messages are discarded.
 * Test infrastructure only.
 */
#ifndef TXREF_LOGGING_H
#define TXREF_LOGGING_H
#include <iostream>
#define BOOST_LOG_TRIVIAL(level) \
    if (true) {                   \
    } else                        \
        std::cerr
#endif
