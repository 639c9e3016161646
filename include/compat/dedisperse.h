/*
 * dedisperse.h -- the globals of the reference's include/dedisperse.h:25-29, which
 * transientx_fil defines (dedisperse_fil.cpp:34-39).  The GPU path reads none of them: its
 * parallelism is the device's.
 */
#ifndef TXG_COMPAT_DEDISPERSE_H
#define TXG_COMPAT_DEDISPERSE_H

extern unsigned int dbscan_radius;
extern unsigned int dbscan_k;
extern unsigned int num_threads;
extern bool repeater;
extern bool dumptim;

#endif
