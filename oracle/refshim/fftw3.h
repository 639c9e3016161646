/*
 * fftw3.h -- stand-in so that src/singlepulse/candidate.cpp of the reference compiles in place
 * for the parity harness.  Only the coherent-dedispersion branch uses FFTW; the harness never
 * takes it, and these stand-ins abort if it ever does.  Test infrastructure only.
 */
#ifndef TXREF_FFTW3_H
#define TXREF_FFTW3_H
#include <cstdlib>
typedef float fftwf_complex[2];
typedef struct txref_fftwf_plan_s *fftwf_plan;
#define FFTW_ESTIMATE 0u
inline int fftwf_init_threads() { return 1; }
inline void fftwf_plan_with_nthreads(int) {}
inline void fftwf_cleanup_threads() {}
inline fftwf_plan fftwf_plan_dft_r2c_1d(int, float *, fftwf_complex *, unsigned) { std::abort(); }
inline fftwf_plan fftwf_plan_dft_c2r_1d(int, fftwf_complex *, float *, unsigned) { std::abort(); }
inline void fftwf_execute_dft_r2c(fftwf_plan, float *, fftwf_complex *) { std::abort(); }
inline void fftwf_execute_dft_c2r(fftwf_plan, fftwf_complex *, float *) { std::abort(); }
inline void fftwf_destroy_plan(fftwf_plan) {}
#endif
