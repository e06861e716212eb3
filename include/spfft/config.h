/* Build configuration of the GB300 SpFFT library (hand-written; the reference generates this file
 * from CMake, include/spfft/config.h.in). This library always has the CUDA backend and the
 * single-precision API, and never MPI. */
#ifndef SPFFT_CONFIG_H
#define SPFFT_CONFIG_H

#define SPFFT_CUDA
#define SPFFT_SINGLE_PRECISION
/* SPFFT_MPI is intentionally not defined: the distributed slab/pencil path is not part of this
 * library. */

#if defined(_WIN32)
#define SPFFT_EXPORT
#define SPFFT_NO_EXPORT
#else
#define SPFFT_EXPORT __attribute__((visibility("default")))
#define SPFFT_NO_EXPORT __attribute__((visibility("hidden")))
#endif

#endif
