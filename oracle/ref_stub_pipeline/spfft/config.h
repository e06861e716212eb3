/* Stand-in for the CMake-generated configuration header of the reference, used only to compile the
 * reference's host transform path (FFTW replaced by oracle/fftw_shim) on the host: OpenMP and the
 * single-precision API on; no GPU backend, no MPI. */
#ifndef SPFFT_CONFIG_H
#define SPFFT_CONFIG_H
#define SPFFT_OMP
#define SPFFT_SINGLE_PRECISION
#define SPFFT_EXPORT __attribute__((visibility("default")))
#define SPFFT_NO_EXPORT __attribute__((visibility("hidden")))
#endif
