/* Stand-in for the CMake-generated configuration header of the reference, used only to compile the
 * reference's GPU transform path (its CUDA kernels plus cuFFT) for the comparison timing in
 * baseline/ref_gpu_bench.cpp: CUDA backend, OpenMP and the single-precision API on; no MPI. The
 * host engine that the reference links alongside is compiled against baseline/fftw_absent and
 * never used (no SPFFT_PU_HOST transform is created). */
#ifndef SPFFT_CONFIG_H
#define SPFFT_CONFIG_H
#define SPFFT_CUDA
#define SPFFT_OMP
#define SPFFT_SINGLE_PRECISION
#define SPFFT_EXPORT __attribute__((visibility("default")))
#define SPFFT_NO_EXPORT __attribute__((visibility("hidden")))
#endif
