/* Stand-in for the CMake-generated configuration header of the reference, used only to compile the
 * reference's index planner (src/parameters/parameters.cpp) and its test index generator on the
 * host: no GPU backend, no MPI, no OpenMP. */
#ifndef SPFFT_CONFIG_H
#define SPFFT_CONFIG_H
#define SPFFT_EXPORT __attribute__((visibility("default")))
#define SPFFT_NO_EXPORT __attribute__((visibility("hidden")))
#endif
