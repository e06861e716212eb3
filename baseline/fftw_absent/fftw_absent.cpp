// Definitions behind fftw3.h for a process that runs the reference's GPU path only: planners
// return no plan (the reference turns that into its FFTW error), executing aborts. Neither is
// reached when only SPFFT_PU_GPU transforms are created.
#include "fftw3.h"

#include <cstdio>
#include <cstdlib>

namespace {
[[noreturn]] void absent(const char* what) {
  std::fprintf(stderr, "%s: FFTW is not available in the GPU comparison build\n", what);
  std::abort();
}
}  // namespace

extern "C" {
fftw_plan fftw_plan_dft_1d(int, fftw_complex*, fftw_complex*, int, unsigned) { return nullptr; }
fftw_plan fftw_plan_many_dft(int, const int*, int, fftw_complex*, const int*, int, int, fftw_complex*,
                             const int*, int, int, int, unsigned) { return nullptr; }
fftw_plan fftw_plan_many_dft_r2c(int, const int*, int, double*, const int*, int, int, fftw_complex*,
                                 const int*, int, int, unsigned) { return nullptr; }
fftw_plan fftw_plan_many_dft_c2r(int, const int*, int, fftw_complex*, const int*, int, int, double*,
                                 const int*, int, int, unsigned) { return nullptr; }
void fftw_execute(const fftw_plan) { absent("fftw_execute"); }
void fftw_execute_dft(const fftw_plan, fftw_complex*, fftw_complex*) { absent("fftw_execute_dft"); }
void fftw_execute_dft_r2c(const fftw_plan, double*, fftw_complex*) { absent("fftw_execute_dft_r2c"); }
void fftw_execute_dft_c2r(const fftw_plan, fftw_complex*, double*) { absent("fftw_execute_dft_c2r"); }
void fftw_destroy_plan(fftw_plan) {}
int fftw_alignment_of(double*) { return 0; }

fftwf_plan fftwf_plan_dft_1d(int, fftwf_complex*, fftwf_complex*, int, unsigned) { return nullptr; }
fftwf_plan fftwf_plan_many_dft(int, const int*, int, fftwf_complex*, const int*, int, int, fftwf_complex*,
                               const int*, int, int, int, unsigned) { return nullptr; }
fftwf_plan fftwf_plan_many_dft_r2c(int, const int*, int, float*, const int*, int, int, fftwf_complex*,
                                   const int*, int, int, unsigned) { return nullptr; }
fftwf_plan fftwf_plan_many_dft_c2r(int, const int*, int, fftwf_complex*, const int*, int, int, float*,
                                   const int*, int, int, unsigned) { return nullptr; }
void fftwf_execute(const fftwf_plan) { absent("fftwf_execute"); }
void fftwf_execute_dft(const fftwf_plan, fftwf_complex*, fftwf_complex*) { absent("fftwf_execute_dft"); }
void fftwf_execute_dft_r2c(const fftwf_plan, float*, fftwf_complex*) { absent("fftwf_execute_dft_r2c"); }
void fftwf_execute_dft_c2r(const fftwf_plan, fftwf_complex*, float*) { absent("fftwf_execute_dft_c2r"); }
void fftwf_destroy_plan(fftwf_plan) {}
int fftwf_alignment_of(float*) { return 0; }
}
