/* Declarations of the FFTW 3 functions that the reference's host transform engine calls
 * (src/fft/fftw_interface.hpp:42-100, src/fft/fftw_plan_1d.hpp:86-139), with FFTW 3's published
 * signatures, so that the reference library compiles where FFTW is not installed. The GPU
 * comparison timing (ref_gpu_bench.cpp) creates GPU transforms only, and the reference constructs
 * its host engine only for SPFFT_PU_HOST transforms, so none of these is ever called there; the
 * definitions in fftw_absent.cpp return no plan and abort if executed. */
#ifndef SPFFT_BASELINE_FFTW_ABSENT_H
#define SPFFT_BASELINE_FFTW_ABSENT_H

#ifdef __cplusplus
extern "C" {
#endif

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)

typedef double fftw_complex[2];
typedef float fftwf_complex[2];
typedef struct absent_plan_s* fftw_plan;
typedef struct absent_plan_s* fftwf_plan;

fftw_plan fftw_plan_dft_1d(int n, fftw_complex* in, fftw_complex* out, int sign, unsigned flags);
fftw_plan fftw_plan_many_dft(int rank, const int* n, int howmany, fftw_complex* in, const int* inembed,
                             int istride, int idist, fftw_complex* out, const int* onembed, int ostride,
                             int odist, int sign, unsigned flags);
fftw_plan fftw_plan_many_dft_r2c(int rank, const int* n, int howmany, double* in, const int* inembed,
                                 int istride, int idist, fftw_complex* out, const int* onembed,
                                 int ostride, int odist, unsigned flags);
fftw_plan fftw_plan_many_dft_c2r(int rank, const int* n, int howmany, fftw_complex* in,
                                 const int* inembed, int istride, int idist, double* out,
                                 const int* onembed, int ostride, int odist, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_execute_dft(const fftw_plan p, fftw_complex* in, fftw_complex* out);
void fftw_execute_dft_r2c(const fftw_plan p, double* in, fftw_complex* out);
void fftw_execute_dft_c2r(const fftw_plan p, fftw_complex* in, double* out);
void fftw_destroy_plan(fftw_plan p);
int fftw_alignment_of(double* p);

fftwf_plan fftwf_plan_dft_1d(int n, fftwf_complex* in, fftwf_complex* out, int sign, unsigned flags);
fftwf_plan fftwf_plan_many_dft(int rank, const int* n, int howmany, fftwf_complex* in, const int* inembed,
                               int istride, int idist, fftwf_complex* out, const int* onembed,
                               int ostride, int odist, int sign, unsigned flags);
fftwf_plan fftwf_plan_many_dft_r2c(int rank, const int* n, int howmany, float* in, const int* inembed,
                                   int istride, int idist, fftwf_complex* out, const int* onembed,
                                   int ostride, int odist, unsigned flags);
fftwf_plan fftwf_plan_many_dft_c2r(int rank, const int* n, int howmany, fftwf_complex* in,
                                   const int* inembed, int istride, int idist, float* out,
                                   const int* onembed, int ostride, int odist, unsigned flags);
void fftwf_execute(const fftwf_plan p);
void fftwf_execute_dft(const fftwf_plan p, fftwf_complex* in, fftwf_complex* out);
void fftwf_execute_dft_r2c(const fftwf_plan p, float* in, fftwf_complex* out);
void fftwf_execute_dft_c2r(const fftwf_plan p, fftwf_complex* in, float* out);
void fftwf_destroy_plan(fftwf_plan p);
int fftwf_alignment_of(float* p);

#ifdef __cplusplus
}
#endif

#endif
