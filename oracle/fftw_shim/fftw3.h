/* FFTW-3 API subset written for this project (test infrastructure only). It lets the reference's
 * host transform path (src/fft/fftw_interface.hpp:42-100, src/fft/fftw_plan_1d.hpp:86-139) compile
 * and run where FFTW itself is not installed: the functions the reference calls, with FFTW 3's
 * published signatures and semantics (rank-1 plans over `howmany` strided sequences, complex,
 * real-to-complex and complex-to-real; sign -1 forward, +1 backward; unnormalised), computed by the
 * mixed-radix DFT of fftw_shim.cpp. Nothing of FFTW's implementation is used or restated. */
#ifndef SPFFT_ORACLE_FFTW_SHIM_H
#define SPFFT_ORACLE_FFTW_SHIM_H

#ifdef __cplusplus
extern "C" {
#endif

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)

typedef double fftw_complex[2];
typedef float fftwf_complex[2];
typedef struct shim_plan_s* fftw_plan;
typedef struct shim_plan_s* fftwf_plan;

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
