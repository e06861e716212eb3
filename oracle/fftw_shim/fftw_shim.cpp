// Implementation of the FFTW-3 API subset of fftw3.h -- test infrastructure only, linked into the
// reference's host pipeline under oracle/_ref and never into the library.
//
// Every plan is a rank-1 transform of length n over `howmany` sequences (element stride, sequence
// distance). The DFT itself is the textbook recursive decimation in time over the prime factors of
// n: a length-n transform is p transforms of length n/p over the decimated sequences, combined by
// X[k + q m] = sum_r w_n^{r (k + q m)} Y_r[k] (m = n/p). Arithmetic is in double precision for
// both APIs (the float API rounds its results), with the roots of unity evaluated in long double.
// Unnormalised; sign -1 forward, +1 backward. A real-to-complex plan returns X[0 .. n/2] of the
// forward DFT of its real input; a complex-to-real plan extends X[0 .. n/2] hermitian (using the
// real parts of X[0] and, for even n, X[n/2]) and returns the real backward DFT.
#include "fftw3.h"

#include <cmath>
#include <complex>
#include <cstddef>
#include <cstdint>
#include <vector>

namespace {

using C = std::complex<double>;

enum class Kind { C2C, R2C, C2R };

class Dft {
public:
  Dft(int n, int sign) : n_(n) {
    for (int m = n, p = 2; m > 1;) {
      if (m % p == 0) {
        factors_.push_back(p);
        m /= p;
      } else {
        p = (p == 2) ? 3 : p + 2;
        if (p * p > m) p = m;
      }
    }
    roots_.resize(n);
    const long double pi = 3.141592653589793238462643383279502884L;
    for (int k = 0; k < n; ++k) {
      const long double a = static_cast<long double>(sign) * 2.0L * pi * k / n;
      roots_[k] = C(static_cast<double>(std::cos(a)), static_cast<double>(std::sin(a)));
    }
  }
  // out[0 .. n) = DFT of in[0], in[is], ..., in[(n-1) is]
  void run(const C* in, std::ptrdiff_t is, C* out) const { rec(in, is, out, n_, 0, 1); }
  int size() const { return n_; }

private:
  void rec(const C* in, std::ptrdiff_t is, C* out, int n, std::size_t fi, int rootStep) const {
    if (n == 1) {
      out[0] = in[0];
      return;
    }
    const int p = factors_[fi], m = n / p;
    std::vector<C> sub(static_cast<std::size_t>(n));
    for (int r = 0; r < p; ++r) rec(in + r * is, is * p, sub.data() + r * m, m, fi + 1, rootStep * p);
    for (int k = 0; k < m; ++k) {
      for (int q = 0; q < p; ++q) {
        const int kk = k + q * m;
        C acc = 0.0;
        for (int r = 0; r < p; ++r) {
          const long long e = (static_cast<long long>(r) * kk) % n;
          acc += roots_[static_cast<std::size_t>(e * rootStep)] * sub[static_cast<std::size_t>(r * m + k)];
        }
        out[kk] = acc;
      }
    }
  }

  int n_;
  std::vector<int> factors_;
  std::vector<C> roots_;
};

}  // namespace

struct shim_plan_s {
  Kind kind;
  int n, howmany, istride, idist, ostride, odist;
  void* in;
  void* out;
  Dft dft;
  shim_plan_s(Kind k, int n_, int hm, int is, int id, int os, int od, int sign, void* i, void* o)
      : kind(k), n(n_), howmany(hm), istride(is), idist(id), ostride(os), odist(od), in(i), out(o),
        dft(n_, sign) {}
};

namespace {

// T = double or float; CT = the API's complex array type (T[2]).
template <typename T>
void run_plan(const shim_plan_s* p, void* inPtr, void* outPtr) {
  const int n = p->n;
  std::vector<C> seq(static_cast<std::size_t>(n)), res(static_cast<std::size_t>(n));
  for (int t = 0; t < p->howmany; ++t) {
    if (p->kind == Kind::C2C) {
      const T* in = static_cast<const T*>(inPtr) + 2 * static_cast<std::ptrdiff_t>(t) * p->idist;
      for (int j = 0; j < n; ++j) {
        const T* v = in + 2 * static_cast<std::ptrdiff_t>(j) * p->istride;
        seq[j] = C(v[0], v[1]);
      }
      p->dft.run(seq.data(), 1, res.data());
      T* out = static_cast<T*>(outPtr) + 2 * static_cast<std::ptrdiff_t>(t) * p->odist;
      for (int j = 0; j < n; ++j) {
        T* v = out + 2 * static_cast<std::ptrdiff_t>(j) * p->ostride;
        v[0] = static_cast<T>(res[j].real());
        v[1] = static_cast<T>(res[j].imag());
      }
    } else if (p->kind == Kind::R2C) {
      const T* in = static_cast<const T*>(inPtr) + static_cast<std::ptrdiff_t>(t) * p->idist;
      for (int j = 0; j < n; ++j) seq[j] = C(in[static_cast<std::ptrdiff_t>(j) * p->istride], 0.0);
      p->dft.run(seq.data(), 1, res.data());
      T* out = static_cast<T*>(outPtr) + 2 * static_cast<std::ptrdiff_t>(t) * p->odist;
      for (int k = 0; k <= n / 2; ++k) {
        T* v = out + 2 * static_cast<std::ptrdiff_t>(k) * p->ostride;
        v[0] = static_cast<T>(res[k].real());
        v[1] = static_cast<T>(res[k].imag());
      }
    } else {
      const T* in = static_cast<const T*>(inPtr) + 2 * static_cast<std::ptrdiff_t>(t) * p->idist;
      for (int k = 0; k <= n / 2; ++k) {
        const T* v = in + 2 * static_cast<std::ptrdiff_t>(k) * p->istride;
        const bool selfConjugate = (k == 0) || (2 * k == n);
        seq[k] = C(v[0], selfConjugate ? 0.0 : v[1]);
      }
      for (int k = n / 2 + 1; k < n; ++k) seq[k] = std::conj(seq[n - k]);
      p->dft.run(seq.data(), 1, res.data());
      T* out = static_cast<T*>(outPtr) + static_cast<std::ptrdiff_t>(t) * p->odist;
      for (int j = 0; j < n; ++j) out[static_cast<std::ptrdiff_t>(j) * p->ostride] = static_cast<T>(res[j].real());
    }
  }
}

shim_plan_s* make(Kind kind, int rank, const int* n, int howmany, void* in, int istride, int idist, void* out,
                  int ostride, int odist, int sign) {
  if (rank != 1 || !n || n[0] < 1 || howmany < 0) return nullptr;
  return new shim_plan_s(kind, n[0], howmany, istride, idist, ostride, odist, sign, in, out);
}

int alignment(const void* p) { return static_cast<int>(reinterpret_cast<std::uintptr_t>(p) % 16); }

}  // namespace

extern "C" {

fftw_plan fftw_plan_dft_1d(int n, fftw_complex* in, fftw_complex* out, int sign, unsigned) {
  return make(Kind::C2C, 1, &n, 1, in, 1, n, out, 1, n, sign);
}
fftw_plan fftw_plan_many_dft(int rank, const int* n, int howmany, fftw_complex* in, const int*, int istride,
                             int idist, fftw_complex* out, const int*, int ostride, int odist, int sign,
                             unsigned) {
  return make(Kind::C2C, rank, n, howmany, in, istride, idist, out, ostride, odist, sign);
}
fftw_plan fftw_plan_many_dft_r2c(int rank, const int* n, int howmany, double* in, const int*, int istride,
                                 int idist, fftw_complex* out, const int*, int ostride, int odist, unsigned) {
  return make(Kind::R2C, rank, n, howmany, in, istride, idist, out, ostride, odist, FFTW_FORWARD);
}
fftw_plan fftw_plan_many_dft_c2r(int rank, const int* n, int howmany, fftw_complex* in, const int*,
                                 int istride, int idist, double* out, const int*, int ostride, int odist,
                                 unsigned) {
  return make(Kind::C2R, rank, n, howmany, in, istride, idist, out, ostride, odist, FFTW_BACKWARD);
}
void fftw_execute(const fftw_plan p) { run_plan<double>(p, p->in, p->out); }
void fftw_execute_dft(const fftw_plan p, fftw_complex* in, fftw_complex* out) { run_plan<double>(p, in, out); }
void fftw_execute_dft_r2c(const fftw_plan p, double* in, fftw_complex* out) { run_plan<double>(p, in, out); }
void fftw_execute_dft_c2r(const fftw_plan p, fftw_complex* in, double* out) { run_plan<double>(p, in, out); }
void fftw_destroy_plan(fftw_plan p) { delete p; }
int fftw_alignment_of(double* p) { return alignment(p); }

fftwf_plan fftwf_plan_dft_1d(int n, fftwf_complex* in, fftwf_complex* out, int sign, unsigned) {
  return make(Kind::C2C, 1, &n, 1, in, 1, n, out, 1, n, sign);
}
fftwf_plan fftwf_plan_many_dft(int rank, const int* n, int howmany, fftwf_complex* in, const int*, int istride,
                               int idist, fftwf_complex* out, const int*, int ostride, int odist, int sign,
                               unsigned) {
  return make(Kind::C2C, rank, n, howmany, in, istride, idist, out, ostride, odist, sign);
}
fftwf_plan fftwf_plan_many_dft_r2c(int rank, const int* n, int howmany, float* in, const int*, int istride,
                                   int idist, fftwf_complex* out, const int*, int ostride, int odist,
                                   unsigned) {
  return make(Kind::R2C, rank, n, howmany, in, istride, idist, out, ostride, odist, FFTW_FORWARD);
}
fftwf_plan fftwf_plan_many_dft_c2r(int rank, const int* n, int howmany, fftwf_complex* in, const int*,
                                   int istride, int idist, float* out, const int*, int ostride, int odist,
                                   unsigned) {
  return make(Kind::C2R, rank, n, howmany, in, istride, idist, out, ostride, odist, FFTW_BACKWARD);
}
void fftwf_execute(const fftwf_plan p) { run_plan<float>(p, p->in, p->out); }
void fftwf_execute_dft(const fftwf_plan p, fftwf_complex* in, fftwf_complex* out) { run_plan<float>(p, in, out); }
void fftwf_execute_dft_r2c(const fftwf_plan p, float* in, fftwf_complex* out) { run_plan<float>(p, in, out); }
void fftwf_execute_dft_c2r(const fftwf_plan p, fftwf_complex* in, float* out) { run_plan<float>(p, in, out); }
void fftwf_destroy_plan(fftwf_plan p) { delete p; }
int fftwf_alignment_of(float* p) { return alignment(p); }

}  // extern "C"
