// Host-side self test of the register DFTs and the two-pass FFT shapes (dft.cuh), compiled by the
// CPU test suite with nvcc as host code: every size is checked against a direct DFT evaluated in
// long double. Prints "ok <checks>" or the first failure.
#include <cmath>
#include <complex>
#include <cstdio>
#include <vector>

#include "dd.cuh"
#include "dft.cuh"
#include "fft_plan.hpp"

using namespace spfft::gb300;
using cd = std::complex<long double>;

static std::vector<cd> direct(const std::vector<cd>& x, int sign) {
  const size_t n = x.size();
  std::vector<cd> y(n);
  const long double twoPi = 6.283185307179586476925286766559005768L;
  for (size_t k = 0; k < n; ++k) {
    cd acc = 0;
    for (size_t j = 0; j < n; ++j) {
      long double a = sign * twoPi * static_cast<long double>((k * j) % n) / n;
      acc += x[j] * cd(cosl(a), sinl(a));
    }
    y[k] = acc;
  }
  return y;
}

static int checks = 0;

template <int R, int SIGN>
static bool check_register() {
  double2 v[R];
  std::vector<cd> x(R);
  for (int i = 0; i < R; ++i) {
    x[i] = cd(std::sin(1.0 + 3.1 * i), std::cos(0.3 + 1.7 * i * i));
    v[i] = make_double2(static_cast<double>(x[i].real()), static_cast<double>(x[i].imag()));
  }
  Dft<R, SIGN>::run(v);
  auto y = direct(x, SIGN);
  for (int i = 0; i < R; ++i) {
    const double e = std::abs(std::complex<double>(v[i].x - (double)y[i].real(), v[i].y - (double)y[i].imag()));
    if (e > 1e-13 * R) {
      std::printf("register DFT %d sign %d: element %d error %g\n", R, SIGN, i, e);
      return false;
    }
  }
  ++checks;
  return true;
}

template <int N, int SIGN>
static bool check_two_pass() {
  constexpr int A = Shape<N>::A, B = Shape<N>::B;
  std::vector<double> twd = make_twiddles(N);
  std::vector<double2> tw(N), buf(N);
  for (int i = 0; i < N; ++i) tw[i] = make_double2(twd[2 * i], twd[2 * i + 1]);
  std::vector<cd> x(N);
  for (int i = 0; i < N; ++i) {
    x[i] = cd(std::sin(0.5 + 1.3 * i), std::cos(2.0 - 0.7 * i));
    buf[i] = make_double2((double)x[i].real(), (double)x[i].imag());
  }
  for (int b = 0; b < B; ++b) fft_pass1<N, SIGN>(buf.data(), 1, b, tw.data());
  std::vector<double2> out(N);
  for (int k1 = 0; k1 < A; ++k1) {
    double2 v[B];
    fft_pass2<N, SIGN>(buf.data(), 1, k1, v);
    for (int k2 = 0; k2 < B; ++k2) out[k1 + A * k2] = v[k2];
  }
  // stored-back (transposed) order
  for (int k1 = 0; k1 < A; ++k1) {
    double2 v[B];
    fft_pass2<N, SIGN>(buf.data(), 1, k1, v);
    for (int k2 = 0; k2 < B; ++k2) {
      if (transposed_pos<N>(k1 + A * k2) != k1 * B + k2) {
        std::printf("transposed_pos mismatch N=%d\n", N);
        return false;
      }
    }
  }
  auto y = direct(x, SIGN);
  for (int i = 0; i < N; ++i) {
    const double e = std::abs(std::complex<double>(out[i].x - (double)y[i].real(), out[i].y - (double)y[i].imag()));
    if (e > 2e-14 * N) {
      std::printf("two-pass FFT %d sign %d: element %d error %g\n", N, SIGN, i, e);
      return false;
    }
  }
  ++checks;
  return true;
}

// Double-float arithmetic: the same register DFTs and two-pass shapes in dd, against the same
// long-double reference, at a bound set by the ~48-bit dd mantissa.
template <int N, int SIGN>
static bool check_two_pass_dd() {
  constexpr int A = Shape<N>::A, B = Shape<N>::B;
  std::vector<double> twd = make_twiddles(N);
  std::vector<ddc> tw(N), buf(N);
  for (int i = 0; i < N; ++i) tw[i] = make_c(to_dd(twd[2 * i]), to_dd(twd[2 * i + 1]));
  std::vector<cd> x(N);
  for (int i = 0; i < N; ++i) {
    x[i] = cd(std::sin(0.5 + 1.3 * i), std::cos(2.0 - 0.7 * i));
    buf[i] = make_c(to_dd((double)x[i].real()), to_dd((double)x[i].imag()));
  }
  for (int b = 0; b < B; ++b) fft_pass1<N, SIGN>(buf.data(), 1, b, tw.data());
  std::vector<ddc> out(N);
  for (int k1 = 0; k1 < A; ++k1) {
    ddc v[B];
    fft_pass2<N, SIGN>(buf.data(), 1, k1, v);
    for (int k2 = 0; k2 < B; ++k2) out[k1 + A * k2] = v[k2];
  }
  auto y = direct(x, SIGN);
  long double num = 0, den = 0;
  for (int i = 0; i < N; ++i) {
    const long double er = (long double)to_double(re(out[i])) - y[i].real();
    const long double ei = (long double)to_double(im(out[i])) - y[i].imag();
    num += er * er + ei * ei;
    den += std::norm(y[i]);
  }
  const double rel = std::sqrt((double)(num / den));
  if (rel > 2e-14) {
    std::printf("dd two-pass FFT %d sign %d: rel-L2 error %g\n", N, SIGN, rel);
    return false;
  }
  ++checks;
  return true;
}

#define REG(R) (check_register<R, -1>() && check_register<R, 1>())
#define DD(N) (check_two_pass_dd<N, -1>() && check_two_pass_dd<N, 1>())
#define TWO(N) (check_two_pass<N, -1>() && check_two_pass<N, 1>())

int main() {
  bool ok = REG(2) && REG(3) && REG(4) && REG(5) && REG(6) && REG(7) && REG(8) && REG(9) &&
            REG(10) && REG(12) && REG(15) && REG(16) && REG(18) && REG(20) && REG(24) &&
            REG(25) && REG(27) && REG(30) && REG(32);
  ok = ok && TWO(3) && TWO(4) && TWO(6) && TWO(8) && TWO(12) && TWO(16) && TWO(24) && TWO(30) &&
       TWO(32) && TWO(36) && TWO(45) && TWO(48) && TWO(50) && TWO(54) && TWO(60) && TWO(64) &&
       TWO(72) && TWO(75) && TWO(80) && TWO(90) && TWO(96) && TWO(100) && TWO(108) && TWO(120) &&
       TWO(128) && TWO(144) && TWO(150) && TWO(160) && TWO(180) && TWO(192) && TWO(240) &&
       TWO(256);
  ok = ok && DD(12) && DD(48) && DD(60) && DD(64) && DD(72) && DD(90) && DD(96) && DD(100) &&
       DD(108) && DD(120) && DD(128) && DD(150) && DD(160) && DD(192) && DD(24) && DD(30) &&
       DD(36) && DD(45) && DD(50) && DD(54) && DD(75) && DD(80) && DD(6);
  if (!ok) return 1;
  std::printf("ok %d\n", checks);
  return 0;
}
