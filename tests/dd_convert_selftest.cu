// Host self-test of the integer-only double <-> dd conversions in spfft_gb300/csrc/dd.cuh:
// split exactness (hi + lo within 2^-47 of v * 2^k), round trips, signs, zeros, infinities and the
// rounding of dd_to_double on normalised dd values and on pairs whose lo is not below hi. Prints "ok <checks>" or the first failure.
#include <cmath>
#include <cstdio>
#include <random>

#include "dd.cuh"

using namespace spfft::gb300;

int main() {
  std::mt19937_64 rng(12345);
  std::uniform_real_distribution<double> mant(1.0, 2.0);
  std::uniform_int_distribution<int> ex(-60, 60);
  long checks = 0;
  for (int i = 0; i < 2000000; ++i) {
    double v = mant(rng) * std::ldexp(1.0, ex(rng));
    if (i & 1) v = -v;
    const int k = (i % 7) - 3;
    const dd d = dd_from_double(v, k);
    const long double want = std::ldexp((long double)v, k);
    const long double got = (long double)d.hi + (long double)d.lo;
    if (std::fabs((double)((got - want) / want)) > std::ldexp(1.0, -47)) {
      std::printf("split error v=%.17g k=%d\n", v, k);
      return 1;
    }
    // round trip
    const double back = dd_to_double(d, -k);
    if (std::fabs((back - v) / v) > std::ldexp(1.0, -47)) {
      std::printf("round trip error v=%.17g back=%.17g\n", v, back);
      return 1;
    }
    // dd_to_double of a normalised dd (two_sum output) must equal the correctly rounded sum
    const float a = (float)mant(rng) * std::ldexp(1.0f, ex(rng) / 4), b = (float)mant(rng) * std::ldexp(1.0f, ex(rng) / 4 - 30);
    const dd n = dd_two_sum(a, (i & 2) ? -b : b);
    const double exact = (double)n.hi + (double)n.lo;  // exact: fits in 53 bits here
    if (dd_to_double(n, 0) != exact) {
      std::printf("combine error hi=%.9g lo=%.9g got %.17g want %.17g\n", n.hi, n.lo, dd_to_double(n, 0), exact);
      return 1;
    }
    // pairs that are not normalised (lo in hi's binade or above, zero hi) are still summed exactly
    const float c = (float)mant(rng) * std::ldexp(1.0f, ex(rng) / 4);
    const float e = (i % 5 == 0) ? 0.0f : (float)mant(rng) * std::ldexp(1.0f, ex(rng) / 4 % 3) * ((i & 4) ? -1.0f : 1.0f);
    const double sum = (double)e + (double)c;  // exact: exponents differ by at most 18
    if (dd_to_double(dd(e, c), 0) != sum) {
      std::printf("unnormalised error hi=%.9g lo=%.9g got %.17g want %.17g\n", e, c, dd_to_double(dd(e, c), 0), sum);
      return 1;
    }
    checks += 4;
  }
  // specials
  if (dd_to_double(dd_from_double(0.0, 5), -5) != 0.0) return 2;
  if (!std::signbit(dd_to_double(dd_from_double(-0.0, 0), 0))) return 3;
  if (!std::isinf(dd_to_double(dd_from_double(INFINITY, 0), 0))) return 4;
  if (!std::isnan(dd_to_double(dd_from_double(NAN, 0), 0))) return 5;
  if (dd_exponent_field(1.0) != 1023 || dd_exponent_field(0.0) != 0) return 6;
  std::printf("ok %ld\n", checks + 5);
  return 0;
}
