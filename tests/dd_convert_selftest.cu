// Host self-test of the integer-only double <-> dd conversions in spfft_gb300/csrc/dd.cuh:
// split accuracy (hi + lo within 2^-46 of v * 2^k), round trips, faithful rounding of dd_to_double
// (within one binary64 ulp of the exact sum) on normalised pairs, on pairs whose lo is not below
// hi, on powers of two with a negative lo and on all-ones mantissas with a positive lo, signs,
// zeros, infinities and NaN. Prints "ok <checks>" or the first failure.
#include <cmath>
#include <cstdio>
#include <random>

#include "dd.cuh"

using namespace spfft::gb300;

// |got - want| within one ulp of want (want exactly representable as long double).
static bool faithful(double got, long double want) {
  const double w = (double)want;
  const double ulp = std::fabs(std::nextafter(w, INFINITY) - w);
  return std::fabs((long double)got - want) <= (long double)ulp;
}

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
    if (std::fabs((double)((got - want) / want)) > std::ldexp(1.0, -46)) {
      std::printf("split error v=%.17g k=%d\n", v, k);
      return 1;
    }
    // round trip
    const double back = dd_to_double(d, -k);
    if (std::fabs((back - v) / v) > std::ldexp(1.0, -46)) {
      std::printf("round trip error v=%.17g back=%.17g\n", v, back);
      return 1;
    }
    // dd_to_double of a normalised dd (two_sum output): within one ulp of the exact sum
    const float a = (float)mant(rng) * std::ldexp(1.0f, ex(rng) / 4), b = (float)mant(rng) * std::ldexp(1.0f, ex(rng) / 4 - 30);
    const dd n = dd_two_sum(a, (i & 2) ? -b : b);
    const long double exact = (long double)n.hi + (long double)n.lo;
    if (!faithful(dd_to_double(n, 0), exact)) {
      std::printf("combine error hi=%.9g lo=%.9g got %.17g want %.17Lg\n", n.hi, n.lo, dd_to_double(n, 0), exact);
      return 1;
    }
    // pairs that are not normalised (lo in hi's binade or above, zero hi)
    const float c = (float)mant(rng) * std::ldexp(1.0f, ex(rng) / 4);
    const float e = (i % 5 == 0) ? 0.0f : (float)mant(rng) * std::ldexp(1.0f, ex(rng) / 4 % 3) * ((i & 4) ? -1.0f : 1.0f);
    const long double sum = (long double)e + (long double)c;
    if (!faithful(dd_to_double(dd(e, c), 0), sum)) {
      std::printf("unnormalised error hi=%.9g lo=%.9g got %.17g want %.17Lg\n", e, c, dd_to_double(dd(e, c), 0), (long double)sum);
      return 1;
    }
    // hi a power of two with lo pulling below it, and hi with an all-ones mantissa with lo
    // pushing up to the next binade, with the block scale applied
    const int x = ex(rng) / 2;
    const float p2 = std::ldexp(1.0f, x) * ((i & 8) ? -1.0f : 1.0f);
    const float small = std::ldexp((float)mant(rng), x - 25 - (i % 9));
    const dd below(p2, p2 > 0 ? -small : small);
    if (!faithful(dd_to_double(below, k), std::ldexp((long double)below.hi + (long double)below.lo, k))) {
      std::printf("power-of-two error hi=%.9g lo=%.9g\n", below.hi, below.lo);
      return 1;
    }
    const float ones = std::nextafter(std::ldexp(1.0f, x + 1), 0.0f);
    const dd above(ones, std::ldexp((float)mant(rng), x - 25 - (i % 5)));
    if (!faithful(dd_to_double(above, k), std::ldexp((long double)above.hi + (long double)above.lo, k))) {
      std::printf("all-ones error hi=%.9g lo=%.9g\n", above.hi, above.lo);
      return 1;
    }
    checks += 6;
  }
  // specials
  if (dd_to_double(dd_from_double(0.0, 5), -5) != 0.0) return 2;
  if (!std::signbit(dd_to_double(dd_from_double(-0.0, 0), 0))) return 3;
  if (!std::isinf(dd_to_double(dd_from_double(INFINITY, 0), 0))) return 4;
  if (!std::isnan(dd_to_double(dd_from_double(NAN, 0), 0))) return 5;
  if (dd_exponent_field(1.0) != 1023 || dd_exponent_field(0.0) != 0) return 6;
  if (!std::isinf(dd_to_double(dd(1.5f, 0.0f), 2000))) return 7;
  if (dd_to_double(dd(1.5f, 0.0f), -2000) != 0.0) return 8;
  std::printf("ok %ld\n", checks + 7);
  return 0;
}
