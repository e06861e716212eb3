// Host self-test of the integer-only double <-> dd conversions in spfft_gb300/csrc/dd.cuh:
// split accuracy (hi + lo within 2^-46 of v * 2^k), round trips, faithful rounding of dd_to_double
// (within one binary64 ulp of the exact sum) on normalised pairs, on pairs whose lo is not below
// hi, on powers of two with a negative lo and on all-ones mantissas with a positive lo, signs,
// zeros, infinities and NaN; subnormal binary64 inputs (subnormal key, block scale, split, round
// trip; the exact conversions, which the fast ones match on normal values) and results in the
// subnormal range. Prints "ok <checks>" or the first failure.
#include <cmath>
#include <cstdio>
#include <cstring>
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
    // the exact conversions agree bit for bit with the fast ones on normal values
    const dd de = dd_from_double_exact(v, k);
    if (de.hi != d.hi || de.lo != d.lo) {
      std::printf("exact split differs v=%.17g\n", v);
      return 1;
    }
    // round trip
    const double back = dd_to_double(d, -k);
    if (dd_to_double_exact(d, -k) != back) {
      std::printf("exact combine differs v=%.17g\n", v);
      return 1;
    }
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
  // subnormal binary64 inputs: the subnormal key orders them (below every normal, whose key is
  // its exponent field >= 1), the block scale brings each into [1, 2), the split is exact for up
  // to 47 significant bits (within 2^-46 otherwise) and the round trip returns to the subnormal
  // within that error
  std::uniform_int_distribution<int> subShift(0, 51);
  for (int i = 0; i < 200000; ++i) {
    const unsigned long long frac = (rng() & 0xFFFFFFFFFFFFFull) >> subShift(rng);
    if (frac == 0) continue;
    double v;
    std::memcpy(&v, &frac, 8);
    if (i & 1) v = -v;
    const int key = dd_subnormal_key(v);
    if (key < -52 || key > -1 || dd_exponent_field(v) != 0) {
      std::printf("subnormal key %d for %.17g\n", key, v);
      return 10;
    }
    const int k = dd_block_scale(key);
    const long double scaled = std::fabs(std::ldexp((long double)v, k));
    if (scaled < 1.0L || scaled >= 2.0L) {
      std::printf("subnormal block scale %d for %.17g\n", k, v);
      return 11;
    }
    const int kk = k - (i % 40);  // the value is not always the block maximum
    const dd d = dd_from_double_exact(v, kk);
    const dd flushed = dd_from_double(v, kk);  // the fast conversion flushes subnormals
    if (flushed.hi != 0.0f || flushed.lo != 0.0f) {
      std::printf("fast conversion kept a subnormal v=%.17g\n", v);
      return 8;
    }
    const long double want = std::ldexp((long double)v, kk);
    const long double got = (long double)d.hi + (long double)d.lo;
    if (std::fabs((double)((got - want) / want)) > std::ldexp(1.0, -46)) {
      std::printf("subnormal split error v=%.17g k=%d\n", v, kk);
      return 12;
    }
    const double back = dd_to_double_exact(d, -kk);
    if (std::fabs(back - v) > std::ldexp(std::fabs(v), -46) + std::ldexp(1.0, -1074)) {
      std::printf("subnormal round trip v=%.17g back=%.17g\n", v, back);
      return 13;
    }
    // a subnormal scaled by a normal block maximum's k (2^-1022 .. 2^-1000 maxima)
    const int kn = dd_block_scale(1 + (i % 23));
    const dd dn = dd_from_double_exact(v, kn);
    const long double wn = std::ldexp((long double)v, kn);
    if (std::fabs(wn) >= std::ldexp(1.0L, -100) &&
        std::fabs((double)(((long double)dn.hi + (long double)dn.lo - wn) / wn)) > std::ldexp(1.0, -46)) {
      std::printf("subnormal under a normal block scale v=%.17g k=%d\n", v, kn);
      return 9;
    }
    checks += 4;
  }
  // results in the binary64 subnormal range: within one subnormal unit of the exact scaled sum
  for (int i = 0; i < 200000; ++i) {
    const float a = (float)mant(rng) * ((i & 1) ? -1.0f : 1.0f);
    const float b = (float)mant(rng) * std::ldexp(1.0f, -24 - (i % 8)) * ((i & 2) ? -1.0f : 1.0f);
    const dd n = dd_two_sum(a, b);
    const int k = -1022 - (i % 70);  // 2^k * [1, 2) from the smallest normal down past 2^-1074
    const double got = dd_to_double_exact(n, k);
    const long double want = std::ldexp((long double)n.hi + (long double)n.lo, k);
    if (std::fabs((long double)got - want) > std::ldexp(1.0L, -1074)) {
      std::printf("subnormal result error hi=%.9g lo=%.9g k=%d got %.17g want %.17Lg\n", n.hi, n.lo, k, got, want);
      return 14;
    }
    if (got != 0.0 && std::signbit(got) != std::signbit(a)) return 15;
    checks += 1;
  }
  // key edges
  if (dd_subnormal_key(0.0) != kDdNoSubnormal || dd_subnormal_key(-0.0) != kDdNoSubnormal) return 16;
  if (dd_subnormal_key(4.9406564584124654e-324) != -52) return 17;
  if (dd_subnormal_key(std::nextafter(2.2250738585072014e-308, 0.0)) != -1) return 18;
  if (dd_block_scale(dd_exponent_field(1.0)) != 0 || dd_block_scale(2047) != 0 || dd_block_scale(0) != 0) return 19;
  if (dd_block_scale(-52) != 1074 || dd_block_scale(1) != 1022) return 20;
  // specials
  if (dd_to_double(dd_from_double(0.0, 5), -5) != 0.0) return 2;
  if (!std::signbit(dd_to_double(dd_from_double(-0.0, 0), 0))) return 3;
  if (!std::isinf(dd_to_double(dd_from_double(INFINITY, 0), 0))) return 4;
  if (!std::isnan(dd_to_double(dd_from_double(NAN, 0), 0))) return 5;
  if (dd_exponent_field(1.0) != 1023 || dd_exponent_field(0.0) != 0) return 6;
  if (!std::isinf(dd_to_double(dd(1.5f, 0.0f), 2000))) return 7;
  if (dd_to_double(dd(1.5f, 0.0f), -2000) != 0.0) return 8;
  std::printf("ok %ld\n", checks + 12);
  return 0;
}
