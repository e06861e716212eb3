// Double-float ("dd") arithmetic: a value is the unevaluated sum hi + lo of two floats, lo at most
// a few ulps of hi, giving about 44-48 significant bits on the FP32 pipes. GB300 issues FP32 FMA at
// 57x its FP64 rate, so FFT butterflies in dd arithmetic beat native FP64 several times while
// staying well inside a 1e-12 relative error.
//
// Published building blocks used here (Dekker 1971; Knuth TAOCP vol. 2; Hida, Li, Bailey 2001):
//   two_sum(a, b):      s = a + b, e = exact rounding error of the sum (6 flops, any a, b)
//   fast_two_sum(a, b): the same for |a| >= |b| (3 flops)
//   two_prod(a, b):     p = a * b, e = fma(a, b, -p) (exact error of the product)
// add: two_sum of the high parts, low parts added into the error;
// mul: two_prod of the high parts, cross terms added into the error.
// Neither renormalises (no final fast_two_sum): hi + lo stays the exact value of the pair and only
// the FP32 roundings of the low-order terms cost accuracy. Without renormalisation lo may grow to
// a few ulps of hi within a transform, which costs a few of the ~48 bits, in exchange for 8
// instead of 11 instructions per add and 4 instead of 7 per product. The conversion to binary64
// (dd_to_double) accepts unnormalised pairs.
#pragma once

#include <cuda_runtime.h>

#include <cstring>

namespace spfft {
namespace gb300 {

struct dd {
  float hi, lo;
  dd() = default;
  __host__ __device__ constexpr dd(float h, float l) : hi(h), lo(l) {}
  // Split a double (used for compile-time constants, folded by the compiler).
  __host__ __device__ constexpr explicit dd(double v)
      : hi(static_cast<float>(v)), lo(static_cast<float>(v - static_cast<double>(static_cast<float>(v)))) {}
  __host__ __device__ constexpr explicit dd(int v) : hi(static_cast<float>(v)), lo(0.0f) {}
};

__host__ __device__ __forceinline__ dd dd_two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  const float e = (a - (s - bb)) + (b - bb);
  return dd(s, e);
}
__host__ __device__ __forceinline__ dd dd_fast_two_sum(float a, float b) {
  const float s = a + b;
  return dd(s, b - (s - a));
}

__host__ __device__ __forceinline__ dd operator+(dd a, dd b) {
  const dd s = dd_two_sum(a.hi, b.hi);
  return dd(s.hi, s.lo + (a.lo + b.lo));
}
__host__ __device__ __forceinline__ dd operator-(dd a) { return dd(-a.hi, -a.lo); }
__host__ __device__ __forceinline__ dd operator-(dd a, dd b) { return a + (-b); }
__host__ __device__ __forceinline__ dd operator*(dd a, dd b) {
  const float p = a.hi * b.hi;
#ifdef __CUDA_ARCH__
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
#else
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
#endif
  return dd(p, e);
}
// Multiplication by 1/2 (exact in both parts).
__host__ __device__ __forceinline__ dd half_of(dd a) { return dd(0.5f * a.hi, 0.5f * a.lo); }
// Multiplication by +1 / -1 (the sign factors of the butterflies).
__host__ __device__ __forceinline__ dd operator*(int s, dd a) { return s >= 0 ? a : -a; }
__host__ __device__ __forceinline__ bool operator!=(dd a, int z) {
  return a.hi != static_cast<float>(z) || a.lo != 0.0f;
}

struct ddc {
  dd x, y;
};
static_assert(sizeof(ddc) == 16, "ddc must match double2");

__host__ __device__ __forceinline__ ddc make_c(dd x, dd y) { return ddc{x, y}; }

// double <-> dd conversion by FP64 instructions (host side and constants).
__host__ __device__ __forceinline__ dd to_dd(double v) {
  const float h = static_cast<float>(v);
  return dd(h, static_cast<float>(v - static_cast<double>(h)));
}
__host__ __device__ __forceinline__ double to_double(dd v) {
  return static_cast<double>(v.hi) + static_cast<double>(v.lo);
}

// ---- integer-only conversions (GB300's FP64 pipe is slow, its integer pipes are not) ----------
// Bit layouts are those of IEEE 754 binary64 (1 sign, 11 exponent, 52 fraction bits) and binary32
// (1, 8, 23). Both conversions fold an exact scaling by 2^k into the exponent.

__host__ __device__ __forceinline__ unsigned long long dd_bits64(double v) {
#ifdef __CUDA_ARCH__
  return static_cast<unsigned long long>(__double_as_longlong(v));
#else
  unsigned long long u;
  memcpy(&u, &v, 8);
  return u;
#endif
}
__host__ __device__ __forceinline__ double dd_double_from_bits(unsigned long long u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double(static_cast<long long>(u));
#else
  double v;
  memcpy(&v, &u, 8);
  return v;
#endif
}
__host__ __device__ __forceinline__ float dd_float_from_bits(unsigned u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float f;
  memcpy(&f, &u, 4);
  return f;
#endif
}
__host__ __device__ __forceinline__ unsigned dd_bits32(float f) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(f);
#else
  unsigned u;
  memcpy(&u, &f, 4);
  return u;
#endif
}
__host__ __device__ __forceinline__ int dd_clz32(unsigned x) {
#ifdef __CUDA_ARCH__
  return __clz(static_cast<int>(x));
#else
  return x ? __builtin_clz(x) : 32;
#endif
}
__host__ __device__ __forceinline__ int dd_clz64(unsigned long long x) {
#ifdef __CUDA_ARCH__
  return __clzll(static_cast<long long>(x));
#else
  return x ? __builtin_clzll(x) : 64;
#endif
}

// Biased binary64 exponent field of v (0 for zero / subnormal, 2047 for inf / NaN).
__host__ __device__ __forceinline__ int dd_exponent_field(double v) {
  return static_cast<int>((dd_bits64(v) >> 52) & 0x7ff);
}

// v * 2^k as dd: hi takes the top 24 significant bits (truncated), lo the next 24. Values whose
// scaled magnitude leaves the binary32 normal range become signed zero (below) or infinity
// (above); callers choose k so that the block maximum lands in [1, 2).
__host__ __device__ __forceinline__ dd dd_from_double(double v, int k) {
  const unsigned long long u = dd_bits64(v);
  const unsigned sign = static_cast<unsigned>(u >> 63) << 31;
  const int E = static_cast<int>((u >> 52) & 0x7ff);
  const unsigned long long m = u & 0xFFFFFFFFFFFFFull;
  if (E == 0x7ff) return dd(dd_float_from_bits(sign | 0x7f800000u | (m ? 0x400000u : 0u)), 0.0f);
  const int e = E - 1023 + k;
  if (E == 0 || e < -126) return dd(dd_float_from_bits(sign), 0.0f);
  if (e > 127) return dd(dd_float_from_bits(sign | 0x7f800000u), 0.0f);
  const float hi = dd_float_from_bits(sign | (static_cast<unsigned>(e + 127) << 23) |
                                      static_cast<unsigned>(m >> 29));
  const unsigned r = static_cast<unsigned>(m & 0x1FFFFFFFu);  // remaining 29 fraction bits
  if (r == 0) return dd(hi, 0.0f);
  const int p = 31 - dd_clz32(r);  // leading one of the remainder
  const int el = e - 52 + p;
  if (el < -126) return dd(hi, 0.0f);
  const unsigned frac = p >= 23 ? (r >> (p - 23)) & 0x7FFFFFu : (r << (23 - p)) & 0x7FFFFFu;
  return dd(hi, dd_float_from_bits(sign | (static_cast<unsigned>(el + 127) << 23) | frac));
}

// (hi + lo) * 2^k as the nearest double (ties to even), for binary32-normal (or zero) hi and lo.
// Inf / NaN in hi pass through. Integer and FP32 instructions only.
__host__ __device__ __forceinline__ double dd_to_double(dd v, int k) {
  unsigned hb = dd_bits32(v.hi), lb = dd_bits32(v.lo);
  if ((lb << 1) != 0 && ((lb >> 23) & 0xff) >= ((hb >> 23) & 0xff)) {
    // lo not below hi's binade (after a cancellation in the unnormalised arithmetic, or a zero
    // hi): renormalise exactly with two_sum on the FP32 pipe, after which lo is at most half an
    // ulp of hi.
    const dd n = dd_two_sum(v.hi, v.lo);
    hb = dd_bits32(n.hi);
    lb = dd_bits32(n.lo);
  }
  const int eh = static_cast<int>((hb >> 23) & 0xff);
  if (eh == 0xff) {
    return dd_double_from_bits((static_cast<unsigned long long>(hb >> 31) << 63) | 0x7ff0000000000000ull |
                               ((hb & 0x7fffff) ? 0x8000000000000ull : 0ull));
  }
  if (eh == 0) return dd_double_from_bits(static_cast<unsigned long long>(hb >> 31) << 63);
  const unsigned long long H = static_cast<unsigned long long>((hb & 0x7FFFFFu) | 0x800000u) << 39;
  unsigned long long S = H;
  const int el = static_cast<int>((lb >> 23) & 0xff);
  if (el != 0) {
    const int shift = 39 - (eh - el);  // < 39: lo lies in a lower binade than hi
    const unsigned long long L = (lb & 0x7FFFFFu) | 0x800000u;
    // Bits of lo shifted out below S's last place are kept as a sticky bit, so that the final
    // rounding (which drops >= 9 bits) sees whether the exact value lies above S.
    unsigned long long Y = 0;
    bool sticky = false;
    if (shift >= 0) {
      Y = L << shift;
    } else if (shift > -24) {
      Y = L >> (-shift);
      sticky = (L & ((1ull << (-shift)) - 1)) != 0;
    } else {
      sticky = true;
    }
    if ((hb ^ lb) >> 31) {
      S = S - Y - (sticky ? 1 : 0);
    } else {
      S = S + Y;
    }
    if (sticky) S |= 1;
  }
  // value = S * 2^(eh - 127 - 23 - 39 + k); normalise S to 53 bits with round-to-nearest-even
  const int lead = 63 - dd_clz64(S);
  int expo = eh - 127 - 62 + lead + k;  // unbiased exponent of the leading bit
  unsigned long long mant;
  const int drop = lead - 52;
  if (drop > 0) {
    mant = S >> drop;
    const unsigned long long rem = S & ((1ull << drop) - 1), half = 1ull << (drop - 1);
    if (rem > half || (rem == half && (mant & 1))) ++mant;
  } else {
    mant = S << (-drop);
  }
  if (expo + 1023 <= 0) return dd_double_from_bits(static_cast<unsigned long long>(hb >> 31) << 63);
  if (expo + 1023 >= 2047) {
    return dd_double_from_bits((static_cast<unsigned long long>(hb >> 31) << 63) | 0x7ff0000000000000ull);
  }
  // mant has its leading one at bit 52 (or 53 after a rounding carry, which the add propagates)
  const unsigned long long bits = (static_cast<unsigned long long>(expo + 1022) << 52) + mant;
  return dd_double_from_bits((static_cast<unsigned long long>(hb >> 31) << 63) | bits);
}

}  // namespace gb300
}  // namespace spfft
