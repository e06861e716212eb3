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

// Complex double-float, stored as the pair of high parts (real, imaginary) and the pair of low
// parts: each pair is one float2, so an operation applied to the real and the imaginary part at
// once runs as one packed FP32x2 instruction (FADD2 / FMUL2 / FFMA2, sm_100 and later) instead of
// two. The 16 bytes hold re.hi, im.hi, re.lo, im.lo.
struct ddc {
  float2 hi, lo;
};
static_assert(sizeof(ddc) == 16, "ddc must match double2");

__host__ __device__ __forceinline__ ddc make_c(dd x, dd y) {
  return ddc{make_float2(x.hi, y.hi), make_float2(x.lo, y.lo)};
}
__host__ __device__ __forceinline__ dd re(ddc c) { return dd(c.hi.x, c.lo.x); }
__host__ __device__ __forceinline__ dd im(ddc c) { return dd(c.hi.y, c.lo.y); }

// Packed FP32x2 arithmetic (one instruction for both lanes on sm_100 and later; each lane rounds
// like the scalar instruction). a - b is b * -1 + a: the product is exact, one rounding.
#if defined(__CUDA_ARCH__) && (__CUDA_ARCH__ >= 1000)
#define SPFFT_GB300_DD_PACKED 1
#endif
__host__ __device__ __forceinline__ float2 f2_add(float2 a, float2 b) {
#ifdef SPFFT_GB300_DD_PACKED
  return __fadd2_rn(a, b);
#else
  return make_float2(a.x + b.x, a.y + b.y);
#endif
}
__host__ __device__ __forceinline__ float2 f2_sub(float2 a, float2 b) {
#ifdef SPFFT_GB300_DD_PACKED
  return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a);
#else
  return make_float2(a.x - b.x, a.y - b.y);
#endif
}
__host__ __device__ __forceinline__ float2 f2_mul(float2 a, float2 b) {
#ifdef SPFFT_GB300_DD_PACKED
  return __fmul2_rn(a, b);
#else
  return make_float2(a.x * b.x, a.y * b.y);
#endif
}
__host__ __device__ __forceinline__ float2 f2_fma(float2 a, float2 b, float2 c) {
#ifdef SPFFT_GB300_DD_PACKED
  return __ffma2_rn(a, b, c);
#else
  return make_float2(fmaf(a.x, b.x, c.x), fmaf(a.y, b.y, c.y));
#endif
}

// Complex double-float operations on both parts at once: the same operation sequence per part as
// the scalar dd operators above (so the same results), in packed instructions.
// a + b: two_sum of the high pairs, low pairs added into the error.
__host__ __device__ __forceinline__ ddc cadd(ddc a, ddc b) {
  const float2 s = f2_add(a.hi, b.hi);
  const float2 bb = f2_sub(s, a.hi);
  const float2 e = f2_add(f2_sub(a.hi, f2_sub(s, bb)), f2_sub(b.hi, bb));
  return ddc{s, f2_add(e, f2_add(a.lo, b.lo))};
}
// a - b = a + (-b): two_sum(a, -b) with (-b) - bb = -(b + bb).
__host__ __device__ __forceinline__ ddc csub(ddc a, ddc b) {
  const float2 s = f2_sub(a.hi, b.hi);
  const float2 bb = f2_sub(s, a.hi);
  const float2 e = f2_sub(f2_sub(a.hi, f2_sub(s, bb)), f2_add(b.hi, bb));
  return ddc{s, f2_add(e, f2_sub(a.lo, b.lo))};
}
// a * s for a real double-float s: two_prod of the high parts, cross terms into the error.
__host__ __device__ __forceinline__ ddc cscale(ddc a, dd s) {
  const float2 sh = make_float2(s.hi, s.hi), sl = make_float2(s.lo, s.lo);
  const float2 p = f2_mul(a.hi, sh);
  float2 e = f2_fma(a.hi, sh, make_float2(-p.x, -p.y));
  e = f2_fma(a.hi, sl, e);
  e = f2_fma(a.lo, sh, e);
  return ddc{p, e};
}
// a * s + b for a real s
__host__ __device__ __forceinline__ ddc cfma_r(ddc a, dd s, ddc b) { return cadd(cscale(a, s), b); }
// a / 2 (exact in both parts)
__host__ __device__ __forceinline__ ddc chalf(ddc a) {
  const float2 h = make_float2(0.5f, 0.5f);
  return ddc{f2_mul(a.hi, h), f2_mul(a.lo, h)};
}
// a - b / 2 (halving is exact in both parts)
__host__ __device__ __forceinline__ ddc csub_half(ddc a, ddc b) {
  return csub(a, chalf(b));
}
__host__ __device__ __forceinline__ ddc cconj(ddc a) {
  return ddc{make_float2(a.hi.x, -a.hi.y), make_float2(a.lo.x, -a.lo.y)};
}
// Multiply by sign * i.
template <int SIGN>
__host__ __device__ __forceinline__ ddc cmul_i(ddc a) {
  return SIGN > 0 ? ddc{make_float2(-a.hi.y, a.hi.x), make_float2(-a.lo.y, a.lo.x)}
                  : ddc{make_float2(a.hi.y, -a.hi.x), make_float2(a.lo.y, -a.lo.x)};
}
// a * (c + i s) for real c, s: a c + (i a) s.
__host__ __device__ __forceinline__ ddc cmul_cs(ddc a, dd c, dd s) { return cfma_r(cmul_i<1>(a), s, cscale(a, c)); }
// General complex products (run-time twiddles) in the same packed form: a b = a re(b) + (i a) im(b).
// Every part is the same two-product and two-sum as in the scalar form
// re(a) re(b) - im(a) im(b), re(a) im(b) + im(a) re(b) (two_sum is exact in either operand order,
// negation is exact), so the results equal it (up to the sign of a zero) with fewer instructions.
__host__ __device__ __forceinline__ ddc cmul(ddc a, ddc b) { return cmul_cs(a, re(b), im(b)); }
// a * conj(b)
__host__ __device__ __forceinline__ ddc cmulc(ddc a, ddc b) { return cmul_cs(a, re(b), -im(b)); }
__host__ __device__ __forceinline__ ddc cneg(ddc a) {
  return ddc{make_float2(-a.hi.x, -a.hi.y), make_float2(-a.lo.x, -a.lo.y)};
}
__host__ __device__ __forceinline__ bool cnonzero(ddc a) {
  return a.hi.x != 0.0f || a.lo.x != 0.0f || a.hi.y != 0.0f || a.lo.y != 0.0f;
}

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

// Block magnitude keys. The largest biased exponent field of a block's values (1..2046 for a
// normal maximum, 2047 when the block holds inf or NaN, 0 for zeros and subnormals only) is the
// key of every block that holds a normal value. A block of zeros and subnormals only is scanned
// again with dd_subnormal_key, whose maximum (the largest subnormal's effective biased exponent
// minus one, -52..-1; kDdNoSubnormal for zeros) becomes the key (0 when the block is all zeros).
constexpr int kDdNoSubnormal = -0x7fffffff - 1;
__host__ __device__ __forceinline__ int dd_subnormal_key(double v) {
  const unsigned long long f = dd_bits64(v) & 0xFFFFFFFFFFFFFull;
  // effective biased exponent of a subnormal: 1 - (shift of its leading bit to the implicit bit)
  // = 12 - clz64(f); the key is one less
  return f ? 11 - dd_clz64(f) : kDdNoSubnormal;
}
// Scale exponent k for a block with magnitude key `key`: 2^k * max in [1, 2). Zero and
// non-finite blocks use k = 0.
__host__ __device__ __forceinline__ int dd_block_scale(int key) {
  return (key == 0 || key == 2047) ? 0 : (key > 0 ? 1023 - key : 1022 - key);
}

// dd from the sign, the scaled exponent e of the leading bit and the fraction bits 1..23 (top) and
// 24..46 (next) of a binary64 value: see dd_from_double.
__host__ __device__ __forceinline__ dd dd_assemble(unsigned sign, int e, unsigned top, unsigned next) {
  const float hi = dd_float_from_bits(e < -126 ? sign : (sign | (static_cast<unsigned>(e + 127) << 23) | top));
  const unsigned base = sign | (static_cast<unsigned>(e + 104) << 23);
  const float lo = e < -103 ? dd_float_from_bits(sign) : dd_float_from_bits(base | next) - dd_float_from_bits(base);
  return dd(hi, lo);
}

// v * 2^k as dd: hi takes the top 24 significant bits of v (truncated), lo the next 23 (the last
// 6 of binary64's 53 are dropped: relative error below 2^-46). lo is formed exactly on the FP32
// pipe as (2^(e-23) * 1.f) - 2^(e-23) from two assembled bit patterns, so no count of leading
// zeros or variable shift is needed. Values whose scaled exponent e is below -126 become signed
// zero (their lo already below e = -103), and so do binary64 subnormals; above 127 they become
// infinity. Callers choose k so that the block maximum lands in [1, 2); subnormals then lie more
// than 2^60 below it unless k >= 962, where the callers use dd_from_double_exact.
__host__ __device__ __forceinline__ dd dd_from_double(double v, int k) {
  const unsigned long long u = dd_bits64(v);
  const unsigned hw = static_cast<unsigned>(u >> 32), lw = static_cast<unsigned>(u);
  const unsigned sign = hw & 0x80000000u;
  const int E = static_cast<int>((hw >> 20) & 0x7ffu);
  const int e = E - 1023 + k;
  if (e > 127) {  // overflow, or inf / NaN (k = 0 for blocks that hold them)
    const bool nan = E == 0x7ff && (((hw & 0xFFFFFu) | lw) != 0u);
    return dd(dd_float_from_bits(sign | 0x7f800000u | (nan ? 0x400000u : 0u)), 0.0f);
  }
  return dd_assemble(sign, E == 0 ? -1000 : e, ((hw & 0xFFFFFu) << 3) | (lw >> 29), (lw >> 6) & 0x7FFFFFu);
}

// dd_from_double for every binary64 class: a subnormal v is normalised first (its fraction
// shifted up to the implicit bit, its exponent lowered to match: E = 1 - shift).
__host__ __device__ __forceinline__ dd dd_from_double_exact(double v, int k) {
  const unsigned long long u = dd_bits64(v);
  const unsigned long long f = u & 0xFFFFFFFFFFFFFull;
  if (((u >> 52) & 0x7ffu) != 0u || f == 0ull) return dd_from_double(v, k);
  const unsigned sign = static_cast<unsigned>(u >> 32) & 0x80000000u;
  const int lz = dd_clz64(f) - 11;  // 1 .. 52
  const unsigned long long m = (f << lz) & 0xFFFFFFFFFFFFFull;
  const unsigned hw = static_cast<unsigned>(m >> 32), lw = static_cast<unsigned>(m);
  const int e = (1 - lz) - 1023 + k;
  if (e > 127) return dd(dd_float_from_bits(sign | 0x7f800000u), 0.0f);
  return dd_assemble(sign, e, (hw << 3) | (lw >> 29), (lw >> 6) & 0x7FFFFFu);
}

// Rounded m * 2^s for s <= 28 (round half up), as an integer count.
__host__ __device__ __forceinline__ unsigned long long dd_shift_round(unsigned m, int s) {
  if (s >= 0) return static_cast<unsigned long long>(m) << s;
  if (s <= -32) return 0ull;
  return (static_cast<unsigned long long>(m) + (1ull << (-s - 1))) >> (-s);
}

// (hi + lo) * 2^k as a double, faithfully rounded (error below one unit in the last place), for
// any pair of binary32 values whose sum is finite: two_sum first makes |lo| <= ulp(hi) / 2, then
// lo is added to hi's binary64 bit pattern as an integer count of binary64 ulps of hi (at most
// 2^28 in magnitude, so the sum never carries into the next binade; when hi is a power of two and
// lo pulls below it the count is doubled, since the ulps there are half as large, except at the
// bottom of the normal range where the subnormal ulps below are not). Scaled results below the
// binary64 normal range become signed zero (dd_to_double_exact assembles them as subnormals),
// above it infinity; inf / NaN in hi pass through. Integer and FP32 instructions only.
__host__ __device__ __forceinline__ double dd_to_double(dd v, int k) {
  const dd n = dd_two_sum(v.hi, v.lo);
  const unsigned hb = dd_bits32(n.hi), lb = dd_bits32(n.lo);
  const unsigned sign = hb & 0x80000000u;
  const int eh = static_cast<int>((hb >> 23) & 0xffu);
  if (eh == 0xff) {
    return dd_double_from_bits((static_cast<unsigned long long>(sign) << 32) | 0x7ff0000000000000ull |
                               ((hb & 0x7fffffu) ? 0x8000000000000ull : 0ull));
  }
  const int E = eh - 127 + k + 1023;  // biased binary64 exponent of hi * 2^k
  if (eh == 0 || E <= 0) return dd_double_from_bits(static_cast<unsigned long long>(sign) << 32);
  if (E >= 2047) return dd_double_from_bits((static_cast<unsigned long long>(sign) << 32) | 0x7ff0000000000000ull);
  const unsigned long long H =
      (static_cast<unsigned long long>(sign | (static_cast<unsigned>(E) << 20) | ((hb >> 3) & 0xFFFFFu)) << 32) |
      static_cast<unsigned long long>(hb << 29);
  const int el = static_cast<int>((lb >> 23) & 0xffu);
  const unsigned ml = el ? ((lb & 0x7FFFFFu) | 0x800000u) : 0u;
  const bool opposite = ((hb ^ lb) >> 31) != 0u;
  const int s = 29 + el - eh + ((opposite && (hb & 0x7FFFFFu) == 0u && E > 1) ? 1 : 0);  // <= 6
  unsigned y;
  if (s >= 0) {
    y = ml << s;
  } else if (s > -25) {
    y = (ml + (1u << (-s - 1))) >> (-s);
  } else {
    y = 0u;
  }
  const unsigned long long Y = static_cast<unsigned long long>(y);
  return dd_double_from_bits(opposite ? H - Y : H + Y);
}

// dd_to_double with results below the binary64 normal range assembled as subnormals: for a
// normalised pair (hb, lb after two_sum, hi normal) with E, the biased binary64 exponent of
// hi * 2^k, at most 0, hi * 2^k = Mh * 2^(E + 28) and lo * 2^k = Ml * 2^(E + 28 + el' - eh) in units
// of 2^-1074 (el' = 1 for a subnormal lo), each rounded to an integer count and added (an error
// of at most one subnormal unit). A count of 2^52 is the smallest normal, which the bit pattern
// encodes by itself. Results below half the smallest subnormal become signed zero.
__host__ __device__ __forceinline__ double dd_to_double_exact(dd v, int k) {
  const dd n = dd_two_sum(v.hi, v.lo);
  const unsigned hb = dd_bits32(n.hi), lb = dd_bits32(n.lo);
  const int eh = static_cast<int>((hb >> 23) & 0xffu);
  const int E = eh - 127 + k + 1023;
  if (eh == 0xff || eh == 0 || E > 0) return dd_to_double(v, k);
  const unsigned sign = hb & 0x80000000u;
  if (E < -60) return dd_double_from_bits(static_cast<unsigned long long>(sign) << 32);
  const int el = static_cast<int>((lb >> 23) & 0xffu);
  const unsigned ml = el ? ((lb & 0x7FFFFFu) | 0x800000u) : (lb & 0x7FFFFFu);
  const int sh = E + 28;
  const unsigned long long H = dd_shift_round((hb & 0x7FFFFFu) | 0x800000u, sh);
  const unsigned long long L = dd_shift_round(ml, sh + (el ? el : 1) - eh);
  const bool opposite = ((hb ^ lb) >> 31) != 0u;
  const unsigned long long T = opposite ? (H > L ? H - L : 0ull) : H + L;
  return dd_double_from_bits((static_cast<unsigned long long>(sign) << 32) | T);
}

}  // namespace gb300
}  // namespace spfft
