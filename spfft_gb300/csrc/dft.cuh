// Register DFTs of compile-time size: Dft<R, SIGN>::run(v) replaces v[0..R) by its length-R DFT
// with root exp(SIGN * 2 pi i / R), in natural order. Sizes 2, 3, 4, 5, 7, 8 are hand-written
// butterflies (fft_core.cuh); composite sizes are built as R = R1 * R2 from two register passes and
// constant twiddles (Cooley-Tukey), fully unrolled so that every value stays in registers.
#pragma once

#include "dd.cuh"
#include "fft_core.cuh"
#include "twiddle_constants.hpp"

namespace spfft {
namespace gb300 {

// cos / sin of 2 pi m / R in the arithmetic type T. Double-float takes the generated float pairs,
// so forming a constant never needs a binary64 instruction.
template <typename T>
struct TwConst {
  __host__ __device__ static T cos(int r, int m) { return T(tw_cos(r, m)); }
  __host__ __device__ static T sin(int r, int m) { return T(tw_sin(r, m)); }
};
template <>
struct TwConst<dd> {
  __host__ __device__ static dd cos(int r, int m) { return dd(tw_cos_pair_hi(r, m), tw_cos_pair_lo(r, m)); }
  __host__ __device__ static dd sin(int r, int m) { return dd(tw_sin_pair_hi(r, m), tw_sin_pair_lo(r, m)); }
};

// Multiply by exp(SIGN * 2 pi i * m / R) with m, R compile-time constants after unrolling.
template <int R, int SIGN, typename C>
__host__ __device__ __forceinline__ C twiddle_const(C a, int m) {
  using T = decltype(re(a));
  m %= R;
  if (m == 0) return a;
  if (2 * m == R) return cneg(a);
  if (4 * m == R) return cmul_i<SIGN>(a);
  if (4 * m == 3 * R) return cmul_i<-SIGN>(a);
  const T c = TwConst<T>::cos(R, m);
  const T s = SIGN > 0 ? TwConst<T>::sin(R, m) : -TwConst<T>::sin(R, m);
  return cmul_cs(a, c, s);
}

template <int R>
struct Factor;  // R = first * second for composite register sizes
template <> struct Factor<6> { static constexpr int first = 3, second = 2; };
template <> struct Factor<9> { static constexpr int first = 3, second = 3; };
template <> struct Factor<10> { static constexpr int first = 5, second = 2; };
template <> struct Factor<12> { static constexpr int first = 4, second = 3; };
template <> struct Factor<15> { static constexpr int first = 5, second = 3; };
template <> struct Factor<16> { static constexpr int first = 4, second = 4; };
template <> struct Factor<18> { static constexpr int first = 9, second = 2; };
template <> struct Factor<20> { static constexpr int first = 5, second = 4; };
template <> struct Factor<24> { static constexpr int first = 8, second = 3; };
template <> struct Factor<25> { static constexpr int first = 5, second = 5; };
template <> struct Factor<27> { static constexpr int first = 9, second = 3; };
template <> struct Factor<30> { static constexpr int first = 6, second = 5; };
template <> struct Factor<32> { static constexpr int first = 8, second = 4; };

template <int R, int SIGN>
struct Dft {
  // Composite: R2 DFTs of size R1 on stride-R2 elements, twiddles, R1 DFTs of size R2.
  template <typename C>
  __host__ __device__ __forceinline__ static void run(C* v);
};

template <int SIGN>
struct Dft<1, SIGN> {
  template <typename C>
  __host__ __device__ __forceinline__ static void run(C*) {}
};
template <int SIGN>
struct Dft<2, SIGN> {
  template <typename C>
  __host__ __device__ __forceinline__ static void run(C* v) { dft2<SIGN>(v); }
};
template <int SIGN>
struct Dft<3, SIGN> {
  template <typename C>
  __host__ __device__ __forceinline__ static void run(C* v) { dft3<SIGN>(v); }
};
template <int SIGN>
struct Dft<4, SIGN> {
  template <typename C>
  __host__ __device__ __forceinline__ static void run(C* v) { dft4<SIGN>(v); }
};
template <int SIGN>
struct Dft<5, SIGN> {
  template <typename C>
  __host__ __device__ __forceinline__ static void run(C* v) { dft5<SIGN>(v); }
};
template <int SIGN>
struct Dft<7, SIGN> {
  template <typename C>
  __host__ __device__ __forceinline__ static void run(C* v) { dft7<SIGN>(v); }
};
template <int SIGN>
struct Dft<8, SIGN> {
  template <typename C>
  __host__ __device__ __forceinline__ static void run(C* v) { dft8<SIGN>(v); }
};

template <int R, int SIGN>
template <typename C>
__host__ __device__ __forceinline__ void Dft<R, SIGN>::run(C* v) {
  constexpr int R1 = Factor<R>::first, R2 = Factor<R>::second;
  C t[R];
#pragma unroll
  for (int i2 = 0; i2 < R2; ++i2) {
    C a[R1];
#pragma unroll
    for (int i1 = 0; i1 < R1; ++i1) a[i1] = v[i1 * R2 + i2];
    Dft<R1, SIGN>::run(a);
#pragma unroll
    for (int k1 = 0; k1 < R1; ++k1) t[k1 * R2 + i2] = twiddle_const<R, SIGN>(a[k1], k1 * i2);
  }
#pragma unroll
  for (int k1 = 0; k1 < R1; ++k1) {
    C b[R2];
#pragma unroll
    for (int i2 = 0; i2 < R2; ++i2) b[i2] = t[k1 * R2 + i2];
    Dft<R2, SIGN>::run(b);
#pragma unroll
    for (int k2 = 0; k2 < R2; ++k2) v[k1 + R1 * k2] = b[k2];
  }
}

// ---- two-pass FFT of length N = A * B on data in shared memory ---------------------------------
//
// Input element n = a*B + b sits at buf[n * stride]. Pass 1 (one work item per b): DFT_A over a,
// multiply by w_N^(k1*b), store back at the same places (k1*B + b). Pass 2 (one work item per
// k1): DFT_B over b; the result X[k1 + A*k2] is left in registers (v[k2]) for the caller, which
// either emits it or stores it back in place at buf[(k1*B + k2) * stride] -- the "transposed"
// order, where X[k] lives at position (k mod A)*B + k div A. tw is the w_N table (forward sign).
template <int N, int V = 0>
struct Shape;  // N = A * B; V = 1 selects the split of the z and split-y kernels
#define SPFFT_GB300_SHAPE(N_, A_, B_)        \
  template <>                              \
  struct Shape<N_, 0> {                    \
    static constexpr int A = A_, B = B_;   \
  };
SPFFT_GB300_SHAPE(3, 3, 1)
SPFFT_GB300_SHAPE(4, 4, 1)
SPFFT_GB300_SHAPE(6, 6, 1)
SPFFT_GB300_SHAPE(8, 8, 1)
SPFFT_GB300_SHAPE(12, 12, 1)
SPFFT_GB300_SHAPE(16, 16, 1)
SPFFT_GB300_SHAPE(24, 8, 3)
SPFFT_GB300_SHAPE(30, 6, 5)
SPFFT_GB300_SHAPE(32, 8, 4)
SPFFT_GB300_SHAPE(36, 6, 6)
SPFFT_GB300_SHAPE(45, 9, 5)
SPFFT_GB300_SHAPE(48, 8, 6)
SPFFT_GB300_SHAPE(50, 10, 5)
SPFFT_GB300_SHAPE(54, 9, 6)
SPFFT_GB300_SHAPE(60, 10, 6)
SPFFT_GB300_SHAPE(64, 8, 8)
SPFFT_GB300_SHAPE(72, 9, 8)
SPFFT_GB300_SHAPE(75, 15, 5)
SPFFT_GB300_SHAPE(80, 10, 8)
SPFFT_GB300_SHAPE(90, 10, 9)
SPFFT_GB300_SHAPE(96, 12, 8)
SPFFT_GB300_SHAPE(100, 10, 10)
SPFFT_GB300_SHAPE(108, 12, 9)
SPFFT_GB300_SHAPE(120, 12, 10)
SPFFT_GB300_SHAPE(128, 16, 8)
SPFFT_GB300_SHAPE(144, 12, 12)
SPFFT_GB300_SHAPE(150, 15, 10)
SPFFT_GB300_SHAPE(160, 16, 10)
SPFFT_GB300_SHAPE(180, 15, 12)
SPFFT_GB300_SHAPE(192, 16, 12)
SPFFT_GB300_SHAPE(240, 16, 15)
SPFFT_GB300_SHAPE(256, 16, 16)
#undef SPFFT_GB300_SHAPE
// Variant 1 is variant 0 except where another split measured faster: 192 = 12 x 16 in the z
// kernels, the split y kernels and the y pass of the fused backward plane kernel (FP64 y backward
// 39.6 -> 35.5 us, FP32 batched z passes 4-6 % and fused backward 1 % faster); the fused forward
// plane kernel keeps 16 x 12, which it runs 4 % faster.
template <int N>
struct Shape<N, 1> : Shape<N, 0> {};
template <>
struct Shape<192, 1> {
  static constexpr int A = 12, B = 16;
};
// Variant 2 swaps the two factors of variant 1 (B x A instead of A x B): the z and split-y kernels
// are built in both orders for every length where the swap differs, and the autotuner chooses one
// per pass.
template <int N>
struct Shape<N, 2> {
  static constexpr int A = Shape<N, 1>::B > 1 ? Shape<N, 1>::B : Shape<N, 1>::A;
  static constexpr int B = Shape<N, 1>::B > 1 ? Shape<N, 1>::A : 1;
};
template <int N>
constexpr bool has_swapped_split() {
  return Shape<N, 2>::A != Shape<N, 1>::A;
}

// Variant 3 is variant 1 run in three passes: the B-point DFT of pass 2 is itself split as
// B = B1 * B2 (Factor<B>) into a pass of B1-point DFTs (pass 2a, with the w_B twiddles) and a
// pass of B2-point DFTs (pass 2b), with one more shared-memory exchange between them. No work item
// then holds more than max(A, B1, B2) values (double-float 16-point DFTs need more registers than
// three blocks per SM leave a thread), and pass 2 has B2 (2a) and B1 (2b) times as many work items.
template <int N>
struct Shape<N, 3> : Shape<N, 1> {};
template <int R>
struct HasFactor {
  static constexpr bool value = false;
};
#define SPFFT_GB300_HAS_FACTOR(R_) \
  template <>                      \
  struct HasFactor<R_> {           \
    static constexpr bool value = true; \
  };
SPFFT_GB300_HAS_FACTOR(12)
SPFFT_GB300_HAS_FACTOR(16)
#undef SPFFT_GB300_HAS_FACTOR
// Lengths that have the three-pass variant: a second factor of 12 or 16.
template <int N>
constexpr bool has_three_pass() {
  return HasFactor<Shape<N, 1>::B>::value;
}
template <int N, bool = has_three_pass<N>()>
struct Split3 {
  static constexpr int A = Shape<N, 1>::A, B = Shape<N, 1>::B, B1 = 1, B2 = 1;
};
template <int N>
struct Split3<N, true> {
  static constexpr int A = Shape<N, 1>::A, B = Shape<N, 1>::B;
  static constexpr int B1 = Factor<B>::first, B2 = Factor<B>::second;
};

// Position of X[k] after pass 2 stored back in place: (k mod A) * B + k div A for the two-pass
// variants; for variant 3, pass 2b leaves X[k1 + A (kk1 + B1 kk2)] at k1 B + kk1 B2 + kk2.
template <int N, int V = 0>
__host__ __device__ __forceinline__ int transposed_pos(int k) {
  constexpr int A = Shape<N, V>::A, B = Shape<N, V>::B;
  if constexpr (V == 3) {
    constexpr int B1 = Split3<N>::B1, B2 = Split3<N>::B2;
    const int k2 = k / A;
    return (k - k2 * A) * B + (k2 % B1) * B2 + k2 / B1;
  } else {
    return (k % A) * B + k / A;
  }
}
// Rotated in-place outputs of the two-pass variants: pass-2 work item k1 stores X[k1 + A k2] at
// k1 B + (k2 + k1 mod B) mod B, still inside its own B slots. Unrotated, the outputs of consecutive
// k1 sit B slots apart, all in one shared-memory bank when B is a multiple of 16; rotated,
// consecutive outputs fall in different banks, and a gather in output order (192 = 12 x 16, 8-byte
// values) takes about 2 wavefronts per half-warp instead of 10. Variant 3 keeps transposed_pos
// (its pass 2b items own B2 slots each, too few to rotate within).
template <int N, int V = 0>
__host__ __device__ __forceinline__ int rotated_slot(int k1, int k2) {
  constexpr int A = Shape<N, V>::A, B = Shape<N, V>::B;
  const int r = A <= B ? k1 : k1 % B;
  const int q = k2 + r;
  return k1 * B + (q >= B ? q - B : q);
}
template <int N, int V = 0>
__host__ __device__ __forceinline__ int rotated_pos(int k) {
  if constexpr (V == 3) {
    return transposed_pos<N, V>(k);
  } else {
    constexpr int A = Shape<N, V>::A;
    const int k2 = k / A;
    return rotated_slot<N, V>(k - k2 * A, k2);
  }
}
// Variant 3: the output index k of the value pass 2b leaves at in-place position e.
template <int N>
__host__ __device__ __forceinline__ int three_pass_index(int e) {
  constexpr int A = Split3<N>::A, B = Split3<N>::B, B1 = Split3<N>::B1, B2 = Split3<N>::B2;
  const int k1 = e / B, r = e - k1 * B, kk1 = r / B2, kk2 = r - kk1 * B2;
  return k1 + A * (kk1 + B1 * kk2);
}

template <int N, int SIGN, int V = 0, typename C>
__host__ __device__ __forceinline__ void fft_pass1(C* buf, int stride, int b, const C* __restrict__ tw) {
  constexpr int A = Shape<N, V>::A, B = Shape<N, V>::B;
  C v[A];
#pragma unroll
  for (int a = 0; a < A; ++a) v[a] = buf[(a * B + b) * stride];
  Dft<A, SIGN>::run(v);
  if (B > 1) {
#pragma unroll
    for (int k1 = 1; k1 < A; ++k1) v[k1] = ctw<SIGN>(v[k1], tw[k1 * b]);
  }
#pragma unroll
  for (int k1 = 0; k1 < A; ++k1) buf[(k1 * B + b) * stride] = v[k1];
}

// Pass 1 with its twiddles in pass-1 order, tw1[k1 * B + b] = w^(k1 b): the work items b of a
// warp read consecutive entries (no bank conflicts; tw[k1 * b] puts b and b + 16 / gcd(k1, 16) in
// one bank) at constant offsets from tw1 + b.
template <int N, int SIGN, int V = 0, typename C>
__host__ __device__ __forceinline__ void fft_pass1_ordered(C* buf, int stride, int b, const C* __restrict__ tw1) {
  constexpr int A = Shape<N, V>::A, B = Shape<N, V>::B;
  C v[A];
#pragma unroll
  for (int a = 0; a < A; ++a) v[a] = buf[(a * B + b) * stride];
  Dft<A, SIGN>::run(v);
  if (B > 1) {
    const C* t = tw1 + b;
#pragma unroll
    for (int k1 = 1; k1 < A; ++k1) v[k1] = ctw<SIGN>(v[k1], t[k1 * B]);
  }
#pragma unroll
  for (int k1 = 0; k1 < A; ++k1) buf[(k1 * B + b) * stride] = v[k1];
}

// Pass 1 with the inputs already in registers (loaded by the caller from elsewhere).
template <int N, int SIGN, int V = 0, typename C>
__host__ __device__ __forceinline__ void fft_pass1_regs(C (&v)[Shape<N, V>::A], int b, const C* __restrict__ tw) {
  constexpr int A = Shape<N, V>::A, B = Shape<N, V>::B;
  Dft<A, SIGN>::run(v);
  if (B > 1) {
#pragma unroll
    for (int k1 = 1; k1 < A; ++k1) v[k1] = ctw<SIGN>(v[k1], tw[k1 * b]);
  }
}

// fft_pass1_regs with the twiddles in pass-1 order (tw1[k1 * B + b] = w^(k1 b), as for
// fft_pass1_ordered).
template <int N, int SIGN, int V = 0, typename C>
__host__ __device__ __forceinline__ void fft_pass1_regs_ordered(C (&v)[Shape<N, V>::A], int b, const C* __restrict__ tw1) {
  constexpr int A = Shape<N, V>::A, B = Shape<N, V>::B;
  Dft<A, SIGN>::run(v);
  if (B > 1) {
    const C* t = tw1 + b;
#pragma unroll
    for (int k1 = 1; k1 < A; ++k1) v[k1] = ctw<SIGN>(v[k1], t[k1 * B]);
  }
}

template <int N, int SIGN, int V = 0, typename C>
__host__ __device__ __forceinline__ void fft_pass2(const C* buf, int stride, int k1, C (&v)[Shape<N, V>::B]) {
  constexpr int B = Shape<N, V>::B;
#pragma unroll
  for (int b = 0; b < B; ++b) v[b] = buf[(k1 * B + b) * stride];
  Dft<B, SIGN>::run(v);
}

// Variant 3, pass 2a (one work item per (k1, i2), after pass 1): the B1-point DFTs over
// b = i1 * B2 + i2 of row k1, times w_B^(kk1 * i2) = w_N^(kk1 * i2 * A) from the same w_N table,
// stored back in place at k1 * B + kk1 * B2 + i2 (the first half of Dft<B>::run).
template <int N, int SIGN, typename C>
__host__ __device__ __forceinline__ void fft_pass2a(C* buf, int stride, int k1, int i2, const C* __restrict__ tw) {
  constexpr int A = Split3<N>::A, B = Split3<N>::B, B1 = Split3<N>::B1, B2 = Split3<N>::B2;
  C v[B1];
#pragma unroll
  for (int i1 = 0; i1 < B1; ++i1) v[i1] = buf[(k1 * B + i1 * B2 + i2) * stride];
  Dft<B1, SIGN>::run(v);
#pragma unroll
  for (int kk1 = 1; kk1 < B1; ++kk1) v[kk1] = ctw<SIGN>(v[kk1], tw[kk1 * i2 * A]);
#pragma unroll
  for (int kk1 = 0; kk1 < B1; ++kk1) buf[(k1 * B + kk1 * B2 + i2) * stride] = v[kk1];
}

// Variant 3, pass 2b (one work item per (k1, kk1), after pass 2a): the B2-point DFT over i2;
// v[kk2] = X[k1 + A * (kk1 + B1 * kk2)] (the second half of Dft<B>::run).
template <int N, int SIGN, typename C>
__host__ __device__ __forceinline__ void fft_pass2b(const C* buf, int stride, int k1, int kk1,
                                                    C (&v)[Split3<N>::B2]) {
  constexpr int B = Split3<N>::B, B2 = Split3<N>::B2;
#pragma unroll
  for (int i2 = 0; i2 < B2; ++i2) v[i2] = buf[(k1 * B + kk1 * B2 + i2) * stride];
  Dft<B2, SIGN>::run(v);
}

}  // namespace gb300
}  // namespace spfft
