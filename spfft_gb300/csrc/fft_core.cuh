// Device FFT core: complex helpers, radix butterflies and a batched Stockham FFT that runs on data
// staged in shared memory.
//
// Stockham formulation (autosort, no bit reversal). For a length n = R_1 * R_2 * ... and a stage
// with radix R that follows stages whose radices multiply to Ns, butterfly j (0 <= j < n/R) reads
//   x_r = src[j + r * n/R],   r = 0..R-1,
// multiplies x_r by w^(r * (j mod Ns)) with w = exp(sign * 2 pi i / (Ns * R)), takes a length-R DFT
// and writes
//   dst[(j / Ns) * Ns * R + (j mod Ns) + q * Ns] = X_q.
// After the last stage dst holds the transform in natural order. sign = -1 is the forward
// (space -> frequency) direction, +1 the backward one, matching the transform definition of the
// reference (docs/source/details.rst:6-13).
#pragma once

#include <cuda_runtime.h>

#include "fft_plan.hpp"

namespace spfft {
namespace gb300 {

template <typename T>
struct Complex;
template <>
struct Complex<double> {
  using type = double2;
};
template <>
struct Complex<float> {
  using type = float2;
};

__host__ __device__ __forceinline__ double2 make_c(double x, double y) { return make_double2(x, y); }
// Real and imaginary parts (double-float complex values define their own).
__host__ __device__ __forceinline__ float re(float2 c) { return c.x; }
__host__ __device__ __forceinline__ float im(float2 c) { return c.y; }
__host__ __device__ __forceinline__ double re(double2 c) { return c.x; }
__host__ __device__ __forceinline__ double im(double2 c) { return c.y; }
// Multiplication by 1/2 (double-float overloads it with an exact two-part scaling).
__host__ __device__ __forceinline__ float half_of(float a) { return 0.5f * a; }
__host__ __device__ __forceinline__ double half_of(double a) { return 0.5 * a; }
__host__ __device__ __forceinline__ float2 make_c(float x, float y) { return make_float2(x, y); }

template <typename C>
__host__ __device__ __forceinline__ C cadd(C a, C b) {
  return make_c(a.x + b.x, a.y + b.y);
}
template <typename C>
__host__ __device__ __forceinline__ C csub(C a, C b) {
  return make_c(a.x - b.x, a.y - b.y);
}
template <typename C>
__host__ __device__ __forceinline__ C cmul(C a, C b) {
  return make_c(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
template <typename C>
__host__ __device__ __forceinline__ C cmulc(C a, C b) {
  return make_c(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
template <typename C, typename T>
__host__ __device__ __forceinline__ C cscale(C a, T s) {
  return make_c(a.x * s, a.y * s);
}
// a * (c + i s) for real c, s
template <typename C, typename T>
__host__ __device__ __forceinline__ C cmul_cs(C a, T c, T s) {
  return make_c(a.x * c - a.y * s, a.x * s + a.y * c);
}
template <typename C>
__host__ __device__ __forceinline__ C cneg(C a) {
  return make_c(-a.x, -a.y);
}
// a * s + b for a real s
template <typename C, typename T>
__host__ __device__ __forceinline__ C cfma_r(C a, T s, C b) {
  return make_c(a.x * s + b.x, a.y * s + b.y);
}
// a / 2
template <typename C>
__host__ __device__ __forceinline__ C chalf(C a) {
  return make_c(half_of(a.x), half_of(a.y));
}
// a - b / 2
template <typename C>
__host__ __device__ __forceinline__ C csub_half(C a, C b) {
  return make_c(a.x - half_of(b.x), a.y - half_of(b.y));
}

// FP32 complex values on sm_100 and later: the real and imaginary parts go through one packed
// FP32x2 instruction (FADD2 / FMUL2 / FFMA2) instead of two, which halves the issue slots of the
// butterflies' additions and real scalings. Each lane rounds exactly like the scalar instruction
// (a - b as b * -1 + a, a - b/2 as b * -0.5 + a: the products are exact, one rounding each).
#if defined(__CUDA_ARCH__) && (__CUDA_ARCH__ >= 1000)
#define SPFFT_GB300_PACKED_F32X2 1
#endif
__host__ __device__ __forceinline__ float2 cadd(float2 a, float2 b) {
#ifdef SPFFT_GB300_PACKED_F32X2
  return __fadd2_rn(a, b);
#else
  return make_float2(a.x + b.x, a.y + b.y);
#endif
}
__host__ __device__ __forceinline__ float2 csub(float2 a, float2 b) {
#ifdef SPFFT_GB300_PACKED_F32X2
  return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a);
#else
  return make_float2(a.x - b.x, a.y - b.y);
#endif
}
__host__ __device__ __forceinline__ float2 cscale(float2 a, float s) {
#ifdef SPFFT_GB300_PACKED_F32X2
  return __fmul2_rn(a, make_float2(s, s));
#else
  return make_float2(a.x * s, a.y * s);
#endif
}
__host__ __device__ __forceinline__ float2 cfma_r(float2 a, float s, float2 b) {
#ifdef SPFFT_GB300_PACKED_F32X2
  return __ffma2_rn(a, make_float2(s, s), b);
#else
  return make_float2(a.x * s + b.x, a.y * s + b.y);
#endif
}
__host__ __device__ __forceinline__ float2 chalf(float2 a) {
#ifdef SPFFT_GB300_PACKED_F32X2
  return __fmul2_rn(a, make_float2(0.5f, 0.5f));
#else
  return make_float2(0.5f * a.x, 0.5f * a.y);
#endif
}
__host__ __device__ __forceinline__ float2 csub_half(float2 a, float2 b) {
#ifdef SPFFT_GB300_PACKED_F32X2
  return __ffma2_rn(b, make_float2(-0.5f, -0.5f), a);
#else
  return make_float2(a.x - 0.5f * b.x, a.y - 0.5f * b.y);
#endif
}
template <typename C>
__host__ __device__ __forceinline__ C cconj(C a) {
  return make_c(a.x, -a.y);
}
// Multiply by sign * i.
template <int SIGN, typename C>
__host__ __device__ __forceinline__ C cmul_i(C a) {
  return SIGN > 0 ? make_c(-a.y, a.x) : make_c(a.y, -a.x);
}
// Multiply by the stage twiddle tw (stored for the forward sign); conjugated for SIGN = +1.
template <int SIGN, typename C>
__host__ __device__ __forceinline__ C ctw(C a, C tw) {
  return SIGN < 0 ? cmul(a, tw) : cmulc(a, tw);
}
template <typename C>
__host__ __device__ __forceinline__ bool cnonzero(C a) {
  return a.x != 0 || a.y != 0;
}

// ---- fixed-radix DFTs on registers (in place, natural output order) ---------------------------

template <int SIGN, typename C>
__host__ __device__ __forceinline__ void dft2(C* v) {
  C a = v[0], b = v[1];
  v[0] = cadd(a, b);
  v[1] = csub(a, b);
}

template <int SIGN, typename C>
__host__ __device__ __forceinline__ void dft3(C* v) {
  using T = decltype(re(v[0]));
  constexpr T h = T(0.8660254037844386467637232);  // sin(2 pi / 3)
  C t1 = cadd(v[1], v[2]);
  C t2 = csub(v[1], v[2]);
  C m = csub_half(v[0], t1);
  C n = cmul_i<SIGN>(cscale(t2, h));
  v[0] = cadd(v[0], t1);
  v[1] = cadd(m, n);
  v[2] = csub(m, n);
}

template <int SIGN, typename C>
__host__ __device__ __forceinline__ void dft4(C* v) {
  C t0 = cadd(v[0], v[2]);
  C t1 = csub(v[0], v[2]);
  C t2 = cadd(v[1], v[3]);
  C t3 = cmul_i<SIGN>(csub(v[1], v[3]));
  v[0] = cadd(t0, t2);
  v[2] = csub(t0, t2);
  v[1] = cadd(t1, t3);
  v[3] = csub(t1, t3);
}

template <int SIGN, typename C>
__host__ __device__ __forceinline__ void dft5(C* v) {
  using T = decltype(re(v[0]));
  constexpr T c1 = T(0.3090169943749474241022934), c2 = T(-0.8090169943749474241022934);
  constexpr T s1 = T(0.9510565162951535721164393), s2 = T(0.5877852522924731291687060);
  C a = cadd(v[1], v[4]), b = cadd(v[2], v[3]);
  C c = csub(v[1], v[4]), d = csub(v[2], v[3]);
  C x0 = v[0];
  v[0] = cadd(x0, cadd(a, b));
  C m1 = cfma_r(b, c2, cfma_r(a, c1, x0));
  C m2 = cfma_r(b, c1, cfma_r(a, c2, x0));
  C n1 = cmul_i<SIGN>(cfma_r(d, s2, cscale(c, s1)));
  C n2 = cmul_i<SIGN>(cfma_r(d, -s1, cscale(c, s2)));
  v[1] = cadd(m1, n1);
  v[4] = csub(m1, n1);
  v[2] = cadd(m2, n2);
  v[3] = csub(m2, n2);
}

template <int SIGN, typename C>
__host__ __device__ __forceinline__ void dft7(C* v) {
  using T = decltype(re(v[0]));
  constexpr T C1 = T(0.6234898018587335305250049), C2 = T(-0.2225209339563144042889026),
              C3 = T(-0.9009688679024191262361023);
  constexpr T S1 = T(0.7818314824680298087084445), S2 = T(0.9749279121818236070181317),
              S3 = T(0.4338837391175581204757683);
  C a1 = cadd(v[1], v[6]), a2 = cadd(v[2], v[5]), a3 = cadd(v[3], v[4]);
  C d1 = csub(v[1], v[6]), d2 = csub(v[2], v[5]), d3 = csub(v[3], v[4]);
  C x0 = v[0];
  v[0] = cadd(x0, cadd(a1, cadd(a2, a3)));
  // q = 1: cos (C1, C2, C3), sin (S1, S2, S3)
  C m = cfma_r(a3, C3, cfma_r(a2, C2, cfma_r(a1, C1, x0)));
  C n = cmul_i<SIGN>(cfma_r(d3, S3, cfma_r(d2, S2, cscale(d1, S1))));
  v[1] = cadd(m, n);
  v[6] = csub(m, n);
  // q = 2: cos (C2, C3, C1), sin (S2, -S3, -S1)
  m = cfma_r(a3, C1, cfma_r(a2, C3, cfma_r(a1, C2, x0)));
  n = cmul_i<SIGN>(cfma_r(d3, -S1, cfma_r(d2, -S3, cscale(d1, S2))));
  v[2] = cadd(m, n);
  v[5] = csub(m, n);
  // q = 3: cos (C3, C1, C2), sin (S3, -S1, S2)
  m = cfma_r(a3, C2, cfma_r(a2, C1, cfma_r(a1, C3, x0)));
  n = cmul_i<SIGN>(cfma_r(d3, S2, cfma_r(d2, -S1, cscale(d1, S3))));
  v[3] = cadd(m, n);
  v[4] = csub(m, n);
}

template <int SIGN, typename C>
__host__ __device__ __forceinline__ void dft8(C* v) {
  using T = decltype(re(v[0]));
  constexpr T r = T(0.7071067811865475244008444);
  C b[4], c[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    b[i] = cadd(v[i], v[i + 4]);
    c[i] = csub(v[i], v[i + 4]);
  }
  // c_r *= exp(sign * 2 pi i r / 8)
  c[1] = cscale(cadd(c[1], cmul_i<SIGN>(c[1])), r);
  c[2] = cmul_i<SIGN>(c[2]);
  c[3] = cscale(csub(cmul_i<SIGN>(c[3]), c[3]), r);
  dft4<SIGN>(b);
  dft4<SIGN>(c);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    v[2 * i] = b[i];
    v[2 * i + 1] = c[i];
  }
}

// One fixed-radix Stockham stage over `count` transforms.
template <int R, int SIGN, typename C>
__device__ __forceinline__ void stage_fixed(const C* __restrict__ src, C* __restrict__ dst,
                                            const C* __restrict__ tw, int n, int Ns, int count,
                                            int stride, int dist, bool fmajor) {
  const int m = n / R;
  const int total = count * m;
  const int twStep = n / (Ns * R);
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    int f, j;
    if (fmajor) {
      j = t / count;
      f = t - j * count;
    } else {
      f = t / m;
      j = t - f * m;
    }
    const int k = j % Ns;
    const C* in = src + f * dist;
    C* out = dst + f * dist;
    C v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = in[(j + r * m) * stride];
    if (k != 0) {
#pragma unroll
      for (int r = 1; r < R; ++r) v[r] = ctw<SIGN>(v[r], tw[r * k * twStep]);
    }
    if (R == 2) dft2<SIGN>(v);
    if (R == 3) dft3<SIGN>(v);
    if (R == 4) dft4<SIGN>(v);
    if (R == 5) dft5<SIGN>(v);
    if (R == 7) dft7<SIGN>(v);
    if (R == 8) dft8<SIGN>(v);
    const int base = (j - k) * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) out[(base + r * Ns) * stride] = v[r];
  }
}

// Generic radix stage (any R dividing n): one thread per output element, O(R) work each.
template <int SIGN, typename C>
__device__ __forceinline__ void stage_generic(const C* __restrict__ src, C* __restrict__ dst,
                                              const C* __restrict__ tw, int n, int R, int Ns,
                                              int count, int stride, int dist, bool fmajor) {
  const int m = n / R;
  const int total = count * m * R;
  const int twStep = n / (Ns * R);
  const int rootStep = n / R;
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    int f, jq;
    if (fmajor) {
      jq = t / count;
      f = t - jq * count;
    } else {
      f = t / (m * R);
      jq = t - f * (m * R);
    }
    const int q = jq / m;
    const int j = jq - q * m;
    const int k = j % Ns;
    const C* in = src + f * dist;
    C acc = make_c(decltype(acc.x)(0), decltype(acc.x)(0));
    int rq = 0;  // (r * q) mod R
    for (int r = 0; r < R; ++r) {
      C x = in[(j + r * m) * stride];
      if (k != 0 && r != 0) x = ctw<SIGN>(x, tw[r * k * twStep]);
      if (rq != 0) x = ctw<SIGN>(x, tw[rq * rootStep]);
      acc = cadd(acc, x);
      rq += q;
      if (rq >= R) rq -= R;
    }
    const int base = (j - k) * R + k;
    dst[f * dist + (base + q * Ns) * stride] = acc;
  }
}

// Batched FFT of `count` sequences of length plan.n held in shared memory.
// Element e of sequence f is at buf[f * dist + e * stride]. `a` holds the input; `b` is scratch of
// the same extent. Returns the buffer that holds the result. `fmajor` selects the thread mapping:
// consecutive threads take consecutive sequences (for strided, column-like data) instead of
// consecutive butterflies. Must be called by all threads of the block; ends with __syncthreads().
template <int SIGN, typename C>
__device__ C* smem_fft(C* a, C* b, const C* __restrict__ tw, const RadixPlan& plan, int count,
                       int stride, int dist, bool fmajor) {
  const int n = plan.n;
  int Ns = 1;
  for (int s = 0; s < plan.numStages; ++s) {
    const int R = plan.radix[s];
    switch (R) {
      case 2: stage_fixed<2, SIGN>(a, b, tw, n, Ns, count, stride, dist, fmajor); break;
      case 3: stage_fixed<3, SIGN>(a, b, tw, n, Ns, count, stride, dist, fmajor); break;
      case 4: stage_fixed<4, SIGN>(a, b, tw, n, Ns, count, stride, dist, fmajor); break;
      case 5: stage_fixed<5, SIGN>(a, b, tw, n, Ns, count, stride, dist, fmajor); break;
      case 7: stage_fixed<7, SIGN>(a, b, tw, n, Ns, count, stride, dist, fmajor); break;
      case 8: stage_fixed<8, SIGN>(a, b, tw, n, Ns, count, stride, dist, fmajor); break;
      default: stage_generic<SIGN>(a, b, tw, n, R, Ns, count, stride, dist, fmajor); break;
    }
    __syncthreads();
    C* t = a;
    a = b;
    b = t;
    Ns *= R;
  }
  return a;
}

}  // namespace gb300
}  // namespace spfft
