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
// Multiplication by 1/2 (double-float overloads it with an exact two-part scaling).
__host__ __device__ __forceinline__ float half_of(float a) { return 0.5f * a; }
__host__ __device__ __forceinline__ double half_of(double a) { return 0.5 * a; }
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
  using T = decltype(v[0].x);
  constexpr T h = T(0.8660254037844386467637232);  // sin(2 pi / 3)
  C t1 = cadd(v[1], v[2]);
  C t2 = csub(v[1], v[2]);
  C m = make_c(v[0].x - half_of(t1.x), v[0].y - half_of(t1.y));
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
  using T = decltype(v[0].x);
  constexpr T c1 = T(0.3090169943749474241022934), c2 = T(-0.8090169943749474241022934);
  constexpr T s1 = T(0.9510565162951535721164393), s2 = T(0.5877852522924731291687060);
  C a = cadd(v[1], v[4]), b = cadd(v[2], v[3]);
  C c = csub(v[1], v[4]), d = csub(v[2], v[3]);
  C x0 = v[0];
  v[0] = cadd(x0, cadd(a, b));
  C m1 = make_c(x0.x + c1 * a.x + c2 * b.x, x0.y + c1 * a.y + c2 * b.y);
  C m2 = make_c(x0.x + c2 * a.x + c1 * b.x, x0.y + c2 * a.y + c1 * b.y);
  C n1 = cmul_i<SIGN>(make_c(s1 * c.x + s2 * d.x, s1 * c.y + s2 * d.y));
  C n2 = cmul_i<SIGN>(make_c(s2 * c.x - s1 * d.x, s2 * c.y - s1 * d.y));
  v[1] = cadd(m1, n1);
  v[4] = csub(m1, n1);
  v[2] = cadd(m2, n2);
  v[3] = csub(m2, n2);
}

template <int SIGN, typename C>
__host__ __device__ __forceinline__ void dft7(C* v) {
  using T = decltype(v[0].x);
  constexpr T C1 = T(0.6234898018587335305250049), C2 = T(-0.2225209339563144042889026),
              C3 = T(-0.9009688679024191262361023);
  constexpr T S1 = T(0.7818314824680298087084445), S2 = T(0.9749279121818236070181317),
              S3 = T(0.4338837391175581204757683);
  C a1 = cadd(v[1], v[6]), a2 = cadd(v[2], v[5]), a3 = cadd(v[3], v[4]);
  C d1 = csub(v[1], v[6]), d2 = csub(v[2], v[5]), d3 = csub(v[3], v[4]);
  C x0 = v[0];
  v[0] = cadd(x0, cadd(a1, cadd(a2, a3)));
  // q = 1: cos (C1, C2, C3), sin (S1, S2, S3)
  C m = make_c(x0.x + C1 * a1.x + C2 * a2.x + C3 * a3.x, x0.y + C1 * a1.y + C2 * a2.y + C3 * a3.y);
  C n = cmul_i<SIGN>(make_c(S1 * d1.x + S2 * d2.x + S3 * d3.x, S1 * d1.y + S2 * d2.y + S3 * d3.y));
  v[1] = cadd(m, n);
  v[6] = csub(m, n);
  // q = 2: cos (C2, C3, C1), sin (S2, -S3, -S1)
  m = make_c(x0.x + C2 * a1.x + C3 * a2.x + C1 * a3.x, x0.y + C2 * a1.y + C3 * a2.y + C1 * a3.y);
  n = cmul_i<SIGN>(make_c(S2 * d1.x - S3 * d2.x - S1 * d3.x, S2 * d1.y - S3 * d2.y - S1 * d3.y));
  v[2] = cadd(m, n);
  v[5] = csub(m, n);
  // q = 3: cos (C3, C1, C2), sin (S3, -S1, S2)
  m = make_c(x0.x + C3 * a1.x + C1 * a2.x + C2 * a3.x, x0.y + C3 * a1.y + C1 * a2.y + C2 * a3.y);
  n = cmul_i<SIGN>(make_c(S3 * d1.x - S1 * d2.x + S2 * d3.x, S3 * d1.y - S1 * d2.y + S2 * d3.y));
  v[3] = cadd(m, n);
  v[4] = csub(m, n);
}

template <int SIGN, typename C>
__host__ __device__ __forceinline__ void dft8(C* v) {
  using T = decltype(v[0].x);
  constexpr T r = T(0.7071067811865475244008444);
  C b[4], c[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    b[i] = cadd(v[i], v[i + 4]);
    c[i] = csub(v[i], v[i + 4]);
  }
  // c_r *= exp(sign * 2 pi i r / 8)
  c[1] = make_c(r * (c[1].x - SIGN * c[1].y), r * (c[1].y + SIGN * c[1].x));
  c[2] = cmul_i<SIGN>(c[2]);
  c[3] = make_c(r * (-c[3].x - SIGN * c[3].y), r * (-c[3].y + SIGN * c[3].x));
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
