// Size-specialised transform kernels (compile-time FFT lengths, register DFTs, one in-place
// shared-memory exchange per 1D FFT). Two launches per direction:
//
//   backward: z kernel   values -> (scatter, stick symmetry, z-FFT) -> sticks[z][s]
//             plane      sticks of plane z -> compact plane in smem -> plane symmetry ->
//                        y-FFT on the non-empty x columns -> x-FFT (C2C, or C2R through a
//                        half-length complex FFT) -> space rows
//   forward:  plane      space rows -> x-FFT (C2C, or R2C through a half-length complex FFT) ->
//                        keep the non-empty columns -> y-FFT -> gather plane z of every stick
//             z kernel   sticks -> z-FFT -> gather (and scale) the values
//
// Replaces, fused: compression_kernels.cu:39-150, symmetry_kernels.cu:38-165,
// local_transpose_kernels.cu:43-201 and the cuFFT calls of transform_1d_gpu.hpp /
// transform_2d_gpu.hpp / transform_real_2d_gpu.hpp (all in the reference's src/). Compared with the
// generic kernels, the y and x passes are one kernel, so the compact plane never goes to HBM.
#pragma once

#include <cuda_runtime.h>

#include "dft.cuh"
#include "kernels.hpp"

namespace spfft {
namespace gb300 {
namespace fast {

template <typename T>
using C = typename Complex<T>::type;

constexpr int kThreads = 256;       // z-pass blocks
constexpr int kPlaneThreads = 512;  // plane blocks (one plane per block, so more warps per SM)

extern __shared__ __align__(16) unsigned char g_fast_smem[];

template <typename T>
__device__ __forceinline__ C<T> czero() {
  return make_c(T(0), T(0));
}

// Asynchronous global -> shared copy of one complex value (cp.async, 8 or 16 bytes). Lets a
// thread keep many loads in flight instead of waiting on each.
template <typename T>
__device__ __forceinline__ void cp_async_c(C<T>* smemDst, const C<T>* gmemSrc) {
  const unsigned dst = static_cast<unsigned>(__cvta_generic_to_shared(smemDst));
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(dst), "l"(gmemSrc),
               "n"(static_cast<int>(sizeof(C<T>)))
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int PENDING>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(PENDING) : "memory");
}

// Conditional conjugate fill along one line, two ordered halves (symmetry_host.hpp:42-90).
template <typename T>
__device__ __forceinline__ void line_fill(C<T>* v, int n, int stride) {
  for (int k = 1 + threadIdx.x; k < n / 2 + 1; k += blockDim.x) {
    C<T> a = v[k * stride];
    if (cnonzero(a)) v[(n - k) * stride] = cconj(a);
  }
  __syncthreads();
  for (int k = n / 2 + 1 + threadIdx.x; k < n; k += blockDim.x) {
    C<T> a = v[k * stride];
    if (cnonzero(a)) v[(n - k) * stride] = cconj(a);
  }
  __syncthreads();
}

// ================================================================================================
// z pass
// ================================================================================================
template <int NZ>
struct ZLayout {
  static constexpr int pitch = NZ | 1;  // odd: conflict-free column access across sticks
};

template <typename T, int NZ>
__global__ void __launch_bounds__(kThreads) z_backward(const PlanView<T> p,
                                                       const T* __restrict__ values, int spb) {
  constexpr int A = Shape<NZ>::A, B = Shape<NZ>::B, PZ = ZLayout<NZ>::pitch;
  C<T>* tw = reinterpret_cast<C<T>*>(g_fast_smem);
  C<T>* buf = tw + NZ;
  const int s0 = blockIdx.x * spb;
  const int nsb = min(spb, p.numSticks - s0);

  const C<T>* twg = reinterpret_cast<const C<T>*>(p.twz);
  for (int i = threadIdx.x; i < NZ; i += blockDim.x) tw[i] = twg[i];
  for (int i = threadIdx.x; i < nsb * PZ; i += blockDim.x) buf[i] = czero<T>();
  __syncthreads();

  const C<T>* vals = reinterpret_cast<const C<T>*>(values);
  const int e0 = p.stickEntryStart[s0], e1 = p.stickEntryStart[s0 + nsb];
  const int base = s0 * NZ;
  // Index loads four at a time, then asynchronous value copies straight to their stick slots.
  for (int e = e0 + threadIdx.x; e < e1; e += 4 * blockDim.x) {
    int pos[4], usr[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int eu = e + u * blockDim.x;
      pos[u] = eu < e1 ? p.entryPos[eu] - base : -1;
      usr[u] = eu < e1 ? p.entryUser[eu] : 0;
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      if (pos[u] >= 0) {
        const int sl = pos[u] / NZ;
        cp_async_c<T>(buf + sl * PZ + (pos[u] - sl * NZ), vals + usr[u]);
      }
    }
  }
  cp_async_commit();
  cp_async_wait<0>();
  __syncthreads();
  const int zz = p.zeroZeroStick - s0;
  if (p.r2c && zz >= 0 && zz < nsb) line_fill<T>(buf + zz * PZ, NZ, 1);

  for (int i = threadIdx.x; i < nsb * B; i += blockDim.x) {
    const int sl = i / B, b = i - sl * B;
    fft_pass1<NZ, +1>(buf + sl * PZ, 1, b, tw);
  }
  __syncthreads();
  C<T>* sticks = reinterpret_cast<C<T>*>(p.sticks) + s0;
  for (int i = threadIdx.x; i < nsb * A; i += blockDim.x) {
    const int k1 = i / nsb, sl = i - k1 * nsb;
    C<T> v[B];
    fft_pass2<NZ, +1>(buf + sl * PZ, 1, k1, v);
#pragma unroll
    for (int k2 = 0; k2 < B; ++k2) sticks[static_cast<size_t>(k1 + A * k2) * p.numSticks + sl] = v[k2];
  }
}

template <typename T, int NZ>
__global__ void __launch_bounds__(kThreads) z_forward(const PlanView<T> p, T* __restrict__ values,
                                                      T scale, int spb) {
  constexpr int A = Shape<NZ>::A, B = Shape<NZ>::B, PZ = ZLayout<NZ>::pitch;
  C<T>* tw = reinterpret_cast<C<T>*>(g_fast_smem);
  C<T>* buf = tw + NZ;
  const int s0 = blockIdx.x * spb;
  const int nsb = min(spb, p.numSticks - s0);

  const C<T>* twg = reinterpret_cast<const C<T>*>(p.twz);
  for (int i = threadIdx.x; i < NZ; i += blockDim.x) tw[i] = twg[i];
  const C<T>* sticks = reinterpret_cast<const C<T>*>(p.sticks) + s0;
  for (int i = threadIdx.x; i < NZ * nsb; i += blockDim.x) {
    const int z = i / nsb, sl = i - z * nsb;
    cp_async_c<T>(buf + sl * PZ + z, sticks + static_cast<size_t>(z) * p.numSticks + sl);
  }
  cp_async_commit();
  cp_async_wait<0>();
  __syncthreads();
  for (int i = threadIdx.x; i < nsb * B; i += blockDim.x) {
    const int sl = i / B, b = i - sl * B;
    fft_pass1<NZ, -1>(buf + sl * PZ, 1, b, tw);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nsb * A; i += blockDim.x) {
    const int k1 = i / nsb, sl = i - k1 * nsb;
    C<T> v[B];
    fft_pass2<NZ, -1>(buf + sl * PZ, 1, k1, v);
#pragma unroll
    for (int k2 = 0; k2 < B; ++k2) buf[sl * PZ + k1 * B + k2] = v[k2];
  }
  __syncthreads();
  C<T>* out = reinterpret_cast<C<T>*>(values);
  const int e0 = p.stickEntryStart[s0], e1 = p.stickEntryStart[s0 + nsb];
  const int base = s0 * NZ;
  for (int e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
    const int pos = p.entryPos[e] - base;
    const int sl = pos / NZ;
    C<T> v = buf[sl * PZ + transposed_pos<NZ>(pos - sl * NZ)];
    if (scale != T(0)) v = cscale(v, scale);
    out[p.entryUser[e]] = v;
  }
}

// ================================================================================================
// plane pass (one block per plane z)
// ================================================================================================
// Shared memory: twy[NY] | twx[NX] | (R2C) twm[M] | colOf[NXF] (int) | P[NY][numColumns] |
//                W[2][rows][LX], with LX = NX (C2C) or M = NX/2 (R2C). The forward pass streams row
//                chunks into the two W halves with cp.async (one chunk in flight while the other
//                is transformed); the backward pass uses one half.
template <int NX, int NY, bool R2C>
struct PlaneLayout {
  static constexpr int M = NX / 2;
  static constexpr int LX = R2C ? M : NX;
  static constexpr int NXF = R2C ? M + 1 : NX;
  // W rows: element e of the x-FFT row sits at e + PAD * (e / Bx), so pass 2 (which reads
  // e = k1*Bx + b across threads k1) strides by an odd number of slots; row pitch WP = Bx mod 16 so
  // two rows of pass 1 fall into different halves of the banks.
  static constexpr int Bx = Shape<LX>::B, Ax = Shape<LX>::A;
  static constexpr int PAD = (Bx % 2 == 0 && Bx > 1) ? 1 : 0;
  static constexpr int ROW = LX + PAD * Ax;
  static constexpr int WP = ROW + ((Bx % 16) - ROW % 16 + 16) % 16;
  __host__ __device__ static constexpr int wpos(int e) { return e + PAD * (e / Bx); }
  template <typename T>
  static size_t bytes(int numColumns, int rows) {
    const size_t c = sizeof(C<T>);
    size_t b = (NY + NX + (R2C ? M : 0)) * c;
    b += ((NXF * sizeof(int) + c - 1) / c) * c;
    b += static_cast<size_t>(NY) * numColumns * c;
    b += 2 * static_cast<size_t>(rows) * WP * c;
    return b;
  }
};

template <typename T, int NX, int NY, bool R2C>
struct PlaneSmem {
  using L = PlaneLayout<NX, NY, R2C>;
  C<T>* twy;
  C<T>* twx;
  C<T>* twm;
  int* colOf;
  C<T>* P;
  C<T>* W;
  __device__ __forceinline__ PlaneSmem(int numColumns) {
    const size_t c = sizeof(C<T>);
    twy = reinterpret_cast<C<T>*>(g_fast_smem);
    twx = twy + NY;
    twm = twx + NX;
    colOf = reinterpret_cast<int*>(twm + (R2C ? L::M : 0));
    P = reinterpret_cast<C<T>*>(reinterpret_cast<unsigned char*>(colOf) +
                                ((L::NXF * sizeof(int) + c - 1) / c) * c);
    W = P + NY * numColumns;
  }
};

template <typename T, int NX, int NY, bool R2C>
__device__ __forceinline__ void plane_load_tables(const PlanView<T>& p, PlaneSmem<T, NX, NY, R2C>& s) {
  using L = PlaneLayout<NX, NY, R2C>;
  const C<T>* ty = reinterpret_cast<const C<T>*>(p.twy);
  const C<T>* tx = reinterpret_cast<const C<T>*>(p.twx);
  for (int i = threadIdx.x; i < NY; i += blockDim.x) s.twy[i] = ty[i];
  for (int i = threadIdx.x; i < NX; i += blockDim.x) s.twx[i] = tx[i];
  if (R2C) {
    for (int i = threadIdx.x; i < L::M; i += blockDim.x) s.twm[i] = tx[2 * i];  // w_M = w_N^2
  }
  for (int i = threadIdx.x; i < L::NXF; i += blockDim.x) s.colOf[i] = -1;
  __syncthreads();
  for (int c = threadIdx.x; c < p.numColumns; c += blockDim.x) s.colOf[p.columnX[c]] = c;
}

template <typename T, int NX, int NY, bool R2C>
__global__ void __launch_bounds__(kPlaneThreads) plane_backward(const PlanView<T> p, T* __restrict__ space,
                                                           int rows) {
  using L = PlaneLayout<NX, NY, R2C>;
  constexpr int Ay = Shape<NY>::A, By = Shape<NY>::B;
  constexpr int Ax = Shape<L::LX>::A, Bx = Shape<L::LX>::B;
  const int z = blockIdx.x;
  const int nc = p.numColumns;
  PlaneSmem<T, NX, NY, R2C> s(nc);
  plane_load_tables<T, NX, NY, R2C>(p, s);
  for (int i = threadIdx.x; i < NY * nc; i += blockDim.x) s.P[i] = czero<T>();
  __syncthreads();

  // sticks of this plane -> compact columns, all copies in flight at once
  const C<T>* sticks = reinterpret_cast<const C<T>*>(p.sticks) + static_cast<size_t>(z) * p.numSticks;
  for (int st = threadIdx.x; st < p.numSticks; st += blockDim.x) {
    cp_async_c<T>(s.P + p.stickY[st] * nc + p.stickColumn[st], sticks + st);
  }
  cp_async_commit();
  cp_async_wait<0>();
  __syncthreads();
  if (R2C && p.columnX[0] == 0) line_fill<T>(s.P, NY, nc);

  // y-FFT on every compact column, result rows left in transposed order
  for (int i = threadIdx.x; i < nc * By; i += blockDim.x) {
    const int b = i / nc, c = i - b * nc;
    fft_pass1<NY, +1>(s.P + c, nc, b, s.twy);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nc * Ay; i += blockDim.x) {
    const int k1 = i / nc, c = i - k1 * nc;
    C<T> v[By];
    fft_pass2<NY, +1>(s.P + c, nc, k1, v);
#pragma unroll
    for (int k2 = 0; k2 < By; ++k2) s.P[(k1 * By + k2) * nc + c] = v[k2];
  }
  __syncthreads();

  // x-FFT of every row
  const C<T>* twl = R2C ? s.twm : s.twx;
  for (int r0 = 0; r0 < NY; r0 += rows) {
    const int nr = min(rows, NY - r0);
    for (int i = threadIdx.x; i < nr * Bx; i += blockDim.x) {
      const int rl = i / Bx, b = i - rl * Bx;
      const C<T>* prow = s.P + transposed_pos<NY>(r0 + rl) * nc;
      C<T> v[Ax];
#pragma unroll
      for (int a = 0; a < Ax; ++a) {
        const int k = a * Bx + b;
        if (!R2C) {
          const int col = s.colOf[k];
          v[a] = col >= 0 ? prow[col] : czero<T>();
        } else {
          // Half-length C2R: Z'[k] = (X[k] + conj X[M-k]) + i e^{+2 pi i k/N} (X[k] - conj X[M-k]),
          // with only the real parts of X[0] and X[M] (the C2R convention).
          const int ck = s.colOf[k], cm = s.colOf[L::M - k];
          const C<T> xk = ck >= 0 ? prow[ck] : czero<T>();
          const C<T> xm = cm >= 0 ? prow[cm] : czero<T>();
          if (k == 0) {
            v[a] = make_c(xk.x + xm.x, xk.x - xm.x);
          } else {
            const C<T> sum = make_c(xk.x + xm.x, xk.y - xm.y);
            const C<T> dif = make_c(xk.x - xm.x, xk.y + xm.y);
            const C<T> u = cmulc(dif, s.twx[k]);
            v[a] = make_c(sum.x - u.y, sum.y + u.x);
          }
        }
      }
      fft_pass1_regs<L::LX, +1>(v, b, twl);
      C<T>* wrow = s.W + rl * L::WP;
#pragma unroll
      for (int k1 = 0; k1 < Ax; ++k1) wrow[L::wpos(k1 * Bx + b)] = v[k1];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nr * Ax; i += blockDim.x) {
      const int rl = i / Ax, k1 = i - rl * Ax;
      C<T> v[Bx];
      fft_pass2<L::LX, +1>(s.W + rl * L::WP + k1 * L::PAD, 1, k1, v);
      // C2C: complex x row; C2R: pairs (x[2m], x[2m+1]) of the real row
      C<T>* out = reinterpret_cast<C<T>*>(space + (static_cast<size_t>(z) * NY + r0 + rl) * NX * (R2C ? 1 : 2));
#pragma unroll
      for (int k2 = 0; k2 < Bx; ++k2) out[k1 + Ax * k2] = v[k2];
    }
    __syncthreads();
  }
}

template <typename T, int NX, int NY, bool R2C>
__global__ void __launch_bounds__(kPlaneThreads) plane_forward(const PlanView<T> p,
                                                          const T* __restrict__ space, int rows) {
  using L = PlaneLayout<NX, NY, R2C>;
  constexpr int Ay = Shape<NY>::A, By = Shape<NY>::B;
  constexpr int Ax = Shape<L::LX>::A, Bx = Shape<L::LX>::B;
  const int z = blockIdx.x;
  const int nc = p.numColumns;
  PlaneSmem<T, NX, NY, R2C> s(nc);
  plane_load_tables<T, NX, NY, R2C>(p, s);
  __syncthreads();

  const C<T>* twl = R2C ? s.twm : s.twx;
  // Row chunks of plane z are contiguous in the space buffer: stream chunk i+1 into the other
  // half of W while chunk i is transformed.
  const C<T>* plane = reinterpret_cast<const C<T>*>(space + static_cast<size_t>(z) * NY * NX * (R2C ? 1 : 2));
  const int nchunks = (NY + rows - 1) / rows;
  auto issue_chunk = [&](int chunk) {
    const int r0 = chunk * rows, nr = min(rows, NY - r0);
    C<T>* dst = s.W + (chunk & 1) * rows * L::WP;
    const C<T>* src = plane + static_cast<size_t>(r0) * L::LX;
    for (int i = threadIdx.x; i < nr * L::LX; i += blockDim.x) {
      const int rl = i / L::LX, e = i - rl * L::LX;
      cp_async_c<T>(dst + rl * L::WP + L::wpos(e), src + i);
    }
    cp_async_commit();
  };
  issue_chunk(0);
  for (int chunk = 0; chunk < nchunks; ++chunk) {
    const int r0 = chunk * rows, nr = min(rows, NY - r0);
    C<T>* wbase = s.W + (chunk & 1) * rows * L::WP;
    if (chunk + 1 < nchunks) {
      issue_chunk(chunk + 1);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nr * Bx; i += blockDim.x) {
      const int rl = i / Bx, b = i - rl * Bx;
      // padded row: element a*Bx + b sits at a*(Bx + PAD) + b
      C<T>* wrow = wbase + rl * L::WP;
      C<T> v[Ax];
#pragma unroll
      for (int a = 0; a < Ax; ++a) v[a] = wrow[a * (Bx + L::PAD) + b];
      fft_pass1_regs<L::LX, -1>(v, b, twl);
#pragma unroll
      for (int k1 = 0; k1 < Ax; ++k1) wrow[k1 * (Bx + L::PAD) + b] = v[k1];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nr * Ax; i += blockDim.x) {
      const int rl = i / Ax, k1 = i - rl * Ax;
      C<T> v[Bx];
      C<T>* wrow = wbase + rl * L::WP + k1 * L::PAD;
      fft_pass2<L::LX, -1>(wrow, 1, k1, v);
      if (!R2C) {
        C<T>* prow = s.P + (r0 + rl) * nc;
#pragma unroll
        for (int k2 = 0; k2 < Bx; ++k2) {
          const int col = s.colOf[k1 + Ax * k2];
          if (col >= 0) prow[col] = v[k2];
        }
      } else {
#pragma unroll
        for (int k2 = 0; k2 < Bx; ++k2) wrow[k1 * Bx + k2] = v[k2];  // wrow is offset by k1*PAD
      }
    }
    __syncthreads();
    if (R2C) {
      // X[k] = (Z[k] + conj Z[M-k]) / 2 - i/2 e^{-2 pi i k/N} (Z[k] - conj Z[M-k]), Z[M] = Z[0]
      for (int i = threadIdx.x; i < nr * nc; i += blockDim.x) {
        const int rl = i / nc, c = i - rl * nc;
        const int k = p.columnX[c];
        const C<T>* wrow = wbase + rl * L::WP;
        const C<T> zk = wrow[L::wpos(transposed_pos<L::LX>(k % L::M))];
        const C<T> zm = wrow[L::wpos(transposed_pos<L::LX>((L::M - k) % L::M))];
        const C<T> dif = make_c(zk.x - zm.x, zk.y + zm.y);
        const C<T> u = cmul(dif, s.twx[k]);
        s.P[(r0 + rl) * nc + c] = make_c(T(0.5) * (zk.x + zm.x + u.y), T(0.5) * (zk.y - zm.y - u.x));
      }
      __syncthreads();
    }
  }

  for (int i = threadIdx.x; i < nc * By; i += blockDim.x) {
    const int b = i / nc, c = i - b * nc;
    fft_pass1<NY, -1>(s.P + c, nc, b, s.twy);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nc * Ay; i += blockDim.x) {
    const int k1 = i / nc, c = i - k1 * nc;
    C<T> v[By];
    fft_pass2<NY, -1>(s.P + c, nc, k1, v);
#pragma unroll
    for (int k2 = 0; k2 < By; ++k2) s.P[(k1 * By + k2) * nc + c] = v[k2];
  }
  __syncthreads();
  C<T>* sticks = reinterpret_cast<C<T>*>(p.sticks) + static_cast<size_t>(z) * p.numSticks;
  for (int st = threadIdx.x; st < p.numSticks; st += blockDim.x) {
    sticks[st] = s.P[transposed_pos<NY>(p.stickY[st]) * nc + p.stickColumn[st]];
  }
}

// ================================================================================================
// host-side launchers (instantiated per size in kernels_fast_*.cu)
// ================================================================================================
template <typename T, int NZ>
struct ZKernels {
  static size_t smem(int spb) { return (NZ + static_cast<size_t>(spb) * ZLayout<NZ>::pitch) * sizeof(C<T>); }
  static cudaError_t prepare(size_t maxSmem) {
    cudaError_t e1 = cudaFuncSetAttribute(z_backward<T, NZ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          static_cast<int>(maxSmem));
    cudaError_t e2 = cudaFuncSetAttribute(z_forward<T, NZ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          static_cast<int>(maxSmem));
    return e1 != cudaSuccess ? e1 : e2;
  }
  static void backward(const PlanView<T>& p, int spb, const T* values, cudaStream_t st) {
    const int g = (p.numSticks + spb - 1) / spb;
    z_backward<T, NZ><<<g, kThreads, smem(spb), st>>>(p, values, spb);
  }
  static void forward(const PlanView<T>& p, int spb, T* values, T scale, cudaStream_t st) {
    const int g = (p.numSticks + spb - 1) / spb;
    z_forward<T, NZ><<<g, kThreads, smem(spb), st>>>(p, values, scale, spb);
  }
};

template <typename T, int NX, int NY, bool R2C>
struct PlaneKernels {
  using L = PlaneLayout<NX, NY, R2C>;
  static size_t smem(int numColumns, int rows) { return L::template bytes<T>(numColumns, rows); }
  static cudaError_t prepare(size_t maxSmem) {
    cudaError_t e1 = cudaFuncSetAttribute(plane_backward<T, NX, NY, R2C>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(maxSmem));
    cudaError_t e2 = cudaFuncSetAttribute(plane_forward<T, NX, NY, R2C>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(maxSmem));
    return e1 != cudaSuccess ? e1 : e2;
  }
  static void backward(const PlanView<T>& p, int rows, T* space, cudaStream_t st) {
    plane_backward<T, NX, NY, R2C><<<p.dimZ, kPlaneThreads, smem(p.numColumns, rows), st>>>(p, space, rows);
  }
  static void forward(const PlanView<T>& p, int rows, const T* space, cudaStream_t st) {
    plane_forward<T, NX, NY, R2C><<<p.dimZ, kPlaneThreads, smem(p.numColumns, rows), st>>>(p, space, rows);
  }
};

}  // namespace fast
}  // namespace gb300
}  // namespace spfft
