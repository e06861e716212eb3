// Generic transform kernels: correct for every size the planner accepts. Three passes per
// direction, each a single launch over all of its work:
//
//   backward:  z-pass   sparse values -> (scatter, stick symmetry, z-FFT) -> sticks[z][s]
//              y-pass   sticks -> (scatter to compact columns, plane symmetry, y-FFT) -> planes
//              x-pass   planes -> (expand to full rows, hermitian fill for R2C, x-FFT) -> space
//   forward:   the mirror image, with the gather (and optional scaling) fused into the z-pass.
//
// Reference operators these passes replace (all in src/):
//   compression/gpu_kernels/compression_kernels.cu:39-150 (decompress/compress, scaled compress)
//   symmetry/gpu_kernels/symmetry_kernels.cu:38-165      (stick and plane symmetry)
//   transpose/gpu_kernels/local_transpose_kernels.cu:43-201 (stick <-> plane transpose)
//   fft/transform_1d_gpu.hpp, transform_2d_gpu.hpp, transform_real_2d_gpu.hpp (cuFFT calls)
// The stick and plane zero-fills of the reference (compression_gpu.hpp:74-76,
// transpose_gpu.hpp:95-104) happen in shared memory and never touch HBM.
#include <cstdint>

#include "fft_core.cuh"
#include "kernels.hpp"

namespace spfft {
namespace gb300 {

namespace {

template <typename T>
using C = typename Complex<T>::type;

extern __shared__ __align__(16) unsigned char g_smem[];

template <typename T>
__device__ __forceinline__ void load_twiddles(C<T>* dst, const T* src, int n) {
  const C<T>* s = reinterpret_cast<const C<T>*>(src);
  for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = s[i];
}

template <typename T>
__device__ __forceinline__ void zero_fill(C<T>* dst, int n) {
  const C<T> z = make_c(T(0), T(0));
  for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = z;
}

// Conjugate fill of one hermitian line: for k in [1, n/2] then [n/2+1, n), v[n-k] = conj(v[k])
// wherever v[k] != 0. Two ordered halves, as the reference does on host and GPU
// (symmetry_host.hpp:72-90, symmetry_kernels.cu:104-165).
template <typename T>
__device__ __forceinline__ void hermitian_line_fill(C<T>* v, int n, int stride) {
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

// ---------------------------------------------------------------------------------------------
// z-pass, backward: one block per group of sticksPerBlock consecutive sticks.
template <typename T>
__global__ void z_backward_kernel(const PlanView<T> p, const T* __restrict__ values, int spb,
                                  int pitch) {
  C<T>* tw = reinterpret_cast<C<T>*>(g_smem);
  C<T>* a = tw + p.dimZ;
  C<T>* b = a + spb * pitch;
  const int s0 = blockIdx.x * spb;
  const int nsb = min(spb, p.numSticks - s0);
  const int nz = p.dimZ;

  load_twiddles<T>(tw, p.twz, nz);
  zero_fill<T>(a, nsb * pitch);
  __syncthreads();

  const C<T>* vals = reinterpret_cast<const C<T>*>(values);
  const int e0 = p.stickEntryStart[s0], e1 = p.stickEntryStart[s0 + nsb];
  const int base = s0 * nz;
  for (int e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
    const int pos = p.entryPos[e] - base;
    const int sl = pos / nz;
    const int z = pos - sl * nz;
    a[sl * pitch + z] = vals[p.entryUser[e]];
  }
  __syncthreads();

  const int zz = p.zeroZeroStick - s0;
  if (p.r2c && zz >= 0 && zz < nsb) hermitian_line_fill<T>(a + zz * pitch, nz, 1);

  C<T>* res = smem_fft<+1>(a, b, tw, p.fz, nsb, 1, pitch, false);

  C<T>* sticks = reinterpret_cast<C<T>*>(p.sticks);
  for (int i = threadIdx.x; i < nz * nsb; i += blockDim.x) {
    const int z = i / nsb;
    const int sl = i - z * nsb;
    sticks[static_cast<size_t>(z) * p.numSticks + s0 + sl] = res[sl * pitch + z];
  }
}

// y-pass, backward: block (column group, z).
template <typename T>
__global__ void y_backward_kernel(const PlanView<T> p, int cpb) {
  C<T>* tw = reinterpret_cast<C<T>*>(g_smem);
  C<T>* a = tw + p.dimY;
  C<T>* b = a + p.dimY * cpb;
  const int c0 = blockIdx.x * cpb;
  const int ncb = min(cpb, p.numColumns - c0);
  const int z = blockIdx.y;
  const int ny = p.dimY;

  load_twiddles<T>(tw, p.twy, ny);
  zero_fill<T>(a, ny * ncb);
  __syncthreads();

  const C<T>* sticks = reinterpret_cast<const C<T>*>(p.sticks) + static_cast<size_t>(z) * p.numSticks;
  const int sBegin = p.columnStickStart[c0], sEnd = p.columnStickStart[c0 + ncb];
  for (int s = sBegin + threadIdx.x; s < sEnd; s += blockDim.x) {
    a[p.stickY[s] * ncb + (p.stickColumn[s] - c0)] = sticks[s];
  }
  __syncthreads();

  // Plane symmetry on the x = 0 column (symmetry_gpu.hpp:45-61 applies it to every plane).
  if (p.r2c && c0 == 0 && p.columnX[0] == 0) hermitian_line_fill<T>(a, ny, ncb);

  C<T>* res = smem_fft<+1>(a, b, tw, p.fy, ncb, ncb, 1, true);

  C<T>* planes = reinterpret_cast<C<T>*>(p.planes) + static_cast<size_t>(z) * ny * p.numColumns;
  for (int i = threadIdx.x; i < ny * ncb; i += blockDim.x) {
    const int y = i / ncb;
    const int cl = i - y * ncb;
    planes[static_cast<size_t>(y) * p.numColumns + c0 + cl] = res[y * ncb + cl];
  }
}

// x-pass, backward: block (row group, z). C2C writes complex rows, R2C real rows.
template <typename T>
__global__ void x_backward_kernel(const PlanView<T> p, T* __restrict__ space, int rpb, int pitch) {
  C<T>* tw = reinterpret_cast<C<T>*>(g_smem);
  C<T>* a = tw + p.dimX;
  C<T>* b = a + rpb * pitch;
  const int y0 = blockIdx.x * rpb;
  const int nrb = min(rpb, p.dimY - y0);
  const int z = blockIdx.y;
  const int nx = p.dimX;

  load_twiddles<T>(tw, p.twx, nx);
  zero_fill<T>(a, nrb * pitch);
  __syncthreads();

  const C<T>* planes = reinterpret_cast<const C<T>*>(p.planes) +
                       (static_cast<size_t>(z) * p.dimY + y0) * p.numColumns;
  for (int i = threadIdx.x; i < nrb * p.numColumns; i += blockDim.x) {
    const int yl = i / p.numColumns;
    const int c = i - yl * p.numColumns;
    a[yl * pitch + p.columnX[c]] = planes[i];
  }
  __syncthreads();

  if (p.r2c) {
    // Hermitian extension of each row: X[x] = conj(X[nx - x]) for x > nx/2. The real part of the
    // full inverse DFT then equals the C2R result, which ignores the imaginary parts of the
    // x = 0 and x = nx/2 bins.
    const int upper = nx - p.dimXFreq;  // number of x > nx/2
    for (int i = threadIdx.x; i < nrb * upper; i += blockDim.x) {
      const int yl = i / upper;
      const int x = p.dimXFreq + (i - yl * upper);
      a[yl * pitch + x] = cconj(a[yl * pitch + (nx - x)]);
    }
    __syncthreads();
  }

  C<T>* res = smem_fft<+1>(a, b, tw, p.fx, nrb, 1, pitch, false);

  const size_t rowBase = (static_cast<size_t>(z) * p.dimY + y0) * nx;
  if (p.r2c) {
    for (int i = threadIdx.x; i < nrb * nx; i += blockDim.x) {
      const int yl = i / nx;
      const int x = i - yl * nx;
      space[rowBase + i] = res[yl * pitch + x].x;
    }
  } else {
    C<T>* out = reinterpret_cast<C<T>*>(space);
    for (int i = threadIdx.x; i < nrb * nx; i += blockDim.x) {
      const int yl = i / nx;
      const int x = i - yl * nx;
      out[rowBase + i] = res[yl * pitch + x];
    }
  }
}

// ---------------------------------------------------------------------------------------------
// x-pass, forward: rows of the space domain -> compact columns of the plane buffer.
template <typename T>
__global__ void x_forward_kernel(const PlanView<T> p, const T* __restrict__ space, int rpb,
                                 int pitch) {
  C<T>* tw = reinterpret_cast<C<T>*>(g_smem);
  C<T>* a = tw + p.dimX;
  C<T>* b = a + rpb * pitch;
  const int y0 = blockIdx.x * rpb;
  const int nrb = min(rpb, p.dimY - y0);
  const int z = blockIdx.y;
  const int nx = p.dimX;

  load_twiddles<T>(tw, p.twx, nx);
  const size_t rowBase = (static_cast<size_t>(z) * p.dimY + y0) * nx;
  if (p.r2c) {
    for (int i = threadIdx.x; i < nrb * nx; i += blockDim.x) {
      const int yl = i / nx;
      const int x = i - yl * nx;
      a[yl * pitch + x] = make_c(space[rowBase + i], T(0));
    }
  } else {
    const C<T>* in = reinterpret_cast<const C<T>*>(space);
    for (int i = threadIdx.x; i < nrb * nx; i += blockDim.x) {
      const int yl = i / nx;
      const int x = i - yl * nx;
      a[yl * pitch + x] = in[rowBase + i];
    }
  }
  __syncthreads();

  C<T>* res = smem_fft<-1>(a, b, tw, p.fx, nrb, 1, pitch, false);

  C<T>* planes = reinterpret_cast<C<T>*>(p.planes) +
                 (static_cast<size_t>(z) * p.dimY + y0) * p.numColumns;
  for (int i = threadIdx.x; i < nrb * p.numColumns; i += blockDim.x) {
    const int yl = i / p.numColumns;
    const int c = i - yl * p.numColumns;
    planes[i] = res[yl * pitch + p.columnX[c]];
  }
}

// y-pass, forward: compact columns -> y-FFT -> gather stick values at plane z.
template <typename T>
__global__ void y_forward_kernel(const PlanView<T> p, int cpb) {
  C<T>* tw = reinterpret_cast<C<T>*>(g_smem);
  C<T>* a = tw + p.dimY;
  C<T>* b = a + p.dimY * cpb;
  const int c0 = blockIdx.x * cpb;
  const int ncb = min(cpb, p.numColumns - c0);
  const int z = blockIdx.y;
  const int ny = p.dimY;

  load_twiddles<T>(tw, p.twy, ny);
  const C<T>* planes = reinterpret_cast<const C<T>*>(p.planes) + static_cast<size_t>(z) * ny * p.numColumns;
  for (int i = threadIdx.x; i < ny * ncb; i += blockDim.x) {
    const int y = i / ncb;
    const int cl = i - y * ncb;
    a[y * ncb + cl] = planes[static_cast<size_t>(y) * p.numColumns + c0 + cl];
  }
  __syncthreads();

  C<T>* res = smem_fft<-1>(a, b, tw, p.fy, ncb, ncb, 1, true);

  C<T>* sticks = reinterpret_cast<C<T>*>(p.sticks) + static_cast<size_t>(z) * p.numSticks;
  const int sBegin = p.columnStickStart[c0], sEnd = p.columnStickStart[c0 + ncb];
  for (int s = sBegin + threadIdx.x; s < sEnd; s += blockDim.x) {
    sticks[s] = res[p.stickY[s] * ncb + (p.stickColumn[s] - c0)];
  }
}

// z-pass, forward: sticks -> z-FFT -> gather (and scale) the sparse values.
template <typename T>
__global__ void z_forward_kernel(const PlanView<T> p, T* __restrict__ values, T scale, int spb,
                                 int pitch) {
  C<T>* tw = reinterpret_cast<C<T>*>(g_smem);
  C<T>* a = tw + p.dimZ;
  C<T>* b = a + spb * pitch;
  const int s0 = blockIdx.x * spb;
  const int nsb = min(spb, p.numSticks - s0);
  const int nz = p.dimZ;

  load_twiddles<T>(tw, p.twz, nz);
  const C<T>* sticks = reinterpret_cast<const C<T>*>(p.sticks);
  for (int i = threadIdx.x; i < nz * nsb; i += blockDim.x) {
    const int z = i / nsb;
    const int sl = i - z * nsb;
    a[sl * pitch + z] = sticks[static_cast<size_t>(z) * p.numSticks + s0 + sl];
  }
  __syncthreads();

  C<T>* res = smem_fft<-1>(a, b, tw, p.fz, nsb, 1, pitch, false);

  C<T>* out = reinterpret_cast<C<T>*>(values);
  const int e0 = p.stickEntryStart[s0], e1 = p.stickEntryStart[s0 + nsb];
  const int base = s0 * nz;
  for (int e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
    const int pos = p.entryPos[e] - base;
    const int sl = pos / nz;
    const int z = pos - sl * nz;
    C<T> v = res[sl * pitch + z];
    // Scaling multiplies by T(1 / (Nx Ny Nz)) like compress_kernel_scaled
    // (compression_kernels.cu:106-128).
    if (scale != T(0)) v = cscale(v, scale);
    out[p.entryUser[e]] = v;
  }
}

template <typename T>
__global__ void weight_values_kernel(const T* __restrict__ in, T* out, const unsigned char* __restrict__ w,
                                     int n, T factor, int divide) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    T f = factor;
    if (w) f = divide ? factor / T(w[i]) : factor * T(w[i]);
    out[2 * i] = in[2 * i] * f;
    out[2 * i + 1] = in[2 * i + 1] * f;
  }
}

}  // namespace

template <typename T>
cudaError_t launch_weight_values(const T* in, T* out, const unsigned char* weight, int n, T factor,
                                 int divide, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  const int blocks = (n + 255) / 256 < 4 * 152 ? (n + 255) / 256 : 4 * 152;
  weight_values_kernel<T><<<blocks, 256, 0, stream>>>(in, out, weight, n, factor, divide);
  return cudaGetLastError();
}
template cudaError_t launch_weight_values<double>(const double*, double*, const unsigned char*, int,
                                                  double, int, cudaStream_t);
template cudaError_t launch_weight_values<float>(const float*, float*, const unsigned char*, int, float,
                                                 int, cudaStream_t);

template <typename T>
cudaError_t prepare_kernels(size_t maxSmem) {
  const int bytes = static_cast<int>(maxSmem);
  cudaError_t err = cudaSuccess;
  auto set = [&](const void* fn) {
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e != cudaSuccess && err == cudaSuccess) err = e;
  };
  set(reinterpret_cast<const void*>(&z_backward_kernel<T>));
  set(reinterpret_cast<const void*>(&y_backward_kernel<T>));
  set(reinterpret_cast<const void*>(&x_backward_kernel<T>));
  set(reinterpret_cast<const void*>(&x_forward_kernel<T>));
  set(reinterpret_cast<const void*>(&y_forward_kernel<T>));
  set(reinterpret_cast<const void*>(&z_forward_kernel<T>));
  return err;
}

template <typename T>
cudaError_t launch_generic(GenericPass pass, const PlanView<T>& p, const LaunchConfig& c,
                           const T* in, T* out, T scale, cudaStream_t stream) {
  const int gz = (p.numSticks + c.sticksPerBlock - 1) / c.sticksPerBlock;
  const dim3 gy((p.numColumns + c.columnsPerBlock - 1) / c.columnsPerBlock, p.dimZ);
  const dim3 gx((p.dimY + c.rowsPerBlock - 1) / c.rowsPerBlock, p.dimZ);
  switch (pass) {
    case GenericPass::ZBackward:
      if (p.numSticks > 0)
        z_backward_kernel<T><<<gz, c.threads, c.smemZ, stream>>>(p, in, c.sticksPerBlock, c.zPitch);
      break;
    case GenericPass::YBackward:
      if (p.numSticks > 0) y_backward_kernel<T><<<gy, c.threads, c.smemY, stream>>>(p, c.columnsPerBlock);
      break;
    case GenericPass::XBackward:
      x_backward_kernel<T><<<gx, c.threads, c.smemX, stream>>>(p, out, c.rowsPerBlock, c.xPitch);
      break;
    case GenericPass::XForward:
      if (p.numSticks > 0)
        x_forward_kernel<T><<<gx, c.threads, c.smemX, stream>>>(p, in, c.rowsPerBlock, c.xPitch);
      break;
    case GenericPass::YForward:
      if (p.numSticks > 0) y_forward_kernel<T><<<gy, c.threads, c.smemY, stream>>>(p, c.columnsPerBlock);
      break;
    case GenericPass::ZForward:
      if (p.numSticks > 0)
        z_forward_kernel<T><<<gz, c.threads, c.smemZ, stream>>>(p, out, scale, c.sticksPerBlock,
                                                                c.zPitch);
      break;
  }
  return cudaGetLastError();
}

template cudaError_t prepare_kernels<double>(size_t);
template cudaError_t prepare_kernels<float>(size_t);
template cudaError_t launch_generic<double>(GenericPass, const PlanView<double>&,
                                            const LaunchConfig&, const double*, double*, double,
                                            cudaStream_t);
template cudaError_t launch_generic<float>(GenericPass, const PlanView<float>&, const LaunchConfig&,
                                           const float*, float*, float, cudaStream_t);

}  // namespace gb300
}  // namespace spfft
