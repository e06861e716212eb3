// Batched specialised kernels: one launch per pass covers every transform of a shape group. Each
// block finds its transform from the per-transform block offsets (binary search) and runs the same
// body as the single-transform kernel with its local block coordinates. Lets many small transforms
// fill the GPU and hide each block's load latency behind the others.
#pragma once

#include "kernels_fast.cuh"

namespace spfft {
namespace gb300 {

namespace fast {

__device__ __forceinline__ int find_transform(const int* __restrict__ starts, int count, int b) {
  int lo = 0, hi = count;  // starts[lo] <= b < starts[hi]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(starts + mid) <= b) lo = mid;
    else hi = mid;
  }
  return lo;
}

template <typename S, typename A, int NZ>
__global__ void __launch_bounds__(kThreads, ZBackwardMinBlocks<A>::value) z_backward_batch(const BatchView<S> bv, int spb) {
  __shared__ int sExp[2];
  const int t = find_transform(bv.starts, bv.count, blockIdx.x);
  z_backward_body<S, A, NZ>(bv.views[t], bv.in[t], spb, blockIdx.x - bv.starts[t], sExp);
}

template <typename S, typename A, int NZ>
__global__ void __launch_bounds__(kThreads) z_forward_batch(const BatchView<S> bv, int spb) {
  __shared__ int sExp[2];
  const int t = find_transform(bv.starts, bv.count, blockIdx.x);
  z_forward_body<S, A, NZ>(bv.views[t], bv.out[t], bv.scale, spb, blockIdx.x - bv.starts[t], sExp);
}

template <typename S, typename A, int NY>
__global__ void __launch_bounds__(kThreads, YMinBlocks<A>::value) y_backward_batch(const BatchView<S> bv, int cpb) {
  __shared__ int sExp[2];
  const int t = find_transform(bv.starts, bv.count, blockIdx.x);
  const PlanView<S>& p = bv.views[t];
  const int lb = blockIdx.x - bv.starts[t];
  const int gx = (p.numColumns + cpb - 1) / cpb;
  y_backward_body<S, A, NY>(p, cpb, lb % gx, lb / gx, sExp);
}

template <typename S, typename A, int NY>
__global__ void __launch_bounds__(kThreads, YMinBlocks<A>::value) y_forward_batch(const BatchView<S> bv, int cpb) {
  __shared__ int sExp[2];
  const int t = find_transform(bv.starts, bv.count, blockIdx.x);
  const PlanView<S>& p = bv.views[t];
  const int lb = blockIdx.x - bv.starts[t];
  const int gx = (p.numColumns + cpb - 1) / cpb;
  y_forward_body<S, A, NY>(p, cpb, lb % gx, lb / gx, sExp);
}

template <typename S, typename A, int NX, bool R2C>
__global__ void __launch_bounds__(kThreads) x_backward_batch(const BatchView<S> bv, int rpb) {
  __shared__ int sExp[2];
  const int t = find_transform(bv.starts, bv.count, blockIdx.x);
  const PlanView<S>& p = bv.views[t];
  const int lb = blockIdx.x - bv.starts[t];
  const int gx = (p.dimY + rpb - 1) / rpb;
  x_backward_body<S, A, NX, R2C>(p, bv.out[t], rpb, lb % gx, lb / gx, sExp);
}

template <typename S, typename A, int NX, bool R2C>
__global__ void __launch_bounds__(kThreads) x_forward_batch(const BatchView<S> bv, int rpb) {
  __shared__ int sExp[2];
  const int t = find_transform(bv.starts, bv.count, blockIdx.x);
  const PlanView<S>& p = bv.views[t];
  const int lb = blockIdx.x - bv.starts[t];
  const int gx = (p.dimY + rpb - 1) / rpb;
  x_forward_body<S, A, NX, R2C>(p, bv.in[t], rpb, lb % gx, lb / gx, sExp);
}

// Fused y + x passes, one block per plane (cubic planes): starts count planes. `groups` row groups
// share the x pass (RowGroups; blockDim.x / groups a multiple of 32, rows / groups >= 1).
template <typename S, typename A, int N, bool R2C>
__global__ void __launch_bounds__(BatchPlaneThreads<A>::value, 2)
    plane_backward_batch(const BatchView<S> bv, int rows, int groups) {
  __shared__ int sExp[2];
  const int t = find_transform(bv.starts, bv.count, blockIdx.x);
  plane_backward_body<S, A, N, N, R2C>(bv.views[t], bv.out[t], rows, blockIdx.x - bv.starts[t], sExp, groups);
}

template <typename S, typename A, int N, bool R2C>
__global__ void __launch_bounds__(BatchPlaneThreads<A>::value, 2)
    plane_forward_batch(const BatchView<S> bv, int rows, int wRows, int groups) {
  __shared__ int sExp[2];
  const int t = find_transform(bv.starts, bv.count, blockIdx.x);
  plane_forward_body<S, A, N, N, R2C>(bv.views[t], bv.in[t], rows, wRows, blockIdx.x - bv.starts[t], sExp,
                                      groups);
}

template <typename S, typename A, int N>
struct BatchKernels {
  static cudaError_t prepare(size_t maxSmem) {
    cudaError_t e = allow_dynamic_smem(z_backward_batch<S, A, N>, maxSmem);
    if (e == cudaSuccess) e = allow_dynamic_smem(z_forward_batch<S, A, N>, maxSmem);
    if (e == cudaSuccess) e = allow_dynamic_smem(y_backward_batch<S, A, N>, maxSmem);
    if (e == cudaSuccess) e = allow_dynamic_smem(y_forward_batch<S, A, N>, maxSmem);
    if (e == cudaSuccess) e = allow_dynamic_smem(x_backward_batch<S, A, N, false>, maxSmem);
    if (e == cudaSuccess) e = allow_dynamic_smem(x_backward_batch<S, A, N, true>, maxSmem);
    if (e == cudaSuccess) e = allow_dynamic_smem(x_forward_batch<S, A, N, false>, maxSmem);
    if (e == cudaSuccess) e = allow_dynamic_smem(x_forward_batch<S, A, N, true>, maxSmem);
    if (e == cudaSuccess) e = allow_dynamic_smem(plane_backward_batch<S, A, N, false>, maxSmem);
    if (e == cudaSuccess) e = allow_dynamic_smem(plane_backward_batch<S, A, N, true>, maxSmem);
    if (e == cudaSuccess) e = allow_dynamic_smem(plane_forward_batch<S, A, N, false>, maxSmem);
    if (e == cudaSuccess) e = allow_dynamic_smem(plane_forward_batch<S, A, N, true>, maxSmem);
    return e;
  }
};

}  // namespace fast
}  // namespace gb300
}  // namespace spfft
