// Host interface of the size-specialised kernels (kernels_fast.cuh), instantiated in size groups
// (kernels_fast_group_*.cu) so the library's translation units compile in parallel.
#pragma once

#include <cuda_runtime.h>

#include "kernels.hpp"

namespace spfft {
namespace gb300 {

enum class FastOp {
  Has,
  Prepare,
  ZBackward,
  ZForward,
  PlaneBackward,
  PlaneForward,
  PlaneSmem,
  ZSmem,
  ZOccupancy,  // resident z_backward blocks per SM for param sticks per block (into *smemOut)
  YBackward,  // split y pass (n = dimY), param = columns per block
  YForward,
  YSmem,
  XBackward,  // split x pass (n = dimX), param = rows per block
  XForward,
  XSmem,
  // batched passes over a shape group (args.batch, args.blocks, args.smem): n is the z length for
  // BatchZ*, the y length for BatchY*, the x length for BatchX*
  BatchZBackward,
  BatchZForward,
  BatchYBackward,
  BatchYForward,
  BatchXBackward,
  BatchXForward,
  // batched fused plane passes (n = the cubic plane size; param = rows per x chunk)
  BatchPlaneBackward,
  BatchPlaneForward,
  // first-pass radix A of a kernel's split N = A * B into *smemOut (0: no such split);
  // param: 0 z pass, 1 split y pass (both with args.split: 0 default, 1 swapped, 2 three-pass),
  // 2 / 3 y pass of the fused plane backward / forward kernel, 4 x pass (C2C, or R2C with r2c
  // set: the half-length complex FFT)
  SplitRadix,
  // first factor B1 of B = B1 * B2 of the three-pass split of the z and split-y passes into
  // *smemOut (0: the length has no three-pass split in this precision)
  ThreePassFactor
};

// Threads of a batched fused plane block (two blocks per SM): 384 in FP32 (80 registers), 256 in
// double-float (T = double; its register demand would spill at 384).
template <typename T>
constexpr int batch_plane_threads() {
  return sizeof(T) == sizeof(float) ? 384 : 256;
}

template <typename T>
struct FastArgs {
  const PlanView<T>* plan = nullptr;
  int param = 0;  // sticks per block (z) or rows per chunk (plane)
  int split = 0;  // z and split y passes: 1 the swapped two-pass split, 2 the three-pass split
  int param2 = 0;  // batched plane forward: rows of the chunk buffer (2 * param double-buffers)
  int groups = 1;  // batched plane passes: independent row groups of the x pass
  int zBegin = 0, zCount = -1;  // split y and x passes: plane range (zCount < 0: to the last plane)
  const T* in = nullptr;
  T* out = nullptr;
  T scale = T(0);
  cudaStream_t stream = nullptr;
  size_t maxSmem = 0;
  int numColumns = 0;
  size_t* smemOut = nullptr;
  const BatchView<T>* batch = nullptr;
  int blocks = 0;
  size_t smem = 0;
};

// Each group handles its own sizes: returns true if `n` (the z length for z ops, the cubic plane
// size for plane ops) belongs to the group and the op was performed.
template <typename T>
bool fast_group_a(FastOp op, int n, bool r2c, const FastArgs<T>& args);
template <typename T>
bool fast_group_b(FastOp op, int n, bool r2c, const FastArgs<T>& args);
template <typename T>
bool fast_group_c(FastOp op, int n, bool r2c, const FastArgs<T>& args);
template <typename T>
bool fast_group_d(FastOp op, int n, bool r2c, const FastArgs<T>& args);
template <typename T>
bool fast_group_e(FastOp op, int n, bool r2c, const FastArgs<T>& args);
template <typename T>
bool fast_group_f(FastOp op, int n, bool r2c, const FastArgs<T>& args);
template <typename T>
bool fast_group_g(FastOp op, int n, bool r2c, const FastArgs<T>& args);
template <typename T>
bool fast_group_h(FastOp op, int n, bool r2c, const FastArgs<T>& args);
template <typename T>
bool fast_group_i(FastOp op, int n, bool r2c, const FastArgs<T>& args);

// Lengths with specialised kernels: 12, 48, 60, 64, 72, 90, 96, 100, 108, 120, 128, 144, 150, 160,
// 180, 192, 240, 256.
template <typename T>
inline bool fast_dispatch(FastOp op, int n, bool r2c, const FastArgs<T>& args) {
  return fast_group_a<T>(op, n, r2c, args) || fast_group_b<T>(op, n, r2c, args) ||
         fast_group_c<T>(op, n, r2c, args) || fast_group_d<T>(op, n, r2c, args) ||
         fast_group_e<T>(op, n, r2c, args) || fast_group_f<T>(op, n, r2c, args) ||
         fast_group_g<T>(op, n, r2c, args) || fast_group_h<T>(op, n, r2c, args) ||
         fast_group_i<T>(op, n, r2c, args);
}

}  // namespace gb300
}  // namespace spfft
