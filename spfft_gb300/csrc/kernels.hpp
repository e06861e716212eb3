// Device-side view of a transform plan and the launch entry points of the transform kernels.
// Shared between the host engine (engine.cpp) and the kernels (kernels_generic.cu).
#pragma once

#include <cuda_runtime.h>

#include "fft_plan.hpp"

namespace spfft {
namespace gb300 {

// Everything a kernel needs to know about one transform. Device pointers only.
//
// HBM layouts:
//   sticks  [dimZ][numSticks]          complex  z-major: row z holds every stick's value at z
//   planes  [dimZ][dimY][numColumns]   complex  y-transformed compact columns (x = columnX[c])
//   space   [dimZ][dimY][dimX]         complex (C2C) or real (R2C), the user's layout
//   values  [numValues]                interleaved complex, user order
template <typename T>
struct PlanView {
  int dimX, dimY, dimZ, dimXFreq;
  int numSticks, numColumns;
  int zeroZeroStick;  // -1 when absent or C2C
  int r2c;
  RadixPlan fz, fy, fx;
  const T* twz;  // interleaved (cos, -sin) tables of length dimZ / dimY / dimX
  const T* twy;
  const T* twx;
  const int* stickColumn;
  const int* stickY;
  const int* stickPlanePos;  // stickY * numColumns + stickColumn: the stick's slot in a compact plane
  const int* columnX;
  const int* columnStickStart;
  const int* entryPos;
  const int* entryUser;
  const int* stickEntryStart;
  const unsigned char* hermitianWeight;  // R2C: per user value, 1 or 2; null for C2C
  T* sticks;
  T* planes;
  // Double precision: the split y and x kernels keep the compact planes in double-float form
  // (hi, lo floats in the 16 bytes of a complex double, scaled by a power of two per column or
  // per row) instead of converting them to binary64 and back; planeExp holds those exponents.
  int* planeExp;
  int planesRaw;
  // The same for the sticks between the z and the split y kernels (single transforms on the
  // split path): per-stick exponents from the z pass (backward), per-(plane, column) exponents
  // from the y pass (forward).
  int* stickExp;
  int sticksRaw;
};

// Device tables of one shape group of a batch for one pass (all device pointers); read by the
// batched kernels (kernels_batch.cuh).
template <typename S>
struct BatchView {
  const PlanView<S>* views;  // [count]
  const int* starts;         // [count + 1] first block of each transform in this pass
  int count;
  const S* const* in;   // per transform: values (backward z) or space (forward x)
  S* const* out;        // per transform: space (backward x) or values (forward z)
  S scale;              // forward scaling factor, 0 = none
};

// Tile shapes of the generic kernels, chosen by the host (engine.cpp: choose_launch_config).
struct LaunchConfig {
  int threads;            // threads per block (all kernels)
  int sticksPerBlock;     // z kernels
  int zPitch;             // padded stick length in shared memory
  int columnsPerBlock;    // y kernels
  int rowsPerBlock;       // x kernels
  int xPitch;             // padded row length in shared memory
  size_t smemZ, smemY, smemX;
};

// Optional events recorded before pass 0 and after each pass (stage timing).
struct StageEvents {
  cudaEvent_t ev[4];
};

// The six passes of the generic kernels. Backward: z (values -> sticks), y (sticks -> planes),
// x (planes -> space). Forward: x (space -> planes), y (planes -> sticks), z (sticks -> values,
// scaled unless scale == 0). `in` / `out` are the values or space pointers where a pass touches
// them and are ignored otherwise.
enum class GenericPass { ZBackward, YBackward, XBackward, XForward, YForward, ZForward };
template <typename T>
cudaError_t launch_generic(GenericPass pass, const PlanView<T>& p, const LaunchConfig& c,
                           const T* in, T* out, T scale, cudaStream_t stream);
// out[i] = in[i] * factor * w_i (divide = 0) or in[i] * factor / w_i (divide = 1) for the n complex
// values, with w_i = weight[i] (1 when weight is null). In place allowed.
template <typename T>
cudaError_t launch_weight_values(const T* in, T* out, const unsigned char* weight, int n, T factor,
                                 int divide, cudaStream_t stream);

// One-time per-process attribute setup (dynamic shared memory limits).
template <typename T>
cudaError_t prepare_kernels(size_t maxSmem);

}  // namespace gb300
}  // namespace spfft
