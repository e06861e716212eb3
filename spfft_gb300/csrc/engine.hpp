// Device-resident plan of one transform: index tables, twiddles and tile shapes, plus the launch
// sequence of a backward or forward transform on a stream. Replaces the reference's GPU execution
// engine (src/execution/execution_gpu.cpp:47-115 construction, :253-410 execution) with this
// library's fused kernels.
#pragma once

#include <cuda_runtime.h>

#include <array>
#include <memory>
#include <utility>
#include <vector>

#include "kernels.hpp"
#include "planner.hpp"
#include "runtime.hpp"

namespace spfft {
namespace gb300 {

// Bytes of scratch one transform needs, and where each part starts inside it.
struct ScratchLayout {
  size_t sticksOffset = 0, planesOffset = 0, expOffset = 0, stickExpOffset = 0, valuesOffset = 0, total = 0;
};

template <typename T>
class GpuPlan {
public:
  GpuPlan(const IndexPlan& plan, int device);

  const ScratchLayout& scratch_layout() const { return layout_; }
  const LaunchConfig& launch_config() const { return config_; }

  // values/space are device pointers; scratch points to scratch_layout().total bytes.
  void backward(const T* values, T* space, void* scratch, cudaStream_t stream,
                const StageEvents* events = nullptr) const;
  void forward(const T* space, T* values, bool scaled, void* scratch, cudaStream_t stream,
               const StageEvents* events = nullptr) const;

  // Transforms whose space domain lives in host memory, staged through the device buffer
  // `devSpace` in plane chunks so that the host link and the x pass overlap: the forward copies
  // chunk c on `copyStream` while the x pass of chunk c - 1 runs on `stream`; the backward copies
  // chunk c back while the x pass of chunk c + 1 runs. `events` holds kStagedEvents events. Both
  // return false, doing nothing, when the plan has no split x pass (the caller then copies the
  // whole domain at once).
  // Plane chunks per staged transform (stagedSizes_, in the backward's order; the forward takes them
  // in reverse): by default sizes doubling from about dimZ / 24 planes; SPFFT_GB300_STAGED_CHUNKS=n
  // (1 .. kMaxStagedChunks) at plan creation selects n equal chunks.
  static constexpr int kMaxStagedChunks = 32, kStagedEvents = kMaxStagedChunks + 1;
  int staged_chunks() const { return static_cast<int>(stagedSizes_.size()); }
  bool forward_staged(const T* hostSpace, T* devSpace, T* values, bool scaled, void* scratch,
                      cudaStream_t stream, cudaStream_t copyStream, cudaEvent_t* events) const;
  bool backward_staged(const T* values, T* devSpace, T* hostSpace, void* scratch, cudaStream_t stream,
                       cudaStream_t copyStream, cudaEvent_t* events) const;

  // Adjoints (with respect to the real inner product Re <a, b>): of backward (space gradient ->
  // value gradient) and of forward (value gradient -> space gradient).
  void adjoint_backward(const T* gradSpace, T* gradValues, void* scratch, cudaStream_t stream) const;
  void adjoint_forward(const T* gradValues, T* gradSpace, bool scaled, void* scratch,
                       cudaStream_t stream) const;

  // How the y and x passes run: generic kernels, one fused specialised kernel per plane, or
  // specialised y and x kernels over column / row groups with the compact plane in HBM.
  enum class PlanePath { Generic, Fused, Split };
  // Which kernels run: bit 0 = size-specialised z pass, bit 1 = fused plane pass, bit 2 = split
  // specialised y and x passes.
  int path_flags() const {
    return (fastZ_ ? 1 : 0) | (planePath_ == PlanePath::Fused ? 2 : 0) | (planePath_ == PlanePath::Split ? 4 : 0);
  }

  // Tile shapes and plane strategy the kernels run with.
  struct Tuning {
    int spb = 0;           // sticks per z block (0: generic z kernels)
    int path = 0;          // 0 generic, 1 fused plane, 2 split y and x
    int fusedRows = 0;     // fused: half of the x chunk buffer rows
    int fusedThreads = 0;  // fused: threads per block (256: two blocks per SM, 512: one)
    int cpb = 0, rpb = 0;  // split: columns per y block, rows per x forward block
    int rpbB = 0;          // split: rows per x backward block
    int radix[3] = {0, 0, 0};  // generic kernels: radix plan of z, y, x (index into radix_plans())
    // size-specialised z backward, z forward, split y backward, split y forward passes: 1 runs
    // the swapped two-pass split of the length (B x A instead of A x B), 2 the three-pass split
    // (A x B1 x B2 with B = B1 * B2), where the length has one
    int split[4] = {0, 0, 0, 0};
  };
  // First-pass radix A of the split (length = A * B) each pass runs with: z backward,
  // z forward, y backward, y forward, x backward, x forward; 0 for a pass on the generic kernels.
  void split_radices(int* radices) const;
  // The radices of each pass's split, stages[3 * pass + 0..2]: (A, B, 0) for a two-pass split,
  // (A, B1, B2) for a three-pass split, zeros for a pass on the generic kernels (pass order as in
  // split_radices).
  void split_stages(int* stages) const;
  // Radix plans available to the generic kernels for the z, y and x lengths (dim 0, 1, 2), and
  // the ones in use.
  const std::vector<RadixPlan>& radix_plans(int dim) const { return radixCands_[dim]; }
  RadixPlan radix_plan(int dim) const { return dim == 0 ? base_.fz : dim == 1 ? base_.fy : base_.fx; }
  Tuning tuning() const;
  // Every tuning this plan can run (all combinations of the valid z, fused and split shapes).
  std::vector<Tuning> candidates() const;
  // Throws InvalidParameterError for a tuning that is not among candidates().
  void set_tuning(const Tuning& t);
  // Autotuner: times `reps` backward + scaled forward pairs per candidate on `values` / `space`
  // (device buffers of this plan's sizes, overwritten) on `stream`, first over the z shapes with
  // the current plane strategy, then over the plane strategies and tile shapes with the best z
  // shape, then over the two-pass split (default or swapped) of each specialised z and split-y
  // pass, then -- for the lengths that run on the generic kernels -- over their radix plans one
  // length at a time, and keeps the fastest. Returns its time per pair in milliseconds. No other
  // work of this plan may run meanwhile.
  float autotune(T* values, T* space, void* scratch, cudaStream_t stream, int reps);

  // Device view of this plan with its intermediates in `scratch` (used by batched execution).
  PlanView<T> device_view(void* scratch) const { return view(scratch); }
  T forward_scale() const { return scale_; }

  // Device pointer of the value staging area inside `scratch` (host input / output path).
  T* staging(void* scratch) const {
    return reinterpret_cast<T*>(static_cast<char*>(scratch) + layout_.valuesOffset);
  }

private:
  PlanView<T> view(void* scratch) const;

  void check_alignment(const T* values, const T* space, bool* planeAligned) const;

  PlanView<T> base_{};
  LaunchConfig config_{};
  bool fastZ_ = false;
  PlanePath planePath_ = PlanePath::Generic;
  // valid shapes, for the autotuner
  std::vector<int> zCands_;
  std::vector<std::pair<int, int>> fusedCands_;  // (rows, threads)
  std::vector<std::array<int, 3>> splitCands_;  // (cpb, rpb, rpbB)
  int fastSpb_ = 0, fastRows_ = 0, splitCpb_ = 0, splitRpb_ = 0, splitRpbB_ = 0, fusedThreads_ = 512;
  std::vector<int> stagedSizes_;
  std::vector<RadixPlan> radixCands_[3];
  int radixChoice_[3] = {0, 0, 0};
  int splitChoice_[4] = {0, 0, 0, 0};  // Tuning::split
  bool zSwap_ = false, ySwap_ = false;  // the z / split y length has a swapped split
  bool zThree_ = false, yThree_ = false;  // the z / split y length has a three-pass split
  // Whether split variant v (0 default, 1 swapped, 2 three-pass) exists for pass i (0 z backward,
  // 1 z forward, 2 y backward, 3 y forward); `active`: the pass runs on the specialised z kernels
  // (i < 2) or on the split y kernels (i >= 2). Variant 0 is always valid.
  bool split_valid(int i, int v, bool active) const {
    if (v == 0) return true;
    if (!active) return false;
    if (v == 1) return i < 2 ? zSwap_ : ySwap_;
    if (v == 2) return i < 2 ? zThree_ : yThree_;
    return false;
  }
  ScratchLayout layout_{};
  T scale_ = T(1);
  int numValues_ = 0;
  DeviceBuffer tables_;
  std::shared_ptr<const DeviceIndexTables> sharedTables_;  // device-planned index tables
};

// Opt-in shared memory per block of `device`, and one-time attribute setup of the specialised
// kernels of length n (false if n has no specialised kernels).
size_t smem_optin(int device);
template <typename T>
bool fast_prepare(int device, int n);

extern template class GpuPlan<double>;
extern template class GpuPlan<float>;

}  // namespace gb300
}  // namespace spfft
