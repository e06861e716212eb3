// Batched execution of many independent transforms: the GB300 form of the reference's
// multi-transform (src/spfft/multi_transform_internal.hpp:63-174). Transforms are grouped by
// shape; each pass of each group is ONE launch over all of the group's transforms (batched
// kernels, kernels_batch.cuh), and a whole backward + forward pair can be captured once into a
// CUDA graph and replayed.
#pragma once

#include <cuda_runtime.h>

#include <memory>
#include <vector>

#include "internal.hpp"
#include "kernels.hpp"
#include "runtime.hpp"

namespace spfft {
namespace gb300 {

template <typename T>
class BatchPlan {
public:
  // The transforms must be GPU transforms on distinct grids.
  explicit BatchPlan(std::vector<std::shared_ptr<TransformInternal<T>>> transforms);
  ~BatchPlan();
  BatchPlan(const BatchPlan&) = delete;
  BatchPlan& operator=(const BatchPlan&) = delete;

  // Device buffers of every transform: values[i] (interleaved complex) and spaces[i] (the space
  // domain). Both must be aligned to the complex size. Replaces earlier bindings; captured graphs
  // stay valid (they read the bound pointers from a device table), unless the buffers of an
  // unbatched transform change (those are kernel arguments; the graphs are then captured anew).
  // Synchronous by default, so no work of this batch may be in flight; with `async` the table is
  // written in the order of `stream` instead, which then must be the stream the batch runs on.
  void bind(const T* const* values, T* const* spaces, cudaStream_t stream = nullptr, bool async = false);

  // With more than one shape group (or unbatched transforms), the groups run as concurrent
  // branches: each on its own stream, forked from and joined back into `stream`.
  void backward(cudaStream_t stream);
  void forward(bool scaled, cudaStream_t stream);
  // backward then forward as one CUDA graph, captured on the first call for this scaling (on
  // `stream`, which must not be the legacy default stream) and replayed afterwards. Each group's
  // six launches form one chain of the graph; the chains of different groups run concurrently.
  void pair_graph(bool scaled, cudaStream_t stream);
  // The same for one direction (what: 1 backward, 2 forward, 3 backward then forward).
  void graph(int what, bool scaled, cudaStream_t stream);
  // One direction (0 backward, 1 forward) with the groups run pass by pass on `stream` and events
  // between the passes; waits and returns the three pass times in milliseconds (z, y, x for the
  // backward, x, y, z for the forward; a fused group runs its plane kernel in the y slot).
  void stage_times(int direction, bool scaled, cudaStream_t stream, float ms[3]);

  // Autotuner: per shape group, times `reps` backward + scaled forward pairs of the group alone on
  // the bound buffers (overwriting them) for each plane strategy that fits (fused, split) and each
  // sticks-per-z-block size, and keeps the fastest; drops captured graphs. Returns the sum over
  // the groups of their best times per pair in milliseconds. Synchronous.
  float autotune(cudaStream_t stream, int reps);

  int num_transforms() const { return static_cast<int>(tp_.size()); }
  // Stop keeping the transforms alive (for an owner that tracks their lifetime itself and drops
  // the plan before any of them goes away).
  void release_transforms() { transforms_.clear(); }
  // Pointers currently bound (nullptr before the first bind).
  const T* bound_values(int t) const { return bound_ ? values_[t] : nullptr; }
  const T* bound_space(int t) const { return bound_ ? spaces_[t] : nullptr; }
  int num_groups() const { return static_cast<int>(groups_.size()); }
  int num_unbatched() const { return static_cast<int>(fallback_.size()); }
  // Groups whose y and x passes run as one fused plane kernel.
  int num_fused_groups() const;
  // 0 unbatched, 1 batched with split y and x passes, 2 batched with the fused plane pass.
  int transform_path(int t) const;
  // Row groups of the fused plane passes' x pass for transform t (0 when its passes are not fused).
  int row_groups(int t) const;
  // Kernel launches of one backward + forward pair.
  int launches_per_pair() const;

private:
  struct Group;
  void upload_views();
  void check_bound() const;
  // Passes of one group on `s`: bit 0 backward, bit 1 forward (after the backward).
  void run_group(Group& g, int what, bool scaled, cudaStream_t s);
  void run_pass(Group& g, int pass, int direction, bool scaled, cudaStream_t s);
  void set_z_shape(Group& g, int spb);
  void run_fallback(int what, bool scaled, cudaStream_t s);
  // Every group (and the unbatched transforms) as concurrent branches of `stream`.
  void run(int what, bool scaled, cudaStream_t stream);

  std::vector<std::shared_ptr<TransformInternal<T>>> transforms_;  // ownership (may be released)
  std::vector<TransformInternal<T>*> tp_;
  std::vector<std::unique_ptr<Group>> groups_;
  std::vector<int> fallback_;
  std::vector<const T*> values_;
  std::vector<T*> spaces_;
  std::vector<void*> scratchSeen_;
  bool bound_ = false;
  cudaGraphExec_t graphs_[8] = {};  // index 2 * what + scaled
  int device_ = 0;
  // fork / join of the concurrent branches (created with the plan when there is more than one)
  std::vector<std::unique_ptr<Stream>> branchStreams_;
  std::vector<std::unique_ptr<Event>> branchDone_;
  std::unique_ptr<Event> fork_;
};

extern template class BatchPlan<double>;
extern template class BatchPlan<float>;

}  // namespace gb300
}  // namespace spfft
