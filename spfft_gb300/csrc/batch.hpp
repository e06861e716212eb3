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
  // domain). Both must be aligned to the complex size. Replaces earlier bindings and drops any
  // captured graph.
  void bind(const T* const* values, T* const* spaces);

  void backward(cudaStream_t stream);
  void forward(bool scaled, cudaStream_t stream);
  // backward then forward as one CUDA graph, captured on the first call for this scaling (on
  // `stream`, which must not be the legacy default stream) and replayed afterwards.
  void pair_graph(bool scaled, cudaStream_t stream);

  int num_transforms() const { return static_cast<int>(transforms_.size()); }
  int num_groups() const { return static_cast<int>(groups_.size()); }
  int num_unbatched() const { return static_cast<int>(fallback_.size()); }
  // Kernel launches of one backward + forward pair.
  int launches_per_pair() const;

private:
  struct Group;
  void upload_views();
  void check_bound() const;

  std::vector<std::shared_ptr<TransformInternal<T>>> transforms_;
  std::vector<std::unique_ptr<Group>> groups_;
  std::vector<int> fallback_;
  std::vector<const T*> values_;
  std::vector<T*> spaces_;
  std::vector<void*> scratchSeen_;
  bool bound_ = false;
  cudaGraphExec_t graphs_[2] = {nullptr, nullptr};
  int device_ = 0;
};

extern template class BatchPlan<double>;
extern template class BatchPlan<float>;

}  // namespace gb300
}  // namespace spfft
