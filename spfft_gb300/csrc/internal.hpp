// Grid and transform internals behind the public spfft::Grid / spfft::Transform handles.
//
// GridInternal owns the memory a transform executes in (reference: src/spfft/grid_internal.cpp:
// 49-104): the internal device space-domain buffer, its pinned host mirror and the device scratch
// (sticks, compact planes, value staging). TransformInternal validates a plan against its grid
// (reference: src/spfft/transform_internal.cpp:45-137) and runs the stream / event protocol of
// src/execution/execution_gpu.cpp:253-410 around the kernels.
#pragma once

#include <cuda_runtime.h>

#include <memory>
#include <mutex>

#include "engine.hpp"
#include "planner.hpp"
#include "runtime.hpp"
#include "spfft/types.h"

namespace spfft {

template <typename T>
class GridInternal {
public:
  GridInternal(int maxDimX, int maxDimY, int maxDimZ, int maxNumLocalZColumns,
               SpfftProcessingUnitType processingUnit, int numThreads);
  // A copy has the same limits and fresh memory (grid_internal.cpp:233-263).
  GridInternal(const GridInternal& other);

  int max_dim_x() const { return maxDimX_; }
  int max_dim_y() const { return maxDimY_; }
  int max_dim_z() const { return maxDimZ_; }
  int max_num_local_z_columns() const { return maxNumLocalZColumns_; }
  int max_local_z_length() const { return maxDimZ_; }
  SpfftProcessingUnitType processing_unit() const { return processingUnit_; }
  int device_id() const { return deviceId_; }
  int num_threads() const { return numThreads_; }

  // Internal space-domain buffers: maxDimX * maxDimY * maxDimZ complex values.
  T* space_device() { return static_cast<T*>(space_.get()); }
  T* space_host();
  // Device scratch of at least `bytes`. Grown when transforms are created, never while one runs.
  void reserve_scratch(size_t bytes);
  void* scratch() { return scratch_.get(); }

private:
  int maxDimX_, maxDimY_, maxDimZ_, maxNumLocalZColumns_;
  SpfftProcessingUnitType processingUnit_;
  int numThreads_;
  int deviceId_ = 0;
  gb300::DeviceBuffer space_;
  gb300::DeviceBuffer scratch_;
  gb300::PinnedBuffer spaceHost_;
  std::mutex mutex_;
};

template <typename T>
class TransformInternal {
public:
  TransformInternal(SpfftProcessingUnitType processingUnit, std::shared_ptr<GridInternal<T>> grid,
                    std::shared_ptr<const gb300::IndexPlan> plan);

  // Same parameters, new grid with the same limits (transform_internal.cpp:178-182).
  std::shared_ptr<TransformInternal<T>> clone() const;

  void forward(SpfftProcessingUnitType inputLocation, T* output, SpfftScalingType scaling);
  void forward(const T* input, T* output, SpfftScalingType scaling);
  void backward(const T* input, SpfftProcessingUnitType outputLocation);
  void backward(const T* input, T* output);

  // Split execution used by the multi-transform functions: enqueue, then synchronize.
  void forward_enqueue(const T* input, T* output, SpfftScalingType scaling);
  void backward_enqueue(const T* input, T* output);
  void synchronize();

  T* space_domain_data(SpfftProcessingUnitType location);

  SpfftTransformType type() const { return plan_->type; }
  int dim_x() const { return plan_->dimX; }
  int dim_y() const { return plan_->dimY; }
  int dim_z() const { return plan_->dimZ; }
  int local_z_length() const { return plan_->dimZ; }
  int local_z_offset() const { return 0; }
  long long global_size() const {
    return static_cast<long long>(plan_->dimX) * plan_->dimY * plan_->dimZ;
  }
  int num_local_elements() const { return plan_->numValues; }
  long long num_global_elements() const { return plan_->numValues; }
  SpfftProcessingUnitType processing_unit() const { return processingUnit_; }
  int device_id() const { return grid_->device_id(); }
  int num_threads() const { return grid_->num_threads(); }
  SpfftExecType execution_mode() const { return execMode_; }
  void set_execution_mode(SpfftExecType mode);
  bool shared_grid(const TransformInternal<T>& other) const { return grid_ == other.grid_; }

  // ---- extensions of this library -------------------------------------------------------------
  // Run on `stream` directly (no internal stream, no default-stream ordering); nullptr restores
  // the reference protocol.
  void set_stream(cudaStream_t stream) { userStream_ = stream; hasUserStream_ = (stream != nullptr); }
  bool has_user_stream() const { return hasUserStream_; }
  // Device address of a user buffer: device memory as it is, pinned host memory through its mapped
  // alias when kernels access host buffers directly, nullptr for anything else.
  template <typename P>
  P* device_address(P* p) const {
    auto split = gb300::split_pointer(p);
    if (split.second) return split.second;
    return directHost_ ? gb300::mapped_host_alias(split.first) : nullptr;
  }
  const gb300::IndexPlan& index_plan() const { return *plan_; }
  const gb300::GpuPlan<T>& gpu_plan() const { return *gpu_; }
  int path_flags() const { return gpu_->path_flags(); }
  GridInternal<T>& grid() { return *grid_; }
  // Kernel-only entry points on device pointers, on the stream the caller gives.
  void backward_device(const T* values, T* space, cudaStream_t stream);
  void forward_device(const T* space, T* values, bool scaled, cudaStream_t stream);
  // Adjoint passes on device pointers (see GpuPlan::adjoint_backward / adjoint_forward).
  void adjoint_backward_device(const T* gradSpace, T* gradValues, cudaStream_t stream) {
    gb300::DeviceGuard guard(grid_->device_id());
    gpu_->adjoint_backward(gradSpace, gradValues, grid_->scratch(), stream);
  }
  void adjoint_forward_device(const T* gradValues, T* gradSpace, bool scaled, cudaStream_t stream) {
    gb300::DeviceGuard guard(grid_->device_id());
    gpu_->adjoint_forward(gradValues, gradSpace, scaled, grid_->scratch(), stream);
  }
  // Autotuner over the plan's tile shapes on the grid's own buffers (see GpuPlan::autotune); on
  // the user stream if one is set, else the internal stream; synchronous.
  float autotune(int reps);
  // One pass in `direction` (0 backward, 1 forward) on device pointers with events between the
  // three kernels; waits for completion and returns the kernel times in milliseconds.
  void stage_times(int direction, const T* in, T* out, bool scaled, cudaStream_t stream,
                   float ms[3]);

private:
  cudaStream_t begin();       // preceding-error check, stream ordering; returns the exec stream
  void finish(cudaStream_t);  // sync or async completion
  size_t space_elements() const;  // T elements of the space domain

  SpfftProcessingUnitType processingUnit_;
  SpfftExecType execMode_ = SPFFT_EXEC_SYNCHRONOUS;
  std::shared_ptr<GridInternal<T>> grid_;
  std::shared_ptr<const gb300::IndexPlan> plan_;
  std::unique_ptr<gb300::GpuPlan<T>> gpu_;
  std::unique_ptr<gb300::Stream> stream_;
  std::unique_ptr<gb300::Event> startEvent_, endEvent_;
  cudaStream_t userStream_ = nullptr;
  bool hasUserStream_ = false;
  bool directHost_ = true;  // kernels access pinned host buffers directly (else: staged copies)
  // second stream and events of the chunked host <-> device copies (created on first use)
  gb300::Stream& copy_stream();
  cudaEvent_t* staged_events();
  std::unique_ptr<gb300::Stream> copyStream_;
  std::unique_ptr<gb300::EventSet> stagedEvents_;
};

extern template class GridInternal<double>;
extern template class GridInternal<float>;
extern template class TransformInternal<double>;
extern template class TransformInternal<float>;

}  // namespace spfft
