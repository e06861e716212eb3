// GridInternal / TransformInternal implementation.
#include "internal.hpp"

#include <cstdlib>
#include <cstring>
#include <thread>

namespace spfft {

using gb300::check_cuda;
using gb300::DeviceGuard;

// ------------------------------------------------------------------------------------------------
// GridInternal
// ------------------------------------------------------------------------------------------------
template <typename T>
GridInternal<T>::GridInternal(int maxDimX, int maxDimY, int maxDimZ, int maxNumLocalZColumns,
                              SpfftProcessingUnitType processingUnit, int numThreads)
    : maxDimX_(maxDimX),
      maxDimY_(maxDimY),
      maxDimZ_(maxDimZ),
      maxNumLocalZColumns_(maxNumLocalZColumns),
      processingUnit_(processingUnit),
      numThreads_(numThreads) {
  // Input checks of grid_internal.cpp:61-67.
  if (maxDimX <= 0 || maxDimY <= 0 || maxDimZ <= 0 || maxNumLocalZColumns < 0) {
    throw InvalidParameterError();
  }
  if (!(processingUnit & (SPFFT_PU_HOST | SPFFT_PU_GPU))) throw InvalidParameterError();
  if (numThreads_ < 1) {
    numThreads_ = static_cast<int>(std::thread::hardware_concurrency());
    if (numThreads_ < 1) numThreads_ = 1;
  }
  if (processingUnit & SPFFT_PU_GPU) {
    check_cuda(cudaGetDevice(&deviceId_));
    const size_t elems = static_cast<size_t>(maxDimX) * maxDimY * maxDimZ;
    space_ = gb300::DeviceBuffer(elems * 2 * sizeof(T));
  }
}

template <typename T>
GridInternal<T>::GridInternal(const GridInternal& other)
    : maxDimX_(other.maxDimX_),
      maxDimY_(other.maxDimY_),
      maxDimZ_(other.maxDimZ_),
      maxNumLocalZColumns_(other.maxNumLocalZColumns_),
      processingUnit_(other.processingUnit_),
      numThreads_(other.numThreads_),
      deviceId_(other.deviceId_) {
  if (processingUnit_ & SPFFT_PU_GPU) {
    DeviceGuard guard(deviceId_);
    const size_t elems = static_cast<size_t>(maxDimX_) * maxDimY_ * maxDimZ_;
    space_ = gb300::DeviceBuffer(elems * 2 * sizeof(T));
    if (other.scratch_.size()) scratch_ = gb300::DeviceBuffer(other.scratch_.size());
  }
}

template <typename T>
T* GridInternal<T>::space_host() {
  std::lock_guard<std::mutex> lock(mutex_);
  const size_t elems = static_cast<size_t>(maxDimX_) * maxDimY_ * maxDimZ_;
  spaceHost_.reserve(elems * 2 * sizeof(T));
  return static_cast<T*>(spaceHost_.get());
}

template <typename T>
void GridInternal<T>::reserve_scratch(size_t bytes) {
  std::lock_guard<std::mutex> lock(mutex_);
  DeviceGuard guard(deviceId_);
  scratch_.reserve(bytes);
}

// ------------------------------------------------------------------------------------------------
// TransformInternal
// ------------------------------------------------------------------------------------------------
template <typename T>
TransformInternal<T>::TransformInternal(SpfftProcessingUnitType processingUnit,
                                        std::shared_ptr<GridInternal<T>> grid,
                                        std::shared_ptr<const gb300::IndexPlan> plan)
    : processingUnit_(processingUnit), grid_(std::move(grid)), plan_(std::move(plan)) {
  // Checks of transform_internal.cpp:52-77, in the same order.
  if (!grid_) throw InvalidParameterError();
  if (plan_->num_sticks() > grid_->max_num_local_z_columns()) throw InvalidParameterError();
  if (plan_->dimX > grid_->max_dim_x() || plan_->dimY > grid_->max_dim_y() ||
      plan_->dimZ > grid_->max_dim_z()) {
    throw InvalidParameterError();
  }
  if (!(processingUnit & grid_->processing_unit())) throw InvalidParameterError();
  if (processingUnit != SPFFT_PU_HOST && processingUnit != SPFFT_PU_GPU) {
    throw InvalidParameterError();
  }
  // This library executes on the GPU only; the reference's host engine (FFTW + OpenMP) is not
  // part of it.
  if (processingUnit != SPFFT_PU_GPU) throw InvalidParameterError();

  DeviceGuard guard(grid_->device_id());
  gpu_.reset(new gb300::GpuPlan<T>(*plan_, grid_->device_id()));
  grid_->reserve_scratch(gpu_->scratch_layout().total);
  stream_.reset(new gb300::Stream());
  startEvent_.reset(new gb300::Event());
  endEvent_.reset(new gb300::Event());
  // SPFFT_GB300_HOST_ACCESS=copy restores the reference's staged host <-> device copies for pinned
  // host buffers; by default kernels read and write them directly.
  const char* access = std::getenv("SPFFT_GB300_HOST_ACCESS");
  directHost_ = !(access && std::strcmp(access, "copy") == 0);
}

template <typename T>
std::shared_ptr<TransformInternal<T>> TransformInternal<T>::clone() const {
  std::shared_ptr<GridInternal<T>> newGrid(new GridInternal<T>(*grid_));
  return std::make_shared<TransformInternal<T>>(processingUnit_, std::move(newGrid), plan_);
}

template <typename T>
size_t TransformInternal<T>::space_elements() const {
  const size_t n = static_cast<size_t>(plan_->dimX) * plan_->dimY * plan_->dimZ;
  return plan_->type == SPFFT_TRANS_C2C ? 2 * n : n;
}

template <typename T>
void TransformInternal<T>::set_execution_mode(SpfftExecType mode) {
  if (mode != SPFFT_EXEC_SYNCHRONOUS && mode != SPFFT_EXEC_ASYNCHRONOUS) {
    throw InvalidParameterError();
  }
  execMode_ = mode;
}

template <typename T>
cudaStream_t TransformInternal<T>::begin() {
  // A pending CUDA error from earlier calls aborts before any work (execution_gpu.cpp:256-258).
  if (cudaGetLastError() != cudaSuccess) throw GPUPrecedingError();
  if (hasUserStream_) return userStream_;
  // Order after the legacy default stream (execution_gpu.cpp:260-261, 333-344).
  startEvent_->order(cudaStreamLegacy, stream_->get());
  return stream_->get();
}

template <typename T>
void TransformInternal<T>::finish(cudaStream_t s) {
  if (execMode_ == SPFFT_EXEC_ASYNCHRONOUS) {
    if (!hasUserStream_) endEvent_->order(s, cudaStreamLegacy);
  } else {
    check_cuda(cudaStreamSynchronize(s));
  }
}

template <typename T>
T* TransformInternal<T>::space_domain_data(SpfftProcessingUnitType location) {
  if (location == SPFFT_PU_GPU) return grid_->space_device();
  if (location == SPFFT_PU_HOST) return grid_->space_host();
  throw InvalidParameterError();
}

template <typename T>
gb300::Stream& TransformInternal<T>::copy_stream() {
  if (!copyStream_) copyStream_.reset(new gb300::Stream());
  return *copyStream_;
}

template <typename T>
cudaEvent_t* TransformInternal<T>::staged_events() {
  if (!stagedEvents_) stagedEvents_.reset(new gb300::EventSet(gb300::GpuPlan<T>::kStagedEvents));
  return stagedEvents_->data();
}

template <typename T>
void TransformInternal<T>::backward_enqueue(const T* input, T* output) {
  cudaStream_t s = begin();
  auto in = gb300::split_pointer(input);
  auto out = gb300::split_pointer(output);
  // pinned host values: the z pass reads them over the coherent host link
  if (directHost_ && in.first) {
    if (const T* d = gb300::mapped_host_alias(in.first)) in = {nullptr, d};
  }
  void* scratch = grid_->scratch();
  const T* values = in.second;
  if (in.first) {
    T* staging = gpu_->staging(scratch);
    if (plan_->numValues > 0) {
      check_cuda(cudaMemcpyAsync(staging, in.first, sizeof(T) * 2 * plan_->numValues,
                                 cudaMemcpyHostToDevice, s));
    }
    values = staging;
  }
  // host space domain: the y and x passes run in plane chunks into the grid's device buffer and
  // each chunk is copied back while the next one is transformed
  if (out.first && gpu_->backward_staged(values, grid_->space_device(), out.first, scratch, s,
                                         copy_stream().get(), staged_events())) {
    return;
  }
  // otherwise (no split passes) pinned memory is written by the x pass directly
  if (directHost_ && out.first) {
    if (T* d = gb300::mapped_host_alias(out.first)) out = {nullptr, d};
  }
  T* space = out.second ? out.second : grid_->space_device();
  gpu_->backward(values, space, scratch, s);
  if (out.first) {
    check_cuda(cudaMemcpyAsync(out.first, space, sizeof(T) * space_elements(),
                               cudaMemcpyDeviceToHost, s));
  }
}

template <typename T>
void TransformInternal<T>::forward_enqueue(const T* input, T* output, SpfftScalingType scaling) {
  cudaStream_t s = begin();
  auto in = gb300::split_pointer(input);
  auto out = gb300::split_pointer(output);
  if (directHost_ && out.first) {
    if (T* d = gb300::mapped_host_alias(out.first)) out = {nullptr, d};
  }
  void* scratch = grid_->scratch();
  T* values = out.second ? out.second : gpu_->staging(scratch);
  // Host input: copy plane chunks to the device buffer, each chunk's x pass starting when it has
  // arrived (faster than kernels reading host memory, whose reads stall the x pass).
  if (in.first && gpu_->forward_staged(in.first, grid_->space_device(), values, scaling == SPFFT_FULL_SCALING,
                                       scratch, s, copy_stream().get(), staged_events())) {
    if (out.first && plan_->numValues > 0) {
      check_cuda(cudaMemcpyAsync(out.first, values, sizeof(T) * 2 * plan_->numValues,
                                 cudaMemcpyDeviceToHost, s));
    }
    return;
  }
  if (directHost_ && in.first) {
    if (const T* d = gb300::mapped_host_alias(in.first)) in = {nullptr, d};
  }
  const T* space = in.second;
  if (in.first) {
    check_cuda(cudaMemcpyAsync(grid_->space_device(), in.first, sizeof(T) * space_elements(),
                               cudaMemcpyHostToDevice, s));
    space = grid_->space_device();
  }
  gpu_->forward(space, values, scaling == SPFFT_FULL_SCALING, scratch, s);
  if (out.first && plan_->numValues > 0) {
    check_cuda(cudaMemcpyAsync(out.first, values, sizeof(T) * 2 * plan_->numValues,
                               cudaMemcpyDeviceToHost, s));
  }
}

template <typename T>
void TransformInternal<T>::synchronize() {
  DeviceGuard guard(grid_->device_id());
  finish(hasUserStream_ ? userStream_ : stream_->get());
}

template <typename T>
void TransformInternal<T>::backward(const T* input, T* output) {
  DeviceGuard guard(grid_->device_id());
  backward_enqueue(input, output);
  finish(hasUserStream_ ? userStream_ : stream_->get());
}

template <typename T>
void TransformInternal<T>::forward(const T* input, T* output, SpfftScalingType scaling) {
  DeviceGuard guard(grid_->device_id());
  forward_enqueue(input, output, scaling);
  finish(hasUserStream_ ? userStream_ : stream_->get());
}

template <typename T>
void TransformInternal<T>::backward(const T* input, SpfftProcessingUnitType outputLocation) {
  backward(input, space_domain_data(outputLocation));
}

template <typename T>
void TransformInternal<T>::forward(SpfftProcessingUnitType inputLocation, T* output,
                                   SpfftScalingType scaling) {
  forward(space_domain_data(inputLocation), output, scaling);
}

template <typename T>
void TransformInternal<T>::backward_device(const T* values, T* space, cudaStream_t stream) {
  DeviceGuard guard(grid_->device_id());
  gpu_->backward(values, space, grid_->scratch(), stream);
}

template <typename T>
void TransformInternal<T>::forward_device(const T* space, T* values, bool scaled,
                                          cudaStream_t stream) {
  DeviceGuard guard(grid_->device_id());
  gpu_->forward(space, values, scaled, grid_->scratch(), stream);
}

template <typename T>
float TransformInternal<T>::autotune(int reps) {
  DeviceGuard guard(grid_->device_id());
  cudaStream_t s = begin();
  void* scratch = grid_->scratch();
  T* values = gpu_->staging(scratch);
  T* space = grid_->space_device();
  // zero data: finite everywhere, so every candidate runs its ordinary arithmetic
  if (plan_->numValues > 0) check_cuda(cudaMemsetAsync(values, 0, sizeof(T) * 2 * plan_->numValues, s));
  check_cuda(cudaMemsetAsync(space, 0, sizeof(T) * space_elements(), s));
  const float ms = gpu_->autotune(values, space, scratch, s, reps);
  check_cuda(cudaStreamSynchronize(s));
  return ms;
}

template <typename T>
void TransformInternal<T>::stage_times(int direction, const T* in, T* out, bool scaled,
                                       cudaStream_t stream, float ms[3]) {
  DeviceGuard guard(grid_->device_id());
  gb300::StageEvents ev{};
  for (auto& e : ev.ev) check_cuda(cudaEventCreate(&e));
  try {
    if (direction == 0) {
      gpu_->backward(in, out, grid_->scratch(), stream, &ev);
    } else {
      gpu_->forward(in, out, scaled, grid_->scratch(), stream, &ev);
    }
    check_cuda(cudaEventSynchronize(ev.ev[3]));
    for (int i = 0; i < 3; ++i) check_cuda(cudaEventElapsedTime(&ms[i], ev.ev[i], ev.ev[i + 1]));
  } catch (...) {
    for (auto& e : ev.ev) (void)cudaEventDestroy(e);
    throw;
  }
  for (auto& e : ev.ev) (void)cudaEventDestroy(e);
}

template class GridInternal<double>;
template class GridInternal<float>;
template class TransformInternal<double>;
template class TransformInternal<float>;

}  // namespace spfft
