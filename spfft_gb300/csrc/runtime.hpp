// CUDA runtime helpers: status -> exception mapping, RAII owners for device / pinned memory,
// streams and events, and a device guard.
//
// The status mapping follows the reference's check_status (src/gpu_util/gpu_runtime_api.hpp:
// 113-125); the guard follows GPUDeviceGuard (src/gpu_util/gpu_device_guard.hpp:38-63).
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstddef>
#include <utility>

#include "spfft/exceptions.hpp"

namespace spfft {
namespace gb300 {

inline void check_cuda(cudaError_t error) {
  if (error == cudaSuccess) return;
  if (error == cudaErrorMemoryAllocation) throw GPUAllocationError();
  if (error == cudaErrorLaunchOutOfResources) throw GPULaunchError();
  if (error == cudaErrorNoDevice || error == cudaErrorInsufficientDriver) throw GPUNoDeviceError();
  if (error == cudaErrorInvalidValue) throw GPUInvalidValueError();
  if (error == cudaErrorInvalidDevicePointer) throw GPUInvalidDevicePointerError();
  throw GPUError();
}

// Kernel launch failures are reported as launch errors.
inline void check_launch(cudaError_t error) {
  if (error == cudaSuccess) return;
  if (error == cudaErrorInvalidConfiguration || error == cudaErrorLaunchOutOfResources ||
      error == cudaErrorInvalidDeviceFunction || error == cudaErrorNoKernelImageForDevice)
    throw GPULaunchError();
  check_cuda(error);
}

// Fault injection for the tests of the allocation-failure paths: with the countdown at n >= 0 the
// next n device or pinned host allocations of the library succeed and the one after fails, once,
// with the exception a failing CUDA allocator raises (without calling it). -1 turns it off.
inline std::atomic<int>& allocation_countdown() {
  static std::atomic<int> countdown{-1};
  return countdown;
}
inline bool injected_allocation_failure() {
  int c = allocation_countdown().load();
  while (c >= 0) {
    if (allocation_countdown().compare_exchange_weak(c, c - 1)) return c == 0;
  }
  return false;
}

class DeviceGuard {
public:
  explicit DeviceGuard(int device) : target_(device) {
    check_cuda(cudaGetDevice(&original_));
    if (original_ != target_) check_cuda(cudaSetDevice(target_));
  }
  ~DeviceGuard() {
    if (original_ != target_) (void)cudaSetDevice(original_);
  }
  DeviceGuard(const DeviceGuard&) = delete;
  DeviceGuard& operator=(const DeviceGuard&) = delete;

private:
  int target_;
  int original_ = 0;
};

class DeviceBuffer {
public:
  DeviceBuffer() = default;
  explicit DeviceBuffer(size_t bytes) { resize(bytes); }
  ~DeviceBuffer() { release(); }
  DeviceBuffer(const DeviceBuffer&) = delete;
  DeviceBuffer& operator=(const DeviceBuffer&) = delete;
  DeviceBuffer(DeviceBuffer&& o) noexcept { swap(o); }
  DeviceBuffer& operator=(DeviceBuffer&& o) noexcept {
    if (this != &o) {
      release();
      swap(o);
    }
    return *this;
  }
  // Grows (never shrinks) to at least `bytes`. Contents are not preserved.
  void reserve(size_t bytes) {
    if (bytes <= bytes_) return;
    resize(bytes);
  }
  void* get() const { return ptr_; }
  size_t size() const { return bytes_; }

private:
  void resize(size_t bytes) {
    release();
    if (bytes == 0) return;
    if (injected_allocation_failure()) throw GPUAllocationError();
    check_cuda(cudaMalloc(&ptr_, bytes));
    bytes_ = bytes;
  }
  void release() {
    if (ptr_) (void)cudaFree(ptr_);
    ptr_ = nullptr;
    bytes_ = 0;
  }
  void swap(DeviceBuffer& o) {
    std::swap(ptr_, o.ptr_);
    std::swap(bytes_, o.bytes_);
  }
  void* ptr_ = nullptr;
  size_t bytes_ = 0;
};

class PinnedBuffer {
public:
  PinnedBuffer() = default;
  ~PinnedBuffer() {
    if (ptr_) (void)cudaFreeHost(ptr_);
  }
  PinnedBuffer(const PinnedBuffer&) = delete;
  PinnedBuffer& operator=(const PinnedBuffer&) = delete;
  void reserve(size_t bytes) {
    if (bytes <= bytes_) return;
    if (ptr_) (void)cudaFreeHost(ptr_);
    ptr_ = nullptr;
    bytes_ = 0;
    if (injected_allocation_failure()) throw HostAllocationError();
    if (cudaMallocHost(&ptr_, bytes) != cudaSuccess) {
      ptr_ = nullptr;
      throw HostAllocationError();
    }
    bytes_ = bytes;
  }
  void* get() const { return ptr_; }

private:
  void* ptr_ = nullptr;
  size_t bytes_ = 0;
};

class Stream {
public:
  Stream() { check_cuda(cudaStreamCreateWithFlags(&s_, cudaStreamNonBlocking)); }
  ~Stream() {
    if (s_) (void)cudaStreamDestroy(s_);
  }
  Stream(const Stream&) = delete;
  Stream& operator=(const Stream&) = delete;
  cudaStream_t get() const { return s_; }

private:
  cudaStream_t s_ = nullptr;
};

class Event {
public:
  Event() { check_cuda(cudaEventCreateWithFlags(&e_, cudaEventDisableTiming)); }
  ~Event() {
    if (e_) (void)cudaEventDestroy(e_);
  }
  Event(const Event&) = delete;
  Event& operator=(const Event&) = delete;
  // Record on `from`, make `to` wait for it.
  void order(cudaStream_t from, cudaStream_t to) {
    check_cuda(cudaEventRecord(e_, from));
    check_cuda(cudaStreamWaitEvent(to, e_, 0));
  }
  void record(cudaStream_t s) { check_cuda(cudaEventRecord(e_, s)); }
  void wait_on(cudaStream_t s) { check_cuda(cudaStreamWaitEvent(s, e_, 0)); }

private:
  cudaEvent_t e_ = nullptr;
};

// A fixed set of events without timing, for fork / join patterns.
class EventSet {
public:
  explicit EventSet(int n) : n_(n), e_(new cudaEvent_t[n]()) {
    for (int i = 0; i < n; ++i) {
      if (cudaEventCreateWithFlags(&e_[i], cudaEventDisableTiming) != cudaSuccess) {
        destroy();
        throw GPUError();
      }
    }
  }
  ~EventSet() { destroy(); }
  EventSet(const EventSet&) = delete;
  EventSet& operator=(const EventSet&) = delete;
  cudaEvent_t* data() { return e_; }

private:
  void destroy() {
    if (!e_) return;
    for (int i = 0; i < n_; ++i) {
      if (e_[i]) (void)cudaEventDestroy(e_[i]);
    }
    delete[] e_;
    e_ = nullptr;
  }
  int n_;
  cudaEvent_t* e_;
};

// Host or device? Mirrors translate_gpu_pointer (src/gpu_util/gpu_pointer_translation.hpp:41-71):
// only memory of type cudaMemoryTypeDevice counts as device memory; managed and registered host
// memory take the host path.
template <typename T>
inline std::pair<T*, T*> split_pointer(T* p) {
  cudaPointerAttributes attr{};
  cudaError_t st = cudaPointerGetAttributes(&attr, static_cast<const void*>(p));
  if (st != cudaSuccess) {
    (void)cudaGetLastError();
    if (st != cudaErrorInvalidValue) check_cuda(st);
    return {p, nullptr};
  }
  if (attr.type == cudaMemoryTypeDevice) {
    return {nullptr, static_cast<T*>(attr.devicePointer)};
  }
  return {attr.hostPointer ? static_cast<T*>(attr.hostPointer) : p, nullptr};
}

// Device-accessible alias of pinned (page-locked, mapped) host memory, or nullptr for any other
// pointer. On GB300 the Grace host memory sits behind the coherent NVLink-C2C link, so kernels can
// read and write such buffers directly instead of staging them through device memory.
template <typename T>
inline T* mapped_host_alias(T* p) {
  if (!p) return nullptr;
  cudaPointerAttributes attr{};
  if (cudaPointerGetAttributes(&attr, static_cast<const void*>(p)) != cudaSuccess) {
    (void)cudaGetLastError();
    return nullptr;
  }
  if (attr.type != cudaMemoryTypeHost || !attr.devicePointer) return nullptr;
  return static_cast<T*>(attr.devicePointer);
}

}  // namespace gb300
}  // namespace spfft
