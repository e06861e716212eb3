// Batched multi-transform execution with a one-entry plan cache per precision.
#include "multi_batch.hpp"

#include <atomic>
#include <mutex>

#include "batch.hpp"

namespace spfft {
namespace gb300 {

namespace {

std::atomic<long long> batchedCalls{0};

// The batch plan of the most recent qualifying call. It does not keep the transforms alive: the
// weak pointers tell whether the transforms it was built for still exist, and a call with other
// transforms replaces it.
template <typename T>
struct Entry {
  std::vector<TransformInternal<T>*> raw;
  std::vector<std::weak_ptr<TransformInternal<T>>> alive;
  std::unique_ptr<BatchPlan<T>> plan;
  std::unique_ptr<Stream> stream;
  std::unique_ptr<Event> start, end;
  int device = 0;
};

template <typename T>
struct Cache {
  std::mutex mutex;
  std::unique_ptr<Entry<T>> entry;
};

// Never destroyed: the CUDA runtime may already be gone when static destructors run.
template <typename T>
Cache<T>& cache() {
  static Cache<T>* c = new Cache<T>();
  return *c;
}

template <typename T>
bool run(const std::vector<std::shared_ptr<TransformInternal<T>>>& ts, const T* const* values,
         T* const* spaces, int what, bool scaled) {
  const size_t n = ts.size();
  if (n < 2) return false;
  // A pending CUDA error aborts before any work, as in the one-by-one path.
  if (cudaGetLastError() != cudaSuccess) throw GPUPrecedingError();
  const int device = ts[0]->device_id();
  for (const auto& t : ts) {
    if (t->processing_unit() != SPFFT_PU_GPU || t->has_user_stream() || t->device_id() != device) return false;
  }
  DeviceGuard guard(device);
  const uintptr_t c = 2 * sizeof(T);
  std::vector<const T*> v(n, nullptr);
  std::vector<T*> s(n, nullptr);
  for (size_t t = 0; t < n; ++t) {
    s[t] = ts[t]->device_address(spaces[t]);
    if (!s[t] || reinterpret_cast<uintptr_t>(s[t]) % c) return false;
    if (ts[t]->num_local_elements() > 0) {
      v[t] = ts[t]->device_address(values[t]);
      if (!v[t] || reinterpret_cast<uintptr_t>(v[t]) % c) return false;
    }
  }

  Cache<T>& cache_ = cache<T>();
  std::lock_guard<std::mutex> lock(cache_.mutex);
  Entry<T>* e = cache_.entry.get();
  bool match = e && e->raw.size() == n && e->device == device;
  for (size_t t = 0; match && t < n; ++t) {
    match = e->raw[t] == ts[t].get() && e->alive[t].lock() == ts[t];
  }
  if (!match) {
    cache_.entry.reset();
    std::unique_ptr<Entry<T>> ne(new Entry<T>());
    ne->device = device;
    for (const auto& t : ts) {
      ne->raw.push_back(t.get());
      ne->alive.push_back(t);
    }
    ne->plan.reset(new BatchPlan<T>(ts));
    ne->plan->release_transforms();
    ne->stream.reset(new Stream());
    ne->start.reset(new Event());
    ne->end.reset(new Event());
    cache_.entry = std::move(ne);
    e = cache_.entry.get();
  }

  cudaStream_t st = e->stream->get();
  // Order after the legacy default stream (execution_gpu.cpp:260-261), rebind in stream order,
  // then replay the direction's graph.
  e->start->order(cudaStreamLegacy, st);
  bool same = true;
  for (size_t t = 0; same && t < n; ++t) {
    same = e->plan->bound_values(static_cast<int>(t)) == v[t] && e->plan->bound_space(static_cast<int>(t)) == s[t];
  }
  if (!same) e->plan->bind(v.data(), s.data(), st, true);
  e->plan->graph(what, scaled, st);
  // Completion: asynchronous transforms make the default stream wait, synchronous ones wait here
  // (execution_gpu.cpp:402-410).
  bool anySync = false, anyAsync = false;
  for (const auto& t : ts) {
    if (t->execution_mode() == SPFFT_EXEC_ASYNCHRONOUS) anyAsync = true;
    else anySync = true;
  }
  if (anyAsync) e->end->order(st, cudaStreamLegacy);
  if (anySync) check_cuda(cudaStreamSynchronize(st));
  ++batchedCalls;
  return true;
}

}  // namespace

template <typename T>
bool multi_backward_batched(const std::vector<std::shared_ptr<TransformInternal<T>>>& transforms,
                            const T* const* values, T* const* spaces) {
  return run<T>(transforms, values, spaces, 1, false);
}

template <typename T>
bool multi_forward_batched(const std::vector<std::shared_ptr<TransformInternal<T>>>& transforms,
                           const T* const* spaces, T* const* values, const SpfftScalingType* scalings) {
  const size_t n = transforms.size();
  if (n < 2) return false;
  for (size_t t = 1; t < n; ++t) {
    if (scalings[t] != scalings[0]) return false;
  }
  // the bound table wants writable value pointers and const space pointers the other way round;
  // both point at the same buffers
  std::vector<const T*> v(values, values + n);
  std::vector<T*> s(n);
  for (size_t t = 0; t < n; ++t) s[t] = const_cast<T*>(spaces[t]);
  return run<T>(transforms, v.data(), s.data(), 2, scalings[0] == SPFFT_FULL_SCALING);
}

long long multi_batched_calls() { return batchedCalls.load(); }

template bool multi_backward_batched<double>(const std::vector<std::shared_ptr<TransformInternal<double>>>&,
                                             const double* const*, double* const*);
template bool multi_backward_batched<float>(const std::vector<std::shared_ptr<TransformInternal<float>>>&,
                                            const float* const*, float* const*);
template bool multi_forward_batched<double>(const std::vector<std::shared_ptr<TransformInternal<double>>>&,
                                            const double* const*, double* const*, const SpfftScalingType*);
template bool multi_forward_batched<float>(const std::vector<std::shared_ptr<TransformInternal<float>>>&,
                                           const float* const*, float* const*, const SpfftScalingType*);

}  // namespace gb300
}  // namespace spfft
