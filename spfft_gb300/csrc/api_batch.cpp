// C interface of batched execution (include/spfft/spfft_gb300.h).
#include <memory>
#include <vector>

#include "access.hpp"
#include "batch.hpp"
#include "multi_batch.hpp"
#include "spfft/spfft_gb300.h"
#include "spfft/transform.hpp"
#include "spfft/transform_float.hpp"

namespace {

struct BatchHandle {
  std::unique_ptr<spfft::gb300::BatchPlan<double>> d;
  std::unique_ptr<spfft::gb300::BatchPlan<float>> f;
};

template <typename F>
SpfftError guarded(F&& f) {
  try {
    f();
  } catch (const spfft::GenericError& e) {
    return e.error_code();
  } catch (...) {
    return SPFFT_UNKNOWN_ERROR;
  }
  return SPFFT_SUCCESS;
}

template <typename H, typename T>
std::vector<std::shared_ptr<spfft::TransformInternal<T>>> collect(int n, const void* const* transforms) {
  if (n <= 0 || !transforms) throw spfft::InvalidParameterError();
  std::vector<std::shared_ptr<spfft::TransformInternal<T>>> v;
  for (int i = 0; i < n; ++i) {
    if (!transforms[i]) throw spfft::InvalidParameterError();
    H& h = *reinterpret_cast<H*>(const_cast<void*>(transforms[i]));
    v.push_back(spfft::TransformAccess::share(h));
  }
  return v;
}

template <typename F>
SpfftError with_batch(void* batch, F&& f) {
  if (!batch) return SPFFT_INVALID_HANDLE_ERROR;
  return guarded([&] { f(*reinterpret_cast<BatchHandle*>(batch)); });
}

}  // namespace

extern "C" {

SpfftError spfft_gb300_batch_create(SpfftGb300Batch* batch, int numTransforms,
                                    const SpfftTransform* transforms) {
  if (!batch) return SPFFT_INVALID_PARAMETER_ERROR;
  return guarded([&] {
    auto h = std::make_unique<BatchHandle>();
    h->d = std::make_unique<spfft::gb300::BatchPlan<double>>(
        collect<spfft::Transform, double>(numTransforms, transforms));
    *batch = h.release();
  });
}

SpfftError spfft_gb300_float_batch_create(SpfftGb300Batch* batch, int numTransforms,
                                          const SpfftFloatTransform* transforms) {
  if (!batch) return SPFFT_INVALID_PARAMETER_ERROR;
  return guarded([&] {
    auto h = std::make_unique<BatchHandle>();
    h->f = std::make_unique<spfft::gb300::BatchPlan<float>>(
        collect<spfft::TransformFloat, float>(numTransforms, transforms));
    *batch = h.release();
  });
}

SpfftError spfft_gb300_batch_destroy(SpfftGb300Batch batch) {
  if (!batch) return SPFFT_INVALID_HANDLE_ERROR;
  return guarded([&] { delete reinterpret_cast<BatchHandle*>(batch); });
}

SpfftError spfft_gb300_batch_bind(SpfftGb300Batch batch, void* const* values, void* const* spaces) {
  return with_batch(batch, [&](BatchHandle& h) {
    if (h.d) {
      h.d->bind(reinterpret_cast<const double* const*>(values), reinterpret_cast<double* const*>(spaces));
    } else {
      h.f->bind(reinterpret_cast<const float* const*>(values), reinterpret_cast<float* const*>(spaces));
    }
  });
}

SpfftError spfft_gb300_batch_backward(SpfftGb300Batch batch, void* stream) {
  return with_batch(batch, [&](BatchHandle& h) {
    if (h.d) h.d->backward(static_cast<cudaStream_t>(stream));
    else h.f->backward(static_cast<cudaStream_t>(stream));
  });
}

SpfftError spfft_gb300_batch_forward(SpfftGb300Batch batch, SpfftScalingType scaling, void* stream) {
  return with_batch(batch, [&](BatchHandle& h) {
    const bool s = scaling == SPFFT_FULL_SCALING;
    if (h.d) h.d->forward(s, static_cast<cudaStream_t>(stream));
    else h.f->forward(s, static_cast<cudaStream_t>(stream));
  });
}

SpfftError spfft_gb300_batch_pair_graph(SpfftGb300Batch batch, SpfftScalingType scaling, void* stream) {
  return with_batch(batch, [&](BatchHandle& h) {
    const bool s = scaling == SPFFT_FULL_SCALING;
    if (h.d) h.d->pair_graph(s, static_cast<cudaStream_t>(stream));
    else h.f->pair_graph(s, static_cast<cudaStream_t>(stream));
  });
}

SpfftError spfft_gb300_batch_info(SpfftGb300Batch batch, int* numGroups, int* numUnbatched,
                                  int* launchesPerPair) {
  return with_batch(batch, [&](BatchHandle& h) {
    if (h.d) {
      if (numGroups) *numGroups = h.d->num_groups();
      if (numUnbatched) *numUnbatched = h.d->num_unbatched();
      if (launchesPerPair) *launchesPerPair = h.d->launches_per_pair();
    } else {
      if (numGroups) *numGroups = h.f->num_groups();
      if (numUnbatched) *numUnbatched = h.f->num_unbatched();
      if (launchesPerPair) *launchesPerPair = h.f->launches_per_pair();
    }
  });
}

SpfftError spfft_gb300_batch_autotune(SpfftGb300Batch batch, int repetitions, void* stream, float* msPerPair) {
  return with_batch(batch, [&](BatchHandle& h) {
    if (repetitions < 1) throw spfft::InvalidParameterError();
    const float ms = h.d ? h.d->autotune(static_cast<cudaStream_t>(stream), repetitions)
                         : h.f->autotune(static_cast<cudaStream_t>(stream), repetitions);
    if (msPerPair) *msPerPair = ms;
  });
}

SpfftError spfft_gb300_batch_transform_path(SpfftGb300Batch batch, int index, int* path) {
  return with_batch(batch, [&](BatchHandle& h) {
    if (!path) throw spfft::InvalidParameterError();
    *path = h.d ? h.d->transform_path(index) : h.f->transform_path(index);
  });
}

SpfftError spfft_gb300_batch_row_groups(SpfftGb300Batch batch, int index, int* groups) {
  return with_batch(batch, [&](BatchHandle& h) {
    if (!groups) throw spfft::InvalidParameterError();
    *groups = h.d ? h.d->row_groups(index) : h.f->row_groups(index);
  });
}

SpfftError spfft_gb300_multi_batched_calls(long long* count) {
  if (!count) return SPFFT_INVALID_PARAMETER_ERROR;
  *count = spfft::gb300::multi_batched_calls();
  return SPFFT_SUCCESS;
}

SpfftError spfft_gb300_batch_stage_times(SpfftGb300Batch batch, int direction, SpfftScalingType scaling,
                                         void* stream, float* stageMs) {
  return with_batch(batch, [&](BatchHandle& h) {
    if (!stageMs || (direction != 0 && direction != 1)) throw spfft::InvalidParameterError();
    const bool s = scaling == SPFFT_FULL_SCALING;
    if (h.d) h.d->stage_times(direction, s, static_cast<cudaStream_t>(stream), stageMs);
    else h.f->stage_times(direction, s, static_cast<cudaStream_t>(stream), stageMs);
  });
}

}  // extern "C"
