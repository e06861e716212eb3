// The C interface: every function converts exceptions into SpfftError codes, like the reference's
// src/spfft/{grid,transform,multi_transform}{,_float}.cpp C sections (e.g. transform.cpp:179-562).
#include <algorithm>
#include <vector>

#include "access.hpp"
#include "internal.hpp"
#include "planner.hpp"
#include "planner_gpu.hpp"
#include "spfft/spfft.h"
#include "spfft/spfft.hpp"
#include "spfft/spfft_gb300.h"

namespace {

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

template <typename H>
std::vector<H> collect_handles(int n, void** transforms) {
  std::vector<H> v;
  v.reserve(n);
  for (int i = 0; i < n; ++i) {
    if (!transforms[i]) throw spfft::InvalidParameterError();
    v.push_back(*reinterpret_cast<H*>(transforms[i]));
  }
  return v;
}

template <typename H, typename F>
SpfftError with_handle(void* handle, F&& f) {
  if (!handle) return SPFFT_INVALID_HANDLE_ERROR;
  return guarded([&] { f(*reinterpret_cast<H*>(handle)); });
}

}  // namespace

extern "C" {

// ---------------------------------------------------------------------------------------------
// Grid (grid.cpp / grid_float.cpp)
// ---------------------------------------------------------------------------------------------
#define SPFFT_GB300_GRID_C_API(PREFIX, GRID)                                                      \
  SpfftError PREFIX##create(void** grid, int maxDimX, int maxDimY, int maxDimZ,                  \
                            int maxNumLocalZColumns, SpfftProcessingUnitType processingUnit,      \
                            int maxNumThreads) {                                                  \
    if (!grid) return SPFFT_INVALID_PARAMETER_ERROR;                                              \
    return guarded([&] {                                                                          \
      *grid = new spfft::GRID(maxDimX, maxDimY, maxDimZ, maxNumLocalZColumns, processingUnit,     \
                              maxNumThreads);                                                     \
    });                                                                                           \
  }                                                                                               \
  SpfftError PREFIX##destroy(void* grid) {                                                        \
    if (!grid) return SPFFT_INVALID_HANDLE_ERROR;                                                 \
    return guarded([&] { delete reinterpret_cast<spfft::GRID*>(grid); });                         \
  }                                                                                               \
  SpfftError PREFIX##max_dim_x(void* grid, int* v) {                                              \
    return with_handle<spfft::GRID>(grid, [&](spfft::GRID& g) { *v = g.max_dim_x(); });           \
  }                                                                                               \
  SpfftError PREFIX##max_dim_y(void* grid, int* v) {                                              \
    return with_handle<spfft::GRID>(grid, [&](spfft::GRID& g) { *v = g.max_dim_y(); });           \
  }                                                                                               \
  SpfftError PREFIX##max_dim_z(void* grid, int* v) {                                              \
    return with_handle<spfft::GRID>(grid, [&](spfft::GRID& g) { *v = g.max_dim_z(); });           \
  }                                                                                               \
  SpfftError PREFIX##max_num_local_z_columns(void* grid, int* v) {                                \
    return with_handle<spfft::GRID>(grid,                                                         \
                                    [&](spfft::GRID& g) { *v = g.max_num_local_z_columns(); });   \
  }                                                                                               \
  SpfftError PREFIX##max_local_z_length(void* grid, int* v) {                                     \
    return with_handle<spfft::GRID>(grid, [&](spfft::GRID& g) { *v = g.max_local_z_length(); });  \
  }                                                                                               \
  SpfftError PREFIX##processing_unit(void* grid, SpfftProcessingUnitType* v) {                    \
    return with_handle<spfft::GRID>(grid, [&](spfft::GRID& g) { *v = g.processing_unit(); });     \
  }                                                                                               \
  SpfftError PREFIX##device_id(void* grid, int* v) {                                              \
    return with_handle<spfft::GRID>(grid, [&](spfft::GRID& g) { *v = g.device_id(); });           \
  }                                                                                               \
  SpfftError PREFIX##num_threads(void* grid, int* v) {                                            \
    return with_handle<spfft::GRID>(grid, [&](spfft::GRID& g) { *v = g.num_threads(); });         \
  }

SPFFT_GB300_GRID_C_API(spfft_grid_, Grid)
SPFFT_GB300_GRID_C_API(spfft_float_grid_, GridFloat)
#undef SPFFT_GB300_GRID_C_API

// ---------------------------------------------------------------------------------------------
// Transform (transform.cpp / transform_float.cpp)
// ---------------------------------------------------------------------------------------------
#define SPFFT_GB300_TRANSFORM_C_API(PREFIX, GPREFIX, GRID, TRANSFORM, T)                          \
  SpfftError PREFIX##create(void** transform, void* grid, SpfftProcessingUnitType processingUnit, \
                            SpfftTransformType transformType, int dimX, int dimY, int dimZ,       \
                            int localZLength, int numLocalElements,                               \
                            SpfftIndexFormatType indexFormat, const int* indices) {               \
    if (!grid) return SPFFT_INVALID_HANDLE_ERROR;                                                 \
    if (!transform) return SPFFT_INVALID_PARAMETER_ERROR;                                         \
    return guarded([&] {                                                                          \
      *transform = new spfft::TRANSFORM(reinterpret_cast<spfft::GRID*>(grid)->create_transform(   \
          processingUnit, transformType, dimX, dimY, dimZ, localZLength, numLocalElements,        \
          indexFormat, indices));                                                                 \
    });                                                                                           \
  }                                                                                               \
  SpfftError PREFIX##create_independent(void** transform, int maxNumThreads,                      \
                                        SpfftProcessingUnitType processingUnit,                   \
                                        SpfftTransformType transformType, int dimX, int dimY,     \
                                        int dimZ, int numLocalElements,                           \
                                        SpfftIndexFormatType indexFormat, const int* indices) {   \
    if (!transform) return SPFFT_INVALID_PARAMETER_ERROR;                                         \
    return guarded([&] {                                                                          \
      *transform = new spfft::TRANSFORM(maxNumThreads, processingUnit, transformType, dimX, dimY, \
                                        dimZ, numLocalElements, indexFormat, indices);            \
    });                                                                                           \
  }                                                                                               \
  SpfftError PREFIX##destroy(void* transform) {                                                   \
    if (!transform) return SPFFT_INVALID_HANDLE_ERROR;                                            \
    return guarded([&] { delete reinterpret_cast<spfft::TRANSFORM*>(transform); });              \
  }                                                                                               \
  SpfftError PREFIX##clone(void* transform, void** newTransform) {                                \
    return with_handle<spfft::TRANSFORM>(transform, [&](spfft::TRANSFORM& t) {                    \
      *newTransform = new spfft::TRANSFORM(t.clone());                                            \
    });                                                                                           \
  }                                                                                               \
  SpfftError PREFIX##forward(void* transform, SpfftProcessingUnitType inputLocation, T* output,   \
                             SpfftScalingType scaling) {                                          \
    return with_handle<spfft::TRANSFORM>(                                                         \
        transform, [&](spfft::TRANSFORM& t) { t.forward(inputLocation, output, scaling); });      \
  }                                                                                               \
  SpfftError PREFIX##forward_ptr(void* transform, const T* input, T* output,                      \
                                 SpfftScalingType scaling) {                                      \
    return with_handle<spfft::TRANSFORM>(                                                         \
        transform, [&](spfft::TRANSFORM& t) { t.forward(input, output, scaling); });              \
  }                                                                                               \
  SpfftError PREFIX##backward(void* transform, const T* input,                                    \
                              SpfftProcessingUnitType outputLocation) {                           \
    return with_handle<spfft::TRANSFORM>(                                                         \
        transform, [&](spfft::TRANSFORM& t) { t.backward(input, outputLocation); });              \
  }                                                                                               \
  SpfftError PREFIX##backward_ptr(void* transform, const T* input, T* output) {                   \
    return with_handle<spfft::TRANSFORM>(transform,                                               \
                                         [&](spfft::TRANSFORM& t) { t.backward(input, output); }); \
  }                                                                                               \
  SpfftError PREFIX##get_space_domain(void* transform, SpfftProcessingUnitType dataLocation,      \
                                      T** data) {                                                 \
    return with_handle<spfft::TRANSFORM>(                                                         \
        transform, [&](spfft::TRANSFORM& t) { *data = t.space_domain_data(dataLocation); });      \
  }                                                                                               \
  SpfftError PREFIX##dim_x(void* transform, int* v) {                                             \
    return with_handle<spfft::TRANSFORM>(transform, [&](spfft::TRANSFORM& t) { *v = t.dim_x(); });\
  }                                                                                               \
  SpfftError PREFIX##dim_y(void* transform, int* v) {                                             \
    return with_handle<spfft::TRANSFORM>(transform, [&](spfft::TRANSFORM& t) { *v = t.dim_y(); });\
  }                                                                                               \
  SpfftError PREFIX##dim_z(void* transform, int* v) {                                             \
    return with_handle<spfft::TRANSFORM>(transform, [&](spfft::TRANSFORM& t) { *v = t.dim_z(); });\
  }                                                                                               \
  SpfftError PREFIX##local_z_length(void* transform, int* v) {                                    \
    return with_handle<spfft::TRANSFORM>(transform,                                               \
                                         [&](spfft::TRANSFORM& t) { *v = t.local_z_length(); });  \
  }                                                                                               \
  SpfftError PREFIX##local_slice_size(void* transform, int* v) {                                  \
    return with_handle<spfft::TRANSFORM>(transform,                                               \
                                         [&](spfft::TRANSFORM& t) { *v = t.local_slice_size(); });\
  }                                                                                               \
  SpfftError PREFIX##local_z_offset(void* transform, int* v) {                                    \
    return with_handle<spfft::TRANSFORM>(transform,                                               \
                                         [&](spfft::TRANSFORM& t) { *v = t.local_z_offset(); });  \
  }                                                                                               \
  SpfftError PREFIX##global_size(void* transform, long long int* v) {                             \
    return with_handle<spfft::TRANSFORM>(transform,                                               \
                                         [&](spfft::TRANSFORM& t) { *v = t.global_size(); });     \
  }                                                                                               \
  SpfftError PREFIX##num_local_elements(void* transform, int* v) {                                \
    return with_handle<spfft::TRANSFORM>(                                                         \
        transform, [&](spfft::TRANSFORM& t) { *v = t.num_local_elements(); });                   \
  }                                                                                               \
  SpfftError PREFIX##num_global_elements(void* transform, long long int* v) {                     \
    return with_handle<spfft::TRANSFORM>(                                                         \
        transform, [&](spfft::TRANSFORM& t) { *v = t.num_global_elements(); });                  \
  }                                                                                               \
  SpfftError PREFIX##device_id(void* transform, int* v) {                                         \
    return with_handle<spfft::TRANSFORM>(transform,                                               \
                                         [&](spfft::TRANSFORM& t) { *v = t.device_id(); });       \
  }                                                                                               \
  SpfftError PREFIX##num_threads(void* transform, int* v) {                                       \
    return with_handle<spfft::TRANSFORM>(transform,                                               \
                                         [&](spfft::TRANSFORM& t) { *v = t.num_threads(); });     \
  }                                                                                               \
  SpfftError PREFIX##execution_mode(void* transform, SpfftExecType* v) {                          \
    return with_handle<spfft::TRANSFORM>(transform,                                               \
                                         [&](spfft::TRANSFORM& t) { *v = t.execution_mode(); });  \
  }                                                                                               \
  SpfftError PREFIX##set_execution_mode(void* transform, SpfftExecType mode) {                    \
    return with_handle<spfft::TRANSFORM>(transform,                                               \
                                         [&](spfft::TRANSFORM& t) { t.set_execution_mode(mode); });\
  }                                                                                               \
  SpfftError GPREFIX##set_stream(void* transform, void* stream) {                                 \
    return with_handle<spfft::TRANSFORM>(transform, [&](spfft::TRANSFORM& t) {                    \
      spfft::TransformAccess::get(t).set_stream(static_cast<cudaStream_t>(stream));               \
    });                                                                                           \
  }                                                                                               \
  SpfftError GPREFIX##backward_device(void* transform, const T* values, T* space, void* stream) { \
    return with_handle<spfft::TRANSFORM>(transform, [&](spfft::TRANSFORM& t) {                    \
      spfft::TransformAccess::get(t).backward_device(values, space,                               \
                                                     static_cast<cudaStream_t>(stream));          \
    });                                                                                           \
  }                                                                                               \
  SpfftError GPREFIX##stage_times(void* transform, int direction, const T* input, T* output,     \
                                  SpfftScalingType scaling, void* stream, float* stageMs) {       \
    return with_handle<spfft::TRANSFORM>(transform, [&](spfft::TRANSFORM& t) {                    \
      if (!stageMs || (direction != 0 && direction != 1)) throw spfft::InvalidParameterError();   \
      spfft::TransformAccess::get(t).stage_times(direction, input, output,                        \
                                                 scaling == SPFFT_FULL_SCALING,                   \
                                                 static_cast<cudaStream_t>(stream), stageMs);     \
    });                                                                                           \
  }                                                                                               \
  SpfftError GPREFIX##adjoint_backward(void* transform, const T* gradSpace, T* gradValues,        \
                                       void* stream) {                                            \
    return with_handle<spfft::TRANSFORM>(transform, [&](spfft::TRANSFORM& t) {                    \
      spfft::TransformAccess::get(t).adjoint_backward_device(gradSpace, gradValues,               \
                                                             static_cast<cudaStream_t>(stream));  \
    });                                                                                           \
  }                                                                                               \
  SpfftError GPREFIX##adjoint_forward(void* transform, const T* gradValues, T* gradSpace,         \
                                      SpfftScalingType scaling, void* stream) {                   \
    return with_handle<spfft::TRANSFORM>(transform, [&](spfft::TRANSFORM& t) {                    \
      spfft::TransformAccess::get(t).adjoint_forward_device(gradValues, gradSpace,                \
                                                            scaling == SPFFT_FULL_SCALING,        \
                                                            static_cast<cudaStream_t>(stream));   \
    });                                                                                           \
  }                                                                                               \
  SpfftError GPREFIX##path_info(void* transform, int* flags) {                                    \
    return with_handle<spfft::TRANSFORM>(transform, [&](spfft::TRANSFORM& t) {                    \
      *flags = spfft::TransformAccess::get(t).path_flags();                                       \
    });                                                                                           \
  }                                                                                               \
  SpfftError GPREFIX##autotune(void* transform, int repetitions, float* msPerPair) {              \
    return with_handle<spfft::TRANSFORM>(transform, [&](spfft::TRANSFORM& t) {                    \
      if (repetitions < 1) throw spfft::InvalidParameterError();                                  \
      const float ms = spfft::TransformAccess::get(t).autotune(repetitions);                      \
      if (msPerPair) *msPerPair = ms;                                                             \
    });                                                                                           \
  }                                                                                               \
  SpfftError GPREFIX##tuning(void* transform, int* tuning) {                                      \
    return with_handle<spfft::TRANSFORM>(transform, [&](spfft::TRANSFORM& t) {                    \
      if (!tuning) throw spfft::InvalidParameterError();                                          \
      const auto tu = spfft::TransformAccess::get(t).gpu_plan().tuning();                         \
      tuning[0] = tu.spb;                                                                         \
      tuning[1] = tu.path;                                                                        \
      tuning[2] = tu.fusedRows;                                                                   \
      tuning[3] = tu.fusedThreads;                                                                \
      tuning[4] = tu.cpb;                                                                         \
      tuning[5] = tu.rpb;                                                                         \
    });                                                                                           \
  }                                                                                               \
  SpfftError GPREFIX##x_backward_rows(void* transform, int* rows) {                               \
    return with_handle<spfft::TRANSFORM>(transform, [&](spfft::TRANSFORM& t) {                    \
      if (!rows) throw spfft::InvalidParameterError();                                            \
      *rows = spfft::TransformAccess::get(t).gpu_plan().tuning().rpbB;                            \
    });                                                                                           \
  }                                                                                               \
  SpfftError GPREFIX##splits(void* transform, int* radices) {                                    \
    return with_handle<spfft::TRANSFORM>(transform, [&](spfft::TRANSFORM& t) {                    \
      if (!radices) throw spfft::InvalidParameterError();                                         \
      spfft::TransformAccess::get(t).gpu_plan().split_radices(radices);                           \
    });                                                                                           \
  }                                                                                               \
  SpfftError GPREFIX##split_stages(void* transform, int* stages) {                               \
    return with_handle<spfft::TRANSFORM>(transform, [&](spfft::TRANSFORM& t) {                    \
      if (!stages) throw spfft::InvalidParameterError();                                          \
      spfft::TransformAccess::get(t).gpu_plan().split_stages(stages);                             \
    });                                                                                           \
  }                                                                                               \
  SpfftError GPREFIX##radix_plans(void* transform, int* numStages, int* radices) {                \
    return with_handle<spfft::TRANSFORM>(transform, [&](spfft::TRANSFORM& t) {                    \
      if (!numStages || !radices) throw spfft::InvalidParameterError();                           \
      const auto& plan = spfft::TransformAccess::get(t).gpu_plan();                               \
      int split[18];                                                                              \
      plan.split_stages(split);                                                                   \
      for (int d = 0; d < 3; ++d) {                                                               \
        for (int i = 0; i < spfft::gb300::kMaxStages; ++i) radices[d * spfft::gb300::kMaxStages + i] = 0; \
        /* size-specialised backward pass of this length: the radices of its two- or three-pass */ \
        /* split, of the complex FFT length (half the x length for the R2C x pass) */             \
        const int* sp = split + 3 * (d == 0 ? 0 : d == 1 ? 2 : 4);                                 \
        if (sp[0] > 0) {                                                                          \
          numStages[d] = sp[2] > 0 ? 3 : 2;                                                       \
          for (int i = 0; i < numStages[d]; ++i) radices[d * spfft::gb300::kMaxStages + i] = sp[i]; \
          continue;                                                                               \
        }                                                                                         \
        const spfft::gb300::RadixPlan r = plan.radix_plan(d);                                     \
        numStages[d] = r.numStages;                                                               \
        for (int i = 0; i < spfft::gb300::kMaxStages; ++i)                                        \
          radices[d * spfft::gb300::kMaxStages + i] = i < r.numStages ? r.radix[i] : 0;           \
      }                                                                                           \
    });                                                                                           \
  }                                                                                               \
  SpfftError GPREFIX##forward_device(void* transform, const T* space, T* values,                  \
                                     SpfftScalingType scaling, void* stream) {                    \
    return with_handle<spfft::TRANSFORM>(transform, [&](spfft::TRANSFORM& t) {                    \
      spfft::TransformAccess::get(t).forward_device(space, values, scaling == SPFFT_FULL_SCALING,  \
                                                    static_cast<cudaStream_t>(stream));           \
    });                                                                                           \
  }

SPFFT_GB300_TRANSFORM_C_API(spfft_transform_, spfft_gb300_transform_, Grid, Transform, double)
SPFFT_GB300_TRANSFORM_C_API(spfft_float_transform_, spfft_gb300_float_transform_, GridFloat,
                            TransformFloat, float)
#undef SPFFT_GB300_TRANSFORM_C_API

// ---------------------------------------------------------------------------------------------
// Multi-transform (multi_transform.cpp / multi_transform_float.cpp)
// ---------------------------------------------------------------------------------------------
#define SPFFT_GB300_MULTI_C_API(PREFIX, TRANSFORM, T)                                             \
  SpfftError PREFIX##forward(int n, void** transforms,                                            \
                             const SpfftProcessingUnitType* inputLocations,                       \
                             T* const* outputPointers, const SpfftScalingType* scalingTypes) {    \
    if (n > 0 && !transforms) return SPFFT_INVALID_HANDLE_ERROR;                                  \
    return guarded([&] {                                                                          \
      auto v = collect_handles<spfft::TRANSFORM>(n, transforms);                                                    \
      spfft::multi_transform_forward(n, v.data(), inputLocations, outputPointers, scalingTypes);   \
    });                                                                                           \
  }                                                                                               \
  SpfftError PREFIX##forward_ptr(int n, void** transforms, const T* const* inputPointers,         \
                                 T* const* outputPointers, const SpfftScalingType* scalingTypes) {\
    if (n > 0 && !transforms) return SPFFT_INVALID_HANDLE_ERROR;                                  \
    return guarded([&] {                                                                          \
      auto v = collect_handles<spfft::TRANSFORM>(n, transforms);                                                    \
      spfft::multi_transform_forward(n, v.data(), inputPointers, outputPointers, scalingTypes);    \
    });                                                                                           \
  }                                                                                               \
  SpfftError PREFIX##backward(int n, void** transforms, const T* const* inputPointers,            \
                              const SpfftProcessingUnitType* outputLocations) {                   \
    if (n > 0 && !transforms) return SPFFT_INVALID_HANDLE_ERROR;                                  \
    return guarded([&] {                                                                          \
      auto v = collect_handles<spfft::TRANSFORM>(n, transforms);                                                    \
      spfft::multi_transform_backward(n, v.data(), inputPointers, outputLocations);               \
    });                                                                                           \
  }                                                                                               \
  SpfftError PREFIX##backward_ptr(int n, void** transforms, const T* const* inputPointers,        \
                                  T* const* outputPointers) {                                     \
    if (n > 0 && !transforms) return SPFFT_INVALID_HANDLE_ERROR;                                  \
    return guarded([&] {                                                                          \
      auto v = collect_handles<spfft::TRANSFORM>(n, transforms);                                                    \
      spfft::multi_transform_backward(n, v.data(), inputPointers, outputPointers);                \
    });                                                                                           \
  }

SPFFT_GB300_MULTI_C_API(spfft_multi_transform_, Transform, double)
SPFFT_GB300_MULTI_C_API(spfft_float_multi_transform_, TransformFloat, float)
#undef SPFFT_GB300_MULTI_C_API

// ---------------------------------------------------------------------------------------------
// Host-only planning
// ---------------------------------------------------------------------------------------------
SpfftError spfft_gb300_plan_indices(SpfftTransformType transformType, int dimX, int dimY, int dimZ,
                                    int numLocalElements, const int* indices, int* valueIndices,
                                    int* stickKeys, int maxSticks, int* numSticks,
                                    int* zeroZeroStick) {
  return guarded([&] {
    if (numLocalElements < 0 || (!indices && numLocalElements > 0)) {
      throw spfft::InvalidParameterError();
    }
    auto plan = spfft::gb300::make_index_plan(transformType, dimX, dimY, dimZ, numLocalElements,
                                              indices);
    if (valueIndices) {
      for (int i = 0; i < numLocalElements; ++i) valueIndices[i] = plan.valueIndices[i];
    }
    if (stickKeys) {
      if (plan.num_sticks() > maxSticks) throw spfft::InvalidParameterError();
      for (int s = 0; s < plan.num_sticks(); ++s) stickKeys[s] = plan.stickKeys[s];
    }
    if (numSticks) *numSticks = plan.num_sticks();
    if (zeroZeroStick) *zeroZeroStick = plan.zeroZeroStick;
  });
}

// Every table of the index plan, from the host or the device planner (for verification).
SpfftError spfft_gb300_plan_tables(int planner, SpfftTransformType transformType, int dimX, int dimY,
                                   int dimZ, int numLocalElements, const int* indices, int* tables,
                                   long long capacity, long long* size, int* usedDevice) {
  return guarded([&] {
    if (numLocalElements < 0 || (!indices && numLocalElements > 0) || !size) {
      throw spfft::InvalidParameterError();
    }
    if (planner != 0 && planner != 1) throw spfft::InvalidParameterError();
    spfft::gb300::IndexPlan plan;
    bool device = false;
    if (planner == 1) {
      device = spfft::gb300::make_index_plan_device(transformType, dimX, dimY, dimZ,
                                                    numLocalElements, indices, &plan);
    }
    if (!device) {
      plan = spfft::gb300::make_index_plan(transformType, dimX, dimY, dimZ, numLocalElements, indices);
    }
    const spfft::gb300::IndexPlan h = spfft::gb300::download_index_plan(plan);
    const long long ns = h.numSticks, ncol = h.numColumns, nv = h.numValues;
    const long long need = 4 + nv + 5 * ns + ncol + (ncol + 1) + 2 * nv + (ns + 1) +
                           static_cast<long long>(h.hermitianWeight.size());
    *size = need;
    if (usedDevice) *usedDevice = device ? 1 : 0;
    if (!tables || capacity < need) return;
    int* o = tables;
    *o++ = h.numSticks;
    *o++ = h.numColumns;
    *o++ = h.zeroZeroStick;
    *o++ = h.identityOrder ? 1 : 0;
    auto put = [&o](const std::vector<int>& v) { o = std::copy(v.begin(), v.end(), o); };
    put(h.valueIndices);
    put(h.stickKeys);
    put(h.stickColumn);
    put(h.stickY);
    std::vector<int> planePos(ns);
    for (long long st = 0; st < ns; ++st) planePos[st] = h.stickY[st] * h.numColumns + h.stickColumn[st];
    put(planePos);
    put(h.columnX);
    put(h.columnStickStart);
    put(h.entryPos);
    put(h.entryUser);
    put(h.stickEntryStart);
    for (unsigned char w : h.hermitianWeight) *o++ = w;
  });
}

SpfftError spfft_gb300_inject_allocation_failure(int afterAllocations, int* previous) {
  if (afterAllocations < -1) return SPFFT_INVALID_PARAMETER_ERROR;
  const int old = spfft::gb300::allocation_countdown().exchange(afterAllocations);
  if (previous) *previous = old;
  return SPFFT_SUCCESS;
}

SpfftError spfft_gb300_plan_cache_size(int* count) {
  return guarded([&] {
    if (!count) throw spfft::InvalidParameterError();
    *count = spfft::gb300::index_plan_cache_size();
  });
}

}  // extern "C"
