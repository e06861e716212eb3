// C++ handle classes spfft::Grid / Transform (double) and GridFloat / TransformFloat (float), and
// the multi-transform functions. Thin wrappers over GridInternal / TransformInternal, like the
// reference's src/spfft/{grid,transform,multi_transform}{,_float}.cpp.
#include <memory>
#include <vector>

#include "access.hpp"
#include "internal.hpp"
#include "multi_batch.hpp"
#include "planner.hpp"
#include "planner_gpu.hpp"
#include "spfft/grid.hpp"
#include "spfft/grid_float.hpp"
#include "spfft/multi_transform.hpp"
#include "spfft/multi_transform_float.hpp"
#include "spfft/transform.hpp"
#include "spfft/transform_float.hpp"

namespace spfft {

namespace {

// Argument checks of the reference Transform constructors (transform.cpp:51-54, 74-77).
void check_transform_args(int dimX, int dimY, int dimZ, int localZLength, int numLocalElements,
                          const int* indices) {
  if (dimX < 0 || dimY < 0 || dimZ < 0 || localZLength < 0 || numLocalElements < 0 ||
      (!indices && numLocalElements > 0)) {
    throw InvalidParameterError();
  }
}

// The plan of a transform: shared with a live transform of the same index set on the same device,
// else made by the device planner (large sets of GPU transforms) or the host planner. `device` is
// the grid's device, or -1 for the current one.
std::shared_ptr<const gb300::IndexPlan> make_plan(SpfftTransformType type, int dimX, int dimY,
                                                  int dimZ, int numLocalElements,
                                                  SpfftIndexFormatType indexFormat,
                                                  const int* indices,
                                                  SpfftProcessingUnitType processingUnit,
                                                  int device) {
  // Only index triplets are defined (parameters.cpp:159-162 raises InternalError otherwise).
  if (indexFormat != SPFFT_INDEX_TRIPLETS) throw InternalError();
  const bool gpu = processingUnit == SPFFT_PU_GPU;
  if (gpu && device >= 0) {
    gb300::DeviceGuard guard(device);
    return gb300::shared_index_plan(type, dimX, dimY, dimZ, numLocalElements, indices, true);
  }
  return gb300::shared_index_plan(type, dimX, dimY, dimZ, numLocalElements, indices, gpu);
}

template <typename TransformType, typename ValueType>
void multi_forward(int n, TransformType* transforms, const ValueType* const* inputs,
                   ValueType* const* outputs, const SpfftScalingType* scalings) {
  if (n < 0 || (n > 0 && (!transforms || !inputs || !outputs || !scalings))) {
    throw InvalidParameterError();
  }
  // Transforms must not share a grid (multi_transform_internal.hpp:69-76).
  for (int a = 0; a < n; ++a)
    for (int b = a + 1; b < n; ++b)
      if (TransformAccess::get(transforms[a]).shared_grid(TransformAccess::get(transforms[b])))
        throw InvalidParameterError();
  // One batched execution when the call qualifies (multi_batch.hpp).
  std::vector<decltype(TransformAccess::share(transforms[0]))> shared;
  for (int t = 0; t < n; ++t) shared.push_back(TransformAccess::share(transforms[t]));
  if (gb300::multi_forward_batched(shared, inputs, outputs, scalings)) return;
  // Otherwise enqueue every transform before waiting on any (multi_transform_internal.hpp:78-111).
  for (int t = 0; t < n; ++t) {
    auto& ti = TransformAccess::get(transforms[t]);
    gb300::DeviceGuard guard(ti.device_id());
    ti.forward_enqueue(inputs[t], outputs[t], scalings[t]);
  }
  for (int t = 0; t < n; ++t) TransformAccess::get(transforms[t]).synchronize();
}

template <typename TransformType, typename ValueType>
void multi_backward(int n, TransformType* transforms, const ValueType* const* inputs,
                    ValueType* const* outputs) {
  if (n < 0 || (n > 0 && (!transforms || !inputs || !outputs))) throw InvalidParameterError();
  for (int a = 0; a < n; ++a)
    for (int b = a + 1; b < n; ++b)
      if (TransformAccess::get(transforms[a]).shared_grid(TransformAccess::get(transforms[b])))
        throw InvalidParameterError();
  std::vector<decltype(TransformAccess::share(transforms[0]))> shared;
  for (int t = 0; t < n; ++t) shared.push_back(TransformAccess::share(transforms[t]));
  if (gb300::multi_backward_batched(shared, inputs, outputs)) return;
  for (int t = 0; t < n; ++t) {
    auto& ti = TransformAccess::get(transforms[t]);
    gb300::DeviceGuard guard(ti.device_id());
    ti.backward_enqueue(inputs[t], outputs[t]);
  }
  for (int t = 0; t < n; ++t) TransformAccess::get(transforms[t]).synchronize();
}

}  // namespace

// ================================================================================================
// The handle classes are written once as a macro over (Grid, Transform, value type) so the double
// and float APIs stay identical.
// ================================================================================================
#define SPFFT_GB300_DEFINE_HANDLES(GRID, TRANSFORM, T)                                            \
  GRID::GRID(int maxDimX, int maxDimY, int maxDimZ, int maxNumLocalZColumns,                    \
             SpfftProcessingUnitType processingUnit, int maxNumThreads)                          \
      : grid_(new GridInternal<T>(maxDimX, maxDimY, maxDimZ, maxNumLocalZColumns, processingUnit, \
                                  maxNumThreads)) {}                                             \
  GRID::GRID(const GRID& other) : grid_(new GridInternal<T>(*other.grid_)) {}                    \
  GRID& GRID::operator=(const GRID& other) {                                                    \
    if (this != &other) grid_.reset(new GridInternal<T>(*other.grid_));                         \
    return *this;                                                                                \
  }                                                                                              \
  TRANSFORM GRID::create_transform(SpfftProcessingUnitType processingUnit,                       \
                                   SpfftTransformType transformType, int dimX, int dimY,          \
                                   int dimZ, int localZLength, int numLocalElements,              \
                                   SpfftIndexFormatType indexFormat, const int* indices) const {  \
    return TRANSFORM(grid_, processingUnit, transformType, dimX, dimY, dimZ, localZLength,       \
                     numLocalElements, indexFormat, indices);                                     \
  }                                                                                              \
  int GRID::max_dim_x() const { return grid_->max_dim_x(); }                                     \
  int GRID::max_dim_y() const { return grid_->max_dim_y(); }                                     \
  int GRID::max_dim_z() const { return grid_->max_dim_z(); }                                     \
  int GRID::max_num_local_z_columns() const { return grid_->max_num_local_z_columns(); }         \
  int GRID::max_local_z_length() const { return grid_->max_local_z_length(); }                   \
  SpfftProcessingUnitType GRID::processing_unit() const { return grid_->processing_unit(); }     \
  int GRID::device_id() const { return grid_->device_id(); }                                     \
  int GRID::num_threads() const { return grid_->num_threads(); }                                 \
                                                                                                 \
  TRANSFORM::TRANSFORM(const std::shared_ptr<GridInternal<T>>& grid,                             \
                       SpfftProcessingUnitType processingUnit, SpfftTransformType transformType,  \
                       int dimX, int dimY, int dimZ, int localZLength, int numLocalElements,      \
                       SpfftIndexFormatType indexFormat, const int* indices) {                    \
    check_transform_args(dimX, dimY, dimZ, localZLength, numLocalElements, indices);             \
    const int device = grid && (grid->processing_unit() & SPFFT_PU_GPU) ? grid->device_id() : -1; \
    auto plan = make_plan(transformType, dimX, dimY, dimZ, numLocalElements, indexFormat,        \
                          indices, processingUnit, device);                                      \
    transform_ = std::make_shared<TransformInternal<T>>(processingUnit, grid, std::move(plan));  \
  }                                                                                              \
  TRANSFORM::TRANSFORM(int maxNumThreads, SpfftProcessingUnitType processingUnit,                \
                       SpfftTransformType transformType, int dimX, int dimY, int dimZ,            \
                       int numLocalElements, SpfftIndexFormatType indexFormat,                    \
                       const int* indices) {                                                      \
    check_transform_args(dimX, dimY, dimZ, 0, numLocalElements, indices);                        \
    auto plan = make_plan(transformType, dimX, dimY, dimZ, numLocalElements, indexFormat,        \
                          indices, processingUnit, -1);                                          \
    std::shared_ptr<GridInternal<T>> grid(new GridInternal<T>(                                   \
        dimX, dimY, dimZ, plan->num_sticks(), processingUnit, maxNumThreads));                   \
    transform_ = std::make_shared<TransformInternal<T>>(processingUnit, std::move(grid),         \
                                                        std::move(plan));                        \
  }                                                                                              \
  TRANSFORM::TRANSFORM(std::shared_ptr<TransformInternal<T>> transform)                          \
      : transform_(std::move(transform)) {}                                                      \
  TRANSFORM TRANSFORM::clone() const { return TRANSFORM(transform_->clone()); }                  \
  SpfftTransformType TRANSFORM::type() const { return transform_->type(); }                      \
  int TRANSFORM::dim_x() const { return transform_->dim_x(); }                                   \
  int TRANSFORM::dim_y() const { return transform_->dim_y(); }                                   \
  int TRANSFORM::dim_z() const { return transform_->dim_z(); }                                   \
  int TRANSFORM::local_z_length() const { return transform_->local_z_length(); }                 \
  int TRANSFORM::local_z_offset() const { return transform_->local_z_offset(); }                 \
  int TRANSFORM::local_slice_size() const {                                                      \
    return static_cast<int>(transform_->global_size());                                          \
  }                                                                                              \
  long long int TRANSFORM::global_size() const { return transform_->global_size(); }             \
  int TRANSFORM::num_local_elements() const { return transform_->num_local_elements(); }         \
  long long int TRANSFORM::num_global_elements() const {                                         \
    return transform_->num_global_elements();                                                    \
  }                                                                                              \
  SpfftProcessingUnitType TRANSFORM::processing_unit() const {                                   \
    return transform_->processing_unit();                                                        \
  }                                                                                              \
  int TRANSFORM::device_id() const { return transform_->device_id(); }                           \
  int TRANSFORM::num_threads() const { return transform_->num_threads(); }                       \
  SpfftExecType TRANSFORM::execution_mode() const { return transform_->execution_mode(); }       \
  void TRANSFORM::set_execution_mode(SpfftExecType mode) { transform_->set_execution_mode(mode); } \
  T* TRANSFORM::space_domain_data(SpfftProcessingUnitType dataLocation) {                        \
    return transform_->space_domain_data(dataLocation);                                          \
  }                                                                                              \
  void TRANSFORM::forward(SpfftProcessingUnitType inputLocation, T* output,                      \
                          SpfftScalingType scaling) {                                            \
    transform_->forward(inputLocation, output, scaling);                                         \
  }                                                                                              \
  void TRANSFORM::forward(const T* input, T* output, SpfftScalingType scaling) {                 \
    transform_->forward(input, output, scaling);                                                 \
  }                                                                                              \
  void TRANSFORM::backward(const T* input, SpfftProcessingUnitType outputLocation) {             \
    transform_->backward(input, outputLocation);                                                 \
  }                                                                                              \
  void TRANSFORM::backward(const T* input, T* output) { transform_->backward(input, output); }

SPFFT_GB300_DEFINE_HANDLES(Grid, Transform, double)
SPFFT_GB300_DEFINE_HANDLES(GridFloat, TransformFloat, float)
#undef SPFFT_GB300_DEFINE_HANDLES

// Multi-transform (multi_transform.cpp / multi_transform_float.cpp of the reference).
void multi_transform_forward(int n, Transform* transforms, const SpfftProcessingUnitType* inputLocations,
                             double* const* outputPointers, const SpfftScalingType* scalingTypes) {
  if (n > 0 && (!transforms || !inputLocations)) throw InvalidParameterError();
  std::vector<const double*> inputs(n > 0 ? n : 0);
  for (int t = 0; t < n; ++t) inputs[t] = transforms[t].space_domain_data(inputLocations[t]);
  multi_forward(n, transforms, inputs.data(), outputPointers, scalingTypes);
}
void multi_transform_forward(int n, Transform* transforms, const double* const* inputPointers,
                             double* const* outputPointers, const SpfftScalingType* scalingTypes) {
  multi_forward(n, transforms, inputPointers, outputPointers, scalingTypes);
}
void multi_transform_backward(int n, Transform* transforms, const double* const* inputPointers,
                              const SpfftProcessingUnitType* outputLocations) {
  if (n > 0 && (!transforms || !outputLocations)) throw InvalidParameterError();
  std::vector<double*> outputs(n > 0 ? n : 0);
  for (int t = 0; t < n; ++t) outputs[t] = transforms[t].space_domain_data(outputLocations[t]);
  multi_backward(n, transforms, inputPointers, outputs.data());
}
void multi_transform_backward(int n, Transform* transforms, const double* const* inputPointers,
                              double* const* outputPointers) {
  multi_backward(n, transforms, inputPointers, outputPointers);
}

void multi_transform_forward(int n, TransformFloat* transforms,
                             const SpfftProcessingUnitType* inputLocations,
                             float* const* outputPointers, const SpfftScalingType* scalingTypes) {
  if (n > 0 && (!transforms || !inputLocations)) throw InvalidParameterError();
  std::vector<const float*> inputs(n > 0 ? n : 0);
  for (int t = 0; t < n; ++t) inputs[t] = transforms[t].space_domain_data(inputLocations[t]);
  multi_forward(n, transforms, inputs.data(), outputPointers, scalingTypes);
}
void multi_transform_forward(int n, TransformFloat* transforms, const float* const* inputPointers,
                             float* const* outputPointers, const SpfftScalingType* scalingTypes) {
  multi_forward(n, transforms, inputPointers, outputPointers, scalingTypes);
}
void multi_transform_backward(int n, TransformFloat* transforms, const float* const* inputPointers,
                              const SpfftProcessingUnitType* outputLocations) {
  if (n > 0 && (!transforms || !outputLocations)) throw InvalidParameterError();
  std::vector<float*> outputs(n > 0 ? n : 0);
  for (int t = 0; t < n; ++t) outputs[t] = transforms[t].space_domain_data(outputLocations[t]);
  multi_backward(n, transforms, inputPointers, outputs.data());
}
void multi_transform_backward(int n, TransformFloat* transforms, const float* const* inputPointers,
                              float* const* outputPointers) {
  multi_backward(n, transforms, inputPointers, outputPointers);
}

}  // namespace spfft
