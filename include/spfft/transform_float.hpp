/* C++ single-precision Transform handle (reference include/spfft/transform_float.hpp:56-318, local constructors only).
 * Copies share one plan; clone() creates an independent plan with its own grid memory. */
#ifndef SPFFT_TRANSFORM_FLOAT_HPP
#define SPFFT_TRANSFORM_FLOAT_HPP

#include <memory>
#include "spfft/config.h"
#include "spfft/types.h"

namespace spfft {

template <typename T>
class TransformInternal;
template <typename T>
class GridInternal;
class GridFloat;
struct TransformAccess;

class SPFFT_EXPORT TransformFloat {
public:
  using ValueType = float;

  /* Transform with its own grid sized exactly for this problem (transform.hpp:76-95). */
  TransformFloat(int maxNumThreads, SpfftProcessingUnitType processingUnit,
            SpfftTransformType transformType, int dimX, int dimY, int dimZ, int numLocalElements,
            SpfftIndexFormatType indexFormat, const int* indices);

  TransformFloat(const TransformFloat&) = default;
  TransformFloat(TransformFloat&&) = default;
  TransformFloat& operator=(const TransformFloat&) = default;
  TransformFloat& operator=(TransformFloat&&) = default;

  TransformFloat clone() const;

  SpfftTransformType type() const;
  int dim_x() const;
  int dim_y() const;
  int dim_z() const;
  int local_z_length() const;
  int local_z_offset() const;
  int local_slice_size() const;
  long long int global_size() const;
  int num_local_elements() const;
  long long int num_global_elements() const;
  SpfftProcessingUnitType processing_unit() const;
  int device_id() const;
  int num_threads() const;
  SpfftExecType execution_mode() const;
  void set_execution_mode(SpfftExecType mode);

  float* space_domain_data(SpfftProcessingUnitType dataLocation);

  void forward(SpfftProcessingUnitType inputLocation, float* output,
               SpfftScalingType scaling = SPFFT_NO_SCALING);
  void forward(const float* input, float* output, SpfftScalingType scaling = SPFFT_NO_SCALING);
  void backward(const float* input, SpfftProcessingUnitType outputLocation);
  void backward(const float* input, float* output);

private:
  friend GridFloat;
  friend struct TransformAccess;
  SPFFT_NO_EXPORT TransformFloat(const std::shared_ptr<GridInternal<float>>& grid,
                            SpfftProcessingUnitType processingUnit,
                            SpfftTransformType transformType, int dimX, int dimY, int dimZ,
                            int localZLength, int numLocalElements,
                            SpfftIndexFormatType indexFormat, const int* indices);
  SPFFT_NO_EXPORT explicit TransformFloat(std::shared_ptr<TransformInternal<float>> transform);

  std::shared_ptr<TransformInternal<float>> transform_;
};

}  // namespace spfft
#endif
