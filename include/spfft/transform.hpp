/* C++ Transform handle (reference include/spfft/transform.hpp:56-315, local constructors only).
 * Copies share one plan; clone() creates an independent plan with its own grid memory. */
#ifndef SPFFT_TRANSFORM_HPP
#define SPFFT_TRANSFORM_HPP

#include <memory>
#include "spfft/config.h"
#include "spfft/types.h"

namespace spfft {

template <typename T>
class TransformInternal;
template <typename T>
class GridInternal;
class Grid;
struct TransformAccess;

class SPFFT_EXPORT Transform {
public:
  using ValueType = double;

  /* Transform with its own grid sized exactly for this problem (transform.hpp:76-95). */
  Transform(int maxNumThreads, SpfftProcessingUnitType processingUnit,
            SpfftTransformType transformType, int dimX, int dimY, int dimZ, int numLocalElements,
            SpfftIndexFormatType indexFormat, const int* indices);

  Transform(const Transform&) = default;
  Transform(Transform&&) = default;
  Transform& operator=(const Transform&) = default;
  Transform& operator=(Transform&&) = default;

  Transform clone() const;

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

  double* space_domain_data(SpfftProcessingUnitType dataLocation);

  void forward(SpfftProcessingUnitType inputLocation, double* output,
               SpfftScalingType scaling = SPFFT_NO_SCALING);
  void forward(const double* input, double* output, SpfftScalingType scaling = SPFFT_NO_SCALING);
  void backward(const double* input, SpfftProcessingUnitType outputLocation);
  void backward(const double* input, double* output);

private:
  friend Grid;
  friend struct TransformAccess;
  SPFFT_NO_EXPORT Transform(const std::shared_ptr<GridInternal<double>>& grid,
                            SpfftProcessingUnitType processingUnit,
                            SpfftTransformType transformType, int dimX, int dimY, int dimZ,
                            int localZLength, int numLocalElements,
                            SpfftIndexFormatType indexFormat, const int* indices);
  SPFFT_NO_EXPORT explicit Transform(std::shared_ptr<TransformInternal<double>> transform);

  std::shared_ptr<TransformInternal<double>> transform_;
};

}  // namespace spfft
#endif
