/* Execute several independent transforms together (reference include/spfft/multi_transform.hpp:
 * 40-95). Transforms must not share a grid. */
#ifndef SPFFT_MULTI_TRANSFORM_HPP
#define SPFFT_MULTI_TRANSFORM_HPP

#include "spfft/config.h"
#include "spfft/transform.hpp"
#include "spfft/types.h"

namespace spfft {

SPFFT_EXPORT void multi_transform_forward(int numTransforms, Transform* transforms,
                                          const SpfftProcessingUnitType* inputLocations,
                                          double* const* outputPointers,
                                          const SpfftScalingType* scalingTypes);
SPFFT_EXPORT void multi_transform_forward(int numTransforms, Transform* transforms,
                                          const double* const* inputPointers,
                                          double* const* outputPointers,
                                          const SpfftScalingType* scalingTypes);
SPFFT_EXPORT void multi_transform_backward(int numTransforms, Transform* transforms,
                                           const double* const* inputPointers,
                                           const SpfftProcessingUnitType* outputLocations);
SPFFT_EXPORT void multi_transform_backward(int numTransforms, Transform* transforms,
                                           const double* const* inputPointers,
                                           double* const* outputPointers);

}  // namespace spfft
#endif
