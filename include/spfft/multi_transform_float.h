/* Execute several independent transforms together (reference include/spfft/multi_transform_float.h:
 * 49-96). Transforms must not share a grid. All GPU work is enqueued before any call waits. */
#ifndef SPFFT_MULTI_TRANSFORM_FLOAT_H
#define SPFFT_MULTI_TRANSFORM_FLOAT_H

#include "spfft/config.h"
#include "spfft/transform_float.h"
#include "spfft/types.h"

#ifdef __cplusplus
extern "C" {
#endif

SPFFT_EXPORT SpfftError spfft_float_multi_transform_forward(int numTransforms, SpfftFloatTransform* transforms,
                                                      const SpfftProcessingUnitType* inputLocations,
                                                      float* const* outputPointers,
                                                      const SpfftScalingType* scalingTypes);
SPFFT_EXPORT SpfftError spfft_float_multi_transform_forward_ptr(int numTransforms,
                                                          SpfftFloatTransform* transforms,
                                                          const float* const* inputPointers,
                                                          float* const* outputPointers,
                                                          const SpfftScalingType* scalingTypes);
SPFFT_EXPORT SpfftError spfft_float_multi_transform_backward(
    int numTransforms, SpfftFloatTransform* transforms, const float* const* inputPointers,
    const SpfftProcessingUnitType* outputLocations);
SPFFT_EXPORT SpfftError spfft_float_multi_transform_backward_ptr(int numTransforms,
                                                           SpfftFloatTransform* transforms,
                                                           const float* const* inputPointers,
                                                           float* const* outputPointers);

#ifdef __cplusplus
}
#endif
#endif
