/* Execute several independent transforms together (reference include/spfft/multi_transform.h:
 * 49-96). Transforms must not share a grid. All GPU work is enqueued before any call waits. */
#ifndef SPFFT_MULTI_TRANSFORM_H
#define SPFFT_MULTI_TRANSFORM_H

#include "spfft/config.h"
#include "spfft/transform.h"
#include "spfft/types.h"

#ifdef __cplusplus
extern "C" {
#endif

SPFFT_EXPORT SpfftError spfft_multi_transform_forward(int numTransforms, SpfftTransform* transforms,
                                                      const SpfftProcessingUnitType* inputLocations,
                                                      double* const* outputPointers,
                                                      const SpfftScalingType* scalingTypes);
SPFFT_EXPORT SpfftError spfft_multi_transform_forward_ptr(int numTransforms,
                                                          SpfftTransform* transforms,
                                                          const double* const* inputPointers,
                                                          double* const* outputPointers,
                                                          const SpfftScalingType* scalingTypes);
SPFFT_EXPORT SpfftError spfft_multi_transform_backward(
    int numTransforms, SpfftTransform* transforms, const double* const* inputPointers,
    const SpfftProcessingUnitType* outputLocations);
SPFFT_EXPORT SpfftError spfft_multi_transform_backward_ptr(int numTransforms,
                                                           SpfftTransform* transforms,
                                                           const double* const* inputPointers,
                                                           double* const* outputPointers);

#ifdef __cplusplus
}
#endif
#endif
