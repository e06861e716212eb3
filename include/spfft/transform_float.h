/* C interface of the single-precision Transform: a sparse 3D FFT plan executed on one GPU.
 * Mirrors include/spfft/transform_float.h:70-340 of the reference, without the MPI entry points.
 *
 * Layouts: frequency values are interleaved complex (re, im), one per index triplet, in the order
 * the triplets were given. The space domain is (z * dimY + y) * dimX + x, interleaved complex for
 * C2C and real for R2C. backward() is the unnormalised e^{+2 pi i k n / N} transform, forward() the
 * e^{-2 pi i k n / N} one, optionally scaled by 1 / (dimX * dimY * dimZ). */
#ifndef SPFFT_TRANSFORM_FLOAT_H
#define SPFFT_TRANSFORM_FLOAT_H

#include "spfft/config.h"
#include "spfft/errors.h"
#include "spfft/grid_float.h"
#include "spfft/types.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef void* SpfftFloatTransform;

/* Create a transform that executes in the memory of `grid` (transform.h:68-90). localZLength must
 * equal dimZ (local grids only). indices holds numLocalElements (x, y, z) triplets. */
SPFFT_EXPORT SpfftError spfft_float_transform_create(SpfftFloatTransform* transform, SpfftFloatGrid grid,
                                               SpfftProcessingUnitType processingUnit,
                                               SpfftTransformType transformType, int dimX, int dimY,
                                               int dimZ, int localZLength, int numLocalElements,
                                               SpfftIndexFormatType indexFormat,
                                               const int* indices);

/* Create a transform with its own, exactly sized grid (transform.h:92-113). */
SPFFT_EXPORT SpfftError spfft_float_transform_create_independent(
    SpfftFloatTransform* transform, int maxNumThreads, SpfftProcessingUnitType processingUnit,
    SpfftTransformType transformType, int dimX, int dimY, int dimZ, int numLocalElements,
    SpfftIndexFormatType indexFormat, const int* indices);

SPFFT_EXPORT SpfftError spfft_float_transform_destroy(SpfftFloatTransform transform);

/* New transform with the same parameters and a new, independent grid (transform.h:151-158). */
SPFFT_EXPORT SpfftError spfft_float_transform_clone(SpfftFloatTransform transform,
                                              SpfftFloatTransform* newTransform);

/* Space -> frequency. Input is the internal space buffer at inputLocation; output may be a host or
 * device pointer (transform.h:160-175). */
SPFFT_EXPORT SpfftError spfft_float_transform_forward(SpfftFloatTransform transform,
                                                SpfftProcessingUnitType inputLocation,
                                                float* output, SpfftScalingType scaling);
/* Space -> frequency with an external space buffer (host or device; may equal output). */
SPFFT_EXPORT SpfftError spfft_float_transform_forward_ptr(SpfftFloatTransform transform, const float* input,
                                                    float* output, SpfftScalingType scaling);

/* Frequency -> space into the internal space buffer at outputLocation (transform.h:192-205). */
SPFFT_EXPORT SpfftError spfft_float_transform_backward(SpfftFloatTransform transform, const float* input,
                                                 SpfftProcessingUnitType outputLocation);
/* Frequency -> space into an external buffer (host or device; may equal input). */
SPFFT_EXPORT SpfftError spfft_float_transform_backward_ptr(SpfftFloatTransform transform, const float* input,
                                                     float* output);

/* Pointer to the internal space-domain buffer on the host (pinned) or on the GPU. */
SPFFT_EXPORT SpfftError spfft_float_transform_get_space_domain(SpfftFloatTransform transform,
                                                         SpfftProcessingUnitType dataLocation,
                                                         float** data);

SPFFT_EXPORT SpfftError spfft_float_transform_dim_x(SpfftFloatTransform transform, int* dimX);
SPFFT_EXPORT SpfftError spfft_float_transform_dim_y(SpfftFloatTransform transform, int* dimY);
SPFFT_EXPORT SpfftError spfft_float_transform_dim_z(SpfftFloatTransform transform, int* dimZ);
SPFFT_EXPORT SpfftError spfft_float_transform_local_z_length(SpfftFloatTransform transform, int* localZLength);
SPFFT_EXPORT SpfftError spfft_float_transform_local_slice_size(SpfftFloatTransform transform, int* size);
SPFFT_EXPORT SpfftError spfft_float_transform_local_z_offset(SpfftFloatTransform transform, int* offset);
SPFFT_EXPORT SpfftError spfft_float_transform_global_size(SpfftFloatTransform transform,
                                                    long long int* globalSize);
/* Number of frequency elements of this transform. (The reference C function returns the local z
 * length here, transform.cpp:433-445; this library returns the element count, like the C++
 * num_local_elements().) */
SPFFT_EXPORT SpfftError spfft_float_transform_num_local_elements(SpfftFloatTransform transform,
                                                           int* numLocalElements);
SPFFT_EXPORT SpfftError spfft_float_transform_num_global_elements(SpfftFloatTransform transform,
                                                            long long int* numGlobalElements);
SPFFT_EXPORT SpfftError spfft_float_transform_device_id(SpfftFloatTransform transform, int* deviceId);
SPFFT_EXPORT SpfftError spfft_float_transform_num_threads(SpfftFloatTransform transform, int* numThreads);
SPFFT_EXPORT SpfftError spfft_float_transform_execution_mode(SpfftFloatTransform transform,
                                                       SpfftExecType* mode);
SPFFT_EXPORT SpfftError spfft_float_transform_set_execution_mode(SpfftFloatTransform transform,
                                                           SpfftExecType mode);

#ifdef __cplusplus
}
#endif
#endif
