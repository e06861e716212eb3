/* C interface of the single-precision Grid: a reusable pool of device and pinned host memory that
 * transforms up to the given maximum size execute in. Mirrors include/spfft/grid_float.h:61-180 of the
 * reference; the distributed (MPI) constructor and communicator getter are not provided. */
#ifndef SPFFT_GRID_FLOAT_H
#define SPFFT_GRID_FLOAT_H

#include "spfft/config.h"
#include "spfft/errors.h"
#include "spfft/types.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef void* SpfftFloatGrid;

/* Create a grid for transforms with dims up to maxDimX x maxDimY x maxDimZ and up to
 * maxNumLocalZColumns z-sticks. processingUnit is a mask of SPFFT_PU_HOST / SPFFT_PU_GPU; memory is
 * bound to the CUDA device that is current at this call. (reference grid.h:61-71) */
SPFFT_EXPORT SpfftError spfft_float_grid_create(SpfftFloatGrid* grid, int maxDimX, int maxDimY, int maxDimZ,
                                          int maxNumLocalZColumns,
                                          SpfftProcessingUnitType processingUnit,
                                          int maxNumThreads);

/* Release the handle. Transforms created from it keep the memory alive. (grid.h:102) */
SPFFT_EXPORT SpfftError spfft_float_grid_destroy(SpfftFloatGrid grid);

SPFFT_EXPORT SpfftError spfft_float_grid_max_dim_x(SpfftFloatGrid grid, int* dimX);
SPFFT_EXPORT SpfftError spfft_float_grid_max_dim_y(SpfftFloatGrid grid, int* dimY);
SPFFT_EXPORT SpfftError spfft_float_grid_max_dim_z(SpfftFloatGrid grid, int* dimZ);
SPFFT_EXPORT SpfftError spfft_float_grid_max_num_local_z_columns(SpfftFloatGrid grid,
                                                           int* maxNumLocalZColumns);
SPFFT_EXPORT SpfftError spfft_float_grid_max_local_z_length(SpfftFloatGrid grid, int* maxLocalZLength);
SPFFT_EXPORT SpfftError spfft_float_grid_processing_unit(SpfftFloatGrid grid,
                                                   SpfftProcessingUnitType* processingUnit);
SPFFT_EXPORT SpfftError spfft_float_grid_device_id(SpfftFloatGrid grid, int* deviceId);
SPFFT_EXPORT SpfftError spfft_float_grid_num_threads(SpfftFloatGrid grid, int* numThreads);

#ifdef __cplusplus
}
#endif
#endif
