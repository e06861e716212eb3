/* C interface of the double-precision Grid: a reusable pool of device and pinned host memory that
 * transforms up to the given maximum size execute in. Mirrors include/spfft/grid.h:61-175 of the
 * reference; the distributed (MPI) constructor and communicator getter are not provided. */
#ifndef SPFFT_GRID_H
#define SPFFT_GRID_H

#include "spfft/config.h"
#include "spfft/errors.h"
#include "spfft/types.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef void* SpfftGrid;

/* Create a grid for transforms with dims up to maxDimX x maxDimY x maxDimZ and up to
 * maxNumLocalZColumns z-sticks. processingUnit is a mask of SPFFT_PU_HOST / SPFFT_PU_GPU; memory is
 * bound to the CUDA device that is current at this call. (reference grid.h:61-71) */
SPFFT_EXPORT SpfftError spfft_grid_create(SpfftGrid* grid, int maxDimX, int maxDimY, int maxDimZ,
                                          int maxNumLocalZColumns,
                                          SpfftProcessingUnitType processingUnit,
                                          int maxNumThreads);

/* Release the handle. Transforms created from it keep the memory alive. (grid.h:102) */
SPFFT_EXPORT SpfftError spfft_grid_destroy(SpfftGrid grid);

SPFFT_EXPORT SpfftError spfft_grid_max_dim_x(SpfftGrid grid, int* dimX);
SPFFT_EXPORT SpfftError spfft_grid_max_dim_y(SpfftGrid grid, int* dimY);
SPFFT_EXPORT SpfftError spfft_grid_max_dim_z(SpfftGrid grid, int* dimZ);
SPFFT_EXPORT SpfftError spfft_grid_max_num_local_z_columns(SpfftGrid grid,
                                                           int* maxNumLocalZColumns);
SPFFT_EXPORT SpfftError spfft_grid_max_local_z_length(SpfftGrid grid, int* maxLocalZLength);
SPFFT_EXPORT SpfftError spfft_grid_processing_unit(SpfftGrid grid,
                                                   SpfftProcessingUnitType* processingUnit);
SPFFT_EXPORT SpfftError spfft_grid_device_id(SpfftGrid grid, int* deviceId);
SPFFT_EXPORT SpfftError spfft_grid_num_threads(SpfftGrid grid, int* numThreads);

#ifdef __cplusplus
}
#endif
#endif
