/* Enumerations of the SpFFT interface. Values are fixed by the ABI of the reference
 * (include/spfft/types.h:33-117) so that binaries built against it keep their meaning. */
#ifndef SPFFT_TYPES_H
#define SPFFT_TYPES_H

#include "spfft/config.h"

/* MPI exchange flavours. Accepted for source compatibility only; this library is single-GPU. */
enum SpfftExchangeType {
  SPFFT_EXCH_DEFAULT,
  SPFFT_EXCH_BUFFERED,
  SPFFT_EXCH_BUFFERED_FLOAT,
  SPFFT_EXCH_COMPACT_BUFFERED,
  SPFFT_EXCH_COMPACT_BUFFERED_FLOAT,
  SPFFT_EXCH_UNBUFFERED
};

/* Where a transform executes or where a buffer lives. Used as a bit mask by grid creation. */
enum SpfftProcessingUnitType { SPFFT_PU_HOST = 1, SPFFT_PU_GPU = 2 };

/* Sparse index format: interleaved (x, y, z) triplets. */
enum SpfftIndexFormatType { SPFFT_INDEX_TRIPLETS };

/* Complex-to-complex, or real space domain with hermitian frequency data. */
enum SpfftTransformType { SPFFT_TRANS_C2C, SPFFT_TRANS_R2C };

/* Optional 1/(Nx*Ny*Nz) scaling of the forward (space -> frequency) transform. */
enum SpfftScalingType { SPFFT_NO_SCALING, SPFFT_FULL_SCALING };

/* Synchronous: calls return after the GPU finished. Asynchronous: the default stream (or the
 * stream attached with spfft_gb300_transform_set_stream) is made to wait for the work instead. */
enum SpfftExecType { SPFFT_EXEC_SYNCHRONOUS, SPFFT_EXEC_ASYNCHRONOUS };

#ifndef __cplusplus
typedef enum SpfftExchangeType SpfftExchangeType;
typedef enum SpfftProcessingUnitType SpfftProcessingUnitType;
typedef enum SpfftTransformType SpfftTransformType;
typedef enum SpfftIndexFormatType SpfftIndexFormatType;
typedef enum SpfftScalingType SpfftScalingType;
typedef enum SpfftExecType SpfftExecType;
#endif
#endif
