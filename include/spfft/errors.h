/* Error codes returned by every C function. Values are fixed by the reference ABI
 * (include/spfft/errors.h:33-126). */
#ifndef SPFFT_ERRORS_H
#define SPFFT_ERRORS_H

#include "spfft/config.h"

enum SpfftError {
  SPFFT_SUCCESS,                      /* no error */
  SPFFT_UNKNOWN_ERROR,                /* unexpected exception */
  SPFFT_INVALID_HANDLE_ERROR,         /* null grid / transform handle */
  SPFFT_OVERFLOW_ERROR,               /* integer overflow in a size computation */
  SPFFT_ALLOCATION_ERROR,             /* host allocation failed */
  SPFFT_INVALID_PARAMETER_ERROR,      /* invalid argument */
  SPFFT_DUPLICATE_INDICES_ERROR,      /* duplicate z-stick */
  SPFFT_INVALID_INDICES_ERROR,        /* index outside the allowed range */
  SPFFT_MPI_SUPPORT_ERROR,            /* distributed call in a build without MPI (always here) */
  SPFFT_MPI_ERROR,                    /* MPI failure (never raised here) */
  SPFFT_MPI_PARAMETER_MISMATCH_ERROR, /* ranks disagree (never raised here) */
  SPFFT_HOST_EXECUTION_ERROR,         /* host execution failed */
  SPFFT_FFTW_ERROR,                   /* FFT library / internal error */
  SPFFT_GPU_ERROR,                    /* generic CUDA error */
  SPFFT_GPU_PRECEDING_ERROR,          /* a CUDA error was pending before the call */
  SPFFT_GPU_SUPPORT_ERROR,            /* GPU requested but unavailable */
  SPFFT_GPU_ALLOCATION_ERROR,         /* device allocation failed */
  SPFFT_GPU_LAUNCH_ERROR,             /* kernel launch failed */
  SPFFT_GPU_NO_DEVICE_ERROR,          /* no CUDA device */
  SPFFT_GPU_INVALID_VALUE_ERROR,      /* invalid value passed to CUDA */
  SPFFT_GPU_INVALID_DEVICE_PTR_ERROR, /* invalid device pointer */
  SPFFT_GPU_COPY_ERROR,               /* host <-> device copy failed */
  SPFFT_GPU_FFT_ERROR                 /* FFT kernel failure (bad plan / device status word) */
};

#ifndef __cplusplus
typedef enum SpfftError SpfftError;
#endif
#endif
