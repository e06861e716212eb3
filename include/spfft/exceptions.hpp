/* C++ exceptions of the SpFFT interface. Each carries the C error code it maps to; the class names
 * and codes follow the reference (include/spfft/exceptions.hpp:40-297), including InternalError
 * reporting SPFFT_FFTW_ERROR. */
#ifndef SPFFT_EXCEPTIONS_H
#define SPFFT_EXCEPTIONS_H

#include <stdexcept>
#include "spfft/config.h"
#include "spfft/errors.h"

namespace spfft {

class SPFFT_EXPORT GenericError : public std::exception {
public:
  const char* what() const noexcept override { return "SpFFT: Generic error"; }
  virtual SpfftError error_code() const noexcept { return SPFFT_UNKNOWN_ERROR; }
};

#define SPFFT_GB300_DEFINE_ERROR(NAME, BASE, MESSAGE, CODE)                      \
  class SPFFT_EXPORT NAME : public BASE {                                        \
  public:                                                                        \
    const char* what() const noexcept override { return MESSAGE; }              \
    SpfftError error_code() const noexcept override { return CODE; }            \
  };

SPFFT_GB300_DEFINE_ERROR(OverflowError, GenericError, "SpFFT: Overflow error", SPFFT_OVERFLOW_ERROR)
SPFFT_GB300_DEFINE_ERROR(HostAllocationError, GenericError, "SpFFT: Host allocation error",
                         SPFFT_ALLOCATION_ERROR)
SPFFT_GB300_DEFINE_ERROR(InvalidParameterError, GenericError, "SpFFT: Invalid parameter error",
                         SPFFT_INVALID_PARAMETER_ERROR)
SPFFT_GB300_DEFINE_ERROR(DuplicateIndicesError, GenericError, "SpFFT: Duplicate indices error",
                         SPFFT_DUPLICATE_INDICES_ERROR)
SPFFT_GB300_DEFINE_ERROR(InvalidIndicesError, GenericError, "SpFFT: Invalid indices error",
                         SPFFT_INVALID_INDICES_ERROR)
SPFFT_GB300_DEFINE_ERROR(MPISupportError, GenericError, "SpFFT: Not compiled with MPI support",
                         SPFFT_MPI_SUPPORT_ERROR)
SPFFT_GB300_DEFINE_ERROR(MPIError, GenericError, "SpFFT: MPI error", SPFFT_MPI_ERROR)
SPFFT_GB300_DEFINE_ERROR(MPIParameterMismatchError, GenericError,
                         "SpFFT: Mismatched parameters between MPI ranks",
                         SPFFT_MPI_PARAMETER_MISMATCH_ERROR)
SPFFT_GB300_DEFINE_ERROR(HostExecutionError, GenericError, "SpFFT: Host execution error",
                         SPFFT_HOST_EXECUTION_ERROR)
SPFFT_GB300_DEFINE_ERROR(FFTWError, GenericError, "SpFFT: FFTW error", SPFFT_FFTW_ERROR)
SPFFT_GB300_DEFINE_ERROR(InternalError, GenericError, "SpFFT: Internal error", SPFFT_FFTW_ERROR)
SPFFT_GB300_DEFINE_ERROR(GPUError, GenericError, "SpFFT: GPU error", SPFFT_GPU_ERROR)
SPFFT_GB300_DEFINE_ERROR(GPUSupportError, GPUError, "SpFFT: Not compiled with GPU support",
                         SPFFT_GPU_SUPPORT_ERROR)
SPFFT_GB300_DEFINE_ERROR(GPUPrecedingError, GPUError,
                         "SpFFT: Detected error from preceding GPU calls.",
                         SPFFT_GPU_PRECEDING_ERROR)
SPFFT_GB300_DEFINE_ERROR(GPUAllocationError, GPUError, "SpFFT: GPU allocation error",
                         SPFFT_GPU_ALLOCATION_ERROR)
SPFFT_GB300_DEFINE_ERROR(GPULaunchError, GPUError, "SpFFT: GPU launch error",
                         SPFFT_GPU_LAUNCH_ERROR)
SPFFT_GB300_DEFINE_ERROR(GPUNoDeviceError, GPUError, "SpFFT: no GPU available",
                         SPFFT_GPU_NO_DEVICE_ERROR)
SPFFT_GB300_DEFINE_ERROR(GPUInvalidValueError, GPUError, "SpFFT: GPU call with invalid value",
                         SPFFT_GPU_INVALID_VALUE_ERROR)
SPFFT_GB300_DEFINE_ERROR(GPUInvalidDevicePointerError, GPUError, "SpFFT: Invalid GPU pointer",
                         SPFFT_GPU_INVALID_DEVICE_PTR_ERROR)
SPFFT_GB300_DEFINE_ERROR(GPUCopyError, GPUError, "SpFFT: GPU Memory copy error",
                         SPFFT_GPU_COPY_ERROR)
SPFFT_GB300_DEFINE_ERROR(GPUFFTError, GPUError, "SpFFT: GPU FFT error", SPFFT_GPU_FFT_ERROR)

#undef SPFFT_GB300_DEFINE_ERROR

}  // namespace spfft
#endif
