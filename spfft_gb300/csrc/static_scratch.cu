// Allocation-free backward transform: the same kernels as spfft_transform_backward_ptr, with the
// transform's intermediates (the z-stick buffer and the compact plane buffer) placed in one
// file-scope static device array instead of the grid's cudaMalloc'ed scratch.
//
// Who needs this: callers that are not allowed to make the library allocate device memory on
// their behalf -- for example an application whose device memory is owned and budgeted by its own
// pool allocator, or code that runs inside CUDA stream capture, where cudaMalloc/cudaFree are not
// permitted. The transform handle must already exist (its index tables are created with it, where
// allocation is allowed); this call itself allocates nothing.
#include <cuda_runtime.h>

#include <mutex>

#include "access.hpp"
#include "internal.hpp"
#include "spfft/spfft_gb300.h"

namespace {

// Maximum intermediate size served by the static array: 64 MiB per GPU. The array is part of this
// library's device image, so every GPU that loads the library holds these 64 MiB until the process
// exits.
constexpr size_t kStaticScratchBytes = size_t(64) << 20;
__device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
void* g_scratch_address[kMaxDevices] = {};

// Device address of g_static_scratch on `device`, which must be current. In host code the name
// g_static_scratch is only a host-side stand-in, so the address is looked up once per device.
void* scratch_address(int device) {
  if (device < 0 || device >= kMaxDevices) throw spfft::InvalidParameterError();
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_address[device]) {
    void* ptr = nullptr;
    const cudaError_t st = cudaGetSymbolAddress(&ptr, g_static_scratch);
    if (st != cudaSuccess || !ptr) {
      (void)cudaGetLastError();
      spfft::gb300::check_cuda(st == cudaSuccess ? cudaErrorInvalidSymbol : st);
    }
    g_scratch_address[device] = ptr;
  }
  return g_scratch_address[device];
}

}  // namespace

extern "C" SpfftError spfft_gb300_transform_backward_noalloc(SpfftTransform transform,
                                                             const double* values, double* space,
                                                             void* stream) {
  if (!transform) return SPFFT_INVALID_HANDLE_ERROR;
  try {
    auto& t = spfft::TransformAccess::get(*reinterpret_cast<spfft::Transform*>(transform));
    spfft::gb300::DeviceGuard guard(t.device_id());
    const auto& plan = t.gpu_plan();
    // Sticks and planes only; the host-staging part of the regular scratch is not used here.
    if (plan.scratch_layout().valuesOffset > kStaticScratchBytes) {
      return SPFFT_INVALID_PARAMETER_ERROR;
    }
    // Both intermediates are fully written by one kernel before the next one reads them, so
    // nothing in the shared array has to start at zero.
    plan.backward(values, space, scratch_address(t.device_id()), static_cast<cudaStream_t>(stream));
  } catch (const spfft::GenericError& e) {
    return e.error_code();
  } catch (...) {
    return SPFFT_UNKNOWN_ERROR;
  }
  return SPFFT_SUCCESS;
}
