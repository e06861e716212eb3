// Allocation-free backward transform: the same kernels as spfft_transform_backward_ptr, with the
// transform's intermediates (the z-stick buffer and the compact plane buffer) placed in one
// file-scope static device array instead of the grid's cudaMalloc'ed scratch.
//
// Who needs this: callers that cannot let a library allocate device memory on their behalf. An
// application whose device memory is owned by its own pool or arena allocator (which reserves most
// of the GPU up front and budgets every byte) would see a library cudaMalloc fail or break its
// budget; a latency-critical loop cannot afford cudaMalloc/cudaFree, which may synchronise the
// device and take unpredictable time; a plug-in may run inside a host application that forbids
// its plug-ins to allocate. The transform handle must already exist (its index tables are
// created with it, where allocation is allowed); this call itself allocates nothing.
#include <cuda.h>
#include <cudaTypedefs.h>
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
struct ScratchSlot {
  void* address = nullptr;
  unsigned long long context = 0;  // context the address belongs to (0: unknown)
};
ScratchSlot g_scratch[kMaxDevices];

// Unique id of the calling thread's current CUDA context (0 if it cannot be found), through the
// driver entry points the runtime hands out, so the library needs no link to the driver library.
unsigned long long current_context_id() {
  static std::once_flag once;
  static PFN_cuCtxGetCurrent_v4000 get_current = nullptr;
  static PFN_cuCtxGetId_v12000 get_id = nullptr;
  std::call_once(once, [] {
    cudaDriverEntryPointQueryResult q;
    void* fn = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(fn);
    fn = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<PFN_cuCtxGetId_v12000>(fn);
    (void)cudaGetLastError();
  });
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx) return 0;
  if (get_id(ctx, &id) != CUDA_SUCCESS) return 0;
  return id;
}

// Device address of g_static_scratch on `device`, which must be current. In host code the name
// g_static_scratch is only a host-side stand-in, so the address is looked up with
// cudaGetSymbolAddress once per device, and again only if the device's context has changed
// since (after a cudaDeviceReset the old address is gone).
void* scratch_address(int device) {
  if (device < 0 || device >= kMaxDevices) throw spfft::InvalidParameterError();
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  ScratchSlot& slot = g_scratch[device];
  const unsigned long long ctx = current_context_id();
  if (!slot.address || ctx == 0 || ctx != slot.context) {
    void* ptr = nullptr;
    const cudaError_t st = cudaGetSymbolAddress(&ptr, g_static_scratch);
    if (st != cudaSuccess || !ptr) {
      (void)cudaGetLastError();
      spfft::gb300::check_cuda(st == cudaSuccess ? cudaErrorInvalidSymbol : st);
    }
    slot.address = ptr;
    slot.context = ctx ? ctx : current_context_id();
  }
  return slot.address;
}

// True when p is device memory of `device` (not pageable or pinned host memory, not managed
// memory, not another GPU's memory). cudaPointerGetAttributes allocates nothing.
bool device_memory_of(const void* p, int device) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    (void)cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice && a.device == device;
}

}  // namespace

extern "C" SpfftError spfft_gb300_transform_backward_noalloc(SpfftTransform transform,
                                                             const double* values, double* space,
                                                             void* stream) {
  if (!transform) return SPFFT_INVALID_HANDLE_ERROR;
  try {
    auto& t = spfft::TransformAccess::get(*reinterpret_cast<spfft::Transform*>(transform));
    spfft::gb300::DeviceGuard guard(t.device_id());
    // A pending CUDA error from earlier work aborts before anything runs, as in the regular
    // entry points.
    if (cudaGetLastError() != cudaSuccess) return SPFFT_GPU_PRECEDING_ERROR;
    // Both buffers must be device memory of the transform's GPU: there is no staging buffer to
    // copy host memory through, and the kernels must never be handed a host address.
    if (!space || !device_memory_of(space, t.device_id())) return SPFFT_INVALID_PARAMETER_ERROR;
    if (t.num_local_elements() > 0 && (!values || !device_memory_of(values, t.device_id()))) {
      return SPFFT_INVALID_PARAMETER_ERROR;
    }
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
