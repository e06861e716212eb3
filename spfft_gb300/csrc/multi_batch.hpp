// The reference's multi-transform calls (src/spfft/multi_transform_internal.hpp:63-174) on the
// batched kernels: when every transform of a call runs on the same GPU through the library's own
// streams and every buffer is device-addressable, the call becomes one batched, graph-replayed
// execution instead of one kernel sequence per transform.
#pragma once

#include <memory>
#include <vector>

#include "internal.hpp"
#include "spfft/types.h"

namespace spfft {
namespace gb300 {

// Backward of transform t: values[t] -> spaces[t]. Returns false, having done nothing, when the
// call does not qualify (fewer than two transforms, a user stream, several devices, a buffer the
// kernels cannot address, a misaligned buffer); the caller then runs the transforms one by one.
template <typename T>
bool multi_backward_batched(const std::vector<std::shared_ptr<TransformInternal<T>>>& transforms,
                            const T* const* values, T* const* spaces);
// Forward of transform t: spaces[t] -> values[t], with one scaling for all (mixed scalings do not
// qualify).
template <typename T>
bool multi_forward_batched(const std::vector<std::shared_ptr<TransformInternal<T>>>& transforms,
                           const T* const* spaces, T* const* values, const SpfftScalingType* scalings);

// Number of multi-transform calls so far (process-wide) that ran batched.
long long multi_batched_calls();

}  // namespace gb300
}  // namespace spfft
