// Device index planner: the planner of planner.hpp run as CUDA kernels, for large index sets.
//
// It computes the same plan as make_index_plan() (the rules of the reference's
// convert_index_triplets, src/compression/indices.hpp:120-186, and of the local Parameters
// constructor, src/parameters/parameters.cpp:143-180) with presence flags and prefix sums instead
// of an ordered map: stick index = number of occupied xy keys below the stick's key, entry index =
// number of occupied stick positions below the value's position. The derived tables stay on the
// device, where the transform's kernels read them.
#pragma once

#include <memory>

#include "planner.hpp"
#include "runtime.hpp"

namespace spfft {
namespace gb300 {

// The derived index tables of an IndexPlan in the memory of one device, laid out back to back in
// one allocation (each table 256-byte aligned).
struct DeviceIndexTables {
  int device = 0;
  DeviceBuffer buffer;
  const int* stickColumn = nullptr;       // [numSticks]
  const int* stickY = nullptr;            // [numSticks]
  const int* stickPlanePos = nullptr;     // [numSticks] stickY * numColumns + stickColumn
  const int* columnX = nullptr;           // [numColumns]
  const int* columnStickStart = nullptr;  // [numColumns + 1]
  const int* entryPos = nullptr;          // [numValues]
  const int* entryUser = nullptr;         // [numValues]
  const int* stickEntryStart = nullptr;   // [numSticks + 1]
  const unsigned char* hermitianWeight = nullptr;  // [numValues], R2C only (else null)
};

// Plans on the current device. Throws what make_index_plan() throws for the same invalid input.
// Returns false, leaving `out` untouched, where the device planner does not apply and the host
// planner must run instead: more than 2^26 xy keys or 2^27 stick positions, or triplets that
// occur more than once (the host planner keeps their user order).
bool make_index_plan_device(SpfftTransformType type, int dimX, int dimY, int dimZ, int numValues,
                            const int* triplets, IndexPlan* out);

// A copy of `p` whose host tables are filled (valueIndices and stickKeys included), downloaded
// from its device tables when it was planned on the device; `p` itself otherwise.
IndexPlan download_index_plan(const IndexPlan& p);

// Planner choice of transform creation: the device planner when `allowDevice` (a GPU transform),
// a device is present, the set has at least kDevicePlanMinValues values and SPFFT_GB300_PLANNER
// is not "host" ("device" lowers the threshold to 1); otherwise, or where the device planner
// declines or fails with a GPU error, the host planner.
constexpr int kDevicePlanMinValues = 16384;
IndexPlan make_index_plan_auto(SpfftTransformType type, int dimX, int dimY, int dimZ, int numValues,
                               const int* triplets, bool allowDevice);

// Plans shared between transforms: a transform created with the same type, sizes and index
// triplets (compared element by element) as a live one on the same device reuses its plan,
// device tables included. SPFFT_GB300_PLAN_CACHE=0 turns the sharing off. The cache keeps a copy
// of each cached plan's triplets while the plan lives (at most 1 GiB of them in total).
std::shared_ptr<const IndexPlan> shared_index_plan(SpfftTransformType type, int dimX, int dimY,
                                                   int dimZ, int numValues, const int* triplets,
                                                   bool allowDevice);
// Live plans in the cache (for tests).
int index_plan_cache_size();

}  // namespace gb300
}  // namespace spfft
