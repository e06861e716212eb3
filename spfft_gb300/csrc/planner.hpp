// Index planner: turns the user's sparse (x, y, z) triplets into the z-stick layout that every
// kernel of this library works on, plus the derived lookup tables the fused kernels need.
//
// The first half (value indices, sorted stick keys, zero-zero stick) follows the reference's
// conversion rules bit-exactly:
//   * convert_index_triplets  -- src/compression/indices.hpp:120-186
//   * to_storage_index        -- src/compression/indices.hpp:49-55
//   * Parameters (local ctor) -- src/parameters/parameters.cpp:143-180
// The second half (compact x-columns, CSR of values per stick) is this library's own layout.
#pragma once

#include <cstdint>
#include <memory>
#include <vector>

#include "spfft/types.h"

namespace spfft {
namespace gb300 {

struct DeviceIndexTables;  // planner_gpu.hpp

struct IndexPlan {
  SpfftTransformType type = SPFFT_TRANS_C2C;
  int dimX = 0, dimY = 0, dimZ = 0;
  int dimXFreq = 0;  // dimX/2+1 for R2C, dimX for C2C (parameters.cpp:148)
  int numValues = 0;
  int numSticks = 0, numColumns = 0;
  bool centered = false;

  // --- reference-compatible part -------------------------------------------------------------
  // Per user value i: stickIndex * dimZ + zStorage (indices.hpp:167-176).
  std::vector<int> valueIndices;
  // Sorted unique storage keys xStorage * dimY + yStorage of the z-sticks (indices.hpp:151-180).
  std::vector<int> stickKeys;
  // Position of key 0 in stickKeys, or numSticks if absent (parameters.cpp:173-179).
  int zeroZeroStick = 0;

  // --- derived layout used by the GPU kernels --------------------------------------------------
  // Distinct storage x of the sticks, ascending. A "column" is one such x; only columns hold data
  // after the z-pass, so the y-pass runs over columns only (pruned y transform).
  std::vector<int> columnX;
  // Sticks of column c are stickKeys[columnStickStart[c] .. columnStickStart[c+1]).
  std::vector<int> columnStickStart;
  // Per stick: its column index and its storage y.
  std::vector<int> stickColumn;
  std::vector<int> stickY;
  // Values sorted by valueIndices (stable): entryPos[e] = stick*dimZ + z, entryUser[e] = user index.
  std::vector<int> entryPos;
  std::vector<int> entryUser;
  // Entries of stick s are [stickEntryStart[s], stickEntryStart[s+1]).
  std::vector<int> stickEntryStart;
  // True when entryUser[e] == e for every e (values already in stick order).
  bool identityOrder = true;
  // R2C only, per user value: how many times the value enters the real space field (1 or 2),
  // counting the hermitian mirror that the C2R convention and the stick / plane symmetry fills
  // imply. 2 unless the frequency is self-conjugate, on the x Nyquist plane, or on the y Nyquist
  // row of the x = 0 plane (where the plane fill conjugates in place). Used by the adjoints.
  std::vector<unsigned char> hermitianWeight;

  // Set when the plan was made by the device planner: the derived tables (stickColumn ..
  // hermitianWeight, plus the stick plane positions) live on that device only, and the host
  // vectors above are empty (download_index_plan() in planner_gpu.hpp brings them back).
  std::shared_ptr<const DeviceIndexTables> deviceTables;

  int num_sticks() const { return numSticks; }
  int num_columns() const { return numColumns; }
};

// Throws the same exception types as the reference for the same inputs:
//   InvalidParameterError  numValues > dimX*dimY*dimZ, or a non-positive dimension
//   InvalidIndicesError    an index outside the allowed (plain or centered) range
//   OverflowError          numSticks * dimZ does not fit a 32-bit int
IndexPlan make_index_plan(SpfftTransformType type, int dimX, int dimY, int dimZ, int numValues,
                          const int* triplets);

}  // namespace gb300
}  // namespace spfft
