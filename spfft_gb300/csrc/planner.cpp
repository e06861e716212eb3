// Index planner. The validation order, the centered-index rule, the stick ordering and the value
// index formula restate src/compression/indices.hpp:120-186 and src/parameters/parameters.cpp:
// 143-180 of the reference; the derived tables at the end are this library's own.
#include "planner.hpp"

#include <algorithm>
#include <climits>
#include <numeric>

#include "spfft/exceptions.hpp"

namespace spfft {
namespace gb300 {

namespace {
// Negative (centered) frequency index -> storage index in [0, dim) (indices.hpp:49-55).
inline int storage_index(int dim, int index) { return index < 0 ? dim + index : index; }
}  // namespace

IndexPlan make_index_plan(SpfftTransformType type, int dimX, int dimY, int dimZ, int numValues,
                          const int* triplets) {
  if (dimX <= 0 || dimY <= 0 || dimZ <= 0 || numValues < 0) throw InvalidParameterError();
  if (numValues > 0 && !triplets) throw InvalidParameterError();
  const bool hermitian = (type == SPFFT_TRANS_R2C);
  if (type != SPFFT_TRANS_C2C && type != SPFFT_TRANS_R2C) throw InvalidParameterError();

  // More values than grid points is rejected first (indices.hpp:124-127).
  const unsigned long long gridPoints = static_cast<unsigned long long>(dimX) *
                                        static_cast<unsigned long long>(dimY) *
                                        static_cast<unsigned long long>(dimZ);
  if (static_cast<unsigned long long>(numValues) > gridPoints) throw InvalidParameterError();

  IndexPlan p;
  p.type = type;
  p.dimX = dimX;
  p.dimY = dimY;
  p.dimZ = dimZ;
  p.dimXFreq = hermitian ? dimX / 2 + 1 : dimX;
  p.numValues = numValues;

  // A single negative index anywhere switches all three dimensions to centered bounds
  // (indices.hpp:128-135).
  bool centered = false;
  for (int i = 0; i < numValues && !centered; ++i) {
    if (triplets[3 * i] < 0 || triplets[3 * i + 1] < 0 || triplets[3 * i + 2] < 0) centered = true;
  }
  p.centered = centered;

  // Allowed ranges (indices.hpp:137-149): [0, n-1], or [floor(n/2)-n+1, floor(n/2)] when centered;
  // x is always [0, floor(n/2)] for R2C.
  const int maxX = (hermitian || centered ? dimX / 2 + 1 : dimX) - 1;
  const int maxY = (centered ? dimY / 2 + 1 : dimY) - 1;
  const int maxZ = (centered ? dimZ / 2 + 1 : dimZ) - 1;
  const int minX = hermitian ? 0 : maxX - dimX + 1;
  const int minY = maxY - dimY + 1;
  const int minZ = maxZ - dimZ + 1;
  for (int i = 0; i < numValues; ++i) {
    const int x = triplets[3 * i], y = triplets[3 * i + 1], z = triplets[3 * i + 2];
    if (x < minX || x > maxX) throw InvalidIndicesError();
    if (y < minY || y > maxY) throw InvalidIndicesError();
    if (z < minZ || z > maxZ) throw InvalidIndicesError();
  }

  // Unique stick keys x*dimY + y in ascending order; a stick's index is its rank in that order
  // (indices.hpp:151-165). Keys are bounded by dimX * dimY, so a presence table gives the same
  // order as the reference's ordered map in O(values + keys); very large xy planes fall back to a
  // sort + unique.
  std::vector<int> keyOfValue(numValues);
  for (int i = 0; i < numValues; ++i) {
    keyOfValue[i] = storage_index(dimX, triplets[3 * i]) * dimY +
                    storage_index(dimY, triplets[3 * i + 1]);
  }
  const long long keyRange = static_cast<long long>(dimX) * dimY;
  constexpr long long kTableLimit = 1LL << 24;
  std::vector<int> rankOfKey;  // key -> stick index (-1: no stick), when the table is used
  if (keyRange <= kTableLimit) {
    rankOfKey.assign(static_cast<size_t>(keyRange), -1);
    for (int key : keyOfValue) rankOfKey[key] = 0;
    int rank = 0;
    for (long long key = 0; key < keyRange; ++key) {
      if (rankOfKey[key] == 0) {
        rankOfKey[key] = rank++;
        p.stickKeys.push_back(static_cast<int>(key));
      }
    }
  } else {
    p.stickKeys = keyOfValue;
    std::sort(p.stickKeys.begin(), p.stickKeys.end());
    p.stickKeys.erase(std::unique(p.stickKeys.begin(), p.stickKeys.end()), p.stickKeys.end());
  }
  const int numSticks = static_cast<int>(p.stickKeys.size());
  p.numSticks = numSticks;
  if (static_cast<long long>(numSticks) * dimZ > INT_MAX) throw OverflowError();

  // Value index = stickIndex * dimZ + zStorage (indices.hpp:167-176).
  p.valueIndices.resize(numValues);
  for (int i = 0; i < numValues; ++i) {
    const int stick = !rankOfKey.empty()
                          ? rankOfKey[keyOfValue[i]]
                          : static_cast<int>(std::lower_bound(p.stickKeys.begin(), p.stickKeys.end(),
                                                              keyOfValue[i]) - p.stickKeys.begin());
    p.valueIndices[i] = stick * dimZ + storage_index(dimZ, triplets[3 * i + 2]);
  }

  // Zero-zero stick: position of key 0, or numSticks when absent (parameters.cpp:173-179).
  p.zeroZeroStick = 0;
  for (int key : p.stickKeys) {
    if (key == 0) break;
    ++p.zeroZeroStick;
  }

  // ---- derived tables -------------------------------------------------------------------------
  // Keys are sorted by x first, so the sticks of one column are contiguous.
  p.stickColumn.resize(numSticks);
  p.stickY.resize(numSticks);
  for (int s = 0; s < numSticks; ++s) {
    const int x = p.stickKeys[s] / dimY;
    p.stickY[s] = p.stickKeys[s] - x * dimY;
    if (p.columnX.empty() || p.columnX.back() != x) {
      p.columnX.push_back(x);
      p.columnStickStart.push_back(s);
    }
    p.stickColumn[s] = static_cast<int>(p.columnX.size()) - 1;
  }
  p.columnStickStart.push_back(numSticks);
  p.numColumns = static_cast<int>(p.columnX.size());

  // Values grouped by stick and ordered by position; duplicates keep user order (a counting sort
  // over the value positions, or a stable sort when the position range is very large).
  std::vector<int> order(numValues);
  const long long posRange = static_cast<long long>(numSticks) * dimZ;
  bool increasing = true;  // values already in position order (z-stick order without duplicates)
  for (int i = 1; i < numValues && increasing; ++i) increasing = p.valueIndices[i] > p.valueIndices[i - 1];
  if (increasing) {
    std::iota(order.begin(), order.end(), 0);
  } else if (posRange <= kTableLimit) {
    std::vector<int> start(static_cast<size_t>(posRange) + 1, 0);
    for (int i = 0; i < numValues; ++i) ++start[p.valueIndices[i] + 1];
    for (long long q = 0; q < posRange; ++q) start[q + 1] += start[q];
    for (int i = 0; i < numValues; ++i) order[start[p.valueIndices[i]]++] = i;
  } else {
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return p.valueIndices[a] < p.valueIndices[b]; });
  }
  p.entryPos.resize(numValues);
  p.entryUser.resize(numValues);
  p.identityOrder = true;
  for (int e = 0; e < numValues; ++e) {
    p.entryUser[e] = order[e];
    p.entryPos[e] = p.valueIndices[order[e]];
    if (order[e] != e) p.identityOrder = false;
  }
  if (hermitian) {
    auto nyquist = [](int n, int v) { return n % 2 == 0 && v == n / 2; };
    p.hermitianWeight.resize(numValues);
    for (int i = 0; i < numValues; ++i) {
      const int x = storage_index(dimX, triplets[3 * i]), y = storage_index(dimY, triplets[3 * i + 1]),
                z = storage_index(dimZ, triplets[3 * i + 2]);
      unsigned char m;
      if (x != 0) m = nyquist(dimX, x) ? 1 : 2;
      else if (y != 0) m = nyquist(dimY, y) ? 1 : 2;
      else m = (z != 0 && !nyquist(dimZ, z)) ? 2 : 1;
      p.hermitianWeight[i] = m;
    }
  }

  p.stickEntryStart.assign(numSticks + 1, 0);
  for (int e = 0; e < numValues; ++e) ++p.stickEntryStart[p.entryPos[e] / dimZ + 1];
  for (int s = 0; s < numSticks; ++s) p.stickEntryStart[s + 1] += p.stickEntryStart[s];
  return p;
}

}  // namespace gb300
}  // namespace spfft
