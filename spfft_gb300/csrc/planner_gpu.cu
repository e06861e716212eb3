// Device index planner and the shared-plan cache (planner_gpu.hpp).
//
// Two phases, one host read-back after each:
//   1. classify: bounds flags of every value under the plain and the centered ranges, its xy key
//      and the presence flags of keys and x columns; exclusive prefix sums of the presence flags
//      give every key its stick index and every x its column index. Read back: flags, number of
//      sticks and of columns (the host then raises the reference's errors and sizes the tables).
//   2. tables: per stick (column, y, plane position), per column (x, first stick), per value its
//      stick position stick * dimZ + z and a presence flag per position; the prefix sum of those
//      flags gives every value its entry (its rank in position order), then the entry tables and
//      the first entry of every stick. Read back: duplicate and reordering flags.
// All kernels are grid-stride loops over plain global memory: this is integer bookkeeping run
// once per plan, bound by latency rather than bandwidth.
#include "planner_gpu.hpp"

#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstdlib>
#include <cstring>
#include <list>
#include <mutex>
#include <string>
#include <vector>

#include "spfft/exceptions.hpp"

namespace spfft {
namespace gb300 {

namespace {

constexpr int kThreads = 256;                // threads of every planner block
constexpr int kItems = 16;                   // presence flags per thread in the prefix sums
constexpr int kTile = kThreads * kItems;     // flags per prefix-sum block
constexpr int kSumThreads = 1024;            // the single block that sums the block totals
constexpr long long kMaxKeys = 1LL << 26;
constexpr long long kMaxPositions = 1LL << 27;

enum : unsigned {
  kNegative = 1u,     // some index is negative: the centered ranges apply
  kBadPlain = 2u,     // some index lies outside the plain ranges
  kBadCentered = 4u,  // some index lies outside the centered ranges
  kKeyZero = 8u,      // the xy key 0 holds a stick
  kDuplicate = 16u,   // some stick position is given twice
  kReordered = 32u,   // position order differs from user order
};

struct Bounds {
  int lo[3], hi[3];  // x, y, z
};

// Device results read back by the host.
struct Counters {
  unsigned flags;
  int numSticks;
  int numColumns;
  int numEntries;
};

inline size_t align256(size_t b) { return (b + 255) & ~static_cast<size_t>(255); }

__device__ __forceinline__ void merge_flags(unsigned bits, Counters* c) {
  // every thread of the block reaches this after its grid-stride loop
  bits = __reduce_or_sync(0xffffffffu, bits);
  if ((threadIdx.x & 31) == 0 && bits) atomicOr(&c->flags, bits);
}

__device__ __forceinline__ bool outside(const Bounds& b, int x, int y, int z) {
  return x < b.lo[0] || x > b.hi[0] || y < b.lo[1] || y > b.hi[1] || z < b.lo[2] || z > b.hi[2];
}

// Storage index of a (possibly negative, centered) frequency index (indices.hpp:49-55).
__device__ __forceinline__ int storage(int dim, int v) { return v < 0 ? v + dim : v; }

__global__ void __launch_bounds__(kThreads)
    classify_values(const int* __restrict__ t, int n, Bounds plain, Bounds centered, int dimX,
                    int dimY, int dimZ, int dimXFreq, unsigned char* __restrict__ keyPresent,
                    unsigned char* __restrict__ colPresent, int* __restrict__ keyOfValue,
                    Counters* c) {
  unsigned bits = 0;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    const int x = t[3 * i], y = t[3 * i + 1], z = t[3 * i + 2];
    if ((x | y | z) < 0) bits |= kNegative;
    if (outside(plain, x, y, z)) bits |= kBadPlain;
    if (outside(centered, x, y, z)) bits |= kBadCentered;
    const int xs = storage(dimX, x), ys = storage(dimY, y), zs = storage(dimZ, z);
    int key = -1;
    if (xs >= 0 && xs < dimXFreq && ys >= 0 && ys < dimY && zs >= 0 && zs < dimZ) {
      key = xs * dimY + ys;
      keyPresent[key] = 1;
      colPresent[xs] = 1;
      if (key == 0) bits |= kKeyZero;
    } else {
      bits |= kBadPlain | kBadCentered;  // no valid range maps outside the storage box
    }
    keyOfValue[i] = key;
  }
  merge_flags(bits, c);
}

// Exclusive prefix sum of one value per thread over a block of NT threads; *total receives the
// block's sum. Called once per kernel.
template <int NT>
__device__ __forceinline__ int block_exclusive_sum(int v, int* total) {
  __shared__ int warpSums[NT / 32];
  __shared__ int blockTotal;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int incl = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int o = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= d) incl += o;
  }
  if (lane == 31) warpSums[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    const int w = lane < NT / 32 ? warpSums[lane] : 0;
    int wi = w;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int o = __shfl_up_sync(0xffffffffu, wi, d);
      if (lane >= d) wi += o;
    }
    if (lane < NT / 32) warpSums[lane] = wi - w;
    if (lane == 31) blockTotal = wi;
  }
  __syncthreads();
  *total = blockTotal;
  return warpSums[warp] + incl - v;
}

// The kItems presence flags of one thread starting at j0 (0 past m), as 0 / 1.
__device__ __forceinline__ void load_flags(const unsigned char* __restrict__ f, long long j0, long long m,
                                           int v[kItems]) {
  if (j0 + kItems <= m) {
    const uint4 w = *reinterpret_cast<const uint4*>(f + j0);  // j0 is a multiple of 16
    const unsigned ws[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
    for (int k = 0; k < kItems; ++k) v[k] = ((ws[k >> 2] >> (8 * (k & 3))) & 0xffu) != 0;
  } else {
#pragma unroll
    for (int k = 0; k < kItems; ++k) v[k] = (j0 + k < m) ? (f[j0 + k] != 0) : 0;
  }
}

__global__ void __launch_bounds__(kThreads)
    scan_count(const unsigned char* __restrict__ f, long long m, int* __restrict__ blockSums) {
  const long long j0 = static_cast<long long>(blockIdx.x) * kTile + threadIdx.x * kItems;
  int v[kItems];
  load_flags(f, j0, m, v);
  int s = 0;
#pragma unroll
  for (int k = 0; k < kItems; ++k) s += v[k];
  int total = 0;
  block_exclusive_sum<kThreads>(s, &total);
  if (threadIdx.x == 0) blockSums[blockIdx.x] = total;
}

// In place: block sums -> exclusive block offsets; *total receives the grand total.
__global__ void __launch_bounds__(kSumThreads) scan_block_sums(int* __restrict__ sums, int nb, int* total) {
  const int per = (nb + kSumThreads - 1) / kSumThreads;
  const int b0 = threadIdx.x * per;
  int s = 0;
  for (int b = b0; b < min(nb, b0 + per); ++b) s += sums[b];
  int all = 0;
  int run = block_exclusive_sum<kSumThreads>(s, &all);
  for (int b = b0; b < min(nb, b0 + per); ++b) {
    const int v = sums[b];
    sums[b] = run;
    run += v;
  }
  if (threadIdx.x == 0) *total = all;
}

__global__ void __launch_bounds__(kThreads)
    scan_apply(const unsigned char* __restrict__ f, long long m, const int* __restrict__ offsets,
               int* __restrict__ ranks) {
  const long long j0 = static_cast<long long>(blockIdx.x) * kTile + threadIdx.x * kItems;
  int v[kItems];
  load_flags(f, j0, m, v);
  int s = 0;
#pragma unroll
  for (int k = 0; k < kItems; ++k) s += v[k];
  int total = 0;
  int r = offsets[blockIdx.x] + block_exclusive_sum<kThreads>(s, &total);
  int out[kItems];
#pragma unroll
  for (int k = 0; k < kItems; ++k) {
    out[k] = r;
    r += v[k];
  }
  if (j0 + kItems <= m) {
    int4* dst = reinterpret_cast<int4*>(ranks + j0);  // 64-byte aligned
#pragma unroll
    for (int q = 0; q < kItems / 4; ++q) dst[q] = make_int4(out[4 * q], out[4 * q + 1], out[4 * q + 2], out[4 * q + 3]);
  } else {
#pragma unroll
    for (int k = 0; k < kItems; ++k)
      if (j0 + k < m) ranks[j0 + k] = out[k];
  }
}

// ranks[j] = number of nonzero flags before j; *total = number of nonzero flags.
void exclusive_count(const unsigned char* flags, long long m, int* ranks, int* blockSums, int* total,
                     cudaStream_t s) {
  const long long nb = (m + kTile - 1) / kTile;
  scan_count<<<static_cast<unsigned>(nb), kThreads, 0, s>>>(flags, m, blockSums);
  scan_block_sums<<<1, kSumThreads, 0, s>>>(blockSums, static_cast<int>(nb), total);
  scan_apply<<<static_cast<unsigned>(nb), kThreads, 0, s>>>(flags, m, blockSums, ranks);
  check_launch(cudaGetLastError());
}

__global__ void __launch_bounds__(kThreads)
    stick_tables(const unsigned char* __restrict__ keyPresent, const int* __restrict__ keyRank,
                 int keyRange, const int* __restrict__ colRank, int dimY, int numColumns,
                 int* __restrict__ stickColumn, int* __restrict__ stickY, int* __restrict__ stickPlanePos) {
  for (int k = blockIdx.x * kThreads + threadIdx.x; k < keyRange; k += gridDim.x * kThreads) {
    if (!keyPresent[k]) continue;
    const int s = keyRank[k];
    const int x = k / dimY, y = k - x * dimY;
    const int col = colRank[x];
    stickColumn[s] = col;
    stickY[s] = y;
    stickPlanePos[s] = y * numColumns + col;
  }
}

__global__ void __launch_bounds__(kThreads)
    column_tables(const unsigned char* __restrict__ colPresent, const int* __restrict__ colRank,
                  int dimXFreq, const int* __restrict__ keyRank, int dimY, int numSticks, int numColumns,
                  int* __restrict__ columnX, int* __restrict__ columnStickStart) {
  const int g = blockIdx.x * kThreads + threadIdx.x;
  for (int x = g; x < dimXFreq; x += gridDim.x * kThreads) {
    if (!colPresent[x]) continue;
    const int col = colRank[x];
    columnX[col] = x;
    // sticks are ordered by key = x * dimY + y: those of smaller x come first
    columnStickStart[col] = keyRank[x * dimY];
  }
  if (g == 0) columnStickStart[numColumns] = numSticks;
}

__global__ void __launch_bounds__(kThreads)
    value_positions(const int* __restrict__ t, int n, const int* __restrict__ keyOfValue,
                    const int* __restrict__ keyRank, int dimX, int dimY, int dimZ, int r2c,
                    unsigned char* __restrict__ posPresent, int* __restrict__ valuePos,
                    unsigned char* __restrict__ hermitianWeight, Counters* c) {
  unsigned bits = 0;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    const int zs = storage(dimZ, t[3 * i + 2]);
    // value index = stick * dimZ + z (indices.hpp:167-176)
    const int pos = keyRank[keyOfValue[i]] * dimZ + zs;
    valuePos[i] = pos;
    // byte flag set through its aligned 32-bit word (little-endian byte order)
    unsigned* word = reinterpret_cast<unsigned*>(posPresent + (pos & ~3));
    const unsigned bit = 1u << (8 * (pos & 3));
    if (atomicOr(word, bit) & bit) bits |= kDuplicate;
    if (r2c) {
      const int xs = storage(dimX, t[3 * i]), ys = storage(dimY, t[3 * i + 1]);
      const bool nyX = (dimX % 2 == 0) && xs == dimX / 2, nyY = (dimY % 2 == 0) && ys == dimY / 2,
                 nyZ = (dimZ % 2 == 0) && zs == dimZ / 2;
      unsigned char w;
      if (xs != 0) w = nyX ? 1 : 2;
      else if (ys != 0) w = nyY ? 1 : 2;
      else w = (zs != 0 && !nyZ) ? 2 : 1;
      hermitianWeight[i] = w;
    }
  }
  merge_flags(bits, c);
}

__global__ void __launch_bounds__(kThreads)
    entry_tables(const int* __restrict__ valuePos, int n, const int* __restrict__ entryOf,
                 int* __restrict__ entryPos, int* __restrict__ entryUser, Counters* c) {
  unsigned bits = 0;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    const int pos = valuePos[i];
    const int e = entryOf[pos];
    entryPos[e] = pos;
    entryUser[e] = i;
    if (e != i) bits |= kReordered;
  }
  merge_flags(bits, c);
}

__global__ void __launch_bounds__(kThreads)
    stick_entry_starts(const int* __restrict__ entryOf, int numSticks, int dimZ, int numEntries,
                       int* __restrict__ stickEntryStart) {
  for (int s = blockIdx.x * kThreads + threadIdx.x; s <= numSticks; s += gridDim.x * kThreads) {
    stickEntryStart[s] = s < numSticks ? entryOf[static_cast<long long>(s) * dimZ] : numEntries;
  }
}

// Stream-ordered scratch, freed in stream order.
class AsyncBuffer {
public:
  AsyncBuffer(size_t bytes, cudaStream_t s) : s_(s) {
    if (injected_allocation_failure()) throw GPUAllocationError();
    check_cuda(cudaMallocAsync(&p_, bytes, s));
  }
  ~AsyncBuffer() {
    if (p_) (void)cudaFreeAsync(p_, s_);
  }
  AsyncBuffer(const AsyncBuffer&) = delete;
  AsyncBuffer& operator=(const AsyncBuffer&) = delete;
  char* get() const { return static_cast<char*>(p_); }

private:
  void* p_ = nullptr;
  cudaStream_t s_;
};

unsigned grid_for(long long work, int numSms) {
  const long long blocks = (work + kThreads - 1) / kThreads;
  return static_cast<unsigned>(std::max(1LL, std::min(blocks, 8LL * numSms)));
}

bool device_present() {
  int count = 0;
  const bool ok = cudaGetDeviceCount(&count) == cudaSuccess && count > 0;
  if (!ok) (void)cudaGetLastError();
  return ok;
}

}  // namespace

bool make_index_plan_device(SpfftTransformType type, int dimX, int dimY, int dimZ, int numValues,
                            const int* triplets, IndexPlan* out) {
  // Parameter checks in the host planner's order.
  if (dimX <= 0 || dimY <= 0 || dimZ <= 0 || numValues < 0) throw InvalidParameterError();
  if (numValues > 0 && !triplets) throw InvalidParameterError();
  const bool hermitian = (type == SPFFT_TRANS_R2C);
  if (type != SPFFT_TRANS_C2C && type != SPFFT_TRANS_R2C) throw InvalidParameterError();
  const unsigned long long gridPoints = static_cast<unsigned long long>(dimX) *
                                        static_cast<unsigned long long>(dimY) *
                                        static_cast<unsigned long long>(dimZ);
  if (static_cast<unsigned long long>(numValues) > gridPoints) throw InvalidParameterError();
  if (numValues == 0) return false;
  const int dimXFreq = hermitian ? dimX / 2 + 1 : dimX;
  const long long keyRange = static_cast<long long>(dimXFreq) * dimY;
  if (keyRange > kMaxKeys) return false;

  // Plain and centered ranges (indices.hpp:137-149); x is [0, floor(n/2)] for R2C either way.
  Bounds plain{}, centered{};
  {
    const int dims[3] = {dimX, dimY, dimZ};
    for (int d = 0; d < 3; ++d) {
      const int n = dims[d];
      plain.hi[d] = ((d == 0 && hermitian) ? n / 2 + 1 : n) - 1;
      plain.lo[d] = (d == 0 && hermitian) ? 0 : plain.hi[d] - n + 1;
      centered.hi[d] = n / 2;
      centered.lo[d] = (d == 0 && hermitian) ? 0 : centered.hi[d] - n + 1;
    }
  }

  int device = 0, numSms = 0;
  check_cuda(cudaGetDevice(&device));
  check_cuda(cudaDeviceGetAttribute(&numSms, cudaDevAttrMultiProcessorCount, device));
  Stream stream;
  const cudaStream_t s = stream.get();
  const size_t n = static_cast<size_t>(numValues);
  const size_t keyBlocks = static_cast<size_t>((keyRange + kTile - 1) / kTile);
  const size_t colBlocks = static_cast<size_t>((dimXFreq + kTile - 1) / kTile);

  // phase 1 scratch
  size_t off = 0;
  const size_t oTrip = off;         off += align256(n * 3 * sizeof(int));
  const size_t oKeyPresent = off;   off += align256(static_cast<size_t>(keyRange));
  const size_t oColPresent = off;   off += align256(static_cast<size_t>(dimXFreq));
  const size_t oKeyRank = off;      off += align256(static_cast<size_t>(keyRange) * sizeof(int));
  const size_t oColRank = off;      off += align256(static_cast<size_t>(dimXFreq) * sizeof(int));
  const size_t oKeyOfValue = off;   off += align256(n * sizeof(int));
  const size_t oValuePos = off;     off += align256(n * sizeof(int));
  const size_t oKeySums = off;      off += align256(keyBlocks * sizeof(int));
  const size_t oColSums = off;      off += align256(colBlocks * sizeof(int));
  const size_t oCounters = off;     off += align256(sizeof(Counters));
  AsyncBuffer scratch(off, s);
  char* w = scratch.get();
  int* dTrip = reinterpret_cast<int*>(w + oTrip);
  auto* keyPresent = reinterpret_cast<unsigned char*>(w + oKeyPresent);
  auto* colPresent = reinterpret_cast<unsigned char*>(w + oColPresent);
  int* keyRank = reinterpret_cast<int*>(w + oKeyRank);
  int* colRank = reinterpret_cast<int*>(w + oColRank);
  int* keyOfValue = reinterpret_cast<int*>(w + oKeyOfValue);
  int* valuePos = reinterpret_cast<int*>(w + oValuePos);
  auto* counters = reinterpret_cast<Counters*>(w + oCounters);

  check_cuda(cudaMemcpyAsync(dTrip, triplets, n * 3 * sizeof(int), cudaMemcpyHostToDevice, s));
  // presence flags of keys and columns (adjacent) and the counters
  check_cuda(cudaMemsetAsync(w + oKeyPresent, 0, oKeyRank - oKeyPresent, s));
  check_cuda(cudaMemsetAsync(counters, 0, sizeof(Counters), s));
  classify_values<<<grid_for(numValues, numSms), kThreads, 0, s>>>(
      dTrip, numValues, plain, centered, dimX, dimY, dimZ, dimXFreq, keyPresent, colPresent,
      keyOfValue, counters);
  check_launch(cudaGetLastError());
  exclusive_count(keyPresent, keyRange, keyRank, reinterpret_cast<int*>(w + oKeySums),
                  &counters->numSticks, s);
  exclusive_count(colPresent, dimXFreq, colRank, reinterpret_cast<int*>(w + oColSums),
                  &counters->numColumns, s);
  Counters host{};
  check_cuda(cudaMemcpyAsync(&host, counters, sizeof(Counters), cudaMemcpyDeviceToHost, s));
  check_cuda(cudaStreamSynchronize(s));

  // Errors as the host planner raises them: any index outside the ranges of its mode, then a
  // stick volume beyond 32-bit indexing.
  const bool isCentered = (host.flags & kNegative) != 0;
  if (host.flags & (isCentered ? kBadCentered : kBadPlain)) throw InvalidIndicesError();
  const int ns = host.numSticks, ncol = host.numColumns;
  if (static_cast<long long>(ns) * dimZ > INT_MAX) throw OverflowError();
  const long long posRange = static_cast<long long>(ns) * dimZ;
  if (posRange > kMaxPositions) return false;

  // the tables, as the transform keeps them
  auto tables = std::make_shared<DeviceIndexTables>();
  tables->device = device;
  size_t t = 0;
  const size_t tStickColumn = t;      t += align256(static_cast<size_t>(ns) * sizeof(int));
  const size_t tStickY = t;           t += align256(static_cast<size_t>(ns) * sizeof(int));
  const size_t tStickPlanePos = t;    t += align256(static_cast<size_t>(ns) * sizeof(int));
  const size_t tColumnX = t;          t += align256(static_cast<size_t>(ncol) * sizeof(int));
  const size_t tColumnStart = t;      t += align256(static_cast<size_t>(ncol + 1) * sizeof(int));
  const size_t tEntryPos = t;         t += align256(n * sizeof(int));
  const size_t tEntryUser = t;        t += align256(n * sizeof(int));
  const size_t tStickEntryStart = t;  t += align256(static_cast<size_t>(ns + 1) * sizeof(int));
  const size_t tHermitian = t;        t += hermitian ? align256(n) : 0;
  tables->buffer = DeviceBuffer(t);
  char* d = static_cast<char*>(tables->buffer.get());
  int* stickColumn = reinterpret_cast<int*>(d + tStickColumn);
  int* stickY = reinterpret_cast<int*>(d + tStickY);
  int* stickPlanePos = reinterpret_cast<int*>(d + tStickPlanePos);
  int* columnX = reinterpret_cast<int*>(d + tColumnX);
  int* columnStart = reinterpret_cast<int*>(d + tColumnStart);
  int* entryPos = reinterpret_cast<int*>(d + tEntryPos);
  int* entryUser = reinterpret_cast<int*>(d + tEntryUser);
  int* stickEntryStart = reinterpret_cast<int*>(d + tStickEntryStart);
  auto* hermitianWeight = hermitian ? reinterpret_cast<unsigned char*>(d + tHermitian) : nullptr;

  // phase 2 scratch: position flags (padded to whole 32-bit words) and entry ranks
  const size_t posBlocks = static_cast<size_t>((posRange + kTile - 1) / kTile);
  size_t off2 = 0;
  const size_t oPosPresent = off2;  off2 += align256(static_cast<size_t>(posRange));
  const size_t oEntryOf = off2;     off2 += align256(static_cast<size_t>(posRange) * sizeof(int));
  const size_t oPosSums = off2;     off2 += align256(posBlocks * sizeof(int));
  AsyncBuffer scratch2(off2, s);
  char* w2 = scratch2.get();
  auto* posPresent = reinterpret_cast<unsigned char*>(w2 + oPosPresent);
  int* entryOf = reinterpret_cast<int*>(w2 + oEntryOf);
  check_cuda(cudaMemsetAsync(posPresent, 0, align256(static_cast<size_t>(posRange)), s));

  stick_tables<<<grid_for(keyRange, numSms), kThreads, 0, s>>>(keyPresent, keyRank, static_cast<int>(keyRange),
                                                               colRank, dimY, ncol, stickColumn, stickY,
                                                               stickPlanePos);
  column_tables<<<grid_for(dimXFreq, numSms), kThreads, 0, s>>>(colPresent, colRank, dimXFreq, keyRank, dimY,
                                                                ns, ncol, columnX, columnStart);
  value_positions<<<grid_for(numValues, numSms), kThreads, 0, s>>>(
      dTrip, numValues, keyOfValue, keyRank, dimX, dimY, dimZ, hermitian ? 1 : 0, posPresent, valuePos,
      hermitianWeight, counters);
  check_launch(cudaGetLastError());
  exclusive_count(posPresent, posRange, entryOf, reinterpret_cast<int*>(w2 + oPosSums),
                  &counters->numEntries, s);
  entry_tables<<<grid_for(numValues, numSms), kThreads, 0, s>>>(valuePos, numValues, entryOf, entryPos,
                                                                entryUser, counters);
  stick_entry_starts<<<grid_for(static_cast<long long>(ns) + 1, numSms), kThreads, 0, s>>>(
      entryOf, ns, dimZ, numValues, stickEntryStart);
  check_launch(cudaGetLastError());
  check_cuda(cudaMemcpyAsync(&host, counters, sizeof(Counters), cudaMemcpyDeviceToHost, s));
  check_cuda(cudaStreamSynchronize(s));
  if (host.flags & kDuplicate) return false;

  tables->stickColumn = stickColumn;
  tables->stickY = stickY;
  tables->stickPlanePos = stickPlanePos;
  tables->columnX = columnX;
  tables->columnStickStart = columnStart;
  tables->entryPos = entryPos;
  tables->entryUser = entryUser;
  tables->stickEntryStart = stickEntryStart;
  tables->hermitianWeight = hermitianWeight;

  IndexPlan p;
  p.type = type;
  p.dimX = dimX;
  p.dimY = dimY;
  p.dimZ = dimZ;
  p.dimXFreq = dimXFreq;
  p.numValues = numValues;
  p.numSticks = ns;
  p.numColumns = ncol;
  p.centered = isCentered;
  // position of key 0 among the sorted keys: first when present (parameters.cpp:173-179)
  p.zeroZeroStick = (host.flags & kKeyZero) ? 0 : ns;
  p.identityOrder = (host.flags & kReordered) == 0;
  p.deviceTables = std::move(tables);
  *out = std::move(p);
  return true;
}

IndexPlan download_index_plan(const IndexPlan& p) {
  if (!p.deviceTables) return p;
  const DeviceIndexTables& t = *p.deviceTables;
  DeviceGuard guard(t.device);
  IndexPlan h = p;
  h.deviceTables.reset();
  const int ns = p.numSticks, ncol = p.numColumns, nv = p.numValues;
  auto get = [](std::vector<int>& v, const int* src, int count) {
    v.resize(count);
    if (count > 0) check_cuda(cudaMemcpy(v.data(), src, count * sizeof(int), cudaMemcpyDeviceToHost));
  };
  std::vector<int> planePos;
  get(h.stickColumn, t.stickColumn, ns);
  get(h.stickY, t.stickY, ns);
  get(h.columnX, t.columnX, ncol);
  get(h.columnStickStart, t.columnStickStart, ncol + 1);
  get(h.entryPos, t.entryPos, nv);
  get(h.entryUser, t.entryUser, nv);
  get(h.stickEntryStart, t.stickEntryStart, ns + 1);
  h.hermitianWeight.clear();
  if (t.hermitianWeight) {
    h.hermitianWeight.resize(nv);
    if (nv > 0) check_cuda(cudaMemcpy(h.hermitianWeight.data(), t.hermitianWeight, nv, cudaMemcpyDeviceToHost));
  }
  // the reference-compatible part, from the derived tables
  h.stickKeys.resize(ns);
  for (int s = 0; s < ns; ++s) h.stickKeys[s] = h.columnX[h.stickColumn[s]] * p.dimY + h.stickY[s];
  h.valueIndices.resize(nv);
  for (int e = 0; e < nv; ++e) h.valueIndices[h.entryUser[e]] = h.entryPos[e];
  return h;
}

IndexPlan make_index_plan_auto(SpfftTransformType type, int dimX, int dimY, int dimZ, int numValues,
                               const int* triplets, bool allowDevice) {
  const char* env = std::getenv("SPFFT_GB300_PLANNER");
  const std::string mode = env ? env : "";
  const int threshold = mode == "device" ? 1 : kDevicePlanMinValues;
  if (allowDevice && mode != "host" && numValues >= threshold && device_present()) {
    IndexPlan p;
    try {
      if (make_index_plan_device(type, dimX, dimY, dimZ, numValues, triplets, &p)) return p;
    } catch (const GPUError&) {
      // a device that cannot run the planner (no stream-ordered allocator, out of memory): plan on
      // the host; index errors are not GPU errors and propagate
      (void)cudaGetLastError();
    }
  }
  return make_index_plan(type, dimX, dimY, dimZ, numValues, triplets);
}

// ------------------------------------------------------------------------------------------------
// Shared plans
// ------------------------------------------------------------------------------------------------
namespace {

struct CacheEntry {
  SpfftTransformType type;
  int dimX, dimY, dimZ, numValues, device;
  std::vector<int> triplets;
  std::weak_ptr<const IndexPlan> plan;
};

constexpr size_t kCacheBytesLimit = size_t(1) << 30;

std::mutex& cache_mutex() {
  static std::mutex m;
  return m;
}
std::list<CacheEntry>& cache() {
  static std::list<CacheEntry> c;
  return c;
}

// Drops entries whose plan is gone; returns the bytes of triplets still held. Caller holds the lock.
size_t prune_cache() {
  size_t bytes = 0;
  auto& c = cache();
  for (auto it = c.begin(); it != c.end();) {
    if (it->plan.expired()) {
      it = c.erase(it);
    } else {
      bytes += it->triplets.size() * sizeof(int);
      ++it;
    }
  }
  return bytes;
}

bool cache_enabled() {
  const char* env = std::getenv("SPFFT_GB300_PLAN_CACHE");
  return !(env && std::strcmp(env, "0") == 0);
}

}  // namespace

std::shared_ptr<const IndexPlan> shared_index_plan(SpfftTransformType type, int dimX, int dimY,
                                                   int dimZ, int numValues, const int* triplets,
                                                   bool allowDevice) {
  const bool useCache = cache_enabled() && numValues > 0 && triplets;
  int device = -1;
  if (useCache && allowDevice && device_present()) check_cuda(cudaGetDevice(&device));
  const size_t words = static_cast<size_t>(numValues > 0 ? numValues : 0) * 3;
  if (useCache) {
    std::lock_guard<std::mutex> lock(cache_mutex());
    for (const CacheEntry& e : cache()) {
      if (e.type != type || e.dimX != dimX || e.dimY != dimY || e.dimZ != dimZ ||
          e.numValues != numValues || e.device != device) {
        continue;
      }
      if (std::memcmp(e.triplets.data(), triplets, words * sizeof(int)) != 0) continue;
      if (auto live = e.plan.lock()) return live;
    }
  }
  auto plan = std::make_shared<const IndexPlan>(
      make_index_plan_auto(type, dimX, dimY, dimZ, numValues, triplets, allowDevice));
  if (useCache) {
    std::lock_guard<std::mutex> lock(cache_mutex());
    if (prune_cache() + words * sizeof(int) <= kCacheBytesLimit) {
      cache().push_back(CacheEntry{type, dimX, dimY, dimZ, numValues, device,
                                   std::vector<int>(triplets, triplets + words), plan});
    }
  }
  return plan;
}

int index_plan_cache_size() {
  std::lock_guard<std::mutex> lock(cache_mutex());
  prune_cache();
  return static_cast<int>(cache().size());
}

}  // namespace gb300
}  // namespace spfft
