// GpuPlan: uploads the planner's tables and the twiddles once, picks tile shapes, and issues the
// kernel sequence of each transform.
#include "engine.hpp"
#include "planner_gpu.hpp"

#include <algorithm>
#include <array>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <mutex>
#include <vector>

#include "fft_plan.hpp"
#include "kernels_fast.hpp"

namespace spfft {
namespace gb300 {

namespace {

constexpr size_t kAlign = 256;
inline size_t align_up(size_t v) { return (v + kAlign - 1) / kAlign * kAlign; }

// Shared memory budget per block of the generic kernels: two blocks per SM.
constexpr size_t kSmemBudget = 100 * 1024;

int max_smem_optin(int device) {
  int v = 0;
  check_cuda(cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, device));
  return v;
}

template <typename T>
void prepare_once(int device) {
  static std::mutex mutex;
  static std::vector<int> done;
  std::lock_guard<std::mutex> lock(mutex);
  if (std::find(done.begin(), done.end(), device) != done.end()) return;
  check_cuda(prepare_kernels<T>(static_cast<size_t>(max_smem_optin(device))));
  done.push_back(device);
}

// Per (device, size) attribute setup of the specialised kernels.
template <typename T>
bool prepare_fast_once(int device, int n) {
  static std::mutex mutex;
  static std::vector<std::pair<int, int>> done;
  std::lock_guard<std::mutex> lock(mutex);
  if (std::find(done.begin(), done.end(), std::make_pair(device, n)) != done.end()) return true;
  FastArgs<T> a;
  a.maxSmem = static_cast<size_t>(max_smem_optin(device));
  if (!fast_dispatch<T>(FastOp::Prepare, n, false, a)) {
    (void)cudaGetLastError();
    return false;
  }
  done.emplace_back(device, n);
  return true;
}

// Shared memory budget of one specialised z-pass block (four blocks per SM).
constexpr size_t kFastZBudget = 56 * 1024;

inline int odd_pitch(int n) { return n % 2 == 0 ? n + 1 : n; }

// Plane counts of the staged chunks in the backward's order. By default they double from about
// nz / 24 planes (192: 8, 16, 32, 64, 72): the backward's pipeline fills over a short first chunk
// (its y and x passes run before the first copy can start) and the forward, taking the chunks in
// reverse, drains over a short last one (its passes and the z pass run after the last copy), while
// every other chunk's passes, about a quarter of its copy time on the host link, hide under the
// neighbouring chunk's copy; fewer chunks than equal ones of that first size also mean fewer copy
// calls. `uniform` > 0 asks for that many equal chunks instead.
std::vector<int> staged_chunk_sizes(int nz, int uniform) {
  std::vector<int> sizes;
  if (uniform > 0) {
    const int per = (nz + uniform - 1) / uniform;
    for (int z0 = 0; z0 < nz; z0 += per) sizes.push_back(std::min(per, nz - z0));
    return sizes;
  }
  for (int size = std::max(1, (nz + 12) / 24), rem = nz; rem > 0; size *= 2) {
    const int take = std::min(size, rem);
    sizes.push_back(take);
    rem -= take;
  }
  return sizes;
}

template <typename T>
LaunchConfig choose_launch_config(const IndexPlan& p, int device) {
  const size_t c = 2 * sizeof(T);
  const size_t optin = static_cast<size_t>(max_smem_optin(device));
  LaunchConfig cfg{};
  cfg.threads = 256;

  const int nz = p.dimZ, ny = p.dimY, nx = p.dimX;
  cfg.zPitch = odd_pitch(nz);
  cfg.xPitch = odd_pitch(nx);
  // Every pass needs at least one sequence plus its ping-pong copy and the twiddles on chip.
  const size_t minZ = (nz + 2 * static_cast<size_t>(cfg.zPitch)) * c;
  const size_t minY = (ny + 2 * static_cast<size_t>(ny)) * c;
  const size_t minX = (nx + 2 * static_cast<size_t>(cfg.xPitch)) * c;
  if (minZ > optin || minY > optin || minX > optin) throw InvalidParameterError();
  // The y and x passes put z on gridDim.y.
  if (nz > 65535) throw InvalidParameterError();

  auto fit = [&](size_t fixed, size_t per, int cap) {
    const size_t budget = std::max(kSmemBudget, fixed + per);
    int k = static_cast<int>((budget - fixed) / per);
    return std::max(1, std::min(k, cap));
  };
  cfg.sticksPerBlock = fit(nz * c, 2 * cfg.zPitch * c, 32);
  cfg.sticksPerBlock = std::min(cfg.sticksPerBlock, std::max(1, p.num_sticks()));
  cfg.columnsPerBlock = fit(ny * c, 2 * static_cast<size_t>(ny) * c, 32);
  cfg.columnsPerBlock = std::min(cfg.columnsPerBlock, std::max(1, p.num_columns()));
  cfg.rowsPerBlock = fit(nx * c, 2 * cfg.xPitch * c, 16);
  cfg.rowsPerBlock = std::min(cfg.rowsPerBlock, ny);

  cfg.smemZ = (nz + 2 * static_cast<size_t>(cfg.sticksPerBlock) * cfg.zPitch) * c;
  cfg.smemY = (ny + 2 * static_cast<size_t>(cfg.columnsPerBlock) * ny) * c;
  cfg.smemX = (nx + 2 * static_cast<size_t>(cfg.rowsPerBlock) * cfg.xPitch) * c;
  return cfg;
}

}  // namespace

template <typename T>
GpuPlan<T>::GpuPlan(const IndexPlan& p, int device) {
  prepare_once<T>(device);
  config_ = choose_launch_config<T>(p, device);

  const int ns = p.num_sticks(), ncol = p.num_columns(), nv = p.numValues;
  const size_t c = 2 * sizeof(T);

  // Scratch: sticks, then compact planes, then the value staging area.
  layout_.sticksOffset = 0;
  layout_.planesOffset = align_up(static_cast<size_t>(ns) * p.dimZ * c);
  layout_.expOffset = layout_.planesOffset + align_up(static_cast<size_t>(p.dimZ) * p.dimY * ncol * c);
  // per-plane column or row exponents of the double-float compact planes
  layout_.stickExpOffset =
      layout_.expOffset + align_up(static_cast<size_t>(p.dimZ) * std::max(ncol, p.dimY) * sizeof(int));
  layout_.valuesOffset =
      layout_.stickExpOffset + align_up(std::max(static_cast<size_t>(ns), static_cast<size_t>(p.dimZ) * ncol) * sizeof(int));
  layout_.total = layout_.valuesOffset + align_up(static_cast<size_t>(nv) * c);

  // One allocation for every table: twiddles (T) then int arrays.
  const std::vector<double> twz = make_twiddles(p.dimZ), twy = make_twiddles(p.dimY),
                            twx = make_twiddles(p.dimX);
  struct Part {
    const void* src;
    size_t bytes;
    size_t offset;
  };
  std::vector<T> tz(twz.begin(), twz.end()), ty(twy.begin(), twy.end()), tx(twx.begin(), twx.end());
  // Index tables: a plan made by the device planner on this device is read where it lies (and
  // kept alive with this plan); other plans upload their host tables, downloaded first when the
  // plan was made on another device.
  const DeviceIndexTables* dt =
      (p.deviceTables && p.deviceTables->device == device) ? p.deviceTables.get() : nullptr;
  IndexPlan downloaded;
  const IndexPlan* hp = &p;
  if (p.deviceTables && !dt) {
    downloaded = download_index_plan(p);
    hp = &downloaded;
  }
  if (dt) sharedTables_ = p.deviceTables;
  std::vector<int> planePos;
  if (!dt) {
    planePos.resize(ns);
    for (int st = 0; st < ns; ++st) planePos[st] = hp->stickY[st] * ncol + hp->stickColumn[st];
  }
  std::vector<Part> parts = {
      {tz.data(), tz.size() * sizeof(T), 0},
      {ty.data(), ty.size() * sizeof(T), 0},
      {tx.data(), tx.size() * sizeof(T), 0},
  };
  if (!dt) {
    parts.insert(parts.end(), {
        {hp->stickColumn.data(), hp->stickColumn.size() * sizeof(int), 0},
        {hp->stickY.data(), hp->stickY.size() * sizeof(int), 0},
        {hp->columnX.data(), hp->columnX.size() * sizeof(int), 0},
        {hp->columnStickStart.data(), hp->columnStickStart.size() * sizeof(int), 0},
        {hp->entryPos.data(), hp->entryPos.size() * sizeof(int), 0},
        {hp->entryUser.data(), hp->entryUser.size() * sizeof(int), 0},
        {hp->stickEntryStart.data(), hp->stickEntryStart.size() * sizeof(int), 0},
        {hp->hermitianWeight.data(), hp->hermitianWeight.size(), 0},
        {planePos.data(), planePos.size() * sizeof(int), 0},
    });
  }
  size_t total = 0;
  for (auto& part : parts) {
    part.offset = total;
    total += align_up(std::max<size_t>(part.bytes, 1));
  }
  std::vector<char> host(total, 0);
  for (auto& part : parts) {
    if (part.bytes) std::memcpy(host.data() + part.offset, part.src, part.bytes);
  }
  tables_ = DeviceBuffer(total);
  check_cuda(cudaMemcpy(tables_.get(), host.data(), total, cudaMemcpyHostToDevice));
  char* d = static_cast<char*>(tables_.get());

  base_.dimX = p.dimX;
  base_.dimY = p.dimY;
  base_.dimZ = p.dimZ;
  base_.dimXFreq = p.dimXFreq;
  base_.numSticks = ns;
  base_.numColumns = ncol;
  base_.r2c = p.type == SPFFT_TRANS_R2C ? 1 : 0;
  base_.zeroZeroStick = (base_.r2c && p.zeroZeroStick < ns) ? p.zeroZeroStick : -1;
  // Size-specialised kernels where the lengths are supported and shared memory allows (keeping
  // 1 KB of the opt-in maximum for the kernels' static shared memory).
  {
    const size_t optin = static_cast<size_t>(max_smem_optin(device)) - 1024;
    FastArgs<T> a;
    const int nz = p.dimZ;
    if (ns > 0 && fast_dispatch<T>(FastOp::Has, nz, false, a) && prepare_fast_once<T>(device, nz)) {
      size_t sm = 0;
      a.smemOut = &sm;
      // Sticks per block: of 32, 24, 16, 12 and 8, the one with the least modelled time, waves of
      // resident blocks x (sticks per block + 4 for the fixed cost of a block), ties to the larger
      // (measured on 192^3 R2C: 12 in double-float, 8 in FP32).
      int numSms = 0;
      check_cuda(cudaDeviceGetAttribute(&numSms, cudaDevAttrMultiProcessorCount, device));
      int spb = 32;
      long long best = -1;
      for (int cand : {32, 24, 16, 12, 8}) {
        a.param = cand;
        fast_dispatch<T>(FastOp::ZSmem, nz, false, a);
        if (sm > kFastZBudget) continue;
        size_t perSm = 1;
        a.smemOut = &perSm;
        fast_dispatch<T>(FastOp::ZOccupancy, nz, false, a);
        a.smemOut = &sm;
        const long long slots = static_cast<long long>(numSms) * static_cast<long long>(perSm);
        const long long blocks = (ns + cand - 1) / cand;
        const long long cost = (blocks + slots - 1) / slots * (cand + 4);
        if (best < 0 || cost < best) {
          best = cost;
          spb = cand;
        }
      }
      a.param = spb;
      fast_dispatch<T>(FastOp::ZSmem, nz, false, a);
      if (sm <= optin) {
        fastZ_ = true;
        fastSpb_ = spb;
      }
      // autotuner candidates: also 6 sticks, which with three z blocks per SM (the three-pass
      // double-float z kernels) spreads a few thousand sticks over more than one wave
      for (int cand : {32, 24, 16, 12, 8, 6}) {
        a.param = cand;
        fast_dispatch<T>(FastOp::ZSmem, nz, false, a);
        if (sm <= optin) zCands_.push_back(cand);
      }
      // SPFFT_GB300_Z_STICKS=n: sticks per z block, where n is one of the candidates
      if (const char* zs = std::getenv("SPFFT_GB300_Z_STICKS")) {
        const int want = std::atoi(zs);
        if (fastZ_ && std::find(zCands_.begin(), zCands_.end(), want) != zCands_.end()) fastSpb_ = want;
      }
    }
    const bool r2c = p.type == SPFFT_TRANS_R2C;
    // Candidate plane strategies. SPFFT_GB300_PLANE=fused|split|generic forces one (when it is
    // available for this shape); otherwise fused where two blocks fit an SM and there is a plane
    // per SM, then split, then fused with one block per SM, then generic.
    bool fusedOk = false, splitOk = false;
    int fusedRows = 0, cpb = 0, rpb = 0;
    if (ns > 0 && p.dimX == p.dimY && fast_dispatch<T>(FastOp::Has, p.dimX, r2c, a) &&
        prepare_fast_once<T>(device, p.dimX)) {
      size_t sm = 0;
      a.smemOut = &sm;
      a.numColumns = ncol;
      // x chunk buffer of 2 * rows rows: two 256-thread blocks per SM when the block fits 112 KB
      // of shared memory, else the largest (<= 64 rows) that fits one 512-thread block per SM.
      for (int rows = 16; rows >= 1; rows /= 2) {
        a.param = rows;
        fast_dispatch<T>(FastOp::PlaneSmem, p.dimX, r2c, a);
        if (sm <= 112 * 1024) {
          if (!fusedOk) {
            fusedOk = true;
            fusedRows = rows;
            fusedThreads_ = 256;
          }
          fusedCands_.emplace_back(rows, 256);
        }
      }
      for (int rows = 32; rows >= 1; rows /= 2) {
        a.param = rows;
        fast_dispatch<T>(FastOp::PlaneSmem, p.dimX, r2c, a);
        if (sm <= optin) {
          if (!fusedOk) {
            fusedOk = true;
            fusedRows = rows;
            fusedThreads_ = 512;
          }
          fusedCands_.emplace_back(rows, 512);
        }
      }
    }
    if (ns > 0 && fast_dispatch<T>(FastOp::Has, p.dimX, r2c, a) &&
        fast_dispatch<T>(FastOp::Has, p.dimY, r2c, a) && prepare_fast_once<T>(device, p.dimX) &&
        prepare_fast_once<T>(device, p.dimY)) {
      size_t sm = 0;
      a.smemOut = &sm;
      a.numColumns = ncol;
      // Columns per y block and rows per x block: 16 and 32 (>= 256 work items per pass for the
      // usual lengths) while a block stays within 100 KB, smaller otherwise.
      const size_t budget = 100 * 1024;
      for (cpb = 16; cpb > 1; cpb /= 2) {
        a.param = cpb;
        fast_dispatch<T>(FastOp::YSmem, p.dimY, r2c, a);
        if (sm <= budget) break;
      }
      a.param = cpb;
      fast_dispatch<T>(FastOp::YSmem, p.dimY, r2c, a);
      const bool yFits = sm <= optin;
      for (rpb = 32; rpb > 1; rpb /= 2) {
        a.param = rpb;
        fast_dispatch<T>(FastOp::XSmem, p.dimX, r2c, a);
        if (sm <= budget) break;
      }
      a.param = rpb;
      fast_dispatch<T>(FastOp::XSmem, p.dimX, r2c, a);
      splitOk = yFits && sm <= optin;
      cpb = std::min(cpb, std::max(1, ncol));
      rpb = std::min(rpb, p.dimY);
      if (splitOk) {
        // the x backward kernel holds the compact rows besides the FFT rows, so it may want fewer
        // rows per block (more blocks per SM) than the x forward kernel: its own candidates
        std::vector<int> rowsB;
        for (int r : {8, 12, 16, 24, 32}) {
          a.param = r;
          fast_dispatch<T>(FastOp::XSmem, p.dimX, r2c, a);
          if (sm <= optin && r <= p.dimY) rowsB.push_back(r);
        }
        for (int c : {4, 8, 16, 32}) {
          a.param = c;
          fast_dispatch<T>(FastOp::YSmem, p.dimY, r2c, a);
          if (sm > optin || c > std::max(1, ncol)) continue;
          for (int r : {8, 16, 32}) {
            a.param = r;
            fast_dispatch<T>(FastOp::XSmem, p.dimX, r2c, a);
            if (sm > optin || r > p.dimY) continue;
            for (int rb : rowsB) splitCands_.push_back({c, r, rb});
          }
        }
        const std::array<int, 3> dflt{cpb, rpb, rpb};
        if (std::find(splitCands_.begin(), splitCands_.end(), dflt) == splitCands_.end()) {
          splitCands_.push_back(dflt);
        }
      }
    }
    const char* force = std::getenv("SPFFT_GB300_PLANE");
    const std::string want = force ? force : "";
    int numSms = 0;
    check_cuda(cudaDeviceGetAttribute(&numSms, cudaDevAttrMultiProcessorCount, device));
    if (want == "generic") {
      planePath_ = PlanePath::Generic;
    } else if (want == "fused" && fusedOk) {
      planePath_ = PlanePath::Fused;
    } else if (want == "split" && splitOk) {
      planePath_ = PlanePath::Split;
    } else if (fusedOk && fusedThreads_ == 256 && p.dimZ >= numSms) {
      // two fused plane blocks per SM and at least one plane per SM: the compact planes never go
      // to HBM (192^3 R2C FP32: 12.6k against 11.9k pairs/s split)
      planePath_ = PlanePath::Fused;
    } else if (splitOk) {
      planePath_ = PlanePath::Split;
    } else if (fusedOk) {
      planePath_ = PlanePath::Fused;
    }
    fastRows_ = fusedRows;
    splitCpb_ = cpb;
    splitRpb_ = rpb;
    splitRpbB_ = rpb;
    // SPFFT_GB300_XB_ROWS=n: rows per x backward block, where n is one of the candidates
    if (const char* xb = std::getenv("SPFFT_GB300_XB_ROWS")) {
      const int want = std::atoi(xb);
      for (const auto& c : splitCands_) {
        if (c[0] == cpb && c[1] == rpb && c[2] == want) splitRpbB_ = want;
      }
    }
    // Passes that can run the swapped two-pass split or the three-pass split of their length
    // (FastOp::SplitRadix): the specialised z pass and the split y passes.
    // SPFFT_GB300_SPLITS=zb,zf,yb,yf (each 0 default, 1 swapped, 2 three-pass) chooses per pass at
    // creation (z backward, z forward, y backward, y forward).
    {
      size_t rad = 0;
      a.smemOut = &rad;
      a.split = 1;
      a.param = 0;
      zSwap_ = fastZ_ && fast_dispatch<T>(FastOp::SplitRadix, nz, false, a) && rad > 0;
      a.param = 1;
      ySwap_ = splitOk && fast_dispatch<T>(FastOp::SplitRadix, p.dimY, r2c, a) && rad > 0;
      a.split = 2;
      a.param = 0;
      zThree_ = fastZ_ && fast_dispatch<T>(FastOp::SplitRadix, nz, false, a) && rad > 0;
      a.param = 1;
      yThree_ = splitOk && fast_dispatch<T>(FastOp::SplitRadix, p.dimY, r2c, a) && rad > 0;
      a.split = 0;
      if (const char* sw = std::getenv("SPFFT_GB300_SPLITS")) {
        int v[4] = {0, 0, 0, 0};
        if (std::sscanf(sw, "%d,%d,%d,%d", &v[0], &v[1], &v[2], &v[3]) == 4) {
          for (int i = 0; i < 4; ++i) splitChoice_[i] = split_valid(i, v[i], i < 2 || planePath_ == PlanePath::Split) ? v[i] : 0;
        }
      }
    }
  }

  radixCands_[0] = radix_plan_candidates(p.dimZ);
  radixCands_[1] = radix_plan_candidates(p.dimY);
  radixCands_[2] = radix_plan_candidates(p.dimX);
  base_.fz = radixCands_[0][0];
  base_.fy = radixCands_[1][0];
  base_.fx = radixCands_[2][0];
  base_.twz = reinterpret_cast<const T*>(d + parts[0].offset);
  base_.twy = reinterpret_cast<const T*>(d + parts[1].offset);
  base_.twx = reinterpret_cast<const T*>(d + parts[2].offset);
  if (dt) {
    base_.stickColumn = dt->stickColumn;
    base_.stickY = dt->stickY;
    base_.stickPlanePos = dt->stickPlanePos;
    base_.columnX = dt->columnX;
    base_.columnStickStart = dt->columnStickStart;
    base_.entryPos = dt->entryPos;
    base_.entryUser = dt->entryUser;
    base_.stickEntryStart = dt->stickEntryStart;
    base_.hermitianWeight = dt->hermitianWeight;
  } else {
    base_.stickColumn = reinterpret_cast<const int*>(d + parts[3].offset);
    base_.stickY = reinterpret_cast<const int*>(d + parts[4].offset);
    base_.stickPlanePos = reinterpret_cast<const int*>(d + parts[11].offset);
    base_.columnX = reinterpret_cast<const int*>(d + parts[5].offset);
    base_.columnStickStart = reinterpret_cast<const int*>(d + parts[6].offset);
    base_.entryPos = reinterpret_cast<const int*>(d + parts[7].offset);
    base_.entryUser = reinterpret_cast<const int*>(d + parts[8].offset);
    base_.stickEntryStart = reinterpret_cast<const int*>(d + parts[9].offset);
    base_.hermitianWeight = hp->hermitianWeight.empty()
                                ? nullptr
                                : reinterpret_cast<const unsigned char*>(d + parts[10].offset);
  }
  numValues_ = nv;

  int uniform = 0;
  if (const char* env = std::getenv("SPFFT_GB300_STAGED_CHUNKS")) {
    const int want = std::atoi(env);
    if (want >= 1 && want <= kMaxStagedChunks) uniform = want;
  }
  stagedSizes_ = staged_chunk_sizes(p.dimZ, uniform);

  // Forward scaling factor T(1 / (Nx Ny Nz)) computed in double (execution_gpu.cpp:58-59).
  scale_ = static_cast<T>(1.0 / (static_cast<double>(p.dimX) * p.dimY * p.dimZ));
}

template <typename T>
PlanView<T> GpuPlan<T>::view(void* scratch) const {
  PlanView<T> v = base_;
  char* s = static_cast<char*>(scratch);
  v.sticks = reinterpret_cast<T*>(s + layout_.sticksOffset);
  v.planes = reinterpret_cast<T*>(s + layout_.planesOffset);
  v.planeExp = reinterpret_cast<int*>(s + layout_.expOffset);
  v.planesRaw = sizeof(T) == sizeof(double) ? 1 : 0;
  v.stickExp = reinterpret_cast<int*>(s + layout_.stickExpOffset);
  v.sticksRaw = (sizeof(T) == sizeof(double) && fastZ_ && planePath_ == PlanePath::Split) ? 1 : 0;
  return v;
}

namespace {
inline void mark(const StageEvents* e, int i, cudaStream_t s) {
  if (e) check_cuda(cudaEventRecord(e->ev[i], s));
}
}  // namespace

// Complex data must be aligned to its complex size (the kernels move whole complex values). A
// real R2C space buffer only needs T alignment; unaligned ones take the generic plane passes.
template <typename T>
void GpuPlan<T>::check_alignment(const T* values, const T* space, bool* planeAligned) const {
  const uintptr_t c = 2 * sizeof(T);
  if (base_.numSticks > 0 && values && reinterpret_cast<uintptr_t>(values) % c != 0) {
    throw InvalidParameterError();
  }
  const bool aligned = reinterpret_cast<uintptr_t>(space) % c == 0;
  if (!base_.r2c && !aligned) throw InvalidParameterError();
  if (reinterpret_cast<uintptr_t>(space) % sizeof(T) != 0) throw InvalidParameterError();
  *planeAligned = aligned;
}

template <typename T>
void GpuPlan<T>::backward(const T* values, T* space, void* scratch, cudaStream_t stream,
                          const StageEvents* events) const {
  bool aligned = true;
  check_alignment(values, space, &aligned);
  PlanView<T> v = view(scratch);
  // double-float sticks only between the fast z and the split y kernels (an unaligned R2C space
  // buffer sends this call through the generic plane passes, which exchange binary64 sticks)
  if (!(planePath_ == PlanePath::Split && aligned)) v.sticksRaw = 0;
  FastArgs<T> a;
  a.plan = &v;
  a.stream = stream;
  mark(events, 0, stream);
  if (fastZ_) {
    a.param = fastSpb_;
    a.in = values;
    a.split = splitChoice_[0];
    fast_dispatch<T>(FastOp::ZBackward, base_.dimZ, base_.r2c != 0, a);
  } else {
    check_launch(launch_generic<T>(GenericPass::ZBackward, v, config_, values, nullptr, T(0), stream));
  }
  check_launch(cudaGetLastError());
  mark(events, 1, stream);
  if (planePath_ == PlanePath::Fused && aligned) {
    a.param = fastRows_;
    a.param2 = fusedThreads_;
    a.out = space;
    fast_dispatch<T>(FastOp::PlaneBackward, base_.dimX, base_.r2c != 0, a);
    check_launch(cudaGetLastError());
    mark(events, 2, stream);
  } else if (planePath_ == PlanePath::Split && aligned) {
    a.param = splitCpb_;
    a.split = splitChoice_[2];
    fast_dispatch<T>(FastOp::YBackward, base_.dimY, base_.r2c != 0, a);
    check_launch(cudaGetLastError());
    mark(events, 2, stream);
    a.param = splitRpbB_;
    a.out = space;
    fast_dispatch<T>(FastOp::XBackward, base_.dimX, base_.r2c != 0, a);
    check_launch(cudaGetLastError());
  } else {
    check_launch(launch_generic<T>(GenericPass::YBackward, v, config_, nullptr, nullptr, T(0), stream));
    mark(events, 2, stream);
    check_launch(launch_generic<T>(GenericPass::XBackward, v, config_, nullptr, space, T(0), stream));
  }
  mark(events, 3, stream);
}

// Adjoint of backward: the unnormalised forward transform with its gather (the transpose of the
// backward's scatter), times the hermitian multiplicity of each R2C value.
template <typename T>
void GpuPlan<T>::adjoint_backward(const T* gradSpace, T* gradValues, void* scratch, cudaStream_t stream) const {
  forward(gradSpace, gradValues, false, scratch, stream);
  if (base_.hermitianWeight) {
    check_launch(launch_weight_values<T>(gradValues, gradValues, base_.hermitianWeight, numValues_, T(1), 0,
                                         stream));
  }
}

// Adjoint of forward: the backward transform of the value gradient, divided by the R2C
// multiplicities (the backward's implied mirror terms must not be counted twice) and scaled like
// the forward.
template <typename T>
void GpuPlan<T>::adjoint_forward(const T* gradValues, T* gradSpace, bool scaled, void* scratch,
                                 cudaStream_t stream) const {
  const T* in = gradValues;
  if (base_.hermitianWeight || scaled) {
    T* st = staging(scratch);
    check_launch(launch_weight_values<T>(gradValues, st, base_.hermitianWeight, numValues_,
                                         scaled ? scale_ : T(1), 1, stream));
    in = st;
  }
  backward(in, gradSpace, scratch, stream);
}

template <typename T>
void GpuPlan<T>::forward(const T* space, T* values, bool scaled, void* scratch,
                         cudaStream_t stream, const StageEvents* events) const {
  bool aligned = true;
  check_alignment(values, space, &aligned);
  PlanView<T> v = view(scratch);
  // double-float sticks only between the fast z and the split y kernels (an unaligned R2C space
  // buffer sends this call through the generic plane passes, which exchange binary64 sticks)
  if (!(planePath_ == PlanePath::Split && aligned)) v.sticksRaw = 0;
  FastArgs<T> a;
  a.plan = &v;
  a.stream = stream;
  mark(events, 0, stream);
  if (planePath_ == PlanePath::Fused && aligned) {
    a.param = fastRows_;
    a.param2 = fusedThreads_;
    a.in = space;
    fast_dispatch<T>(FastOp::PlaneForward, base_.dimX, base_.r2c != 0, a);
    check_launch(cudaGetLastError());
    mark(events, 1, stream);
  } else if (planePath_ == PlanePath::Split && aligned) {
    a.param = splitRpb_;
    a.in = space;
    fast_dispatch<T>(FastOp::XForward, base_.dimX, base_.r2c != 0, a);
    check_launch(cudaGetLastError());
    mark(events, 1, stream);
    a.param = splitCpb_;
    a.split = splitChoice_[3];
    fast_dispatch<T>(FastOp::YForward, base_.dimY, base_.r2c != 0, a);
    check_launch(cudaGetLastError());
  } else {
    check_launch(launch_generic<T>(GenericPass::XForward, v, config_, space, nullptr, T(0), stream));
    mark(events, 1, stream);
    check_launch(launch_generic<T>(GenericPass::YForward, v, config_, nullptr, nullptr, T(0), stream));
  }
  mark(events, 2, stream);
  const T scale = scaled ? scale_ : T(0);
  if (fastZ_) {
    a.param = fastSpb_;
    a.out = values;
    a.scale = scale;
    a.split = splitChoice_[1];
    fast_dispatch<T>(FastOp::ZForward, base_.dimZ, base_.r2c != 0, a);
    check_launch(cudaGetLastError());
  } else {
    check_launch(launch_generic<T>(GenericPass::ZForward, v, config_, nullptr, values, scale, stream));
  }
  mark(events, 3, stream);
}

template <typename T>
bool GpuPlan<T>::forward_staged(const T* hostSpace, T* devSpace, T* values, bool scaled, void* scratch,
                                cudaStream_t stream, cudaStream_t copyStream, cudaEvent_t* events) const {
  bool aligned = true;
  check_alignment(values, devSpace, &aligned);
  if (planePath_ != PlanePath::Split || !aligned) return false;
  const PlanView<T> v = view(scratch);
  const size_t plane = static_cast<size_t>(base_.dimX) * base_.dimY * (base_.r2c ? 1 : 2);
  const int nChunks = static_cast<int>(stagedSizes_.size());
  // the copies overwrite devSpace: start them after the work already on `stream`
  check_cuda(cudaEventRecord(events[kMaxStagedChunks], stream));
  check_cuda(cudaStreamWaitEvent(copyStream, events[kMaxStagedChunks], 0));
  FastArgs<T> a;
  a.plan = &v;
  a.stream = stream;
  a.param = splitRpb_;
  a.in = devSpace;
  // each chunk's x and y passes run while the next chunk is copied (the y-FFT of plane z needs
  // only plane z)
  // the chunks in decreasing size: the passes left after the last copy are the smallest chunk's
  for (int c = 0, z0 = 0; c < nChunks; z0 += stagedSizes_[nChunks - 1 - c], ++c) {
    const int cnt = stagedSizes_[nChunks - 1 - c];
    check_cuda(cudaMemcpyAsync(devSpace + z0 * plane, hostSpace + z0 * plane, cnt * plane * sizeof(T),
                               cudaMemcpyHostToDevice, copyStream));
    check_cuda(cudaEventRecord(events[c], copyStream));
    check_cuda(cudaStreamWaitEvent(stream, events[c], 0));
    a.zBegin = z0;
    a.zCount = cnt;
    a.param = splitRpb_;
    fast_dispatch<T>(FastOp::XForward, base_.dimX, base_.r2c != 0, a);
    check_launch(cudaGetLastError());
    a.param = splitCpb_;
    a.split = splitChoice_[3];
    fast_dispatch<T>(FastOp::YForward, base_.dimY, base_.r2c != 0, a);
    check_launch(cudaGetLastError());
  }
  a.zBegin = 0;
  a.zCount = -1;
  const T scale = scaled ? scale_ : T(0);
  if (fastZ_) {
    a.param = fastSpb_;
    a.out = values;
    a.scale = scale;
    a.split = splitChoice_[1];
    fast_dispatch<T>(FastOp::ZForward, base_.dimZ, base_.r2c != 0, a);
    check_launch(cudaGetLastError());
  } else {
    check_launch(launch_generic<T>(GenericPass::ZForward, v, config_, nullptr, values, scale, stream));
  }
  return true;
}

template <typename T>
bool GpuPlan<T>::backward_staged(const T* values, T* devSpace, T* hostSpace, void* scratch, cudaStream_t stream,
                                 cudaStream_t copyStream, cudaEvent_t* events) const {
  bool aligned = true;
  check_alignment(values, devSpace, &aligned);
  if (planePath_ != PlanePath::Split || !aligned) return false;
  const PlanView<T> v = view(scratch);
  FastArgs<T> a;
  a.plan = &v;
  a.stream = stream;
  if (fastZ_) {
    a.param = fastSpb_;
    a.in = values;
    a.split = splitChoice_[0];
    fast_dispatch<T>(FastOp::ZBackward, base_.dimZ, base_.r2c != 0, a);
  } else {
    check_launch(launch_generic<T>(GenericPass::ZBackward, v, config_, values, nullptr, T(0), stream));
  }
  check_launch(cudaGetLastError());
  const size_t plane = static_cast<size_t>(base_.dimX) * base_.dimY * (base_.r2c ? 1 : 2);
  a.out = devSpace;
  // each chunk's y and x passes, then its copy back, which overlaps the next chunk's passes (the
  // chunks in increasing size: the first copy waits for the smallest chunk's passes only)
  for (int c = 0, z0 = 0; c < static_cast<int>(stagedSizes_.size()); z0 += stagedSizes_[c], ++c) {
    const int cnt = stagedSizes_[c];
    a.zBegin = z0;
    a.zCount = cnt;
    a.param = splitCpb_;
    a.split = splitChoice_[2];
    fast_dispatch<T>(FastOp::YBackward, base_.dimY, base_.r2c != 0, a);
    check_launch(cudaGetLastError());
    a.param = splitRpbB_;
    fast_dispatch<T>(FastOp::XBackward, base_.dimX, base_.r2c != 0, a);
    check_launch(cudaGetLastError());
    check_cuda(cudaEventRecord(events[c], stream));
    check_cuda(cudaStreamWaitEvent(copyStream, events[c], 0));
    check_cuda(cudaMemcpyAsync(hostSpace + z0 * plane, devSpace + z0 * plane, cnt * plane * sizeof(T),
                               cudaMemcpyDeviceToHost, copyStream));
  }
  // `stream` continues once every chunk is back in host memory
  check_cuda(cudaEventRecord(events[kMaxStagedChunks], copyStream));
  check_cuda(cudaStreamWaitEvent(stream, events[kMaxStagedChunks], 0));
  return true;
}

template <typename T>
typename GpuPlan<T>::Tuning GpuPlan<T>::tuning() const {
  Tuning t;
  t.spb = fastZ_ ? fastSpb_ : 0;
  t.path = planePath_ == PlanePath::Fused ? 1 : planePath_ == PlanePath::Split ? 2 : 0;
  if (t.path == 1) {
    t.fusedRows = fastRows_;
    t.fusedThreads = fusedThreads_;
  }
  if (t.path == 2) {
    t.cpb = splitCpb_;
    t.rpb = splitRpb_;
    t.rpbB = splitRpbB_;
  }
  for (int d = 0; d < 3; ++d) t.radix[d] = radixChoice_[d];
  for (int i = 0; i < 2; ++i) t.split[i] = fastZ_ ? splitChoice_[i] : 0;
  for (int i = 2; i < 4; ++i) t.split[i] = t.path == 2 ? splitChoice_[i] : 0;
  return t;
}

template <typename T>
void GpuPlan<T>::split_radices(int* radices) const {
  for (int i = 0; i < 6; ++i) radices[i] = 0;
  FastArgs<T> a;
  size_t rad = 0;
  a.smemOut = &rad;
  const bool r2c = base_.r2c != 0;
  auto query = [&](int which, int split, int n) {
    a.param = which;
    a.split = split;
    rad = 0;
    return fast_dispatch<T>(FastOp::SplitRadix, n, r2c, a) ? static_cast<int>(rad) : 0;
  };
  if (fastZ_) {
    radices[0] = query(0, splitChoice_[0], base_.dimZ);
    radices[1] = query(0, splitChoice_[1], base_.dimZ);
  }
  if (planePath_ == PlanePath::Split) {
    radices[2] = query(1, splitChoice_[2], base_.dimY);
    radices[3] = query(1, splitChoice_[3], base_.dimY);
    radices[4] = radices[5] = query(4, 0, base_.dimX);
  } else if (planePath_ == PlanePath::Fused) {
    radices[2] = query(2, 0, base_.dimY);
    radices[3] = query(3, 0, base_.dimY);
    radices[4] = radices[5] = query(4, 0, base_.dimX);
  }
}

template <typename T>
void GpuPlan<T>::split_stages(int* stages) const {
  int first[6];
  split_radices(first);
  for (int i = 0; i < 18; ++i) stages[i] = 0;
  const int lens[6] = {base_.dimZ, base_.dimZ, base_.dimY, base_.dimY,
                       base_.r2c ? base_.dimX / 2 : base_.dimX, base_.r2c ? base_.dimX / 2 : base_.dimX};
  for (int i = 0; i < 6; ++i) {
    if (first[i] <= 0) continue;
    const int b = lens[i] / first[i];
    stages[3 * i] = first[i];
    stages[3 * i + 1] = b;
    if (i < 4 && splitChoice_[i] == 2) {
      FastArgs<T> a;
      size_t b1 = 0;
      a.smemOut = &b1;
      if (fast_dispatch<T>(FastOp::ThreePassFactor, i < 2 ? base_.dimZ : base_.dimY, base_.r2c != 0, a) && b1 > 0) {
        stages[3 * i + 1] = static_cast<int>(b1);
        stages[3 * i + 2] = b / static_cast<int>(b1);
      }
    }
  }
}

template <typename T>
std::vector<typename GpuPlan<T>::Tuning> GpuPlan<T>::candidates() const {
  std::vector<int> zs = zCands_;
  if (zs.empty()) zs.push_back(0);
  std::vector<Tuning> out;
  for (int spb : zs) {
    Tuning t;
    t.spb = spb;
    for (const auto& f : fusedCands_) {
      t.path = 1;
      t.fusedRows = f.first;
      t.fusedThreads = f.second;
      t.cpb = t.rpb = t.rpbB = 0;
      out.push_back(t);
    }
    for (const auto& sp : splitCands_) {
      t.path = 2;
      t.fusedRows = t.fusedThreads = 0;
      t.cpb = sp[0];
      t.rpb = sp[1];
      t.rpbB = sp[2];
      out.push_back(t);
    }
    if (fusedCands_.empty() && splitCands_.empty()) {
      t.path = 0;
      t.fusedRows = t.fusedThreads = t.cpb = t.rpb = t.rpbB = 0;
      out.push_back(t);
    }
  }
  return out;
}

template <typename T>
void GpuPlan<T>::set_tuning(const Tuning& t) {
  bool ok = false;
  for (const Tuning& c : candidates()) {
    ok |= c.spb == t.spb && c.path == t.path && c.fusedRows == t.fusedRows && c.fusedThreads == t.fusedThreads &&
          c.cpb == t.cpb && c.rpb == t.rpb && c.rpbB == t.rpbB;
  }
  for (int d = 0; d < 3; ++d) ok &= t.radix[d] >= 0 && t.radix[d] < static_cast<int>(radixCands_[d].size());
  for (int i = 0; i < 4; ++i) ok &= split_valid(i, t.split[i], i < 2 ? t.spb > 0 : t.path == 2);
  if (!ok) throw InvalidParameterError();
  for (int i = 0; i < 4; ++i) splitChoice_[i] = t.split[i];
  for (int d = 0; d < 3; ++d) radixChoice_[d] = t.radix[d];
  base_.fz = radixCands_[0][t.radix[0]];
  base_.fy = radixCands_[1][t.radix[1]];
  base_.fx = radixCands_[2][t.radix[2]];
  if (t.spb > 0) fastSpb_ = t.spb;
  planePath_ = t.path == 1 ? PlanePath::Fused : t.path == 2 ? PlanePath::Split : PlanePath::Generic;
  if (t.path == 1) {
    fastRows_ = t.fusedRows;
    fusedThreads_ = t.fusedThreads;
  }
  if (t.path == 2) {
    splitCpb_ = t.cpb;
    splitRpb_ = t.rpb;
    splitRpbB_ = t.rpbB;
  }
}

template <typename T>
float GpuPlan<T>::autotune(T* values, T* space, void* scratch, cudaStream_t stream, int reps) {
  if (reps < 1) throw InvalidParameterError();
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  check_cuda(cudaEventCreate(&e0));
  check_cuda(cudaEventCreate(&e1));
  auto time_pair = [&](const Tuning& t) {
    set_tuning(t);
    backward(values, space, scratch, stream);  // warm-up
    forward(space, values, true, scratch, stream);
    check_cuda(cudaEventRecord(e0, stream));
    for (int r = 0; r < reps; ++r) {
      backward(values, space, scratch, stream);
      forward(space, values, true, scratch, stream);
    }
    check_cuda(cudaEventRecord(e1, stream));
    check_cuda(cudaEventSynchronize(e1));
    float ms = 0.0f;
    check_cuda(cudaEventElapsedTime(&ms, e0, e1));
    return ms / reps;
  };
  const Tuning initial = tuning();
  Tuning best = initial;
  float bestMs = 0.0f;
  try {
    bestMs = time_pair(best);
    // pass 0: z shapes with the current plane strategy; pass 1: plane strategies with the best z
    // shape (the split choices carry over where the candidate keeps the pass on the same kernels)
    auto descend = [&](int pass) {
      const Tuning base = best;
      for (Tuning c : candidates()) {
        const bool zOnly = c.path == base.path && c.fusedRows == base.fusedRows &&
                           c.fusedThreads == base.fusedThreads && c.cpb == base.cpb && c.rpb == base.rpb &&
                           c.rpbB == base.rpbB;
        const bool planeOnly = c.spb == base.spb;
        if ((pass == 0 && !zOnly) || (pass == 1 && !planeOnly)) continue;
        if (pass == 0 && c.spb == base.spb) continue;
        for (int d = 0; d < 3; ++d) c.radix[d] = base.radix[d];
        for (int i = 0; i < 4; ++i) c.split[i] = (i < 2 ? c.spb > 0 : c.path == 2) ? base.split[i] : 0;
        const float ms = time_pair(c);
        if (ms < bestMs) {
          bestMs = ms;
          best = c;
        }
      }
    };
    descend(0);
    descend(1);
    // the split of each specialised z and split-y pass: the default order, the swapped order or
    // three passes; for the z passes jointly with the sticks per z block (a three-pass z kernel
    // fits more blocks per SM, so its best block shape differs)
    for (int i = 0; i < 4; ++i) {
      if (i < 2 ? best.spb == 0 : best.path != 2) continue;
      const Tuning base = best;
      const std::vector<int> shapes = i < 2 ? zCands_ : std::vector<int>{base.spb};
      for (int v = 0; v < 3; ++v) {
        if (!split_valid(i, v, true)) continue;
        for (int spb : shapes) {
          if (v == base.split[i] && spb == base.spb) continue;
          Tuning c = best;
          c.split[i] = v;
          c.spb = spb;
          const float ms = time_pair(c);
          if (ms < bestMs) {
            bestMs = ms;
            best = c;
          }
        }
      }
    }
    // radix plans of the lengths the generic kernels transform: z without specialised z kernels,
    // y and x on the generic plane path
    const bool generic[3] = {best.spb == 0, best.path == 0, best.path == 0};
    for (int d = 0; d < 3; ++d) {
      if (!generic[d]) continue;
      const Tuning base = best;
      for (int r = 0; r < static_cast<int>(radixCands_[d].size()); ++r) {
        if (r == base.radix[d]) continue;
        Tuning c = base;
        c.radix[d] = r;
        const float ms = time_pair(c);
        if (ms < bestMs) {
          bestMs = ms;
          best = c;
        }
      }
    }
  } catch (...) {
    (void)cudaEventDestroy(e0);
    (void)cudaEventDestroy(e1);
    set_tuning(initial);
    throw;
  }
  (void)cudaEventDestroy(e0);
  (void)cudaEventDestroy(e1);
  set_tuning(best);
  return bestMs;
}

namespace fast {
bool pdl_enabled() {
  static const bool on = [] {
    const char* e = std::getenv("SPFFT_GB300_PDL");
    return !(e && e[0] == '0');
  }();
  return on;
}
}  // namespace fast

size_t smem_optin(int device) { return static_cast<size_t>(max_smem_optin(device)); }
template <typename T>
bool fast_prepare(int device, int n) {
  FastArgs<T> a;
  return fast_dispatch<T>(FastOp::Has, n, false, a) && prepare_fast_once<T>(device, n);
}
template bool fast_prepare<double>(int, int);
template bool fast_prepare<float>(int, int);

template class GpuPlan<double>;
template class GpuPlan<float>;

}  // namespace gb300
}  // namespace spfft
