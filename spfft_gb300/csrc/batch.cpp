// BatchPlan: groups transforms by shape, uploads their plan views and bound buffer pointers, and
// runs each pass of each group as one batched launch.
#include "batch.hpp"

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <tuple>

#include "engine.hpp"
#include "kernels_fast.hpp"

namespace spfft {
namespace gb300 {

namespace {
constexpr size_t kAlign = 256;
inline size_t align_up(size_t v) { return (v + kAlign - 1) / kAlign * kAlign; }
constexpr size_t kZBudget = 56 * 1024, kPlaneBudget = 100 * 1024;
// A fused plane block (y and x passes of one plane with the compact plane on chip) within this
// budget runs two per SM (228 KB of shared memory per SM, 1 KB of it reserved per block).
constexpr size_t kFusedBudget = 112 * 1024;
}  // namespace

template <typename T>
struct BatchPlan<T>::Group {
  int nx = 0, ny = 0, nz = 0;
  bool r2c = false;
  std::vector<int> members;
  int spb = 0, cpb = 0, rpb = 0;
  size_t smemZ = 0, smemY = 0, smemX = 0;
  int blocksZ = 0, blocksY = 0, blocksX = 0;
  // fused plane passes: one block per plane, rows per x chunk (backward uses both halves of the
  // forward's double buffer, so twice the rows)
  bool fused = false;
  bool fusedAvail = false, splitAvail = false;  // which plane strategies fit (for the autotuner)
  std::vector<int> zCands;                      // sticks per z block that fit (for the autotuner)
  int rowsF = 0, rowsB = 0, blocksP = 0;
  int xGroups = 1;                // row groups of the fused plane passes' x pass
  std::vector<int> groupCands;    // valid row-group counts
  size_t smemP = 0;
  T scale = T(0);
  DeviceBuffer dev;
  size_t offViews = 0, offStartsZ = 0, offStartsY = 0, offStartsX = 0, offStartsP = 0, offValues = 0,
         offSpaces = 0;
  BatchView<T> view(size_t startsOff, T scaleValue) const {
    char* d = static_cast<char*>(dev.get());
    BatchView<T> v;
    v.views = reinterpret_cast<const PlanView<T>*>(d + offViews);
    v.starts = reinterpret_cast<const int*>(d + startsOff);
    v.count = static_cast<int>(members.size());
    v.in = nullptr;
    v.out = nullptr;
    v.scale = scaleValue;
    return v;
  }
};

template <typename T>
BatchPlan<T>::BatchPlan(std::vector<std::shared_ptr<TransformInternal<T>>> transforms)
    : transforms_(std::move(transforms)) {
  for (auto& t : transforms_) {
    if (!t) throw InvalidParameterError();
    tp_.push_back(t.get());
  }
  const int n = static_cast<int>(tp_.size());
  if (n == 0) throw InvalidParameterError();
  device_ = tp_[0]->device_id();
  for (int a = 0; a < n; ++a) {
    if (tp_[a]->device_id() != device_) throw InvalidParameterError();
    for (int b = a + 1; b < n; ++b) {
      if (tp_[a]->shared_grid(*tp_[b])) throw InvalidParameterError();
    }
  }
  DeviceGuard guard(device_);
  const size_t optin = smem_optin(device_) - 1024;

  // group by shape; transforms without specialised kernels for every length run one by one
  std::map<std::tuple<int, int, int, bool>, int> index;
  for (int t = 0; t < n; ++t) {
    const IndexPlan& ip = tp_[t]->index_plan();
    const bool r2c = ip.type == SPFFT_TRANS_R2C;
    const bool ok = ip.num_sticks() > 0 && fast_prepare<T>(device_, ip.dimX) &&
                    fast_prepare<T>(device_, ip.dimY) && fast_prepare<T>(device_, ip.dimZ);
    if (!ok) {
      fallback_.push_back(t);
      continue;
    }
    const auto key = std::make_tuple(ip.dimX, ip.dimY, ip.dimZ, r2c);
    auto it = index.find(key);
    if (it == index.end()) {
      it = index.emplace(key, static_cast<int>(groups_.size())).first;
      groups_.emplace_back(new Group());
      Group& g = *groups_.back();
      g.nx = ip.dimX;
      g.ny = ip.dimY;
      g.nz = ip.dimZ;
      g.r2c = r2c;
      g.scale = static_cast<T>(1.0 / (static_cast<double>(ip.dimX) * ip.dimY * ip.dimZ));
    }
    groups_[it->second]->members.push_back(t);
  }

  // tile shapes per group (sized for the group's widest plane) and device tables
  const char* planeEnv = std::getenv("SPFFT_GB300_BATCH_PLANE");
  const std::string planeMode = planeEnv ? planeEnv : "";
  std::vector<std::unique_ptr<Group>> kept;
  for (auto& gp : groups_) {
    Group& g = *gp;
    int maxCols = 1;
    for (int t : g.members) maxCols = std::max(maxCols, tp_[t]->index_plan().num_columns());
    FastArgs<T> a;
    size_t sm = 0;
    a.smemOut = &sm;
    for (g.spb = 32; g.spb > 1; g.spb /= 2) {
      a.param = g.spb;
      fast_dispatch<T>(FastOp::ZSmem, g.nz, g.r2c, a);
      if (sm <= kZBudget) break;
    }
    a.param = g.spb;
    fast_dispatch<T>(FastOp::ZSmem, g.nz, g.r2c, a);
    g.smemZ = sm;
    for (g.cpb = 16; g.cpb > 1; g.cpb /= 2) {
      a.param = g.cpb;
      fast_dispatch<T>(FastOp::YSmem, g.ny, g.r2c, a);
      if (sm <= kPlaneBudget) break;
    }
    a.param = g.cpb;
    fast_dispatch<T>(FastOp::YSmem, g.ny, g.r2c, a);
    g.smemY = sm;
    a.numColumns = maxCols;
    for (g.rpb = 32; g.rpb > 1; g.rpb /= 2) {
      a.param = g.rpb;
      fast_dispatch<T>(FastOp::XSmem, g.nx, g.r2c, a);
      if (sm <= kPlaneBudget) break;
    }
    a.param = g.rpb;
    fast_dispatch<T>(FastOp::XSmem, g.nx, g.r2c, a);
    g.smemX = sm;
    g.rpb = std::min(g.rpb, g.ny);
    // Fused plane passes for cubic planes whose compact plane fits two blocks per SM (the y and x
    // passes then never write the compact planes to HBM). SPFFT_GB300_BATCH_PLANE=split|fused
    // forces one (fused up to the opt-in shared memory limit).
    if (g.nx == g.ny && planeMode != "split") {
      const size_t limit = planeMode == "fused" ? optin : kFusedBudget;
      for (int rows = 16; rows >= 2; rows /= 2) {
        a.param = rows;
        fast_dispatch<T>(FastOp::PlaneSmem, g.nx, g.r2c, a);
        if (sm <= limit) {
          // the chunk buffer holds 2 * rows rows: the backward and (single-buffered, which measured
          // faster than double-buffered half chunks with two blocks per SM) the forward transform
          // chunks of that many rows
          g.fused = true;
          g.fusedAvail = true;
          g.rowsB = std::min(2 * rows, g.ny);
          g.rowsF = g.rowsB;
          g.smemP = sm;
          // row groups of the x pass: whole warps per group, at least one row per group chunk
          constexpr int threads = batch_plane_threads<T>();
          for (int gr : {1, 2, 3, 4}) {
            if (threads % gr == 0 && (threads / gr) % 32 == 0 && g.rowsB / gr >= 1) g.groupCands.push_back(gr);
          }
          // four groups in FP32 (192^3 R2C, 64 transforms: 26.2k against 25.3k pairs/s with one);
          // SPFFT_GB300_BATCH_ROW_GROUPS=n starts with n row groups where n is valid
          if (sizeof(T) == sizeof(float) &&
              std::find(g.groupCands.begin(), g.groupCands.end(), 4) != g.groupCands.end()) {
            g.xGroups = 4;
          }
          if (const char* env = std::getenv("SPFFT_GB300_BATCH_ROW_GROUPS")) {
            const int want = std::atoi(env);
            if (std::find(g.groupCands.begin(), g.groupCands.end(), want) != g.groupCands.end()) g.xGroups = want;
          }
          // SPFFT_GB300_BATCH_FWD_ROWS=r: forward chunks of r rows (r <= rowsB / 2 double-buffers
          // them per row group)
          if (const char* env = std::getenv("SPFFT_GB300_BATCH_FWD_ROWS")) {
            const int want = std::atoi(env);
            if (want >= g.xGroups && want <= g.rowsB) g.rowsF = want;
          }
          break;
        }
      }
    }
    const bool splitFits = g.smemY <= optin && g.smemX <= optin;
    g.splitAvail = splitFits;
    for (int cand : {8, 16, 32}) {
      a.param = cand;
      fast_dispatch<T>(FastOp::ZSmem, g.nz, g.r2c, a);
      if (sm <= optin) g.zCands.push_back(cand);
    }
    if (g.smemZ > optin || (!g.fused && !splitFits)) {
      for (int t : g.members) fallback_.push_back(t);
      continue;
    }
    const size_t m = g.members.size();
    g.offViews = 0;
    g.offStartsZ = align_up(m * sizeof(PlanView<T>));
    g.offStartsY = g.offStartsZ + align_up((m + 1) * sizeof(int));
    g.offStartsX = g.offStartsY + align_up((m + 1) * sizeof(int));
    g.offStartsP = g.offStartsX + align_up((m + 1) * sizeof(int));
    g.offValues = g.offStartsP + align_up((m + 1) * sizeof(int));
    g.offSpaces = g.offValues + align_up(m * sizeof(T*));
    g.dev = DeviceBuffer(g.offSpaces + align_up(m * sizeof(T*)));
    std::vector<int> sz(m + 1, 0), sy(m + 1, 0), sx(m + 1, 0), sp(m + 1, 0);
    for (size_t i = 0; i < m; ++i) {
      const IndexPlan& ip = tp_[g.members[i]]->index_plan();
      sz[i + 1] = sz[i] + (ip.num_sticks() + g.spb - 1) / g.spb;
      sy[i + 1] = sy[i] + ((ip.num_columns() + g.cpb - 1) / g.cpb) * ip.dimZ;
      sx[i + 1] = sx[i] + ((ip.dimY + g.rpb - 1) / g.rpb) * ip.dimZ;
      sp[i + 1] = sp[i] + ip.dimZ;
    }
    g.blocksZ = sz[m];
    g.blocksY = sy[m];
    g.blocksX = sx[m];
    g.blocksP = sp[m];
    char* d = static_cast<char*>(g.dev.get());
    check_cuda(cudaMemcpy(d + g.offStartsZ, sz.data(), (m + 1) * sizeof(int), cudaMemcpyHostToDevice));
    check_cuda(cudaMemcpy(d + g.offStartsY, sy.data(), (m + 1) * sizeof(int), cudaMemcpyHostToDevice));
    check_cuda(cudaMemcpy(d + g.offStartsX, sx.data(), (m + 1) * sizeof(int), cudaMemcpyHostToDevice));
    check_cuda(cudaMemcpy(d + g.offStartsP, sp.data(), (m + 1) * sizeof(int), cudaMemcpyHostToDevice));
    kept.push_back(std::move(gp));
  }
  groups_ = std::move(kept);
  std::sort(fallback_.begin(), fallback_.end());
  const size_t branches = groups_.size() + (fallback_.empty() ? 0 : 1);
  if (branches > 1) {
    fork_.reset(new Event());
    for (size_t b = 0; b < branches; ++b) {
      branchStreams_.emplace_back(new Stream());
      branchDone_.emplace_back(new Event());
    }
  }
  scratchSeen_.assign(n, nullptr);
  values_.assign(n, nullptr);
  spaces_.assign(n, nullptr);
  upload_views();
}

template <typename T>
BatchPlan<T>::~BatchPlan() {
  for (auto& g : graphs_) {
    if (g) (void)cudaGraphExecDestroy(g);
  }
}

template <typename T>
int BatchPlan<T>::launches_per_pair() const {
  int n = 6 * static_cast<int>(fallback_.size());
  for (const auto& g : groups_) n += g->fused ? 4 : 6;
  return n;
}

template <typename T>
int BatchPlan<T>::transform_path(int t) const {
  if (t < 0 || t >= static_cast<int>(tp_.size())) throw InvalidParameterError();
  for (const auto& g : groups_) {
    if (std::find(g->members.begin(), g->members.end(), t) != g->members.end()) return g->fused ? 2 : 1;
  }
  return 0;
}

template <typename T>
int BatchPlan<T>::row_groups(int t) const {
  if (t < 0 || t >= static_cast<int>(tp_.size())) throw InvalidParameterError();
  for (const auto& g : groups_) {
    if (std::find(g->members.begin(), g->members.end(), t) != g->members.end()) return g->fused ? g->xGroups : 0;
  }
  return 0;
}

template <typename T>
int BatchPlan<T>::num_fused_groups() const {
  int n = 0;
  for (const auto& g : groups_) n += g->fused ? 1 : 0;
  return n;
}

// Plan views embed the grids' scratch pointers; refresh them if a grid's scratch moved (a grid
// grows its scratch when another transform is created on it).
template <typename T>
void BatchPlan<T>::upload_views() {
  bool changed = false;
  for (size_t t = 0; t < tp_.size(); ++t) {
    void* sc = tp_[t]->grid().scratch();
    if (sc != scratchSeen_[t]) changed = true;
    scratchSeen_[t] = sc;
  }
  if (!changed) return;
  DeviceGuard guard(device_);
  for (auto& gp : groups_) {
    Group& g = *gp;
    std::vector<PlanView<T>> views;
    for (int t : g.members) {
      PlanView<T> v = tp_[t]->gpu_plan().device_view(tp_[t]->grid().scratch());
      v.sticksRaw = 0;  // binary64 sticks: a group may run the fused plane kernel
      views.push_back(v);
    }
    check_cuda(cudaMemcpy(static_cast<char*>(g.dev.get()) + g.offViews, views.data(),
                          views.size() * sizeof(PlanView<T>), cudaMemcpyHostToDevice));
  }
}

template <typename T>
void BatchPlan<T>::bind(const T* const* values, T* const* spaces, cudaStream_t stream, bool async) {
  if (!values || !spaces) throw InvalidParameterError();
  const uintptr_t c = 2 * sizeof(T);
  for (size_t t = 0; t < tp_.size(); ++t) {
    if (!spaces[t] || reinterpret_cast<uintptr_t>(spaces[t]) % c) throw InvalidParameterError();
    if (tp_[t]->num_local_elements() > 0 &&
        (!values[t] || reinterpret_cast<uintptr_t>(values[t]) % c)) {
      throw InvalidParameterError();
    }
  }
  // Unbatched transforms take their pointers as kernel arguments, so a graph that contains them
  // holds the old pointers: drop the graphs (an in-flight graph is freed when it completes) and
  // capture them again on their next use.
  bool fallbackMoved = false;
  for (int t : fallback_) {
    fallbackMoved |= values_[t] != values[t] || spaces_[t] != spaces[t];
  }
  if (fallbackMoved) {
    for (auto& g : graphs_) {
      if (g) (void)cudaGraphExecDestroy(g);
      g = nullptr;
    }
  }
  for (size_t t = 0; t < tp_.size(); ++t) {
    values_[t] = values[t];
    spaces_[t] = spaces[t];
  }
  DeviceGuard guard(device_);
  for (auto& gp : groups_) {
    Group& g = *gp;
    std::vector<T*> vp, sp;
    for (int t : g.members) {
      vp.push_back(const_cast<T*>(values_[t]));
      sp.push_back(spaces_[t]);
    }
    char* d = static_cast<char*>(g.dev.get());
    if (async) {
      // pageable source: staged by the CUDA runtime before the call returns, written in stream order
      check_cuda(cudaMemcpyAsync(d + g.offValues, vp.data(), vp.size() * sizeof(T*), cudaMemcpyHostToDevice,
                                 stream));
      check_cuda(cudaMemcpyAsync(d + g.offSpaces, sp.data(), sp.size() * sizeof(T*), cudaMemcpyHostToDevice,
                                 stream));
    } else {
      check_cuda(cudaMemcpy(d + g.offValues, vp.data(), vp.size() * sizeof(T*), cudaMemcpyHostToDevice));
      check_cuda(cudaMemcpy(d + g.offSpaces, sp.data(), sp.size() * sizeof(T*), cudaMemcpyHostToDevice));
    }
  }
  bound_ = true;
}

template <typename T>
void BatchPlan<T>::check_bound() const {
  if (!bound_) throw InvalidParameterError();
}

namespace {
template <typename T>
void launch(FastOp op, int n, bool r2c, const BatchView<T>& bv, int blocks, size_t smem, int param,
            cudaStream_t s, int param2 = 0, int groups = 1) {
  if (blocks == 0) return;
  FastArgs<T> a;
  a.batch = &bv;
  a.blocks = blocks;
  a.smem = smem;
  a.param = param;
  a.param2 = param2;
  a.groups = groups;
  a.stream = s;
  fast_dispatch<T>(op, n, r2c, a);
  check_launch(cudaGetLastError());
}
}  // namespace

// One pass of one group: pass 0 = z, 1 = y (or the fused plane pass), 2 = x (nothing when fused);
// direction 0 backward, 1 forward.
template <typename T>
void BatchPlan<T>::run_pass(Group& g, int pass, int direction, bool scaled, cudaStream_t s) {
  char* d = static_cast<char*>(g.dev.get());
  const T* const* spaces = reinterpret_cast<const T* const*>(d + g.offSpaces);
  T* const* spacesOut = reinterpret_cast<T* const*>(d + g.offSpaces);
  if (pass == 0) {
    BatchView<T> bz = g.view(g.offStartsZ, direction == 1 && scaled ? g.scale : T(0));
    if (direction == 0) bz.in = reinterpret_cast<const T* const*>(d + g.offValues);
    else bz.out = reinterpret_cast<T* const*>(d + g.offValues);
    launch(direction == 0 ? FastOp::BatchZBackward : FastOp::BatchZForward, g.nz, g.r2c, bz, g.blocksZ, g.smemZ,
           g.spb, s);
  } else if (g.fused) {
    if (pass != 1) return;
    BatchView<T> bp = g.view(g.offStartsP, T(0));
    if (direction == 0) {
      bp.out = spacesOut;
      launch(FastOp::BatchPlaneBackward, g.nx, g.r2c, bp, g.blocksP, g.smemP, g.rowsB, s, 0, g.xGroups);
    } else {
      bp.in = spaces;
      launch(FastOp::BatchPlaneForward, g.nx, g.r2c, bp, g.blocksP, g.smemP, g.rowsF, s, g.rowsB, g.xGroups);
    }
  } else if (pass == 1) {
    launch(direction == 0 ? FastOp::BatchYBackward : FastOp::BatchYForward, g.ny, g.r2c, g.view(g.offStartsY, T(0)),
           g.blocksY, g.smemY, g.cpb, s);
  } else {
    BatchView<T> bx = g.view(g.offStartsX, T(0));
    if (direction == 0) bx.out = spacesOut;
    else bx.in = spaces;
    launch(direction == 0 ? FastOp::BatchXBackward : FastOp::BatchXForward, g.nx, g.r2c, bx, g.blocksX, g.smemX,
           g.rpb, s);
  }
}

template <typename T>
void BatchPlan<T>::run_group(Group& g, int what, bool scaled, cudaStream_t s) {
  if (what & 1) {
    for (int pass = 0; pass < 3; ++pass) run_pass(g, pass, 0, false, s);
  }
  if (what & 2) {
    for (int pass = 2; pass >= 0; --pass) run_pass(g, pass, 1, scaled, s);
  }
}

template <typename T>
void BatchPlan<T>::run_fallback(int what, bool scaled, cudaStream_t s) {
  for (int t : fallback_) {
    const GpuPlan<T>& plan = tp_[t]->gpu_plan();
    void* scratch = tp_[t]->grid().scratch();
    if (what & 1) plan.backward(values_[t], spaces_[t], scratch, s);
    if (what & 2) plan.forward(spaces_[t], const_cast<T*>(values_[t]), scaled, scratch, s);
  }
}

template <typename T>
void BatchPlan<T>::run(int what, bool scaled, cudaStream_t stream) {
  if (!fork_) {
    for (auto& gp : groups_) run_group(*gp, what, scaled, stream);
    run_fallback(what, scaled, stream);
    return;
  }
  // fork: every branch starts after the work already on `stream`; join: `stream` continues after
  // every branch (also while `stream` is being captured into a graph)
  fork_->record(stream);
  size_t b = 0;
  for (auto& gp : groups_) {
    cudaStream_t s = branchStreams_[b]->get();
    fork_->wait_on(s);
    run_group(*gp, what, scaled, s);
    branchDone_[b]->record(s);
    ++b;
  }
  if (!fallback_.empty()) {
    cudaStream_t s = branchStreams_[b]->get();
    fork_->wait_on(s);
    run_fallback(what, scaled, s);
    branchDone_[b]->record(s);
    ++b;
  }
  for (size_t i = 0; i < b; ++i) branchDone_[i]->wait_on(stream);
}

template <typename T>
void BatchPlan<T>::backward(cudaStream_t stream) {
  check_bound();
  DeviceGuard guard(device_);
  upload_views();
  run(1, false, stream);
}

template <typename T>
void BatchPlan<T>::forward(bool scaled, cudaStream_t stream) {
  check_bound();
  DeviceGuard guard(device_);
  upload_views();
  run(2, scaled, stream);
}

template <typename T>
void BatchPlan<T>::stage_times(int direction, bool scaled, cudaStream_t stream, float ms[3]) {
  check_bound();
  DeviceGuard guard(device_);
  upload_views();
  StageEvents ev{};
  for (auto& e : ev.ev) check_cuda(cudaEventCreate(&e));
  try {
    // backward runs the passes z, y, x; forward x, y, z (event i+1 closes the i-th of them)
    check_cuda(cudaEventRecord(ev.ev[0], stream));
    for (int i = 0; i < 3; ++i) {
      const int pass = direction == 0 ? i : 2 - i;
      for (auto& gp : groups_) run_pass(*gp, pass, direction, scaled, stream);
      if (i == 2) run_fallback(direction == 0 ? 1 : 2, scaled, stream);
      check_cuda(cudaEventRecord(ev.ev[i + 1], stream));
    }
    check_cuda(cudaEventSynchronize(ev.ev[3]));
    for (int i = 0; i < 3; ++i) check_cuda(cudaEventElapsedTime(&ms[i], ev.ev[i], ev.ev[i + 1]));
  } catch (...) {
    for (auto& e : ev.ev) (void)cudaEventDestroy(e);
    throw;
  }
  for (auto& e : ev.ev) (void)cudaEventDestroy(e);
}

template <typename T>
void BatchPlan<T>::set_z_shape(Group& g, int spb) {
  FastArgs<T> a;
  size_t sm = 0;
  a.smemOut = &sm;
  a.param = spb;
  fast_dispatch<T>(FastOp::ZSmem, g.nz, g.r2c, a);
  const size_t m = g.members.size();
  std::vector<int> sz(m + 1, 0);
  for (size_t i = 0; i < m; ++i) {
    sz[i + 1] = sz[i] + (tp_[g.members[i]]->index_plan().num_sticks() + spb - 1) / spb;
  }
  check_cuda(cudaMemcpy(static_cast<char*>(g.dev.get()) + g.offStartsZ, sz.data(), (m + 1) * sizeof(int),
                        cudaMemcpyHostToDevice));
  g.spb = spb;
  g.smemZ = sm;
  g.blocksZ = sz[m];
}

template <typename T>
float BatchPlan<T>::autotune(cudaStream_t stream, int reps) {
  check_bound();
  if (reps < 1) throw InvalidParameterError();
  DeviceGuard guard(device_);
  upload_views();
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  check_cuda(cudaEventCreate(&e0));
  check_cuda(cudaEventCreate(&e1));
  float total = 0.0f;
  try {
    for (auto& gp : groups_) {
      Group& g = *gp;
      auto time_group = [&]() {
        run_group(g, 3, true, stream);  // warm-up
        check_cuda(cudaEventRecord(e0, stream));
        for (int r = 0; r < reps; ++r) run_group(g, 3, true, stream);
        check_cuda(cudaEventRecord(e1, stream));
        check_cuda(cudaEventSynchronize(e1));
        float ms = 0.0f;
        check_cuda(cudaEventElapsedTime(&ms, e0, e1));
        return ms / reps;
      };
      int bestSpb = g.spb, bestGroups = g.xGroups;
      bool bestFused = g.fused;
      float best = time_group();
      for (int f = 0; f < 2; ++f) {
        const bool fused = f == 1;
        if ((fused && !g.fusedAvail) || (!fused && !g.splitAvail)) continue;
        g.fused = fused;
        for (int spb : g.zCands) {
          set_z_shape(g, spb);
          const float ms = time_group();
          if (ms < best) {
            best = ms;
            bestSpb = spb;
            bestFused = fused;
          }
        }
      }
      g.fused = bestFused;
      set_z_shape(g, bestSpb);
      // row groups of the fused x pass, with the best z shape
      if (g.fused) {
        for (int gr : g.groupCands) {
          if (gr == bestGroups) continue;
          g.xGroups = gr;
          const float ms = time_group();
          if (ms < best) {
            best = ms;
            bestGroups = gr;
          }
        }
        g.xGroups = bestGroups;
      }
      total += best;
    }
  } catch (...) {
    (void)cudaEventDestroy(e0);
    (void)cudaEventDestroy(e1);
    throw;
  }
  (void)cudaEventDestroy(e0);
  (void)cudaEventDestroy(e1);
  // the captured graphs hold the old launch shapes
  for (auto& ge : graphs_) {
    if (ge) (void)cudaGraphExecDestroy(ge);
    ge = nullptr;
  }
  return total;
}

template <typename T>
void BatchPlan<T>::pair_graph(bool scaled, cudaStream_t stream) {
  graph(3, scaled, stream);
}

template <typename T>
void BatchPlan<T>::graph(int what, bool scaled, cudaStream_t stream) {
  check_bound();
  if (stream == nullptr || stream == cudaStreamLegacy || stream == cudaStreamPerThread) {
    throw InvalidParameterError();
  }
  DeviceGuard guard(device_);
  // refresh views outside the capture (a synchronous copy cannot be captured); the graphs read
  // the views and the bound pointers from device tables at fixed addresses, so neither a refresh
  // nor a rebind invalidates them
  upload_views();
  cudaGraphExec_t& exec = graphs_[2 * what + (scaled ? 1 : 0)];
  if (!exec) {
    cudaGraph_t g = nullptr;
    check_cuda(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    try {
      run(what, scaled, stream);
    } catch (...) {
      (void)cudaStreamEndCapture(stream, &g);
      if (g) (void)cudaGraphDestroy(g);
      throw;
    }
    check_cuda(cudaStreamEndCapture(stream, &g));
    const cudaError_t st = cudaGraphInstantiate(&exec, g, 0);
    (void)cudaGraphDestroy(g);
    check_cuda(st);
  }
  check_cuda(cudaGraphLaunch(exec, stream));
}

template class BatchPlan<double>;
template class BatchPlan<float>;

}  // namespace gb300
}  // namespace spfft
