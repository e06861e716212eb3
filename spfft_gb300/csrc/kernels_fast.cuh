// Size-specialised transform kernels (compile-time FFT lengths, register DFTs, one in-place
// shared-memory exchange per 1D FFT). Two launches per direction:
//
//   backward: z kernel   values -> (scatter, stick symmetry, z-FFT) -> sticks[z][s]
//             plane      sticks of plane z -> compact plane in smem -> plane symmetry ->
//                        y-FFT on the non-empty x columns -> x-FFT (C2C, or C2R through a
//                        half-length complex FFT) -> space rows
//   forward:  plane      space rows -> x-FFT (C2C, or R2C through a half-length complex FFT) ->
//                        keep the non-empty columns -> y-FFT -> gather plane z of every stick
//             z kernel   sticks -> z-FFT -> gather (and scale) the values
//
// Replaces, fused: compression_kernels.cu:39-150, symmetry_kernels.cu:38-165,
// local_transpose_kernels.cu:43-201 and the cuFFT calls of transform_1d_gpu.hpp /
// transform_2d_gpu.hpp / transform_real_2d_gpu.hpp (all in the reference's src/). Compared with the
// generic kernels, the y and x passes are one kernel, so the compact plane never goes to HBM.
//
// Types: S is the storage type in HBM (values, sticks, space), A the arithmetic type of the FFTs
// (float for FP32; dd, double-float on the FP32 pipes, for FP64). With A = dd every block finds
// the largest binary64 exponent of the data it loads, converts with an exact power-of-two scale
// that brings that maximum into [1, 2), and undoes the scale when it stores -- so every double
// magnitude is handled, and the FFT arithmetic never touches GB300's slow FP64 pipe.
#pragma once

#include <cuda_runtime.h>

#include <type_traits>

#include "dd.cuh"
#include "dft.cuh"
#include "kernels.hpp"
#include "kernels_fast.hpp"

namespace spfft {
namespace gb300 {
namespace fast {

constexpr int kThreads = 256;       // z-pass blocks
constexpr int kPlaneThreads = 512;  // plane blocks (one plane per block, so more warps per SM)
// Batched plane blocks (two per SM), by arithmetic type: batch_plane_threads() of the storage type.
template <typename A>
struct BatchPlaneThreads {
  static constexpr int value = batch_plane_threads<float>();
};
// Minimum resident blocks per SM asked of the compiler for the split y kernels and the split x
// forward kernel: double-float kernels are capped at 80 registers so that three 256-thread
// blocks share an SM (24 warps to hide the FP32 pipe latencies of the dd dependency chains;
// measured 10% faster than two blocks at 128 registers on the 192^3 R2C transform, while the z
// kernels measured slower that way); FP32 kernels fit three anyway.
template <typename A>
struct YMinBlocks {
  static constexpr int value = 1;
};
template <>
struct YMinBlocks<dd> {
  static constexpr int value = 3;
};
// Minimum resident 256-thread blocks per SM asked of the compiler for the z kernels: double-float
// z backward two (at most 128 registers) with a two-pass split, three (at most 80) with the
// three-pass split (V = 3, at most 12 values per work item), z forward three (at most 80).
template <typename A, int V = 1>
struct ZBackwardMinBlocks {
  static constexpr int value = 4;  // FP32: at most 64 registers (the kernel needs about 50)
};
template <int V>
struct ZBackwardMinBlocks<dd, V> {
  static constexpr int value = V == 3 ? 3 : 2;
};
template <typename A>
struct ZForwardMinBlocks {
  static constexpr int value = 3;  // FP32: at most 80 registers (the kernel needs about 60)
};
template <>
struct ZForwardMinBlocks<dd> {
  static constexpr int value = 3;
};
template <>
struct BatchPlaneThreads<dd> {
  static constexpr int value = batch_plane_threads<double>();
};
// Threads of a split x backward block. The double-float R2C kernel (72 registers) is held to two
// blocks per SM by its shared memory (compact rows and FFT rows of 32 rows), not by registers, so
// its blocks take 384 threads: 24 warps per SM instead of 16, and pass 2 (12 work items per row of
// the 12 x 8 split of 192) fills the block. The C2C kernel (about 100 registers) would fit only one
// such block per SM and keeps 256.
template <typename A, bool R2C>
struct XBackwardThreads {
  static constexpr int value = kThreads;
};
template <>
struct XBackwardThreads<dd, true> {
  static constexpr int value = 384;
};

extern __shared__ __align__(16) unsigned char g_fast_smem[];

// ---- types and conversions ----------------------------------------------------------------------
template <typename A>
struct ArithC;
template <>
struct ArithC<float> {
  using type = float2;
};
template <>
struct ArithC<dd> {
  using type = ddc;
};

template <typename S, typename A>
struct Types {
  using CS = typename Complex<S>::type;
  using CA = typename ArithC<A>::type;
  static constexpr bool kScaled = !std::is_same<S, A>::value;
  static_assert(sizeof(CS) == sizeof(CA), "storage and arithmetic complex must have equal size");
};

template <typename A>
__device__ __forceinline__ typename ArithC<A>::type czero() {
  return make_c(A(0), A(0));
}

// storage -> arithmetic with the block scale 2^k
__device__ __forceinline__ float2 to_arith(float2 v, int) { return v; }
__device__ __forceinline__ ddc to_arith(double2 v, int k) {
  return make_c(dd_from_double(v.x, k), dd_from_double(v.y, k));
}
// arithmetic -> storage, undoing the block scale
__device__ __forceinline__ float2 to_storage(float2 v, int) { return v; }
__device__ __forceinline__ double2 to_storage(ddc v, int k) {
  return make_double2(dd_to_double(re(v), -k), dd_to_double(im(v), -k));
}
// The same conversions for every binary64 class: subnormal inputs normalised, results below
// 2^-1022 assembled as subnormals.
__device__ __forceinline__ float2 to_arith_exact(float2 v, int) { return v; }
__device__ __forceinline__ ddc to_arith_exact(double2 v, int k) {
  return make_c(dd_from_double_exact(v.x, k), dd_from_double_exact(v.y, k));
}
__device__ __forceinline__ float2 to_storage_exact(float2 v, int) { return v; }
__device__ __forceinline__ double2 to_storage_exact(ddc v, int k) {
  return make_double2(dd_to_double_exact(re(v), -k), dd_to_double_exact(im(v), -k));
}
// Which conversions a block needs. A block scaled by k brings its largest magnitude into [1, 2),
// and its largest FFT output is at least that large (Parseval), so binary64 subnormals -- inputs or
// outputs -- lie below 2^(k - 1022) of the block's largest value. Below k = 962 that is under 2^-60
// and the fast conversions flush them to zero; blocks of tiny values (largest magnitude below
// 2^-961) use the exact ones. k is the same for every thread of a block, so every branch on it is
// uniform and the exact code never runs in ordinary blocks.
constexpr int kExactScale = 962;
__device__ __forceinline__ bool exact_block(int k) { return k >= kExactScale; }
struct FastStore {
  template <typename CA>
  __device__ __forceinline__ auto operator()(CA v, int k) const { return to_storage(v, k); }
};
struct ExactStore {
  template <typename CA>
  __device__ __forceinline__ auto operator()(CA v, int k) const { return to_storage_exact(v, k); }
};
// Runs `store(conv)` with the storage conversion the block's scale k needs (outputs held in
// registers).
template <typename F>
__device__ __forceinline__ void with_store(int k, F&& store) {
  if (exact_block(k)) {
    store(ExactStore{});
  } else {
    store(FastStore{});
  }
}
// twiddles: double tables -> dd, float tables as they are
__device__ __forceinline__ float2 tw_arith(float2 v) { return v; }
__device__ __forceinline__ ddc tw_arith(double2 v) {
  return make_c(dd_from_double(v.x, 0), dd_from_double(v.y, 0));
}

// Largest biased binary64 exponent field of a complex value (the first step of a block's
// magnitude key, dd.cuh), and its largest subnormal key (the second step, for blocks of zeros and
// subnormals only).
__device__ __forceinline__ int max_exponent(float2) { return 0; }
__device__ __forceinline__ int max_exponent(double2 v) {
  return max(dd_exponent_field(v.x), dd_exponent_field(v.y));
}
__device__ __forceinline__ int max_subnormal_key(float2) { return kDdNoSubnormal; }
__device__ __forceinline__ int max_subnormal_key(double2 v) {
  return max(dd_subnormal_key(v.x), dd_subnormal_key(v.y));
}
// Scale exponent k for a block with magnitude key e: 2^k * max in [1, 2), subnormal maxima
// included. Zero and non-finite blocks use k = 0.
__device__ __forceinline__ int block_scale(int e) { return dd_block_scale(e); }

// Completes a block's magnitude key once the largest exponent field has been reduced into sExp[0]
// (with sExp[1] = kDdNoSubnormal set before that reduction's barrier, and a barrier after it). A
// block holding a normal or non-finite value keeps that field as its key. A block of zeros and
// subnormals only (sExp[0] == 0, the same for every thread) reduces `scan()`, each thread's largest
// max_subnormal_key, into sExp[1] and stores the exact key (0 for an all-zero block) in sExp[0].
// Returns the key. Only that rare case adds a barrier; every thread has read sExp[0] before it, so
// thread 0's store races with no reader.
// The rare part is a separate function (not inlined) so that it costs the common path no
// registers; `scan` captures by value.
template <typename Scan>
__device__ __noinline__ int subnormal_block_key(int* sExp, Scan scan) {
  atomicMax(sExp + 1, scan());
  __syncthreads();
  const int sub = sExp[1];
  const int key = sub == kDdNoSubnormal ? 0 : sub;
  if (threadIdx.x == 0) sExp[0] = key;
  return key;
}
template <typename Scan>
__device__ __forceinline__ int finish_block_key(int* sExp, Scan scan) {
  const int e0 = sExp[0];
  if (e0 != 0) return e0;
  return subnormal_block_key(sExp, scan);
}
// Outputs that sit in shared memory: a block of tiny values converts them in place to storage
// form first (exactly; n slots from `buf`, strided over `nthreads` threads from `tid`; the caller
// synchronises), and the store loop reads them with stored_value instead of converting.
template <typename S, typename A>
__device__ __forceinline__ void convert_exact_in_place(typename Types<S, A>::CA* buf, int n, int k, int tid,
                                                       int nthreads) {
  using CS = typename Types<S, A>::CS;
  for (int i = tid; i < n; i += nthreads) reinterpret_cast<CS*>(buf)[i] = to_storage_exact(buf[i], k);
}
template <typename S, typename A>
__device__ __forceinline__ typename Types<S, A>::CS stored_value(const typename Types<S, A>::CA* slot, int k,
                                                                 bool converted) {
  using CS = typename Types<S, A>::CS;
  return converted ? *reinterpret_cast<const CS*>(slot) : to_storage(*slot, k);
}

// Double-float compact planes (PlanView::planesRaw): each producing block stores its scaled values
// as they are and records its scale exponent k per column (y pass) or per row (x forward); a
// block of zeros records kZeroExp, which never wins the minimum. A consumer takes the smallest
// exponent of its inputs (the largest magnitude) as its own scale and multiplies every other input
// by 2^(k - k_input) <= 1, exactly (or to zero far below the block maximum).
constexpr int kZeroExp = 1 << 20;
__device__ __forceinline__ int produced_exp(int maxKey, int k) { return maxKey == 0 ? kZeroExp : k; }
__device__ __forceinline__ float2 scale_pow2(float2 v, int) { return v; }
__device__ __forceinline__ ddc scale_pow2(ddc v, int d) {
  const float f = d < -126 ? 0.0f : __uint_as_float(static_cast<unsigned>(d + 127) << 23);
  return ddc{f2_mul(v.hi, make_float2(f, f)), f2_mul(v.lo, make_float2(f, f))};
}

// Programmatic dependent launch (sm_90+): kernels of the same transform are launched so that the
// next kernel's blocks may start while the previous kernel finishes. Each kernel loads only its
// constant plan tables (twiddles, index maps) before pdl_wait(), which returns once the previous
// kernel of the stream has completed and its writes are visible; every read of data another
// kernel produces and every global write comes after it. pdl_trigger() lets the next kernel launch
// once every block of this one has passed it. Both are no-ops for an ordinary launch.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// Thread groups of the plane kernels' x pass: the block splits into `groups` groups of whole warps
// that each own a share of the rows and of the W buffer and synchronise only among themselves
// (named barrier g + 1; barrier 0 is __syncthreads), so one group's barrier wait overlaps another
// group's arithmetic. One group is the whole block.
struct RowGroups {
  int groups, threads, g, t;
  __device__ __forceinline__ explicit RowGroups(int n)
      : groups(n), threads(blockDim.x / n), g(threadIdx.x / (blockDim.x / n)),
        t(threadIdx.x - (threadIdx.x / (blockDim.x / n)) * (blockDim.x / n)) {}
  __device__ __forceinline__ void sync() const {
    if (groups == 1) __syncthreads();
    else asm volatile("bar.sync %0, %1;" ::"r"(g + 1), "r"(threads) : "memory");
  }
  // rows [begin, end) of this group out of n
  __device__ __forceinline__ int begin(int n) const { return g * n / groups; }
  __device__ __forceinline__ int end(int n) const { return (g + 1) * n / groups; }
};

// Walks the flat indices i = start, start + step, ... of a row-major [rows][len] range as (row r,
// column c) pairs, one compare instead of one division per element.
struct RowWalk {
  int r, c;
  int dr, dc, len;
  __device__ __forceinline__ RowWalk(int start, int step, int len_)
      : r(start / len_), c(start - (start / len_) * len_), dr(step / len_), dc(step - (step / len_) * len_),
        len(len_) {}
  __device__ __forceinline__ void next() {
    r += dr;
    c += dc;
    if (c >= len) {
      c -= len;
      ++r;
    }
  }
};

// Division by a block-uniform runtime divisor d in [1, 2^16) for numerators n in [0, 2^16): one
// high multiply by m = floor(2^32 / d) + 1 instead of the division sequence. Exact because
// n * (m - 2^32 / d) < n * 1 < 2^32 / d, i.e. the error stays below one step of n / d.
struct FastDiv {
  unsigned m;
  int d;
  __device__ __forceinline__ explicit FastDiv(int divisor)
      : m(divisor > 1 ? 0xFFFFFFFFu / static_cast<unsigned>(divisor) + 1u : 0u), d(divisor) {}
  __device__ __forceinline__ int div(int n) const {
    return d > 1 ? static_cast<int>(__umulhi(static_cast<unsigned>(n), m)) : n;
  }
};

// Asynchronous global -> shared copy of one complex value (cp.async, 8 or 16 bytes). Lets a
// thread keep many loads in flight instead of waiting on each.
template <typename CS>
__device__ __forceinline__ void cp_async_c(void* smemDst, const CS* gmemSrc) {
  const unsigned dst = static_cast<unsigned>(__cvta_generic_to_shared(smemDst));
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(dst), "l"(gmemSrc),
               "n"(static_cast<int>(sizeof(CS)))
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int PENDING>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(PENDING) : "memory");
}

// After raw storage values were copied into n arithmetic slots: find the block scale (dd only)
// and convert in place. Ends with __syncthreads(). Returns the scale exponent k.
template <typename S, typename A>
__device__ __forceinline__ int convert_block(typename Types<S, A>::CA* slots, int n, int* sExp) {
  using TT = Types<S, A>;
  if (!TT::kScaled) return 0;
  using CS = typename TT::CS;
  if (threadIdx.x == 0) {
    sExp[0] = 0;
    sExp[1] = kDdNoSubnormal;
  }
  __syncthreads();
  int e = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) e = max(e, max_exponent(reinterpret_cast<const CS*>(slots)[i]));
  atomicMax(sExp, e);
  __syncthreads();
  const int k = block_scale(finish_block_key(sExp, [=] {
    int m = kDdNoSubnormal;
    for (int i = threadIdx.x; i < n; i += blockDim.x) m = max(m, max_subnormal_key(reinterpret_cast<const CS*>(slots)[i]));
    return m;
  }));
  if (exact_block(k)) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const CS raw = reinterpret_cast<const CS*>(slots)[i];
      slots[i] = to_arith_exact(raw, k);
    }
  } else {
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const CS raw = reinterpret_cast<const CS*>(slots)[i];
      slots[i] = to_arith(raw, k);
    }
  }
  __syncthreads();
  return k;
}

// Conditional conjugate fill along one line, two ordered halves (symmetry_host.hpp:42-90).
template <typename CA>
__device__ __forceinline__ void line_fill(CA* v, int n, int stride) {
  for (int k = 1 + threadIdx.x; k < n / 2 + 1; k += blockDim.x) {
    CA a = v[k * stride];
    if (cnonzero(a)) v[(n - k) * stride] = cconj(a);
  }
  __syncthreads();
  for (int k = n / 2 + 1 + threadIdx.x; k < n; k += blockDim.x) {
    CA a = v[k * stride];
    if (cnonzero(a)) v[(n - k) * stride] = cconj(a);
  }
  __syncthreads();
}

template <typename S, typename A>
__device__ __forceinline__ void load_twiddles(typename Types<S, A>::CA* dst, const S* src, int n) {
  using CS = typename Types<S, A>::CS;
  const CS* s = reinterpret_cast<const CS*>(src);
  for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = tw_arith(s[i]);
}

// ================================================================================================
// z pass
// ================================================================================================
// The z twiddles in pass-1 order (tw1[k1 * B + b] = w^(k1 b)) and, for the three-pass split, in
// power order as well (pass 2a reads w^(kk1 i2 A)).
template <typename S, typename A, int NZ, int V>
__device__ __forceinline__ void load_z_twiddles(typename Types<S, A>::CA* tw1, typename Types<S, A>::CA* tw,
                                                const S* src) {
  using CS = typename Types<S, A>::CS;
  constexpr int Bz = Shape<NZ, V>::B;
  const CS* s = reinterpret_cast<const CS*>(src);
  for (int i = threadIdx.x; i < NZ; i += blockDim.x) {
    const int k1 = i / Bz;
    tw1[i] = tw_arith(s[k1 * (i - k1 * Bz)]);
    if constexpr (V == 3) tw[i] = tw_arith(s[i]);
  }
}

template <int NZ>
struct ZLayout {
  static constexpr int pitch = NZ | 1;  // odd: conflict-free column access across sticks
};

// Kernel bodies take their block coordinates as arguments, so the single-transform kernels and the
// batched kernels (kernels_batch.cuh) share them.
// V selects the two-pass split of the z length (Shape<NZ, V>: 1 the default, 2 the swapped one).
template <typename S, typename A, int NZ, int V = 1>
__device__ __forceinline__ void z_backward_body(const PlanView<S>& p, const S* __restrict__ values,
                                                int spb, int bx, int* sExpPtr) {
  using TT = Types<S, A>;
  using CS = typename TT::CS;
  using CA = typename TT::CA;
  constexpr int Az = Shape<NZ, V>::A, Bz = Shape<NZ, V>::B, PZ = ZLayout<NZ>::pitch;
  int& sExp = *sExpPtr;
  CA* tw1 = reinterpret_cast<CA*>(g_fast_smem);  // pass-1 order
  CA* tw = tw1 + NZ;                              // power order (pass 2a of variant 3)
  CA* buf = tw + NZ;
  const int s0 = bx * spb;
  const int nsb = min(spb, p.numSticks - s0);
  const FastDiv dns(nsb);

  load_z_twiddles<S, A, NZ, V>(tw1, tw, p.twz);
  for (int i = threadIdx.x; i < nsb * PZ; i += blockDim.x) buf[i] = czero<A>();
  // The value map is a plan table (constant from plan creation on): the block's entry range and
  // this thread's first four entries are read before the wait for the previous kernel.
  const int e0 = p.stickEntryStart[s0], e1 = p.stickEntryStart[s0 + nsb];
  const int base = s0 * NZ;
  int pos0[4], usr0[4];
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int eu = e0 + threadIdx.x + u * blockDim.x;
    pos0[u] = eu < e1 ? p.entryPos[eu] - base : -1;
    usr0[u] = eu < e1 ? p.entryUser[eu] : 0;
  }
  __syncthreads();
  pdl_wait();
  pdl_trigger();

  const CS* vals = reinterpret_cast<const CS*>(values);
  // Index loads four at a time, then asynchronous value copies straight to their stick slots.
  for (int e = e0 + threadIdx.x; e < e1; e += 4 * blockDim.x) {
    int pos[4], usr[4];
    const bool first = e == e0 + threadIdx.x;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int eu = e + u * blockDim.x;
      pos[u] = first ? pos0[u] : (eu < e1 ? p.entryPos[eu] - base : -1);
      usr[u] = first ? usr0[u] : (eu < e1 ? p.entryUser[eu] : 0);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      if (pos[u] >= 0) {
        const int sl = pos[u] / NZ;
        cp_async_c(buf + sl * PZ + (pos[u] - sl * NZ), vals + usr[u]);
      }
    }
  }
  cp_async_commit();
  cp_async_wait<0>();
  __syncthreads();
  const int k = convert_block<S, A>(buf, nsb * PZ, &sExp);

  const int zz = p.zeroZeroStick - s0;
  if (p.r2c && zz >= 0 && zz < nsb) line_fill(buf + zz * PZ, NZ, 1);

  for (int i = threadIdx.x; i < nsb * Bz; i += blockDim.x) {
    const int sl = i / Bz, b = i - sl * Bz;
    fft_pass1_ordered<NZ, +1, V>(buf + sl * PZ, 1, b, tw1);
  }
  __syncthreads();
  CS* sticks = reinterpret_cast<CS*>(p.sticks) + s0;
  const bool raw = TT::kScaled && p.sticksRaw;
  const bool park = TT::kScaled && !raw && exact_block(k);
  if constexpr (V == 3) {
    // pass 2 as pass 2a (B1-point DFTs) and pass 2b (B2-point DFTs); sticks fastest across threads
    constexpr int B1 = Split3<NZ>::B1, B2 = Split3<NZ>::B2;
    for (int i = threadIdx.x; i < nsb * Az * B2; i += blockDim.x) {
      const int r = dns.div(i), sl = i - r * nsb, k1 = r / B2;
      fft_pass2a<NZ, +1>(buf + sl * PZ, 1, k1, r - k1 * B2, tw);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nsb * Az * B1; i += blockDim.x) {
      const int r = dns.div(i), sl = i - r * nsb, k1 = r / B1, kk1 = r - k1 * B1;
      CA v[B2];
      fft_pass2b<NZ, +1>(buf + sl * PZ, 1, k1, kk1, v);
#pragma unroll
      for (int kk2 = 0; kk2 < B2; ++kk2) {
        const size_t at = static_cast<size_t>(k1 + Az * (kk1 + B1 * kk2)) * p.numSticks + sl;
        if (raw) reinterpret_cast<CA*>(sticks)[at] = v[kk2];
        else if (park) buf[sl * PZ + k1 * Bz + kk1 * B2 + kk2] = v[kk2];
        else sticks[at] = to_storage(v[kk2], k);
      }
    }
  } else {
    for (int i = threadIdx.x; i < nsb * Az; i += blockDim.x) {
      const int k1 = dns.div(i), sl = i - k1 * nsb;
      CA v[Bz];
      fft_pass2<NZ, +1, V>(buf + sl * PZ, 1, k1, v);
      if (raw) {
        CA* rs = reinterpret_cast<CA*>(sticks);
#pragma unroll
        for (int k2 = 0; k2 < Bz; ++k2) rs[static_cast<size_t>(k1 + Az * k2) * p.numSticks + sl] = v[k2];
      } else if (park) {
        // blocks of tiny values: results back into this item's own pass-2 slots, stored exactly below
#pragma unroll
        for (int k2 = 0; k2 < Bz; ++k2) buf[sl * PZ + k1 * Bz + k2] = v[k2];
      } else {
#pragma unroll
        for (int k2 = 0; k2 < Bz; ++k2) {
          sticks[static_cast<size_t>(k1 + Az * k2) * p.numSticks + sl] = to_storage(v[k2], k);
        }
      }
    }
  }
  if (park) {
    __syncthreads();
    for (int i = threadIdx.x; i < nsb * NZ; i += blockDim.x) {
      const int sl = i / NZ, e = i - sl * NZ;
      int z;
      if constexpr (V == 3) {
        z = three_pass_index<NZ>(e);
      } else {
        const int k1 = e / Bz;
        z = k1 + Az * (e - k1 * Bz);
      }
      sticks[static_cast<size_t>(z) * p.numSticks + sl] = to_storage_exact(buf[sl * PZ + e], k);
    }
  }
  if (raw && threadIdx.x < nsb) p.stickExp[s0 + threadIdx.x] = produced_exp(sExp, k);
}

template <typename S, typename A, int NZ, int V = 1>
__global__ void __launch_bounds__(kThreads, ZBackwardMinBlocks<A, V>::value) z_backward(const PlanView<S> p,
                                                       const S* __restrict__ values, int spb) {
  __shared__ int sExp[2];
  z_backward_body<S, A, NZ, V>(p, values, spb, blockIdx.x, sExp);
}

template <typename S, typename A, int NZ, int V = 1>
__device__ __forceinline__ void z_forward_body(const PlanView<S>& p, S* __restrict__ values, S scale,
                                               int spb, int bx, int* sExpPtr) {
  using TT = Types<S, A>;
  using CS = typename TT::CS;
  using CA = typename TT::CA;
  constexpr int Az = Shape<NZ, V>::A, Bz = Shape<NZ, V>::B, PZ = ZLayout<NZ>::pitch;
  int& sExp = *sExpPtr;
  CA* tw1 = reinterpret_cast<CA*>(g_fast_smem);  // pass-1 order
  CA* tw = tw1 + NZ;                              // power order (pass 2a of variant 3)
  CA* buf = tw + NZ;
  const int s0 = bx * spb;
  const int nsb = min(spb, p.numSticks - s0);
  const FastDiv dns(nsb);

  load_z_twiddles<S, A, NZ, V>(tw1, tw, p.twz);
  // the block's value range (a plan table, read before the wait for the previous kernel)
  const int e0 = p.stickEntryStart[s0], e1 = p.stickEntryStart[s0 + nsb];
  pdl_wait();
  pdl_trigger();
  const CS* sticks = reinterpret_cast<const CS*>(p.sticks) + s0;
  for (int i = threadIdx.x; i < NZ * nsb; i += blockDim.x) {
    const int z = dns.div(i), sl = i - z * nsb;
    cp_async_c(buf + sl * PZ + z, sticks + static_cast<size_t>(z) * p.numSticks + sl);
  }
  // the pitch padding slots are never read; zero them so the block scale ignores them
  for (int i = threadIdx.x; i < nsb; i += blockDim.x) {
    if (PZ > NZ) buf[i * PZ + NZ] = czero<A>();
  }
  cp_async_commit();
  int k = 0;
  if (TT::kScaled && p.sticksRaw) {
    // double-float sticks from the y pass, one exponent per (plane, column): block scale = the
    // smallest of them, every value brought to it
    if (threadIdx.x == 0) sExp = kZeroExp;
    __syncthreads();
    const int nc = p.numColumns;
    int e = kZeroExp;
    for (int i = threadIdx.x; i < NZ * nsb; i += blockDim.x) {
      const int z = dns.div(i), sl = i - z * nsb;
      e = min(e, p.stickExp[z * nc + p.stickColumn[s0 + sl]]);
    }
    atomicMin(&sExp, e);
    cp_async_wait<0>();
    __syncthreads();
    k = sExp == kZeroExp ? 0 : sExp;
    for (int i = threadIdx.x; i < NZ * nsb; i += blockDim.x) {
      const int z = dns.div(i), sl = i - z * nsb;
      CA& v = buf[sl * PZ + z];
      v = scale_pow2(v, k - p.stickExp[z * nc + p.stickColumn[s0 + sl]]);
    }
    __syncthreads();
  } else {
    cp_async_wait<0>();
    __syncthreads();
    k = convert_block<S, A>(buf, nsb * PZ, &sExp);
  }
  for (int i = threadIdx.x; i < nsb * Bz; i += blockDim.x) {
    const int sl = i / Bz, b = i - sl * Bz;
    fft_pass1_ordered<NZ, -1, V>(buf + sl * PZ, 1, b, tw1);
  }
  __syncthreads();
  if constexpr (V == 3) {
    constexpr int B1 = Split3<NZ>::B1, B2 = Split3<NZ>::B2;
    for (int i = threadIdx.x; i < nsb * Az * B2; i += blockDim.x) {
      const int r = dns.div(i), sl = i - r * nsb, k1 = r / B2;
      fft_pass2a<NZ, -1>(buf + sl * PZ, 1, k1, r - k1 * B2, tw);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nsb * Az * B1; i += blockDim.x) {
      const int r = dns.div(i), sl = i - r * nsb, k1 = r / B1, kk1 = r - k1 * B1;
      CA v[B2];
      fft_pass2b<NZ, -1>(buf + sl * PZ, 1, k1, kk1, v);
#pragma unroll
      for (int kk2 = 0; kk2 < B2; ++kk2) buf[sl * PZ + k1 * Bz + kk1 * B2 + kk2] = v[kk2];
    }
  } else {
    for (int i = threadIdx.x; i < nsb * Az; i += blockDim.x) {
      const int k1 = dns.div(i), sl = i - k1 * nsb;
      CA v[Bz];
      fft_pass2<NZ, -1, V>(buf + sl * PZ, 1, k1, v);
#pragma unroll
      for (int k2 = 0; k2 < Bz; ++k2) buf[sl * PZ + rotated_slot<NZ, V>(k1, k2)] = v[k2];
    }
  }
  __syncthreads();
  CS* out = reinterpret_cast<CS*>(values);
  const int base = s0 * NZ;
  const bool converted = TT::kScaled && exact_block(k);
  if (converted) {
    convert_exact_in_place<S, A>(buf, nsb * PZ, k, threadIdx.x, blockDim.x);
    __syncthreads();
  }
  // Index loads four at a time (their latencies overlap), then the gathers and stores.
  for (int e = e0 + threadIdx.x; e < e1; e += 4 * blockDim.x) {
    int pos[4], usr[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int eu = e + u * blockDim.x;
      pos[u] = eu < e1 ? p.entryPos[eu] - base : -1;
      usr[u] = eu < e1 ? p.entryUser[eu] : 0;
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      if (pos[u] >= 0) {
        const int sl = pos[u] / NZ;
        CS v = stored_value<S, A>(buf + sl * PZ + rotated_pos<NZ, V>(pos[u] - sl * NZ), k, converted);
        // scaling multiplies by S(1 / (Nx Ny Nz)) in S, like compress_kernel_scaled
        // (compression_kernels.cu:106-128)
        if (scale != S(0)) v = cscale(v, scale);
        out[usr[u]] = v;
      }
    }
  }
}

template <typename S, typename A, int NZ, int V = 1>
__global__ void __launch_bounds__(kThreads, ZForwardMinBlocks<A>::value) z_forward(const PlanView<S> p, S* __restrict__ values,
                                                      S scale, int spb) {
  __shared__ int sExp[2];
  z_forward_body<S, A, NZ, V>(p, values, scale, spb, blockIdx.x, sExp);
}

// ================================================================================================
// plane pass (one block per plane z)
// ================================================================================================
// Shared memory: twy[NY] | twx[NX] | (R2C) twm[M] | colOf[NXF] (int) | P[NY][numColumns] |
//                W[2][rows][WP], with LX = NX (C2C) or M = NX/2 (R2C). The forward pass streams
//                row chunks into the two W halves with cp.async (one chunk in flight while the
//                other is transformed); the backward pass uses one half.
template <int NX, int NY, bool R2C>
struct PlaneLayout {
  static constexpr int M = NX / 2;
  static constexpr int LX = R2C ? M : NX;
  static constexpr int NXF = R2C ? M + 1 : NX;
  // W rows: element e of the x-FFT row sits at e + PAD * (e / Bx), so pass 2 (which reads
  // e = k1*Bx + b across threads k1) strides by an odd number of slots; row pitch WP = Bx mod 16 so
  // two rows of pass 1 fall into different halves of the banks.
  static constexpr int Bx = Shape<LX>::B, Ax = Shape<LX>::A;
  static constexpr int PAD = (Bx % 2 == 0 && Bx > 1) ? 1 : 0;
  static constexpr int ROW = LX + PAD * Ax;
  // For LX = 12 x 8 (the x pass of 192 R2C and 96 C2C) pass 2 also conflicts at that pitch (a
  // half-warp of its work items spans two rows whose slots meet); a pitch of 12 (mod 16) keeps pass
  // 2 free of conflicts and, with the rows of pass 1 taken as 0, 2, 1, 3 within each group of four
  // (pass1_row), pass 1 too. Modelled shared-memory wavefronts of a pass-1 + pass-2 row chunk: 432
  // -> 288 for 8-byte and 224 -> 192 for 16-byte elements; every other shape is at its minimum
  // with the rule above.
  static constexpr bool kPermute1 = Ax == 12 && Bx == 8;
  static constexpr int WP = kPermute1 ? ROW + (12 - ROW % 16 + 16) % 16 : ROW + ((Bx % 16) - ROW % 16 + 16) % 16;
  __host__ __device__ static constexpr int wpos(int e) { return e + PAD * (e / Bx); }
  // Row (of the nr rows of a chunk) of pass-1 work-item row q: q itself, or 0, 2, 1, 3 within each
  // complete group of four rows for the permuted layout.
  __host__ __device__ static int pass1_row(int q, int nr) {
    if (!kPermute1) return q;
    const int g = q & ~3;
    return g + 3 < nr ? g + (((q & 1) << 1) | ((q & 2) >> 1)) : q;
  }
  template <typename CA>
  static size_t bytes(int numColumns, int rows) {
    const size_t c = sizeof(CA);
    size_t b = round16((NY + NX + (R2C ? M : 0)) * c);
    b += col_table_bytes<CA>();
    b += static_cast<size_t>(NY) * numColumns * c;
    b += 2 * static_cast<size_t>(rows) * WP * c;
    return b;
  }
  // colOf[NXF] (int), colSlots[NXF] (int), colTw[NXF] (complex), colExp[NXF] (int), each padded to
  // 16 bytes. The tables start on a 16-byte boundary (the twiddle tables before them are padded to
  // one), so every table and the buffers after them are 16-byte aligned for every length (20 * N
  // bytes of FP32 twiddles are not, for N = 90).
  __host__ __device__ static constexpr size_t round16(size_t b) { return (b + 15) / 16 * 16; }
  template <typename CA>
  __host__ __device__ static constexpr size_t col_table_bytes() {
    return 3 * round16(NXF * sizeof(int)) + round16(NXF * sizeof(CA));
  }
  // R2C forward, per output column with x = k: the W slots of Z[k] (low 16 bits) and Z[M-k] (high
  // 16 bits) in one int, and the column's twiddle e^{-2 pi i k/N} beside it (colTw), so that an
  // unpacking work item reads 4 + sizeof(complex) bytes of tables instead of an int4 and a
  // dependent twiddle.
  __host__ __device__ static int col_slots(int kk) {
    return wpos(transposed_pos<LX>(kk % M)) | (wpos(transposed_pos<LX>((M - kk) % M)) << 16);
  }
};

template <typename CA, int NX, int NY, bool R2C>
struct PlaneSmem {
  using L = PlaneLayout<NX, NY, R2C>;
  CA* twy;
  CA* twx;
  CA* twm;
  int* colOf;
  int* colSlots;
  CA* colTw;
  CA* P;
  CA* W;
  __device__ __forceinline__ explicit PlaneSmem(int numColumns) {
    twy = reinterpret_cast<CA*>(g_fast_smem);
    twx = twy + NY;
    twm = twx + NX;
    colOf = reinterpret_cast<int*>(g_fast_smem + L::round16((NY + NX + (R2C ? L::M : 0)) * sizeof(CA)));
    colSlots = reinterpret_cast<int*>(reinterpret_cast<unsigned char*>(colOf) + L::round16(L::NXF * sizeof(int)));
    colTw = reinterpret_cast<CA*>(reinterpret_cast<unsigned char*>(colSlots) + L::round16(L::NXF * sizeof(int)));
    P = reinterpret_cast<CA*>(reinterpret_cast<unsigned char*>(colOf) + L::template col_table_bytes<CA>());
    W = P + NY * numColumns;
  }
};

// The twiddles of pass 1 of the x rows in pass-1 order: entry k1 * Bx + b = w_LX^(k1 b), with
// LX = NX (C2C) or M = NX / 2 (R2C, w_M = w_NX^2). In C2C this is the only use of twx; the R2C
// packing reads w_NX in power order from twx and pass 1 reads twm.
template <typename S, typename A, int NX, bool R2C>
__device__ __forceinline__ void load_x_pass1_twiddles(typename Types<S, A>::CA* dst, const S* src) {
  using CS = typename Types<S, A>::CS;
  constexpr int LX = R2C ? NX / 2 : NX, Bx = Shape<LX>::B, step = R2C ? 2 : 1;
  const CS* tx = reinterpret_cast<const CS*>(src);
  for (int i = threadIdx.x; i < LX; i += blockDim.x) {
    const int k1 = i / Bx;
    dst[i] = tw_arith(tx[step * k1 * (i - k1 * Bx)]);
  }
}

template <typename S, typename A, int NX, int NY, bool R2C>
__device__ __forceinline__ void plane_load_tables(const PlanView<S>& p,
                                                  PlaneSmem<typename Types<S, A>::CA, NX, NY, R2C>& s) {
  using L = PlaneLayout<NX, NY, R2C>;
  using CS = typename Types<S, A>::CS;
  load_twiddles<S, A>(s.twy, p.twy, NY);
  if (R2C) load_twiddles<S, A>(s.twx, p.twx, NX);
  load_x_pass1_twiddles<S, A, NX, R2C>(R2C ? s.twm : s.twx, p.twx);
  for (int i = threadIdx.x; i < L::NXF; i += blockDim.x) s.colOf[i] = -1;
  __syncthreads();
  for (int c = threadIdx.x; c < p.numColumns; c += blockDim.x) {
    const int kk = p.columnX[c];
    s.colOf[kk] = c;
    if (R2C) {
      s.colSlots[c] = L::col_slots(kk);
      s.colTw[c] = tw_arith(reinterpret_cast<const CS*>(p.twx)[kk]);
    }
  }
}

// C2R half-length packing of nr compact rows into the x-FFT rows of W (natural order, slot
// L::wpos(k)): Z[k] = (X[k] + conj X[M-k]) + i e^{+2 pi i k/N} (X[k] - conj X[M-k]) with only the
// real parts of X[0] and X[M] (the C2R convention). One work item per pair (k, M - k): with
// s = X[k] + conj X[M-k], d = X[k] - conj X[M-k] and u = d e^{+2 pi i k/N},
// Z[k] = s + i u and Z[M-k] = conj(s) + i conj(u), so the loads, sums and the product serve both.
// Pairs j = 0 .. floor(M/2) cover every k (for even M the middle pair is k = M/2 alone).
// `row(rl)` gives compact row rl.
template <typename L, typename CA, typename RowFn>
__device__ __forceinline__ void c2r_pack_rows(RowFn row, int nr, CA* W, const int* colOf, const CA* twx,
                                              int tid, int nthreads) {
  using A = decltype(re(CA{}));
  constexpr int M = L::M, H = M / 2;
  for (int i = tid; i < nr * (H + 1); i += nthreads) {
    const int rl = i / (H + 1), j = i - rl * (H + 1);
    const CA* prow = row(rl);
    CA* wrow = W + rl * L::WP;
    const int ck = colOf[j], cm = colOf[M - j];
    const CA xk = ck >= 0 ? prow[ck] : make_c(A(0), A(0));
    const CA xm = cm >= 0 ? prow[cm] : make_c(A(0), A(0));
    if (j == 0) {
      wrow[L::wpos(0)] = make_c(re(xk) + re(xm), re(xk) - re(xm));
    } else {
      // sum = xk + conj xm, dif = xk - conj xm
      const CA xmc = cconj(xm);
      const CA sum = cadd(xk, xmc);
      const CA dif = csub(xk, xmc);
      const CA u = cmulc(dif, twx[j]);
      const CA iu = cmul_i<1>(u);
      wrow[L::wpos(j)] = cadd(sum, iu);  // (sum.x - u.y, sum.y + u.x)
      if (2 * j != M) wrow[L::wpos(M - j)] = cconj(csub(sum, iu));  // (sum.x + u.y, u.x - sum.y); M - j = j only for even M
    }
  }
}

template <typename S, typename A, int NX, int NY, bool R2C>
__device__ __forceinline__ void plane_backward_body(const PlanView<S>& p, S* __restrict__ space, int rows,
                                                    int z, int* sExpPtr, int groups = 1) {
  using TT = Types<S, A>;
  using CS = typename TT::CS;
  using CA = typename TT::CA;
  using L = PlaneLayout<NX, NY, R2C>;
  constexpr int Ay = Shape<NY, 1>::A, By = Shape<NY, 1>::B;
  constexpr int Ax = L::Ax, Bx = L::Bx;
  int& sExp = *sExpPtr;
  const int nc = p.numColumns;
  const FastDiv dnc(nc);
  PlaneSmem<CA, NX, NY, R2C> s(nc);
  plane_load_tables<S, A, NX, NY, R2C>(p, s);
  for (int i = threadIdx.x; i < NY * nc; i += blockDim.x) s.P[i] = czero<A>();
  __syncthreads();
  pdl_wait();
  pdl_trigger();

  // sticks of this plane -> compact columns, all copies in flight at once
  // (slot loads four at a time, so their latencies overlap)
  const CS* sticks = reinterpret_cast<const CS*>(p.sticks) + static_cast<size_t>(z) * p.numSticks;
  const int ns = p.numSticks;
  for (int st0 = threadIdx.x; st0 < ns; st0 += 4 * blockDim.x) {
    int pos[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int st = st0 + u * blockDim.x;
      pos[u] = st < ns ? __ldg(p.stickPlanePos + st) : -1;
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      if (pos[u] >= 0) cp_async_c(s.P + pos[u], sticks + st0 + u * blockDim.x);
    }
  }
  cp_async_commit();
  cp_async_wait<0>();
  __syncthreads();
  const int k = convert_block<S, A>(s.P, NY * nc, &sExp);
  if (R2C && p.columnX[0] == 0) line_fill(s.P, NY, nc);

  // y-FFT on every compact column, result rows left in transposed order
  for (int i = threadIdx.x; i < nc * By; i += blockDim.x) {
    const int b = dnc.div(i), c = i - b * nc;
    fft_pass1<NY, +1, 1>(s.P + c, nc, b, s.twy);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nc * Ay; i += blockDim.x) {
    const int k1 = dnc.div(i), c = i - k1 * nc;
    CA v[By];
    fft_pass2<NY, +1, 1>(s.P + c, nc, k1, v);
#pragma unroll
    for (int k2 = 0; k2 < By; ++k2) s.P[(k1 * By + k2) * nc + c] = v[k2];
  }
  __syncthreads();

  // x-FFT of every row; each row group takes its own rows in chunks of `rows / groups`
  const CA* twl = R2C ? s.twm : s.twx;
  const RowGroups rg(groups);
  const int gRows = rows / groups;
  CA* W = s.W + rg.g * gRows * L::WP;
  const int rEnd = rg.end(NY);
  for (int r0 = rg.begin(NY); r0 < rEnd; r0 += gRows) {
    const int nr = min(gRows, rEnd - r0);
    if (R2C) {
      c2r_pack_rows<L>([&](int rl) { return s.P + transposed_pos<NY, 1>(r0 + rl) * nc; }, nr, W, s.colOf, s.twx,
                       rg.t, rg.threads);
      rg.sync();
    }
    for (int i = rg.t; i < nr * Bx; i += rg.threads) {
      const int q = i / Bx, b = i - q * Bx, rl = L::pass1_row(q, nr);
      const CA* prow = s.P + transposed_pos<NY, 1>(r0 + rl) * nc;
      CA* wrow = W + rl * L::WP;
      CA v[Ax];
#pragma unroll
      for (int a = 0; a < Ax; ++a) {
        const int kk = a * Bx + b;
        if (!R2C) {
          const int col = s.colOf[kk];
          v[a] = col >= 0 ? prow[col] : czero<A>();
        } else {
          v[a] = wrow[a * (Bx + L::PAD) + b];  // L::wpos(kk), b < Bx
        }
      }
      fft_pass1_regs_ordered<L::LX, +1>(v, b, twl);
#pragma unroll
      for (int k1 = 0; k1 < Ax; ++k1) wrow[k1 * (Bx + L::PAD) + b] = v[k1];  // L::wpos(k1 * Bx + b)
    }
    rg.sync();
    const bool park = TT::kScaled && exact_block(k);
    for (int i = rg.t; i < nr * Ax; i += rg.threads) {
      const int rl = i / Ax, k1 = i - rl * Ax;
      CA v[Bx];
      CA* w2 = W + rl * L::WP + k1 * L::PAD;
      fft_pass2<L::LX, +1>(w2, 1, k1, v);
      // C2C: complex x row; C2R: pairs (x[2m], x[2m+1]) of the real row
      CS* out = reinterpret_cast<CS*>(space + (static_cast<size_t>(z) * NY + r0 + rl) * NX * (R2C ? 1 : 2));
      if (park) {
        // blocks of tiny values: results back into this item's own pass-2 slots, stored exactly below
#pragma unroll
        for (int k2 = 0; k2 < Bx; ++k2) w2[k1 * Bx + k2] = v[k2];
      } else {
#pragma unroll
        for (int k2 = 0; k2 < Bx; ++k2) out[k1 + Ax * k2] = to_storage(v[k2], k);
      }
    }
    if (park) {
      rg.sync();
      for (int i = rg.t; i < nr * L::LX; i += rg.threads) {
        const int rl = i / L::LX, e = i - rl * L::LX, k1 = e / Bx, k2 = e - k1 * Bx;
        CS* out = reinterpret_cast<CS*>(space + (static_cast<size_t>(z) * NY + r0 + rl) * NX * (R2C ? 1 : 2));
        out[k1 + Ax * k2] = to_storage_exact(W[rl * L::WP + L::wpos(e)], k);
      }
    }
    rg.sync();
  }
}

template <typename S, typename A, int NX, int NY, bool R2C>
__global__ void __launch_bounds__(kPlaneThreads) plane_backward(const PlanView<S> p,
                                                                S* __restrict__ space, int rows) {
  __shared__ int sExp[2];
  plane_backward_body<S, A, NX, NY, R2C>(p, space, rows, blockIdx.x, sExp);
}

template <typename S, typename A, int NX, int NY, bool R2C>
__device__ __forceinline__ void plane_forward_body(const PlanView<S>& p, const S* __restrict__ space, int rows,
                                                   int wRows, int z, int* sExpPtr, int groups = 1) {
  using TT = Types<S, A>;
  using CS = typename TT::CS;
  using CA = typename TT::CA;
  using L = PlaneLayout<NX, NY, R2C>;
  constexpr int Ay = Shape<NY>::A, By = Shape<NY>::B;
  constexpr int Ax = L::Ax, Bx = L::Bx;
  int& sExp = *sExpPtr;
  const int nc = p.numColumns;
  const FastDiv dnc(nc);
  PlaneSmem<CA, NX, NY, R2C> s(nc);
  plane_load_tables<S, A, NX, NY, R2C>(p, s);

  // Row chunks of plane z are contiguous in the space buffer. Each row group (RowGroups) takes its
  // own rows in chunks of rows / groups. When W holds two chunks per group (wRows >= 2 * rows),
  // each group streams its chunk i+1 into its other half while chunk i is transformed; otherwise
  // each chunk is loaded after the previous one is done (other groups and blocks cover the wait).
  const CS* plane = reinterpret_cast<const CS*>(space + static_cast<size_t>(z) * NY * NX * (R2C ? 1 : 2));
  const RowGroups rg(groups);
  const int gRows = rows / groups;
  const bool dbuf = 2 * rows <= wRows;
  CA* Wg = s.W + rg.g * (dbuf ? 2 : 1) * gRows * L::WP;
  const int gBegin = rg.begin(NY), gEnd = rg.end(NY);
  const int nchunks = (gEnd - gBegin + gRows - 1) / gRows;
  auto issue_chunk = [&](int chunk) {
    const int r0 = gBegin + chunk * gRows, nr = min(gRows, gEnd - r0);
    CA* dst = Wg + (dbuf ? (chunk & 1) : 0) * gRows * L::WP;
    const CS* src = plane + static_cast<size_t>(r0) * L::LX;
    if (rg.threads % L::LX == 0) {
      // every thread keeps one row position: its padded slot is computed once
      const int e = rg.t % L::LX, pe = L::wpos(e), step = rg.threads / L::LX;
      for (int rl = rg.t / L::LX; rl < nr; rl += step) cp_async_c(dst + rl * L::WP + pe, src + rl * L::LX + e);
    } else {
      for (int i = rg.t; i < nr * L::LX; i += rg.threads) {
        const int rl = i / L::LX, e = i - rl * L::LX;
        cp_async_c(dst + rl * L::WP + L::wpos(e), src + i);
      }
    }
    cp_async_commit();
  };
  pdl_wait();
  pdl_trigger();
  issue_chunk(0);

  // Block scale (double-float only): the largest exponent of the whole plane, read once up front
  // while the first chunk is in flight (the plane then stays in L2 for the chunk loads).
  int k = 0;
  if (TT::kScaled) {
    if (threadIdx.x == 0) {
      sExp = 0;
      (&sExp)[1] = kDdNoSubnormal;
    }
    __syncthreads();
    int e = 0;
    for (int i = threadIdx.x; i < NY * L::LX; i += blockDim.x) e = max(e, max_exponent(plane[i]));
    atomicMax(&sExp, e);
  }
  __syncthreads();
  if (TT::kScaled) {
    k = block_scale(finish_block_key(&sExp, [=] {
      int m = kDdNoSubnormal;
      for (int i = threadIdx.x; i < NY * L::LX; i += blockDim.x) m = max(m, max_subnormal_key(plane[i]));
      return m;
    }));
  }

  const CA* twl = R2C ? s.twm : s.twx;
  for (int chunk = 0; chunk < nchunks; ++chunk) {
    const int r0 = gBegin + chunk * gRows, nr = min(gRows, gEnd - r0);
    CA* wbase = Wg + (dbuf ? (chunk & 1) : 0) * gRows * L::WP;
    if (!dbuf && chunk > 0) issue_chunk(chunk);
    if (dbuf && chunk + 1 < nchunks) {
      issue_chunk(chunk + 1);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    rg.sync();
    // a plane of tiny values converts its chunk exactly first (uniform branch)
    const bool pre = TT::kScaled && exact_block(k);
    if (pre) {
      for (int i = rg.t; i < nr * L::LX; i += rg.threads) {
        const int rl = i / L::LX, e = i - rl * L::LX;
        CA* slot = wbase + rl * L::WP + L::wpos(e);
        *slot = to_arith_exact(*reinterpret_cast<const CS*>(slot), k);
      }
      rg.sync();
    }
    for (int i = rg.t; i < nr * Bx; i += rg.threads) {
      const int q = i / Bx, b = i - q * Bx, rl = L::pass1_row(q, nr);
      // padded row: element a*Bx + b sits at a*(Bx + PAD) + b (raw storage values until here)
      CA* wrow = wbase + rl * L::WP;
      CA v[Ax];
#pragma unroll
      for (int a = 0; a < Ax; ++a) {
        const int slot = a * (Bx + L::PAD) + b;
        v[a] = pre ? wrow[slot] : to_arith(reinterpret_cast<const CS*>(wrow)[slot], k);
      }
      fft_pass1_regs_ordered<L::LX, -1>(v, b, twl);
#pragma unroll
      for (int k1 = 0; k1 < Ax; ++k1) wrow[k1 * (Bx + L::PAD) + b] = v[k1];
    }
    rg.sync();
    for (int i = rg.t; i < nr * Ax; i += rg.threads) {
      const int rl = i / Ax, k1 = i - rl * Ax;
      CA v[Bx];
      CA* wrow = wbase + rl * L::WP + k1 * L::PAD;
      fft_pass2<L::LX, -1>(wrow, 1, k1, v);
      if (!R2C) {
        CA* prow = s.P + (r0 + rl) * nc;
#pragma unroll
        for (int k2 = 0; k2 < Bx; ++k2) {
          const int col = s.colOf[k1 + Ax * k2];
          if (col >= 0) prow[col] = v[k2];
        }
      } else {
#pragma unroll
        for (int k2 = 0; k2 < Bx; ++k2) wrow[k1 * Bx + k2] = v[k2];  // wrow is offset by k1*PAD
      }
    }
    rg.sync();
    if (R2C) {
      // X[k] = (Z[k] + conj Z[M-k]) / 2 - i/2 e^{-2 pi i k/N} (Z[k] - conj Z[M-k]), Z[M] = Z[0]
      for (int i = rg.t; i < nr * nc; i += rg.threads) {
        const int rl = dnc.div(i), c = i - rl * nc;
        const int sl = s.colSlots[c];
        const CA tw = s.colTw[c];
        const CA* wrow = wbase + rl * L::WP;
        const CA zk = wrow[sl & 0xffff];
        const CA zm = wrow[sl >> 16];
        const CA zmc = cconj(zm);
        const CA dif = csub(zk, zmc);  // (zk.x - zm.x, zk.y + zm.y)
        const CA u = cmul(dif, tw);
        s.P[(r0 + rl) * nc + c] = chalf(csub(cadd(zk, zmc), cmul_i<1>(u)));
      }
      rg.sync();
    }
  }
  if (groups > 1) __syncthreads();  // every group's rows are in P before the y pass

  for (int i = threadIdx.x; i < nc * By; i += blockDim.x) {
    const int b = dnc.div(i), c = i - b * nc;
    fft_pass1<NY, -1>(s.P + c, nc, b, s.twy);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nc * Ay; i += blockDim.x) {
    const int k1 = dnc.div(i), c = i - k1 * nc;
    CA v[By];
    fft_pass2<NY, -1>(s.P + c, nc, k1, v);
#pragma unroll
    for (int k2 = 0; k2 < By; ++k2) s.P[(k1 * By + k2) * nc + c] = v[k2];
  }
  __syncthreads();
  CS* sticks = reinterpret_cast<CS*>(p.sticks) + static_cast<size_t>(z) * p.numSticks;
  const int ns = p.numSticks;
  const bool converted = TT::kScaled && exact_block(k);
  if (converted) {
    convert_exact_in_place<S, A>(s.P, NY * nc, k, threadIdx.x, blockDim.x);
    __syncthreads();
  }
  for (int st0 = threadIdx.x; st0 < ns; st0 += 4 * blockDim.x) {
    int pos[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int st = st0 + u * blockDim.x;
      pos[u] = st < ns ? __ldg(p.stickPlanePos + st) : -1;
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      if (pos[u] >= 0) {
        const int y = dnc.div(pos[u]), c = pos[u] - y * nc;
        sticks[st0 + u * blockDim.x] = stored_value<S, A>(s.P + transposed_pos<NY>(y) * nc + c, k, converted);
      }
    }
  }
}

template <typename S, typename A, int NX, int NY, bool R2C>
__global__ void __launch_bounds__(kPlaneThreads) plane_forward(const PlanView<S> p,
                                                               const S* __restrict__ space, int rows) {
  __shared__ int sExp[2];
  plane_forward_body<S, A, NX, NY, R2C>(p, space, rows, rows, blockIdx.x, sExp);
}

// ================================================================================================
// host-side launchers (instantiated per size in kernels_fast_group_*.cu)
// ================================================================================================
// Raise a kernel's dynamic shared memory limit to what is left of the opt-in maximum after its
// static shared memory.
template <typename K>
cudaError_t allow_dynamic_smem(K kernel, size_t maxSmem) {
  cudaFuncAttributes attr{};
  cudaError_t e = cudaFuncGetAttributes(&attr, kernel);
  if (e != cudaSuccess) return e;
  const size_t avail = maxSmem > attr.sharedSizeBytes ? maxSmem - attr.sharedSizeBytes : 0;
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(avail));
}
// Launch with programmatic stream serialization (see pdl_wait); SPFFT_GB300_PDL=0 at the first
// launch turns it off for the process. Errors are left for cudaGetLastError like <<<>>> launches.
bool pdl_enabled();
template <typename... KArgs, typename... Args>
inline void launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                       Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl_enabled() ? 1 : 0;
  (void)cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

// `variant`: 0 the default split (Shape<N, 1>), 1 the swapped two-pass split (Shape<N, 2>) where
// the length has one (has_swapped_split<N>), 2 the three-pass split (Shape<N, 3>) where the length
// has one and the arithmetic is double-float (has_three<A, N>); otherwise the default.
template <typename A, int N>
constexpr bool has_three() {
  return std::is_same<A, dd>::value && has_three_pass<N>();
}
template <typename S, typename A, int NZ>
struct ZKernels {
  using CA = typename Types<S, A>::CA;
  static size_t smem(int spb) { return (2 * NZ + static_cast<size_t>(spb) * ZLayout<NZ>::pitch) * sizeof(CA); }
  static cudaError_t prepare(size_t maxSmem) {
    cudaError_t e1 = allow_dynamic_smem(z_backward<S, A, NZ>, maxSmem);
    cudaError_t e2 = allow_dynamic_smem(z_forward<S, A, NZ>, maxSmem);
    if constexpr (has_swapped_split<NZ>()) {
      if (e1 == cudaSuccess) e1 = allow_dynamic_smem(z_backward<S, A, NZ, 2>, maxSmem);
      if (e2 == cudaSuccess) e2 = allow_dynamic_smem(z_forward<S, A, NZ, 2>, maxSmem);
    }
    if constexpr (has_three<A, NZ>()) {
      if (e1 == cudaSuccess) e1 = allow_dynamic_smem(z_backward<S, A, NZ, 3>, maxSmem);
      if (e2 == cudaSuccess) e2 = allow_dynamic_smem(z_forward<S, A, NZ, 3>, maxSmem);
    }
    return e1 != cudaSuccess ? e1 : e2;
  }
  static void backward(const PlanView<S>& p, int spb, const S* values, cudaStream_t st, int variant) {
    const int g = (p.numSticks + spb - 1) / spb;
    if constexpr (has_swapped_split<NZ>()) {
      if (variant == 1) return launch_pdl(z_backward<S, A, NZ, 2>, g, kThreads, smem(spb), st, p, values, spb);
    }
    if constexpr (has_three<A, NZ>()) {
      if (variant == 2) return launch_pdl(z_backward<S, A, NZ, 3>, g, kThreads, smem(spb), st, p, values, spb);
    }
    launch_pdl(z_backward<S, A, NZ>, g, kThreads, smem(spb), st, p, values, spb);
  }
  static void forward(const PlanView<S>& p, int spb, S* values, S scale, cudaStream_t st, int variant) {
    const int g = (p.numSticks + spb - 1) / spb;
    if constexpr (has_swapped_split<NZ>()) {
      if (variant == 1) return launch_pdl(z_forward<S, A, NZ, 2>, g, kThreads, smem(spb), st, p, values, scale, spb);
    }
    if constexpr (has_three<A, NZ>()) {
      if (variant == 2) return launch_pdl(z_forward<S, A, NZ, 3>, g, kThreads, smem(spb), st, p, values, scale, spb);
    }
    launch_pdl(z_forward<S, A, NZ>, g, kThreads, smem(spb), st, p, values, scale, spb);
  }
};

template <typename S, typename A, int NX, int NY, bool R2C>
struct PlaneKernels {
  using L = PlaneLayout<NX, NY, R2C>;
  using CA = typename Types<S, A>::CA;
  static size_t smem(int numColumns, int rows) { return L::template bytes<CA>(numColumns, rows); }
  static cudaError_t prepare(size_t maxSmem) {
    cudaError_t e1 = allow_dynamic_smem(plane_backward<S, A, NX, NY, R2C>, maxSmem);
    cudaError_t e2 = allow_dynamic_smem(plane_forward<S, A, NX, NY, R2C>, maxSmem);
    return e1 != cudaSuccess ? e1 : e2;
  }
  // `half`: the shared memory holds 2 * half rows of x chunk buffer, which both directions use as
  // one chunk of 2 * half rows (single-buffered, like the batched plane passes).
  static void backward(const PlanView<S>& p, int half, S* space, cudaStream_t st, int threads) {
    launch_pdl(plane_backward<S, A, NX, NY, R2C>, p.dimZ, threads, smem(p.numColumns, half), st, p, space, 2 * half);
  }
  static void forward(const PlanView<S>& p, int half, const S* space, cudaStream_t st, int threads) {
    launch_pdl(plane_forward<S, A, NX, NY, R2C>, p.dimZ, threads, smem(p.numColumns, half), st, p, space, 2 * half);
  }
};

// ================================================================================================
// split plane passes: y kernel over column groups, x kernel over row groups, with the compact
// plane [z][y][numColumns] in HBM between them. More traffic than the fused plane kernel but many
// small blocks instead of one large block per plane, so every SM stays busy.
// ================================================================================================
// y backward: block (column group, z); V selects the two-pass split of the y length as in the z
// pass
template <typename S, typename A, int NY, int V = 1>
__device__ __forceinline__ void y_backward_body(const PlanView<S>& p, int cpb, int bx, int z, int* sExpPtr) {
  using TT = Types<S, A>;
  using CS = typename TT::CS;
  using CA = typename TT::CA;
  constexpr int Ay = Shape<NY, V>::A, By = Shape<NY, V>::B;
  int& sExp = *sExpPtr;
  CA* tw = reinterpret_cast<CA*>(g_fast_smem);
  CA* buf = tw + NY;
  const int nc = p.numColumns;
  // ceil(nc / cpb) column groups of balanced sizes (at most cpb columns each)
  const int groups = (nc + cpb - 1) / cpb;
  const int c0 = bx * nc / groups, ncb = (bx + 1) * nc / groups - c0;
  const FastDiv dncb(ncb), dnc(nc);
  load_twiddles<S, A>(tw, p.twy, NY);
  for (int i = threadIdx.x; i < NY * ncb; i += blockDim.x) buf[i] = czero<A>();
  // Plan tables (constant from plan creation on) are read before the wait for the previous kernel:
  // the stick range of the column group and this thread's first four stick slots.
  const int sBegin = p.columnStickStart[c0], sEnd = p.columnStickStart[c0 + ncb];
  int pos0[4];
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int st = sBegin + threadIdx.x + u * blockDim.x;
    pos0[u] = st < sEnd ? __ldg(p.stickPlanePos + st) : -1;
  }
  if (TT::kScaled && p.sticksRaw && threadIdx.x == 0) sExp = kZeroExp;
  __syncthreads();
  pdl_wait();
  pdl_trigger();
  const CS* sticks = reinterpret_cast<const CS*>(p.sticks) + static_cast<size_t>(z) * p.numSticks;
  int k = 0;
  if (TT::kScaled && p.sticksRaw) {
    // double-float sticks from the z pass: block scale = smallest stick exponent; each value is
    // brought to it as it is stored. The first four sticks of every thread (all of them when the
    // group has at most 4 * blockDim.x sticks) stay in registers from the load to the store, so
    // the exponents and the values arrive in one round trip.
    const CA* rs = reinterpret_cast<const CA*>(sticks);
    int ex0[4];
    CA val0[4];
    int e = kZeroExp;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int st = sBegin + threadIdx.x + u * blockDim.x;
      ex0[u] = pos0[u] >= 0 ? p.stickExp[st] : kZeroExp;
      if (pos0[u] >= 0) val0[u] = rs[st];
      e = min(e, ex0[u]);
    }
    for (int st = sBegin + threadIdx.x + 4 * blockDim.x; st < sEnd; st += blockDim.x) e = min(e, p.stickExp[st]);
    atomicMin(&sExp, e);
    __syncthreads();
    k = sExp == kZeroExp ? 0 : sExp;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      if (pos0[u] >= 0) {
        const int y = dnc.div(pos0[u]), c = pos0[u] - y * nc;
        buf[y * ncb + (c - c0)] = scale_pow2(val0[u], k - ex0[u]);
      }
    }
    for (int st0 = sBegin + threadIdx.x + 4 * blockDim.x; st0 < sEnd; st0 += 4 * blockDim.x) {
      int pos[4], ex[4];
      CA val[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int st = st0 + u * blockDim.x;
        pos[u] = st < sEnd ? __ldg(p.stickPlanePos + st) : -1;
        ex[u] = st < sEnd ? p.stickExp[st] : 0;
        if (st < sEnd) val[u] = rs[st];
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        if (pos[u] >= 0) {
          const int y = dnc.div(pos[u]), c = pos[u] - y * nc;
          buf[y * ncb + (c - c0)] = scale_pow2(val[u], k - ex[u]);
        }
      }
    }
    __syncthreads();
  } else {
    for (int st0 = sBegin + threadIdx.x; st0 < sEnd; st0 += 4 * blockDim.x) {
      int pos[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int st = st0 + u * blockDim.x;
        pos[u] = st0 == sBegin + threadIdx.x ? pos0[u] : (st < sEnd ? __ldg(p.stickPlanePos + st) : -1);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        if (pos[u] >= 0) {
          const int y = dnc.div(pos[u]), c = pos[u] - y * nc;
          cp_async_c(buf + y * ncb + (c - c0), sticks + st0 + u * blockDim.x);
        }
      }
    }
    cp_async_commit();
    cp_async_wait<0>();
    __syncthreads();
    k = convert_block<S, A>(buf, NY * ncb, &sExp);
  }
  if (p.r2c && c0 == 0 && p.columnX[0] == 0) line_fill(buf, NY, ncb);
  for (int i = threadIdx.x; i < ncb * By; i += blockDim.x) {
    const int b = dncb.div(i), c = i - b * ncb;
    fft_pass1<NY, +1, V>(buf + c, ncb, b, tw);
  }
  __syncthreads();
  CS* planes = reinterpret_cast<CS*>(p.planes) + static_cast<size_t>(z) * NY * nc + c0;
  const bool raw = TT::kScaled && p.planesRaw;
  const bool park = TT::kScaled && !raw && exact_block(k);
  if constexpr (V == 3) {
    // pass 2 as pass 2a (B1-point DFTs) and pass 2b (B2-point DFTs); columns fastest across threads
    constexpr int B1 = Split3<NY>::B1, B2 = Split3<NY>::B2;
    for (int i = threadIdx.x; i < ncb * Ay * B2; i += blockDim.x) {
      const int r = dncb.div(i), c = i - r * ncb, k1 = r / B2;
      fft_pass2a<NY, +1>(buf + c, ncb, k1, r - k1 * B2, tw);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < ncb * Ay * B1; i += blockDim.x) {
      const int r = dncb.div(i), c = i - r * ncb, k1 = r / B1, kk1 = r - k1 * B1;
      CA v[B2];
      fft_pass2b<NY, +1>(buf + c, ncb, k1, kk1, v);
#pragma unroll
      for (int kk2 = 0; kk2 < B2; ++kk2) {
        const size_t at = static_cast<size_t>(k1 + Ay * (kk1 + B1 * kk2)) * nc + c;
        if (raw) reinterpret_cast<CA*>(planes)[at] = v[kk2];
        else if (park) buf[(k1 * By + kk1 * B2 + kk2) * ncb + c] = v[kk2];
        else planes[at] = to_storage(v[kk2], k);
      }
    }
  } else {
    for (int i = threadIdx.x; i < ncb * Ay; i += blockDim.x) {
      const int k1 = dncb.div(i), c = i - k1 * ncb;
      CA v[By];
      fft_pass2<NY, +1, V>(buf + c, ncb, k1, v);
      if (raw) {
        CA* rp = reinterpret_cast<CA*>(planes);
#pragma unroll
        for (int k2 = 0; k2 < By; ++k2) rp[static_cast<size_t>(k1 + Ay * k2) * nc + c] = v[k2];
      } else if (park) {
        // blocks of tiny values: results back into this item's own pass-2 slots, stored exactly below
#pragma unroll
        for (int k2 = 0; k2 < By; ++k2) buf[(k1 * By + k2) * ncb + c] = v[k2];
      } else {
#pragma unroll
        for (int k2 = 0; k2 < By; ++k2) planes[static_cast<size_t>(k1 + Ay * k2) * nc + c] = to_storage(v[k2], k);
      }
    }
  }
  if (park) {
    __syncthreads();
    for (int i = threadIdx.x; i < NY * ncb; i += blockDim.x) {
      const int e = i / ncb, c = i - e * ncb;
      int y;
      if constexpr (V == 3) {
        y = three_pass_index<NY>(e);
      } else {
        const int k1 = e / By;
        y = k1 + Ay * (e - k1 * By);
      }
      planes[static_cast<size_t>(y) * nc + c] = to_storage_exact(buf[e * ncb + c], k);
    }
  }
  if (raw && threadIdx.x < ncb) p.planeExp[z * nc + c0 + threadIdx.x] = produced_exp(sExp, k);
}

template <typename S, typename A, int NY, int V = 1>
__global__ void __launch_bounds__(kThreads, YMinBlocks<A>::value) y_backward_split(const PlanView<S> p, int cpb,
                                                                                     int z0) {
  __shared__ int sExp[2];
  y_backward_body<S, A, NY, V>(p, cpb, blockIdx.x, z0 + blockIdx.y, sExp);
}

// y forward: block (column group, z)
template <typename S, typename A, int NY, int V = 1>
__device__ __forceinline__ void y_forward_body(const PlanView<S>& p, int cpb, int bx, int z, int* sExpPtr) {
  using TT = Types<S, A>;
  using CS = typename TT::CS;
  using CA = typename TT::CA;
  constexpr int Ay = Shape<NY, V>::A, By = Shape<NY, V>::B;
  int& sExp = *sExpPtr;
  CA* tw = reinterpret_cast<CA*>(g_fast_smem);
  CA* buf = tw + NY;
  const int nc = p.numColumns;
  // ceil(nc / cpb) column groups of balanced sizes (at most cpb columns each)
  const int groups = (nc + cpb - 1) / cpb;
  const int c0 = bx * nc / groups, ncb = (bx + 1) * nc / groups - c0;
  const FastDiv dncb(ncb), dnc(nc);
  load_twiddles<S, A>(tw, p.twy, NY);
  pdl_wait();
  pdl_trigger();
  const CS* planes = reinterpret_cast<const CS*>(p.planes) + static_cast<size_t>(z) * NY * nc + c0;
  for (int i = threadIdx.x; i < NY * ncb; i += blockDim.x) {
    const int y = dncb.div(i), c = i - y * ncb;
    cp_async_c(buf + i, planes + static_cast<size_t>(y) * nc + c);
  }
  cp_async_commit();
  int k = 0;
  if (TT::kScaled && p.planesRaw) {
    // double-float rows from the x pass: scale of the block = smallest row exponent
    int* rowExp = reinterpret_cast<int*>(buf + NY * cpb);
    if (threadIdx.x == 0) sExp = kZeroExp;
    __syncthreads();
    int e = kZeroExp;
    for (int y = threadIdx.x; y < NY; y += blockDim.x) {
      rowExp[y] = p.planeExp[z * NY + y];
      e = min(e, rowExp[y]);
    }
    atomicMin(&sExp, e);
    cp_async_wait<0>();
    __syncthreads();
    k = sExp == kZeroExp ? 0 : sExp;
    for (int i = threadIdx.x; i < NY * ncb; i += blockDim.x) {
      const int y = dncb.div(i);
      buf[i] = scale_pow2(buf[i], k - rowExp[y]);
    }
    __syncthreads();
  } else {
    cp_async_wait<0>();
    __syncthreads();
    k = convert_block<S, A>(buf, NY * ncb, &sExp);
  }
  for (int i = threadIdx.x; i < ncb * By; i += blockDim.x) {
    const int b = dncb.div(i), c = i - b * ncb;
    fft_pass1<NY, -1, V>(buf + c, ncb, b, tw);
  }
  __syncthreads();
  if constexpr (V == 3) {
    constexpr int B1 = Split3<NY>::B1, B2 = Split3<NY>::B2;
    for (int i = threadIdx.x; i < ncb * Ay * B2; i += blockDim.x) {
      const int r = dncb.div(i), c = i - r * ncb, k1 = r / B2;
      fft_pass2a<NY, -1>(buf + c, ncb, k1, r - k1 * B2, tw);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < ncb * Ay * B1; i += blockDim.x) {
      const int r = dncb.div(i), c = i - r * ncb, k1 = r / B1, kk1 = r - k1 * B1;
      CA v[B2];
      fft_pass2b<NY, -1>(buf + c, ncb, k1, kk1, v);
#pragma unroll
      for (int kk2 = 0; kk2 < B2; ++kk2) buf[(k1 * By + kk1 * B2 + kk2) * ncb + c] = v[kk2];
    }
  } else {
    for (int i = threadIdx.x; i < ncb * Ay; i += blockDim.x) {
      const int k1 = dncb.div(i), c = i - k1 * ncb;
      CA v[By];
      fft_pass2<NY, -1, V>(buf + c, ncb, k1, v);
#pragma unroll
      for (int k2 = 0; k2 < By; ++k2) buf[(k1 * By + k2) * ncb + c] = v[k2];
    }
  }
  __syncthreads();
  CS* sticks = reinterpret_cast<CS*>(p.sticks) + static_cast<size_t>(z) * p.numSticks;
  const int sBegin = p.columnStickStart[c0], sEnd = p.columnStickStart[c0 + ncb];
  const bool raw = TT::kScaled && p.sticksRaw;
  const bool converted = TT::kScaled && !raw && exact_block(k);
  if (converted) {
    convert_exact_in_place<S, A>(buf, NY * ncb, k, threadIdx.x, blockDim.x);
    __syncthreads();
  }
  for (int st0 = sBegin + threadIdx.x; st0 < sEnd; st0 += 4 * blockDim.x) {
    int pos[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int st = st0 + u * blockDim.x;
      pos[u] = st < sEnd ? __ldg(p.stickPlanePos + st) : -1;
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      if (pos[u] >= 0) {
        const int y = dnc.div(pos[u]), c = pos[u] - y * nc;
        const CA* slot = buf + transposed_pos<NY, V>(y) * ncb + (c - c0);
        if (raw) reinterpret_cast<CA*>(sticks)[st0 + u * blockDim.x] = *slot;
        else sticks[st0 + u * blockDim.x] = stored_value<S, A>(slot, k, converted);
      }
    }
  }
  // exponent of this block's sticks of plane z, per column (the z forward reads them per stick)
  if (raw && threadIdx.x < ncb) p.stickExp[z * nc + c0 + threadIdx.x] = sExp == kZeroExp ? kZeroExp : k;
}

template <typename S, typename A, int NY, int V = 1>
__global__ void __launch_bounds__(kThreads, YMinBlocks<A>::value) y_forward_split(const PlanView<S> p, int cpb,
                                                                                    int z0) {
  __shared__ int sExp[2];
  y_forward_body<S, A, NY, V>(p, cpb, blockIdx.x, z0 + blockIdx.y, sExp);
}

// Shared memory of the x kernels: twx[NX] | (R2C) twm[M] | colOf[NXF] | P[rows][numColumns] |
// W[rows][WP].
template <typename CA, int NX, bool R2C>
struct RowSmem {
  using L = PlaneLayout<NX, 2, R2C>;
  CA* twx;
  CA* twm;
  int* colOf;
  int* colSlots;
  CA* colTw;
  int* colExp;
  CA* P;
  CA* W;
  // withP = false: no compact-row buffer (the R2C forward stores its output columns straight to
  // HBM), W starts where P would.
  __device__ __forceinline__ RowSmem(int numColumns, int rows, bool withP = true) {
    twx = reinterpret_cast<CA*>(g_fast_smem);
    twm = twx + NX;
    colOf = reinterpret_cast<int*>(g_fast_smem + L::round16((NX + (R2C ? L::M : 0)) * sizeof(CA)));
    colSlots = reinterpret_cast<int*>(reinterpret_cast<unsigned char*>(colOf) + L::round16(L::NXF * sizeof(int)));
    colTw = reinterpret_cast<CA*>(reinterpret_cast<unsigned char*>(colSlots) + L::round16(L::NXF * sizeof(int)));
    colExp = reinterpret_cast<int*>(reinterpret_cast<unsigned char*>(colTw) + L::round16(L::NXF * sizeof(CA)));
    P = reinterpret_cast<CA*>(reinterpret_cast<unsigned char*>(colOf) + L::template col_table_bytes<CA>());
    W = P + (withP ? rows * numColumns : 0);
  }
  template <typename CAT>
  static size_t bytes(int numColumns, int rows, bool withP = true) {
    const size_t c = sizeof(CAT);
    return L::round16((NX + (R2C ? L::M : 0)) * c) + L::template col_table_bytes<CAT>() +
           (withP ? static_cast<size_t>(rows) * numColumns * c : 0) + static_cast<size_t>(rows) * L::WP * c;
  }
};

template <typename S, typename A, int NX, bool R2C>
__device__ __forceinline__ void row_load_tables(const PlanView<S>& p, RowSmem<typename Types<S, A>::CA, NX, R2C>& s) {
  using L = PlaneLayout<NX, 2, R2C>;
  using CS = typename Types<S, A>::CS;
  if (R2C) load_twiddles<S, A>(s.twx, p.twx, NX);
  load_x_pass1_twiddles<S, A, NX, R2C>(R2C ? s.twm : s.twx, p.twx);
  for (int i = threadIdx.x; i < L::NXF; i += blockDim.x) s.colOf[i] = -1;
  __syncthreads();
  for (int c = threadIdx.x; c < p.numColumns; c += blockDim.x) {
    const int kk = p.columnX[c];
    s.colOf[kk] = c;
    if (R2C) {
      s.colSlots[c] = L::col_slots(kk);
      s.colTw[c] = tw_arith(reinterpret_cast<const CS*>(p.twx)[kk]);
    }
  }
}

// x backward: block (row group, z); compact rows from HBM -> x-FFT -> space rows
template <typename S, typename A, int NX, bool R2C>
__device__ __forceinline__ void x_backward_body(const PlanView<S>& p, S* __restrict__ space, int rpb,
                                                int bx, int z, int* sExpPtr) {
  using TT = Types<S, A>;
  using CS = typename TT::CS;
  using CA = typename TT::CA;
  using L = PlaneLayout<NX, 2, R2C>;
  constexpr int Ax = L::Ax, Bx = L::Bx;
  int& sExp = *sExpPtr;
  const int nc = p.numColumns, ny = p.dimY;
  const int y0 = bx * rpb, nr = min(rpb, ny - y0);
  RowSmem<CA, NX, R2C> s(nc, rpb);
  row_load_tables<S, A, NX, R2C>(p, s);
  pdl_wait();
  pdl_trigger();
  const CS* planes = reinterpret_cast<const CS*>(p.planes) + (static_cast<size_t>(z) * ny + y0) * nc;
  for (int i = threadIdx.x; i < nr * nc; i += blockDim.x) cp_async_c(s.P + i, planes + i);
  cp_async_commit();
  int k = 0;
  if (TT::kScaled && p.planesRaw) {
    // double-float columns from the y pass: scale of the block = smallest column exponent
    if (threadIdx.x == 0) sExp = kZeroExp;
    __syncthreads();
    int e = kZeroExp;
    for (int c = threadIdx.x; c < nc; c += blockDim.x) {
      s.colExp[c] = p.planeExp[z * nc + c];
      e = min(e, s.colExp[c]);
    }
    atomicMin(&sExp, e);
    cp_async_wait<0>();
    __syncthreads();
    k = sExp == kZeroExp ? 0 : sExp;
    const FastDiv dnc(nc);
    for (int i = threadIdx.x; i < nr * nc; i += blockDim.x) {
      const int rl = dnc.div(i), c = i - rl * nc;
      s.P[i] = scale_pow2(s.P[i], k - s.colExp[c]);
    }
    __syncthreads();
  } else {
    cp_async_wait<0>();
    __syncthreads();
    k = convert_block<S, A>(s.P, nr * nc, &sExp);
  }
  const CA* twl = R2C ? s.twm : s.twx;
  if (R2C) {
    c2r_pack_rows<L>([&](int rl) { return s.P + rl * nc; }, nr, s.W, s.colOf, s.twx, threadIdx.x, blockDim.x);
    __syncthreads();
  }
  for (int i = threadIdx.x; i < nr * Bx; i += blockDim.x) {
    const int q = i / Bx, b = i - q * Bx, rl = L::pass1_row(q, nr);
    const CA* prow = s.P + rl * nc;
    CA* wrow = s.W + rl * L::WP;
    CA v[Ax];
#pragma unroll
    for (int a = 0; a < Ax; ++a) {
      const int kk = a * Bx + b;
      if (!R2C) {
        const int col = s.colOf[kk];
        v[a] = col >= 0 ? prow[col] : czero<A>();
      } else {
        v[a] = wrow[L::wpos(kk)];
      }
    }
    fft_pass1_regs_ordered<L::LX, +1>(v, b, twl);
#pragma unroll
    for (int k1 = 0; k1 < Ax; ++k1) wrow[k1 * (Bx + L::PAD) + b] = v[k1];  // L::wpos(k1 * Bx + b)
  }
  __syncthreads();
  const bool park = TT::kScaled && exact_block(k);
  for (int i = threadIdx.x; i < nr * Ax; i += blockDim.x) {
    const int rl = i / Ax, k1 = i - rl * Ax;
    CA v[Bx];
    fft_pass2<L::LX, +1>(s.W + rl * L::WP + k1 * L::PAD, 1, k1, v);
    CS* out = reinterpret_cast<CS*>(space + (static_cast<size_t>(z) * ny + y0 + rl) * NX * (R2C ? 1 : 2));
    if (park) {
      // blocks of tiny values: results back into this item's own pass-2 slots, stored exactly below
      CA* w2 = s.W + rl * L::WP + k1 * L::PAD;
#pragma unroll
      for (int k2 = 0; k2 < Bx; ++k2) w2[k1 * Bx + k2] = v[k2];
    } else {
#pragma unroll
      for (int k2 = 0; k2 < Bx; ++k2) out[k1 + Ax * k2] = to_storage(v[k2], k);
    }
  }
  if (park) {
    __syncthreads();
    for (int i = threadIdx.x; i < nr * L::LX; i += blockDim.x) {
      const int rl = i / L::LX, e = i - rl * L::LX, k1 = e / Bx, k2 = e - k1 * Bx;
      CS* out = reinterpret_cast<CS*>(space + (static_cast<size_t>(z) * ny + y0 + rl) * NX * (R2C ? 1 : 2));
      out[k1 + Ax * k2] = to_storage_exact(s.W[rl * L::WP + L::wpos(e)], k);
    }
  }
}

// Planes z0 + blockIdx.y (z0 > 0 when a plane range is transformed on its own).
template <typename S, typename A, int NX, bool R2C>
__global__ void __launch_bounds__(XBackwardThreads<A, R2C>::value) x_backward_split(const PlanView<S> p, S* __restrict__ space,
                                                             int rpb, int z0) {
  __shared__ int sExp[2];
  x_backward_body<S, A, NX, R2C>(p, space, rpb, blockIdx.x, z0 + blockIdx.y, sExp);
}

// x forward: block (row group, z); space rows -> x-FFT -> compact rows to HBM
template <typename S, typename A, int NX, bool R2C>
__device__ __forceinline__ void x_forward_body(const PlanView<S>& p, const S* __restrict__ space, int rpb,
                                               int bx, int z, int* sExpPtr) {
  using TT = Types<S, A>;
  using CS = typename TT::CS;
  using CA = typename TT::CA;
  using L = PlaneLayout<NX, 2, R2C>;
  constexpr int Ax = L::Ax, Bx = L::Bx;
  int& sExp = *sExpPtr;
  const int nc = p.numColumns, ny = p.dimY;
  const FastDiv dnc(nc);
  const int y0 = bx * rpb, nr = min(rpb, ny - y0);
  RowSmem<CA, NX, R2C> s(nc, rpb, !R2C);
  if (TT::kScaled && threadIdx.x == 0) {
    sExp = 0;
    (&sExp)[1] = kDdNoSubnormal;
  }
  row_load_tables<S, A, NX, R2C>(p, s);
  pdl_wait();
  pdl_trigger();
  const CS* rows = reinterpret_cast<const CS*>(space + (static_cast<size_t>(z) * ny + y0) * NX * (R2C ? 1 : 2));
  for (RowWalk w(threadIdx.x, blockDim.x, L::LX); w.r < nr; w.next()) {
    cp_async_c(s.W + w.r * L::WP + L::wpos(w.c), rows + w.r * L::LX + w.c);
  }
  cp_async_commit();
  cp_async_wait<0>();
  int k = 0;
  if (TT::kScaled) {
    // block scale from the thread's own copies, now in shared memory
    int e = 0;
    for (RowWalk w(threadIdx.x, blockDim.x, L::LX); w.r < nr; w.next()) {
      e = max(e, max_exponent(reinterpret_cast<const CS*>(s.W)[w.r * L::WP + L::wpos(w.c)]));
    }
    atomicMax(&sExp, e);
  }
  __syncthreads();
  if (TT::kScaled) {
    k = block_scale(finish_block_key(&sExp, [=] {
      int m = kDdNoSubnormal;
      for (RowWalk w(threadIdx.x, blockDim.x, L::LX); w.r < nr; w.next()) {
        m = max(m, max_subnormal_key(reinterpret_cast<const CS*>(s.W)[w.r * L::WP + L::wpos(w.c)]));
      }
      return m;
    }));
  }
  // blocks of tiny values convert every slot exactly first (uniform branch); the FFT below then
  // reads the converted slots
  const bool pre = TT::kScaled && exact_block(k);
  if (pre) {
    for (RowWalk w(threadIdx.x, blockDim.x, L::LX); w.r < nr; w.next()) {
      CA* slot = s.W + w.r * L::WP + L::wpos(w.c);
      *slot = to_arith_exact(*reinterpret_cast<const CS*>(slot), k);
    }
    __syncthreads();
  }
  const CA* twl = R2C ? s.twm : s.twx;
  for (int i = threadIdx.x; i < nr * Bx; i += blockDim.x) {
    const int q = i / Bx, b = i - q * Bx, rl = L::pass1_row(q, nr);
    CA* wrow = s.W + rl * L::WP;
    CA v[Ax];
#pragma unroll
    for (int a = 0; a < Ax; ++a) {
      const int slot = a * (Bx + L::PAD) + b;
      v[a] = pre ? wrow[slot] : to_arith(reinterpret_cast<const CS*>(wrow)[slot], k);
    }
    fft_pass1_regs_ordered<L::LX, -1>(v, b, twl);
#pragma unroll
    for (int k1 = 0; k1 < Ax; ++k1) wrow[k1 * (Bx + L::PAD) + b] = v[k1];
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nr * Ax; i += blockDim.x) {
    const int rl = i / Ax, k1 = i - rl * Ax;
    CA v[Bx];
    CA* wrow = s.W + rl * L::WP + k1 * L::PAD;
    fft_pass2<L::LX, -1>(wrow, 1, k1, v);
    if (!R2C) {
      CA* prow = s.P + rl * nc;
#pragma unroll
      for (int k2 = 0; k2 < Bx; ++k2) {
        const int col = s.colOf[k1 + Ax * k2];
        if (col >= 0) prow[col] = v[k2];
      }
    } else {
#pragma unroll
      for (int k2 = 0; k2 < Bx; ++k2) wrow[k1 * Bx + k2] = v[k2];
    }
  }
  __syncthreads();
  CS* planes = reinterpret_cast<CS*>(p.planes) + (static_cast<size_t>(z) * ny + y0) * nc;
  const bool raw = TT::kScaled && p.planesRaw;
  CA* rawPlanes = reinterpret_cast<CA*>(planes);
  if (R2C) {
    // output columns straight to the compact plane rows (consecutive threads, consecutive columns)
    with_store(k, [&](auto conv) {
      for (int i = threadIdx.x; i < nr * nc; i += blockDim.x) {
        const int rl = dnc.div(i), c = i - rl * nc;
        const int sl = s.colSlots[c];
        const CA tw = s.colTw[c];
        const CA* wrow = s.W + rl * L::WP;
        const CA zk = wrow[sl & 0xffff];
        const CA zm = wrow[sl >> 16];
        const CA zmc = cconj(zm);
        const CA dif = csub(zk, zmc);  // (zk.x - zm.x, zk.y + zm.y)
        const CA u = cmul(dif, tw);
        const CA xv = chalf(csub(cadd(zk, zmc), cmul_i<1>(u)));
        if (raw) rawPlanes[i] = xv;
        else planes[i] = conv(xv, k);
      }
    });
  } else {
    const bool converted = TT::kScaled && !raw && exact_block(k);
    if (converted) {
      convert_exact_in_place<S, A>(s.P, nr * nc, k, threadIdx.x, blockDim.x);
      __syncthreads();
    }
    for (int i = threadIdx.x; i < nr * nc; i += blockDim.x) {
      if (raw) rawPlanes[i] = s.P[i];
      else planes[i] = stored_value<S, A>(s.P + i, k, converted);
    }
  }
  if (raw && threadIdx.x < nr) p.planeExp[z * ny + y0 + threadIdx.x] = produced_exp(sExp, k);
}

template <typename S, typename A, int NX, bool R2C>
__global__ void __launch_bounds__(kThreads, YMinBlocks<A>::value) x_forward_split(const PlanView<S> p, const S* __restrict__ space,
                                                            int rpb, int z0) {
  __shared__ int sExp[2];
  x_forward_body<S, A, NX, R2C>(p, space, rpb, blockIdx.x, z0 + blockIdx.y, sExp);
}

template <typename S, typename A, int NY>
struct YSplitKernels {
  using CA = typename Types<S, A>::CA;
  // twiddles, the column group, and (forward, double-float planes) the row exponents
  static size_t smem(int cpb) { return (NY + static_cast<size_t>(NY) * cpb) * sizeof(CA) + NY * sizeof(int); }
  static cudaError_t prepare(size_t maxSmem) {
    cudaError_t e1 = allow_dynamic_smem(y_backward_split<S, A, NY>, maxSmem);
    cudaError_t e2 = allow_dynamic_smem(y_forward_split<S, A, NY>, maxSmem);
    if constexpr (has_swapped_split<NY>()) {
      if (e1 == cudaSuccess) e1 = allow_dynamic_smem(y_backward_split<S, A, NY, 2>, maxSmem);
      if (e2 == cudaSuccess) e2 = allow_dynamic_smem(y_forward_split<S, A, NY, 2>, maxSmem);
    }
    if constexpr (has_three<A, NY>()) {
      if (e1 == cudaSuccess) e1 = allow_dynamic_smem(y_backward_split<S, A, NY, 3>, maxSmem);
      if (e2 == cudaSuccess) e2 = allow_dynamic_smem(y_forward_split<S, A, NY, 3>, maxSmem);
    }
    return e1 != cudaSuccess ? e1 : e2;
  }
  // planes [z0, z0 + nz) (nz < 0: all planes from z0); `variant` as in ZKernels
  static void backward(const PlanView<S>& p, int cpb, cudaStream_t st, int z0, int nz, int variant) {
    const dim3 g((p.numColumns + cpb - 1) / cpb, nz < 0 ? p.dimZ - z0 : nz);
    if constexpr (has_swapped_split<NY>()) {
      if (variant == 1) return launch_pdl(y_backward_split<S, A, NY, 2>, g, kThreads, smem(cpb), st, p, cpb, z0);
    }
    if constexpr (has_three<A, NY>()) {
      if (variant == 2) return launch_pdl(y_backward_split<S, A, NY, 3>, g, kThreads, smem(cpb), st, p, cpb, z0);
    }
    launch_pdl(y_backward_split<S, A, NY>, g, kThreads, smem(cpb), st, p, cpb, z0);
  }
  static void forward(const PlanView<S>& p, int cpb, cudaStream_t st, int z0, int nz, int variant) {
    const dim3 g((p.numColumns + cpb - 1) / cpb, nz < 0 ? p.dimZ - z0 : nz);
    if constexpr (has_swapped_split<NY>()) {
      if (variant == 1) return launch_pdl(y_forward_split<S, A, NY, 2>, g, kThreads, smem(cpb), st, p, cpb, z0);
    }
    if constexpr (has_three<A, NY>()) {
      if (variant == 2) return launch_pdl(y_forward_split<S, A, NY, 3>, g, kThreads, smem(cpb), st, p, cpb, z0);
    }
    launch_pdl(y_forward_split<S, A, NY>, g, kThreads, smem(cpb), st, p, cpb, z0);
  }
};

template <typename S, typename A, int NX, bool R2C>
struct XSplitKernels {
  using CA = typename Types<S, A>::CA;
  static size_t smem(int numColumns, int rpb) {
    return RowSmem<CA, NX, R2C>::template bytes<CA>(numColumns, rpb);
  }
  static size_t smem_forward(int numColumns, int rpb) {
    return RowSmem<CA, NX, R2C>::template bytes<CA>(numColumns, rpb, !R2C);
  }
  static cudaError_t prepare(size_t maxSmem) {
    cudaError_t e1 = allow_dynamic_smem(x_backward_split<S, A, NX, R2C>, maxSmem);
    cudaError_t e2 = allow_dynamic_smem(x_forward_split<S, A, NX, R2C>, maxSmem);
    return e1 != cudaSuccess ? e1 : e2;
  }
  // planes [z0, z0 + nz) (nz < 0: all planes from z0)
  static void backward(const PlanView<S>& p, int rpb, S* space, cudaStream_t st, int z0, int nz) {
    const dim3 g((p.dimY + rpb - 1) / rpb, nz < 0 ? p.dimZ - z0 : nz);
    launch_pdl(x_backward_split<S, A, NX, R2C>, g, XBackwardThreads<A, R2C>::value, smem(p.numColumns, rpb), st, p, space, rpb,
               z0);
  }
  static void forward(const PlanView<S>& p, int rpb, const S* space, cudaStream_t st, int z0, int nz) {
    const dim3 g((p.dimY + rpb - 1) / rpb, nz < 0 ? p.dimZ - z0 : nz);
    launch_pdl(x_forward_split<S, A, NX, R2C>, g, kThreads, smem_forward(p.numColumns, rpb), st, p, space, rpb, z0);
  }
};

// First-pass radix A of the split (N = A * B) a kernel of length N runs (FastOp::SplitRadix):
// which = 0 z pass, 1 split y pass (variant 0 the default split, 1 the swapped one, 2 the three-pass
// split; 0 where the length has no such variant), 2 / 3 y pass of the fused plane backward /
// forward kernel, 4 x pass (R2C: the half-length complex FFT).
template <int N, typename A>
int split_radix(int which, int variant, bool r2c) {
  switch (which) {
    case 0:
    case 1:
      if (variant == 1) return has_swapped_split<N>() ? Shape<N, 2>::A : 0;
      if (variant == 2) return has_three<A, N>() ? Shape<N, 3>::A : 0;
      return Shape<N, 1>::A;
    case 2:
      return Shape<N, 1>::A;
    case 3:
      return Shape<N>::A;
    case 4:
      return r2c ? Shape<PlaneLayout<N, N, true>::LX>::A : Shape<N>::A;
    default:
      return 0;
  }
}
// The first factor B1 of B = B1 * B2 in the three-pass split of the z and split-y passes
// (FastOp::ThreePassFactor); 0 where the length has no three-pass variant.
template <int N, typename A>
int three_pass_factor() {
  return has_three<A, N>() ? Split3<N>::B1 : 0;
}

// Arithmetic type of the specialised kernels for a storage type: float for FP32, double-float
// for FP64.
template <typename S>
struct FastArith;
template <>
struct FastArith<float> {
  using type = float;
};
template <>
struct FastArith<double> {
  using type = dd;
};

}  // namespace fast
}  // namespace gb300
}  // namespace spfft
