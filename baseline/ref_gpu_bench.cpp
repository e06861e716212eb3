// Comparison timing of the reference's own GPU transform path (its CUDA kernels plus cuFFT,
// src/execution/execution_gpu.cpp), driven through its public C++ API exactly as its benchmark
// program does in "gpu-gpu" mode (tests/programs/benchmark.cpp:84-96: values in device memory,
// backward then forward, no scaling), with bench.py's timing protocol: device buffers, an external
// out-of-place space domain in device memory, asynchronous execution mode, CUDA events on the
// legacy default stream (which the reference orders its internal stream after), a 256 MB write
// between timed pairs to flush L2, W untimed pairs first.
//
// Measurement infrastructure: compiled from the reference's sources by baseline/Makefile into
// baseline/_ref/build/ref_gpu_bench; never part of the library.
//
// Usage: ref_gpu_bench <input.bin> <64|32> <transforms> <steps> <warmup> [space_out.bin]
// input.bin: int32 type (0 C2C, 1 R2C), int32 n, int32 npts, int32 triplets[3 npts] (centered),
// float64 values[2 npts] (interleaved complex). With `transforms` > 1 the same set runs as that
// many independent transforms (each with its own grid, as the reference's benchmark builds them)
// through the pointer forms of multi_transform_backward / multi_transform_forward. space_out.bin
// receives the space domain of the first backward of transform 0 (in the transform's precision).
#include <cuda_runtime.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <memory>
#include <vector>

#include "spfft/exceptions.hpp"
#include "spfft/spfft.hpp"

// The reference's multi_transform_float.hpp shares its include guard with multi_transform.hpp, so
// after spfft.hpp its float declarations are skipped; these are its pointer forms as it exports
// them (src/spfft/multi_transform_float.cpp).
namespace spfft {
SPFFT_EXPORT void multi_transform_forward(int numTransforms, TransformFloat* transforms,
                                          const float* const* inputPointers, float* const* outputPointers,
                                          const SpfftScalingType* scalingTypes);
SPFFT_EXPORT void multi_transform_backward(int numTransforms, TransformFloat* transforms,
                                           const float* const* inputPointers, float* const* outputPointers);
}  // namespace spfft

namespace {

#define CHECK_CUDA(x)                                                              \
  do {                                                                             \
    cudaError_t e_ = (x);                                                          \
    if (e_ != cudaSuccess) {                                                       \
      std::fprintf(stderr, "CUDA error %s at %s:%d\n", cudaGetErrorString(e_), __FILE__, __LINE__); \
      std::exit(3);                                                                \
    }                                                                              \
  } while (0)

template <typename T, typename TransformT, typename GridT>
int run(int type, int n, const std::vector<int>& idx, const std::vector<double>& vals64, int count,
        int steps, int warmup, const char* outPath) {
  const int npts = static_cast<int>(idx.size() / 3);
  std::vector<T> vals(vals64.begin(), vals64.end());
  const size_t spaceElems = static_cast<size_t>(n) * n * n * (type == 0 ? 2 : 1);

  std::vector<GridT> grids;
  std::vector<TransformT> transforms;
  std::vector<T*> dVals(count), dSpace(count);
  for (int t = 0; t < count; ++t) {
    grids.emplace_back(n, n, n, n * n, SPFFT_PU_GPU, 1);
    transforms.emplace_back(grids.back().create_transform(
        SPFFT_PU_GPU, type == 0 ? SPFFT_TRANS_C2C : SPFFT_TRANS_R2C, n, n, n, n, npts,
        SPFFT_INDEX_TRIPLETS, idx.data()));
    transforms.back().set_execution_mode(SPFFT_EXEC_ASYNCHRONOUS);
    CHECK_CUDA(cudaMalloc(&dVals[t], sizeof(T) * 2 * npts));
    CHECK_CUDA(cudaMalloc(&dSpace[t], sizeof(T) * spaceElems));
    CHECK_CUDA(cudaMemcpy(dVals[t], vals.data(), sizeof(T) * 2 * npts, cudaMemcpyHostToDevice));
  }
  void* flush = nullptr;
  const size_t flushBytes = size_t(256) << 20;
  CHECK_CUDA(cudaMalloc(&flush, flushBytes));

  std::vector<SpfftScalingType> noScale(count, SPFFT_NO_SCALING);
  std::vector<const T*> cVals(dVals.begin(), dVals.end()), cSpace(dSpace.begin(), dSpace.end());
  auto pair = [&]() {
    if (count == 1) {
      transforms[0].backward(dVals[0], dSpace[0]);
      transforms[0].forward(dSpace[0], dVals[0], SPFFT_NO_SCALING);
    } else {
      spfft::multi_transform_backward(count, transforms.data(), cVals.data(), dSpace.data());
      spfft::multi_transform_forward(count, transforms.data(), cSpace.data(), dVals.data(), noScale.data());
    }
  };

  // parity output: the first backward of transform 0
  if (outPath) {
    transforms[0].backward(dVals[0], dSpace[0]);
    CHECK_CUDA(cudaDeviceSynchronize());
    std::vector<T> space(spaceElems);
    CHECK_CUDA(cudaMemcpy(space.data(), dSpace[0], sizeof(T) * spaceElems, cudaMemcpyDeviceToHost));
    std::ofstream(outPath, std::ios::binary).write(reinterpret_cast<const char*>(space.data()),
                                                   sizeof(T) * spaceElems);
  }
  for (int w = 0; w < warmup; ++w) pair();
  CHECK_CUDA(cudaDeviceSynchronize());

  cudaEvent_t a, b;
  CHECK_CUDA(cudaEventCreate(&a));
  CHECK_CUDA(cudaEventCreate(&b));
  double ms = 0.0;
  for (int s = 0; s < steps; ++s) {
    CHECK_CUDA(cudaMemsetAsync(flush, s & 0xff, flushBytes, 0));
    CHECK_CUDA(cudaEventRecord(a, 0));
    pair();
    CHECK_CUDA(cudaEventRecord(b, 0));
    CHECK_CUDA(cudaEventSynchronize(b));
    float t = 0.0f;
    CHECK_CUDA(cudaEventElapsedTime(&t, a, b));
    ms += t;
  }
  std::printf("{\"pairs_per_s\": %.3f, \"ms_per_step\": %.5f, \"transforms\": %d, \"steps\": %d, "
              "\"warmup\": %d, \"precision\": \"%s\"}\n",
              count * steps / (ms * 1e-3), ms / steps, count, steps, warmup,
              sizeof(T) == 8 ? "float64" : "float32");
  for (int t = 0; t < count; ++t) {
    cudaFree(dVals[t]);
    cudaFree(dSpace[t]);
  }
  cudaFree(flush);
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 6) {
    std::fprintf(stderr, "usage: %s input.bin 64|32 transforms steps warmup [space_out.bin]\n", argv[0]);
    return 2;
  }
  std::ifstream in(argv[1], std::ios::binary);
  int head[3];
  if (!in.read(reinterpret_cast<char*>(head), sizeof(head))) return 2;
  const int type = head[0], n = head[1], npts = head[2];
  std::vector<int> idx(3 * static_cast<size_t>(npts));
  std::vector<double> vals(2 * static_cast<size_t>(npts));
  in.read(reinterpret_cast<char*>(idx.data()), sizeof(int) * idx.size());
  in.read(reinterpret_cast<char*>(vals.data()), sizeof(double) * vals.size());
  if (!in) return 2;
  const int precision = std::atoi(argv[2]), count = std::atoi(argv[3]);
  const int steps = std::atoi(argv[4]), warmup = std::atoi(argv[5]);
  const char* out = argc > 6 ? argv[6] : nullptr;
  try {
    if (precision == 64) return run<double, spfft::Transform, spfft::Grid>(type, n, idx, vals, count, steps, warmup, out);
    return run<float, spfft::TransformFloat, spfft::GridFloat>(type, n, idx, vals, count, steps, warmup, out);
  } catch (const spfft::GenericError& e) {
    std::fprintf(stderr, "reference error %d: %s\n", e.error_code(), e.what());
    return 4;
  }
}
