// Test-infrastructure driver around the reference's OWN host transform path (spfft::Transform /
// spfft::TransformFloat on SPFFT_PU_HOST: src/execution/execution_host.cpp and everything it
// calls), compiled from the reference sources where they lie with FFTW replaced by the project's
// FFTW-API shim (fftw_shim/). Built by the Makefile into _ref/libref_pipeline.so; loaded by
// oracle/ref.py with ctypes. It is never linked into the library.
//
//   ref_pipeline_run(precision, type, dimX, dimY, dimZ, n, indices, forwardFirst, valuesIn,
//                    spaceIn, valuesOut, spaceOut, scaling, threads)
//       One independent transform of the given type (0 C2C, 1 R2C) and precision (0 double,
//       1 float) on the host. forwardFirst = 0: backward(valuesIn) -> spaceOut, then
//       forward(spaceOut, scaling) -> valuesOut. forwardFirst = 1: forward(spaceIn, scaling) ->
//       valuesOut, then backward(valuesOut) -> spaceOut (the order of the reference's R2C tests).
//       Values are interleaved complex doubles, space domains dimZ*dimY*dimX complex (C2C) or real
//       (R2C) doubles (converted for the float API). Returns the reference's SpfftError code.
#include <algorithm>
#include <cstddef>
#include <vector>

#include "spfft/exceptions.hpp"
#include "spfft/transform.hpp"
#include "spfft/transform_float.hpp"

namespace {

template <typename TransformT, typename T>
void run(int type, int dimX, int dimY, int dimZ, int n, const int* indices, int forwardFirst,
         const double* valuesIn, const double* spaceIn, double* valuesOut, double* spaceOut, int scaling,
         int threads) {
  TransformT tr(threads, SPFFT_PU_HOST, static_cast<SpfftTransformType>(type), dimX, dimY, dimZ, n,
                SPFFT_INDEX_TRIPLETS, indices);
  const std::size_t nv = 2 * static_cast<std::size_t>(n);
  const std::size_t ns = static_cast<std::size_t>(dimX) * dimY * dimZ * (type == SPFFT_TRANS_C2C ? 2 : 1);
  std::vector<T> values(nv), space(ns);
  const auto sc = static_cast<SpfftScalingType>(scaling);
  if (forwardFirst) {
    std::copy(spaceIn, spaceIn + ns, space.begin());
    tr.forward(space.data(), values.data(), sc);
    std::copy(values.begin(), values.end(), valuesOut);
    tr.backward(values.data(), space.data());
  } else {
    std::copy(valuesIn, valuesIn + nv, values.begin());
    tr.backward(values.data(), space.data());
    tr.forward(space.data(), values.data(), sc);
    std::copy(values.begin(), values.end(), valuesOut);
  }
  std::copy(space.begin(), space.end(), spaceOut);
}

}  // namespace

extern "C" __attribute__((visibility("default"))) int ref_pipeline_run(
    int precision, int type, int dimX, int dimY, int dimZ, int n, const int* indices, int forwardFirst,
    const double* valuesIn, const double* spaceIn, double* valuesOut, double* spaceOut, int scaling, int threads) {
  try {
    if (precision == 0) {
      run<spfft::Transform, double>(type, dimX, dimY, dimZ, n, indices, forwardFirst, valuesIn, spaceIn, valuesOut,
                                    spaceOut, scaling, threads);
    } else {
      run<spfft::TransformFloat, float>(type, dimX, dimY, dimZ, n, indices, forwardFirst, valuesIn, spaceIn,
                                        valuesOut, spaceOut, scaling, threads);
    }
  } catch (const spfft::GenericError& e) {
    return e.error_code();
  } catch (...) {
    return SPFFT_UNKNOWN_ERROR;
  }
  return 0;
}
