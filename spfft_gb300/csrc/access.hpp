// Friend accessor of the public handle classes: gives the multi-transform functions and the
// extension C API access to a handle's internal object.
#pragma once

#include "internal.hpp"
#include "spfft/transform.hpp"
#include "spfft/transform_float.hpp"

namespace spfft {
struct TransformAccess {
  static TransformInternal<double>& get(Transform& t) { return *t.transform_; }
  static TransformInternal<float>& get(TransformFloat& t) { return *t.transform_; }
  static const TransformInternal<double>& get(const Transform& t) { return *t.transform_; }
  static const TransformInternal<float>& get(const TransformFloat& t) { return *t.transform_; }
  static std::shared_ptr<TransformInternal<double>> share(Transform& t) { return t.transform_; }
  static std::shared_ptr<TransformInternal<float>> share(TransformFloat& t) { return t.transform_; }
};
}  // namespace spfft
