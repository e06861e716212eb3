// An SpFFT application in C++ (C++17), as written against the reference's C++ interface, built
// unchanged against this library's headers: spfft::Transform / spfft::TransformFloat created
// independently, backward into an external host space buffer and forward back, and the library's
// exceptions for invalid input.
//
//   app_cpp <type 0|1> <n> <radius> <precision 64|32> <out prefix>
// Writes <prefix>_indices.bin (int32 triplets), <prefix>_values.bin (complex128 input),
// <prefix>_space.bin (backward result, as doubles) and <prefix>_forward.bin (unscaled forward).
#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <vector>

#include "spfft/spfft.hpp"

namespace {

template <typename T>
void write_file(const std::string& prefix, const char* name, const std::vector<T>& v) {
  const std::string path = prefix + "_" + name + ".bin";
  std::FILE* f = std::fopen(path.c_str(), "wb");
  if (!f || std::fwrite(v.data(), sizeof(T), v.size(), f) != v.size()) throw std::runtime_error(path);
  std::fclose(f);
}

template <typename TransformT, typename T>
int run(int type, int n, int radius, const std::string& prefix) {
  const SpfftTransformType ttype = type ? SPFFT_TRANS_R2C : SPFFT_TRANS_C2C;
  const int lo = n / 2 - n + 1, hi = n / 2;
  std::vector<int> idx;
  for (int x = (type ? 0 : lo); x <= hi; ++x)
    for (int y = lo; y <= hi; ++y)
      for (int z = lo; z <= hi; ++z) {
        if (x * x + y * y + z * z > radius * radius) continue;
        if (type && x == 0 && (y < 0 || (y == 0 && z < 0))) continue;
        idx.insert(idx.end(), {x, y, z});
      }
  const int count = static_cast<int>(idx.size() / 3);
  std::vector<T> values(2 * static_cast<size_t>(count)), forward(values.size());
  std::vector<double> values64(values.size());
  for (int i = 0; i < count; ++i) {
    values64[2 * i] = static_cast<double>((i * 29) % 89) / 89.0 - 0.5;
    const bool k0 = idx[3 * i] == 0 && idx[3 * i + 1] == 0 && idx[3 * i + 2] == 0;
    values64[2 * i + 1] = (type && k0) ? 0.0 : static_cast<double>((i * 61) % 83) / 83.0 - 0.5;
    values[2 * i] = static_cast<T>(values64[2 * i]);
    values[2 * i + 1] = static_cast<T>(values64[2 * i + 1]);
  }

  // invalid indices raise the library's exception type with the reference's error code
  try {
    std::vector<int> bad = {n, 0, 0};
    TransformT broken(1, SPFFT_PU_GPU, ttype, n, n, n, 1, SPFFT_INDEX_TRIPLETS, bad.data());
    std::fprintf(stderr, "invalid indices were accepted\n");
    return 1;
  } catch (const spfft::InvalidIndicesError& e) {
    if (e.error_code() != SPFFT_INVALID_INDICES_ERROR) return 1;
  }

  TransformT transform(1, SPFFT_PU_GPU, ttype, n, n, n, count, SPFFT_INDEX_TRIPLETS, idx.data());
  if (transform.num_local_elements() != count || transform.dim_x() != n) return 1;
  std::vector<T> space(static_cast<size_t>(n) * n * n * (type ? 1 : 2));
  transform.backward(values.data(), space.data());  // host pointers: staged by the library
  TransformT copy = transform;                       // shared handle, same transform
  copy.forward(space.data(), forward.data(), SPFFT_NO_SCALING);

  write_file(prefix, "indices", idx);
  write_file(prefix, "values", values64);
  write_file(prefix, "space", std::vector<double>(space.begin(), space.end()));
  write_file(prefix, "forward", std::vector<double>(forward.begin(), forward.end()));
  std::printf("values %d\n", count);
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 6) return 2;
  const int type = std::atoi(argv[1]), n = std::atoi(argv[2]), radius = std::atoi(argv[3]);
  const int precision = std::atoi(argv[4]);
  try {
    return precision == 32 ? run<spfft::TransformFloat, float>(type, n, radius, argv[5])
                           : run<spfft::Transform, double>(type, n, radius, argv[5]);
  } catch (const spfft::GenericError& e) {
    std::fprintf(stderr, "spfft error %d: %s\n", static_cast<int>(e.error_code()), e.what());
    return 1;
  } catch (const std::exception& e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 1;
  }
}
