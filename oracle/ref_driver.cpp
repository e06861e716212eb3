// Test-infrastructure driver around the reference's OWN index code, compiled from the reference
// sources where they lie (see Makefile). It is never linked into the library.
//
//   ref_indices plan <type> <dimX> <dimY> <dimZ> <n>   (3n ints on stdin)
//       Runs spfft::Parameters (src/parameters/parameters.cpp:143-180) and prints
//       "values v0 v1 ...", "sticks k0 k1 ...", "zz z" -- or "error <SpfftError code>".
//   ref_indices gen <dimX> <dimY> <dimZ> <r2c 0|1> <centered 0|1>
//       Reproduces the index sets and values of the reference's local transform tests
//       (tests/test_util/test_transform.hpp:78-276): std::mt19937(42),
//       create_value_indices(...) with fractions 0.7/0.7 (C2C) or 1.0/1.0 (R2C), optional
//       center_indices(...), then one uniform(0,1) draw per value (re, im for C2C; re for R2C).
//       Prints "indices ...", "re ...", "im ..." (17 significant digits).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <random>
#include <string>
#include <vector>

#include "parameters/parameters.hpp"
#include "spfft/exceptions.hpp"
#include "test_util/generate_indices.hpp"

static void print_vec(const char* tag, const std::vector<int>& v) {
  std::printf("%s", tag);
  for (int x : v) std::printf(" %d", x);
  std::printf("\n");
}

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  if (std::strcmp(argv[1], "plan") == 0 && argc == 7) {
    const int type = std::atoi(argv[2]);
    const int dx = std::atoi(argv[3]), dy = std::atoi(argv[4]), dz = std::atoi(argv[5]);
    const int n = std::atoi(argv[6]);
    std::vector<int> idx(3 * static_cast<size_t>(n));
    for (auto& v : idx)
      if (std::scanf("%d", &v) != 1) return 3;
    try {
      spfft::Parameters p(type == 1 ? SPFFT_TRANS_R2C : SPFFT_TRANS_C2C, dx, dy, dz, n,
                          SPFFT_INDEX_TRIPLETS, idx.data());
      print_vec("values", p.local_value_indices());
      auto sv = p.local_z_stick_xy_indices();
      std::vector<int> sticks(sv.data(), sv.data() + sv.size());
      print_vec("sticks", sticks);
      std::printf("zz %llu\n", static_cast<unsigned long long>(p.zero_zero_stick_index()));
    } catch (const spfft::GenericError& e) {
      std::printf("error %d\n", static_cast<int>(e.error_code()));
    }
    return 0;
  }
  if (std::strcmp(argv[1], "gen") == 0 && argc == 7) {
    const int dx = std::atoi(argv[2]), dy = std::atoi(argv[3]), dz = std::atoi(argv[4]);
    const bool r2c = std::atoi(argv[5]) != 0, centered = std::atoi(argv[6]) != 0;
    std::mt19937 randGen(42);
    std::uniform_real_distribution<double> uni(0.0, 1.0);
    const double frac = r2c ? 1.0 : 0.7;
    auto perRank = spfft::create_value_indices(randGen, std::vector<double>(1, 1.0), frac, frac, dx,
                                               dy, dz, r2c);
    std::vector<double> re, im;
    for (std::size_t i = 0; i < perRank[0].size(); i += 3) {
      re.push_back(uni(randGen));
      im.push_back(r2c ? 0.0 : uni(randGen));
    }
    if (centered) spfft::center_indices(dx, dy, dz, perRank);
    print_vec("indices", perRank[0]);
    std::printf("re");
    for (double v : re) std::printf(" %.17g", v);
    std::printf("\nim");
    for (double v : im) std::printf(" %.17g", v);
    std::printf("\n");
    return 0;
  }
  return 2;
}
