/* An SpFFT application in plain C (C99), as written against the reference's C interface, built
 * unchanged against this library's headers: grid + transform creation, backward of host values
 * into the grid's host space buffer, forward back to host values, error checks on every call.
 *
 *   app_c <type 0|1> <n> <radius> <out prefix>
 * Writes <prefix>_indices.bin (int32 triplets), <prefix>_values.bin (complex128 input),
 * <prefix>_space.bin (backward result) and <prefix>_forward.bin (unscaled forward of it). */
#include <stdio.h>
#include <stdlib.h>

#include "spfft/spfft.h"

#define CHECK(call)                                                      \
  do {                                                                   \
    SpfftError e_ = (call);                                              \
    if (e_ != SPFFT_SUCCESS) {                                           \
      fprintf(stderr, "%s failed with %d\n", #call, (int)e_);           \
      return 1;                                                          \
    }                                                                    \
  } while (0)

static int write_file(const char* prefix, const char* name, const void* data, size_t bytes) {
  char path[1024];
  snprintf(path, sizeof(path), "%s_%s.bin", prefix, name);
  FILE* f = fopen(path, "wb");
  if (!f) return 1;
  const size_t w = fwrite(data, 1, bytes, f);
  fclose(f);
  return w == bytes ? 0 : 1;
}

int main(int argc, char** argv) {
  if (argc != 5) return 2;
  const int type = atoi(argv[1]), n = atoi(argv[2]), radius = atoi(argv[3]);
  const SpfftTransformType ttype = type ? SPFFT_TRANS_R2C : SPFFT_TRANS_C2C;
  const int lo = n / 2 - n + 1, hi = n / 2;
  int* idx = malloc(sizeof(int) * 3 * (size_t)n * n * n);
  int count = 0;
  for (int x = (type ? 0 : lo); x <= hi; ++x)
    for (int y = lo; y <= hi; ++y)
      for (int z = lo; z <= hi; ++z) {
        if (x * x + y * y + z * z > radius * radius) continue;
        if (type && x == 0 && (y < 0 || (y == 0 && z < 0))) continue;
        idx[3 * count] = x;
        idx[3 * count + 1] = y;
        idx[3 * count + 2] = z;
        ++count;
      }
  double* values = malloc(sizeof(double) * 2 * (size_t)count);
  double* forward = malloc(sizeof(double) * 2 * (size_t)count);
  for (int i = 0; i < count; ++i) {
    values[2 * i] = (double)((i * 37) % 101) / 101.0 - 0.5;
    values[2 * i + 1] = (idx[3 * i] == 0 && idx[3 * i + 1] == 0 && idx[3 * i + 2] == 0 && type)
                            ? 0.0
                            : (double)((i * 53) % 97) / 97.0 - 0.5;
  }

  SpfftGrid grid = NULL;
  CHECK(spfft_grid_create(&grid, n, n, n, n * n, SPFFT_PU_GPU, -1));
  SpfftTransform transform = NULL;
  CHECK(spfft_transform_create(&transform, grid, SPFFT_PU_GPU, ttype, n, n, n, n, count,
                               SPFFT_INDEX_TRIPLETS, idx));
  /* the transform keeps the grid alive */
  CHECK(spfft_grid_destroy(grid));

  CHECK(spfft_transform_backward(transform, values, SPFFT_PU_HOST));
  double* space = NULL;
  CHECK(spfft_transform_get_space_domain(transform, SPFFT_PU_HOST, &space));
  const size_t spaceDoubles = (size_t)n * n * n * (type ? 1 : 2);
  double* spaceCopy = malloc(sizeof(double) * spaceDoubles);
  for (size_t i = 0; i < spaceDoubles; ++i) spaceCopy[i] = space[i];
  CHECK(spfft_transform_forward(transform, SPFFT_PU_HOST, forward, SPFFT_NO_SCALING));

  long long numGlobal = 0;
  CHECK(spfft_transform_num_global_elements(transform, &numGlobal));
  if (numGlobal != count) {
    fprintf(stderr, "num_global_elements %lld, expected %d\n", numGlobal, count);
    return 1;
  }
  CHECK(spfft_transform_destroy(transform));

  int rc = 0;
  rc |= write_file(argv[4], "indices", idx, sizeof(int) * 3 * (size_t)count);
  rc |= write_file(argv[4], "values", values, sizeof(double) * 2 * (size_t)count);
  rc |= write_file(argv[4], "space", spaceCopy, sizeof(double) * spaceDoubles);
  rc |= write_file(argv[4], "forward", forward, sizeof(double) * 2 * (size_t)count);
  printf("values %d\n", count);
  free(idx);
  free(values);
  free(forward);
  free(spaceCopy);
  return rc;
}
