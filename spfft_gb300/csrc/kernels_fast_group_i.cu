// Specialised kernels (single, split and batched) for one group of FFT lengths; every length is
// even, so the R2C/C2R half-length path applies.
#define SPFFT_GB300_GROUP fast_group_i
#define SPFFT_GB300_SIZES(X) X(240) X(256)
#include "kernels_fast_group.inc"
