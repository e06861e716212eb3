// Specialised kernels for one group of FFT lengths (cubic grids; every length is even so the
// R2C/C2R half-length path applies).
#define SPFFT_GB300_GROUP fast_group_c
#define SPFFT_GB300_SIZES(X) X(120) X(128) X(150)
#include "kernels_fast_group.inc"
