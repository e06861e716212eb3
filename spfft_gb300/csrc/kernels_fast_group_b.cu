// Specialised kernels for one group of FFT lengths (cubic grids; every length is even so the
// R2C/C2R half-length path applies).
#define SPFFT_GB300_GROUP fast_group_b
#define SPFFT_GB300_SIZES(X) X(90) X(96) X(100) X(108)
#include "kernels_fast_group.inc"
