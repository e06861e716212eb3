/* Umbrella header of the C interface (reference include/spfft/spfft.h:31-37). */
#ifndef SPFFT_SPFFT_H
#define SPFFT_SPFFT_H

#include "spfft/config.h"
#include "spfft/grid.h"
#include "spfft/grid_float.h"
#include "spfft/multi_transform.h"
#include "spfft/multi_transform_float.h"
#include "spfft/transform.h"
#include "spfft/transform_float.h"

#endif
