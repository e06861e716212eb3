/* C++ Grid handle (reference include/spfft/grid.hpp:49-203, local constructor only). A Grid owns
 * the device scratch, the internal space-domain buffer and its pinned host mirror. Copies share the
 * memory; transforms created from a grid keep it alive. */
#ifndef SPFFT_GRID_HPP
#define SPFFT_GRID_HPP

#include <memory>
#include "spfft/config.h"
#include "spfft/transform.hpp"
#include "spfft/types.h"

namespace spfft {

template <typename T>
class GridInternal;

class SPFFT_EXPORT Grid {
public:
  Grid(int maxDimX, int maxDimY, int maxDimZ, int maxNumLocalZColumns,
       SpfftProcessingUnitType processingUnit, int maxNumThreads);

  /* Copying a Grid allocates new memory of the same size (reference grid.cpp copy semantics). */
  Grid(const Grid&);
  Grid(Grid&&) = default;
  Grid& operator=(const Grid&);
  Grid& operator=(Grid&&) = default;

  Transform create_transform(SpfftProcessingUnitType processingUnit,
                             SpfftTransformType transformType, int dimX, int dimY, int dimZ,
                             int localZLength, int numLocalElements,
                             SpfftIndexFormatType indexFormat, const int* indices) const;

  int max_dim_x() const;
  int max_dim_y() const;
  int max_dim_z() const;
  int max_num_local_z_columns() const;
  int max_local_z_length() const;
  SpfftProcessingUnitType processing_unit() const;
  int device_id() const;
  int num_threads() const;

private:
  std::shared_ptr<GridInternal<double>> grid_;
};

}  // namespace spfft
#endif
