// Mesh domain helpers of the Apps kernels, with the same index layout as the
// suite's apps/AppsData.hpp: ADomain (real nodes per dimension, 2 ghost
// layers below and 1 above, strides jp/kp, first/last zone indices) and the
// mesh-position / real-zone fills of AppsData.cpp:56-180.
#pragma once

#include "common/RPTypes.hpp"
#include "common/RunParams.hpp"

#include <vector>

namespace rajaperf {
namespace apps {

struct ADomain {
  ADomain(Index_type real_nodes_per_dim, Index_type ndims);

  Index_type ndims, NPNL, NPNR;
  Index_type imin, jmin, kmin, imax, jmax, kmax;
  Index_type jp, kp, nnalls;
  Index_type fpn, lpn, frn, lrn, fpz, lpz;
  Index_type n_real_zones, n_real_nodes;
};

// Host fills (the arrays are then copied to the device).
void setRealZones_2d(std::vector<Index_type>& real_zones, const ADomain& d);
// In the uniform input mode each node is jittered by up to 0.1 cell.
void setMeshPositions_2d(std::vector<Real_type>& x, Real_type dx,
                         std::vector<Real_type>& y, Real_type dy, const ADomain& d,
                         const RunParams& rp);
void setMeshPositions_3d(std::vector<Real_type>& x, Real_type dx,
                         std::vector<Real_type>& y, Real_type dy,
                         std::vector<Real_type>& z, Real_type dz, const ADomain& d);

}  // namespace apps
}  // namespace rajaperf
