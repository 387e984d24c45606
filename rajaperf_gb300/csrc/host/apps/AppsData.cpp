#include "AppsData.hpp"

#include "common/DataUtils.hpp"

namespace rajaperf {
namespace apps {

ADomain::ADomain(Index_type rnpd, Index_type nd) : ndims(nd), NPNL(2), NPNR(1) {
  Index_type NPZL = NPNL - 1;
  Index_type NPZR = NPNR + 1 - 1;
  imin = NPNL;
  imax = NPNL + rnpd - 1;
  nnalls = (imax + 1 - imin + NPNL + NPNR);
  n_real_zones = (imax - imin);
  n_real_nodes = (imax + 1 - imin);
  jmin = jmax = jp = 0;
  kmin = kmax = kp = 0;
  if (ndims >= 2) {
    jmin = NPNL;
    jmax = NPNL + rnpd - 1;
    jp = nnalls;
    nnalls *= (jmax + 1 - jmin + NPNL + NPNR);
    n_real_zones *= (jmax - jmin);
    n_real_nodes *= (jmax + 1 - jmin);
  }
  if (ndims >= 3) {
    kmin = NPNL;
    kmax = NPNL + rnpd - 1;
    kp = nnalls;
    nnalls *= (kmax + 1 - kmin + NPNL + NPNR);
    n_real_zones *= (kmax - kmin);
    n_real_nodes *= (kmax + 1 - kmin);
  }
  frn = kmin * kp + jmin * jp + imin;
  lrn = kmax * kp + jmax * jp + imax;
  fpn = (kmin - NPNL) * kp + (jmin - NPNL) * jp + (imin - NPNL);
  lpn = (kmax + NPNR) * kp + (jmax + NPNR) * jp + (imax + NPNR);
  fpz = (kmin - NPZL) * kp + (jmin - NPZL) * jp + (imin - NPZL);
  lpz = (kmax - 1 + NPZR) * kp + (jmax - 1 + NPZR) * jp + (imax - 1 + NPZR);
}

void setRealZones_2d(std::vector<Index_type>& rz, const ADomain& d) {
  Index_type j_stride = d.imax - d.imin;
  for (Index_type j = d.jmin; j < d.jmax; j++)
    for (Index_type i = d.imin; i < d.imax; i++)
      rz[(i - d.imin) + (j - d.jmin) * j_stride] = i + j * d.jp;
}

void setMeshPositions_2d(std::vector<Real_type>& x, Real_type dx,
                         std::vector<Real_type>& y, Real_type dy, const ADomain& d,
                         const RunParams& rp) {
  const bool jitter = rp.getInitMode() == RunParams::InitUniform;
  for (Index_type j = d.jmin - d.NPNL; j < d.jmax + 1 + d.NPNR; j++)
    for (Index_type i = d.imin - d.NPNL; i < d.imax + 1 + d.NPNR; i++) {
      Index_type in = i + j * d.jp;
      x[in] = i * dx;
      y[in] = j * dy;
      if (jitter) {
        x[in] += dx * uniformValue(rp.getSeed(), 0x2D0001ULL, in, -0.1, 0.1);
        y[in] += dy * uniformValue(rp.getSeed(), 0x2D0002ULL, in, -0.1, 0.1);
      }
    }
}

void setMeshPositions_3d(std::vector<Real_type>& x, Real_type dx,
                         std::vector<Real_type>& y, Real_type dy,
                         std::vector<Real_type>& z, Real_type dz, const ADomain& d) {
  for (Index_type k = d.kmin - d.NPNL; k < d.kmax + 1 + d.NPNR; k++)
    for (Index_type j = d.jmin - d.NPNL; j < d.jmax + 1 + d.NPNR; j++)
      for (Index_type i = d.imin - d.NPNL; i < d.imax + 1 + d.NPNR; i++) {
        Index_type in = i + j * d.jp + k * d.kp;
        x[in] = i * dx;
        y[in] = j * dy;
        z[in] = k * dz;
      }
}

}  // namespace apps
}  // namespace rajaperf
