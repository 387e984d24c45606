// Apps_DEL_DOT_VEC_2D.  Follows the suite's apps/DEL_DOT_VEC_2D.cpp:28-107:
// rzmax = sqrt(size) + 1 + sqrt(2) - 1 real nodes per dimension, regular mesh
// x = i*0.2, y = j*0.1 (jittered in the uniform mode), checksum over div.
#include "Apps.hpp"

#include <cmath>

namespace rajaperf {
namespace apps {

DEL_DOT_VEC_2D::DEL_DOT_VEC_2D(const RunParams& params)
    : KernelBase(rajaperf::Apps_DEL_DOT_VEC_2D, params) {
  setDefaultProblemSize(1000 * 1000);
  setDefaultReps(100);
  Index_type rzmax =
      static_cast<Index_type>(std::sqrt(getTargetProblemSize()) + 1 + std::sqrt(2) - 1);
  m_domain.reset(new ADomain(rzmax, 2));
  m_array_length = m_domain->nnalls;
  setActualProblemSize(m_domain->n_real_zones);
  setItsPerRep(getActualProblemSize());
  setKernelsPerRep(1);
  setBytesReadPerRep(1 * sizeof(Index_type) * getItsPerRep() +
                     4 * sizeof(Real_type) * m_domain->n_real_nodes);
  setBytesWrittenPerRep(1 * sizeof(Index_type) * getItsPerRep());
  setBytesAtomicModifyWrittenPerRep(0);
  setFLOPsPerRep(54 * m_domain->n_real_zones);
  setComplexity(Complexity::N);
  setUsesFeature(Forall);
  setVariantDefined(Base_GB300);
}

void DEL_DOT_VEC_2D::setUp(VariantID vid, size_t) {
  allocAndInitDataConst(m_x, m_array_length, 0.0, vid);
  allocAndInitDataConst(m_y, m_array_length, 0.0, vid);
  allocAndInitDataConst(m_real_zones, m_domain->n_real_zones, static_cast<Index_type>(-1), vid);
  {
    std::vector<Real_type> hx(m_array_length, 0.0), hy(m_array_length, 0.0);
    std::vector<Index_type> hrz(m_domain->n_real_zones, -1);
    setMeshPositions_2d(hx, 0.2, hy, 0.1, *m_domain, run_params);
    setRealZones_2d(hrz, *m_domain);
    copyToDevice(m_x, hx.data(), hx.size() * sizeof(Real_type));
    copyToDevice(m_y, hy.data(), hy.size() * sizeof(Real_type));
    copyToDevice(m_real_zones, hrz.data(), hrz.size() * sizeof(Index_type));
  }
  allocAndInitData(m_xdot, m_array_length, vid);
  allocAndInitData(m_ydot, m_array_length, vid);
  allocAndInitDataConst(m_div, m_array_length, 0.0, vid);
  // --host-data: the zones gather their corner nodes, so the arrays are
  // staged (the zone list is an input like the node arrays)
  for (Real_ptr* p : {&m_x, &m_y, &m_xdot, &m_ydot}) stageArray(*p, m_array_length, kIn);
  stageArray(m_real_zones, m_domain->n_real_zones, kIn);
  stageArray(m_div, m_array_length, kOut);
  m_ptiny = 1.0e-20;
  m_half = 0.5;
}

KernelBase::RepBody DEL_DOT_VEC_2D::makeRepBody(size_t tune_idx) {
  const b200_tune tn = getTune(tune_idx);
  const Index_type nz = m_domain->n_real_zones, jp = m_domain->jp;
  return [=](b200_stream_t s) {
    checkB200(b200_apps_del_dot_vec_2d(m_x, m_y, m_xdot, m_ydot, m_div,
                                       reinterpret_cast<const int64_t*>(m_real_zones), nz,
                                       jp, m_ptiny, m_half, &tn, s),
              "b200_apps_del_dot_vec_2d");
  };
}

void DEL_DOT_VEC_2D::updateChecksum(VariantID vid, size_t tune_idx) {
  checksum[vid][tune_idx] += calcChecksum(m_div, m_array_length, vid);
}

void DEL_DOT_VEC_2D::tearDown(VariantID vid, size_t) {
  deallocData(m_x, vid);
  deallocData(m_y, vid);
  deallocData(m_real_zones, vid);
  deallocData(m_xdot, vid);
  deallocData(m_ydot, vid);
  deallocData(m_div, vid);
}

}  // namespace apps
}  // namespace rajaperf
