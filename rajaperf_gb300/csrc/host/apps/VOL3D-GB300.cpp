// Apps_VOL3D.  Follows the suite's apps/VOL3D.cpp:28-104: rzmax = cbrt(size)
// + 1 + cbrt(3) - 1, mesh x = i*0.3, y = j*0.2, z = k*0.1, zones [fpz, lpz].
#include "Apps.hpp"

#include <cmath>

namespace rajaperf {
namespace apps {

VOL3D::VOL3D(const RunParams& params) : KernelBase(rajaperf::Apps_VOL3D, params) {
  setDefaultProblemSize(100 * 100 * 100);
  setDefaultReps(100);
  Index_type rzmax =
      static_cast<Index_type>(std::cbrt(getTargetProblemSize()) + 1 + std::cbrt(3) - 1);
  m_domain.reset(new ADomain(rzmax, 3));
  m_array_length = m_domain->nnalls;
  setActualProblemSize(m_domain->n_real_zones);
  setItsPerRep(m_domain->lpz + 1 - m_domain->fpz);
  setKernelsPerRep(1);
  setBytesReadPerRep(3 * sizeof(Real_type) *
                     (getItsPerRep() + 1 + m_domain->jp + m_domain->kp));
  setBytesWrittenPerRep(1 * sizeof(Real_type) * getItsPerRep());
  setBytesAtomicModifyWrittenPerRep(0);
  setFLOPsPerRep(72 * (m_domain->lpz + 1 - m_domain->fpz));
  checksum_scale_factor = 0.001 * (static_cast<Checksum_type>(getDefaultProblemSize()) /
                                   getActualProblemSize());
  setComplexity(Complexity::N);
  setUsesFeature(Forall);
  setVariantDefined(Base_GB300);
}

void VOL3D::setUp(VariantID vid, size_t) {
  allocAndInitDataConst(m_x, m_array_length, 0.0, vid);
  allocAndInitDataConst(m_y, m_array_length, 0.0, vid);
  allocAndInitDataConst(m_z, m_array_length, 0.0, vid);
  {
    std::vector<Real_type> hx(m_array_length, 0.0), hy(m_array_length, 0.0),
        hz(m_array_length, 0.0);
    setMeshPositions_3d(hx, 0.3, hy, 0.2, hz, 0.1, *m_domain);
    copyToDevice(m_x, hx.data(), hx.size() * sizeof(Real_type));
    copyToDevice(m_y, hy.data(), hy.size() * sizeof(Real_type));
    copyToDevice(m_z, hz.data(), hz.size() * sizeof(Real_type));
  }
  allocAndInitDataConst(m_vol, m_array_length, 0.0, vid);
  m_vnormq = 0.083333333333333333;
}

KernelBase::RepBody VOL3D::makeRepBody(size_t tune_idx) {
  const b200_tune tn = getTune(tune_idx);
  const Index_type jp = m_domain->jp, kp = m_domain->kp, ib = m_domain->fpz,
                   ie = m_domain->lpz + 1;
  return [=](b200_stream_t s) {
    checkB200(b200_apps_vol3d(m_x, m_y, m_z, m_vol, m_vnormq, jp, kp, ib, ie, &tn, s),
              "b200_apps_vol3d");
  };
}

void VOL3D::updateChecksum(VariantID vid, size_t tune_idx) {
  checksum[vid][tune_idx] += calcChecksum(m_vol, m_array_length, checksum_scale_factor, vid);
}

void VOL3D::tearDown(VariantID vid, size_t) {
  deallocData(m_x, vid);
  deallocData(m_y, vid);
  deallocData(m_z, vid);
  deallocData(m_vol, vid);
}

}  // namespace apps
}  // namespace rajaperf
