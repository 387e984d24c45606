// Lcals_HYDRO_2D.  Follows the suite's lcals/HYDRO_2D.cpp:27-107: a
// kn x jn grid with kn = jn = sqrt(size) + sqrt(2) - 1, three sweeps per rep
// (run as two launches by b200_lcals_hydro_2d), checksum over zzout + zrout.
#include "Lcals.hpp"

#include <cmath>

namespace rajaperf {
namespace lcals {

HYDRO_2D::HYDRO_2D(const RunParams& params) : KernelBase(rajaperf::Lcals_HYDRO_2D, params) {
  m_jn = 1000;
  m_kn = 1000;
  m_s = 0.0041;
  m_t = 0.0037;
  setDefaultProblemSize(m_kn * m_jn);
  setDefaultReps(100);
  m_jn = m_kn = static_cast<Index_type>(std::sqrt(getTargetProblemSize()) + std::sqrt(2) - 1);
  m_array_length = m_kn * m_jn;
  setActualProblemSize(getTargetProblemSize());
  setItsPerRep(3 * getActualProblemSize());
  setKernelsPerRep(3);
  setBytesReadPerRep(4 * sizeof(Real_type) * m_array_length +
                     4 * sizeof(Real_type) * m_array_length +
                     4 * sizeof(Real_type) * (m_kn - 2) * (m_jn - 2));
  setBytesWrittenPerRep(2 * sizeof(Real_type) * (m_kn - 2) * (m_jn - 2) +
                        2 * sizeof(Real_type) * (m_kn - 2) * (m_jn - 2) +
                        2 * sizeof(Real_type) * (m_kn - 2) * (m_jn - 2));
  setBytesAtomicModifyWrittenPerRep(0);
  setFLOPsPerRep((14 + 26 + 4) * (m_jn - 2) * (m_kn - 2));
  checksum_scale_factor = 0.001 * (static_cast<Checksum_type>(getDefaultProblemSize()) /
                                   getActualProblemSize());
  setComplexity(Complexity::N);
  setUsesFeature(Kernel);
  setVariantDefined(Base_GB300);
}

void HYDRO_2D::setUp(VariantID vid, size_t) {
  allocAndInitDataConst(m_zrout, m_array_length, 0.0, vid);
  allocAndInitDataConst(m_zzout, m_array_length, 0.0, vid);
  allocAndInitData(m_za, m_array_length, vid);
  allocAndInitData(m_zb, m_array_length, vid);
  allocAndInitData(m_zm, m_array_length, vid);
  allocAndInitData(m_zp, m_array_length, vid);
  allocAndInitData(m_zq, m_array_length, vid);
  allocAndInitData(m_zr, m_array_length, vid);
  allocAndInitData(m_zu, m_array_length, vid);
  allocAndInitData(m_zv, m_array_length, vid);
  allocAndInitData(m_zz, m_array_length, vid);
  // --host-data: two sweeps, so the arrays are staged; za and zb are
  // rewritten by BODY1 before BODY2 reads them (device scratch)
  for (Real_ptr* p : {&m_zp, &m_zq, &m_zr, &m_zm, &m_zz}) stageArray(*p, m_array_length, kIn);
  stageArray(m_zu, m_array_length, kIn | kOut);
  stageArray(m_zv, m_array_length, kIn | kOut);
  stageArray(m_za, m_array_length, 0);
  stageArray(m_zb, m_array_length, 0);
  stageArray(m_zrout, m_array_length, kOut);
  stageArray(m_zzout, m_array_length, kOut);
}

KernelBase::RepBody HYDRO_2D::makeRepBody(size_t tune_idx) {
  const b200_tune tn = getTune(tune_idx);
  return [=](b200_stream_t s) {
    checkB200(b200_lcals_hydro_2d(m_za, m_zb, m_zm, m_zp, m_zq, m_zr, m_zu, m_zv, m_zz,
                                  m_zrout, m_zzout, m_s, m_t, m_kn, m_jn, &tn, s),
              "b200_lcals_hydro_2d");
  };
}

void HYDRO_2D::updateChecksum(VariantID vid, size_t tune_idx) {
  checksum[vid][tune_idx] += calcChecksum(m_zzout, m_array_length, checksum_scale_factor, vid);
  checksum[vid][tune_idx] += calcChecksum(m_zrout, m_array_length, checksum_scale_factor, vid);
}

void HYDRO_2D::tearDown(VariantID vid, size_t) {
  deallocData(m_zrout, vid);
  deallocData(m_zzout, vid);
  deallocData(m_za, vid);
  deallocData(m_zb, vid);
  deallocData(m_zm, vid);
  deallocData(m_zp, vid);
  deallocData(m_zq, vid);
  deallocData(m_zr, vid);
  deallocData(m_zu, vid);
  deallocData(m_zv, vid);
  deallocData(m_zz, vid);
}

}  // namespace lcals
}  // namespace rajaperf
