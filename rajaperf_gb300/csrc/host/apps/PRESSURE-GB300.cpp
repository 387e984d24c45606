// Apps_PRESSURE.  Follows the suite's apps/PRESSURE.cpp:24-86; both loops run
// as one fused pass (b200_apps_pressure).
#include "Apps.hpp"

namespace rajaperf {
namespace apps {

PRESSURE::PRESSURE(const RunParams& params) : KernelBase(rajaperf::Apps_PRESSURE, params) {
  setDefaultProblemSize(1000000);
  setDefaultReps(700);
  setActualProblemSize(getTargetProblemSize());
  setItsPerRep(2 * getActualProblemSize());
  setKernelsPerRep(2);
  setBytesReadPerRep(1 * sizeof(Real_type) * getActualProblemSize() +
                     3 * sizeof(Real_type) * getActualProblemSize());
  setBytesWrittenPerRep(1 * sizeof(Real_type) * getActualProblemSize() +
                        1 * sizeof(Real_type) * getActualProblemSize());
  setBytesAtomicModifyWrittenPerRep(0);
  setFLOPsPerRep((2 + 1) * getActualProblemSize());
  setComplexity(Complexity::N);
  setUsesFeature(Forall);
  setVariantDefined(Base_GB300);
}

void PRESSURE::setUp(VariantID vid, size_t) {
  const Index_type n = getActualProblemSize();
  allocAndInitData(m_compression, n, vid);
  allocAndInitData(m_bvc, n, vid);
  allocAndInitDataConst(m_p_new, n, 0.0, vid);
  allocAndInitData(m_e_old, n, vid);
  allocAndInitData(m_vnewc, n, vid);
  initData(m_cls, vid);
  initData(m_p_cut, vid);
  initData(m_pmin, vid);
  initData(m_eosvmax, vid);
}

KernelBase::RepBody PRESSURE::makeRepBody(size_t tune_idx) {
  const b200_tune tn = getTune(tune_idx);
  const Index_type n = getActualProblemSize();
  return [=](b200_stream_t s) {
    checkB200(b200_apps_pressure(m_compression, m_bvc, m_p_new, m_e_old, m_vnewc, m_cls,
                                 m_p_cut, m_pmin, m_eosvmax, n, &tn, s),
              "b200_apps_pressure");
  };
}

void PRESSURE::updateChecksum(VariantID vid, size_t tune_idx) {
  checksum[vid][tune_idx] += calcChecksum(m_p_new, getActualProblemSize(), vid);
}

void PRESSURE::tearDown(VariantID vid, size_t) {
  deallocData(m_compression, vid);
  deallocData(m_bvc, vid);
  deallocData(m_p_new, vid);
  deallocData(m_e_old, vid);
  deallocData(m_vnewc, vid);
}

}  // namespace apps
}  // namespace rajaperf
