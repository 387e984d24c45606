// Apps_ENERGY.  Follows the suite's apps/ENERGY.cpp:24-112 (sizes, fifteen
// arrays, four scalars, checksum over e_new and q_new); the six loops run as
// one fused pass (b200_apps_energy).
#include "Apps.hpp"

namespace rajaperf {
namespace apps {

ENERGY::ENERGY(const RunParams& params) : KernelBase(rajaperf::Apps_ENERGY, params) {
  setDefaultProblemSize(1000000);
  setDefaultReps(130);
  setActualProblemSize(getTargetProblemSize());
  setItsPerRep(6 * getActualProblemSize());
  setKernelsPerRep(6);
  setBytesReadPerRep((5 * sizeof(Real_type) + 1 * sizeof(Real_type) + 6 * sizeof(Real_type) +
                      2 * sizeof(Real_type) + 7 * sizeof(Real_type) + 1 * sizeof(Real_type)) *
                     getActualProblemSize());
  setBytesWrittenPerRep(5 * sizeof(Real_type) * getActualProblemSize());
  setBytesAtomicModifyWrittenPerRep(0);
  setFLOPsPerRep((6 + 11 + 8 + 2 + 19 + 9) * getActualProblemSize());
  setComplexity(Complexity::N);
  setUsesFeature(Forall);
  setVariantDefined(Base_GB300);
}

void ENERGY::setUp(VariantID vid, size_t) {
  const Index_type n = getActualProblemSize();
  allocAndInitDataConst(m_e_new, n, 0.0, vid);
  allocAndInitData(m_e_old, n, vid);
  allocAndInitData(m_delvc, n, vid);
  allocAndInitData(m_p_new, n, vid);
  allocAndInitData(m_p_old, n, vid);
  allocAndInitDataConst(m_q_new, n, 0.0, vid);
  allocAndInitData(m_q_old, n, vid);
  allocAndInitData(m_work, n, vid);
  allocAndInitData(m_compHalfStep, n, vid);
  allocAndInitData(m_pHalfStep, n, vid);
  allocAndInitData(m_bvc, n, vid);
  allocAndInitData(m_pbvc, n, vid);
  allocAndInitData(m_ql_old, n, vid);
  allocAndInitData(m_qq_old, n, vid);
  allocAndInitData(m_vnewc, n, vid);
  initData(m_rho0, vid);
  initData(m_e_cut, vid);
  initData(m_emin, vid);
  initData(m_q_cut, vid);
}

KernelBase::RepBody ENERGY::makeRepBody(size_t tune_idx) {
  const b200_tune tn = getTune(tune_idx);
  const Index_type n = getActualProblemSize();
  return [=](b200_stream_t s) {
    checkB200(b200_apps_energy(m_e_new, m_e_old, m_delvc, m_p_new, m_p_old, m_q_new, m_q_old,
                               m_work, m_compHalfStep, m_pHalfStep, m_bvc, m_pbvc, m_ql_old,
                               m_qq_old, m_vnewc, m_rho0, m_e_cut, m_emin, m_q_cut, n, &tn,
                               s),
              "b200_apps_energy");
  };
}

void ENERGY::updateChecksum(VariantID vid, size_t tune_idx) {
  checksum[vid][tune_idx] += calcChecksum(m_e_new, getActualProblemSize(), vid);
  checksum[vid][tune_idx] += calcChecksum(m_q_new, getActualProblemSize(), vid);
}

void ENERGY::tearDown(VariantID vid, size_t) {
  for (Real_ptr* p : {&m_e_new, &m_e_old, &m_delvc, &m_p_new, &m_p_old, &m_q_new, &m_q_old,
                      &m_work, &m_compHalfStep, &m_pHalfStep, &m_bvc, &m_pbvc, &m_ql_old,
                      &m_qq_old, &m_vnewc})
    deallocData(*p, vid);
}

}  // namespace apps
}  // namespace rajaperf
