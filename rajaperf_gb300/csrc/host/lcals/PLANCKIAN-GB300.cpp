// Lcals_PLANCKIAN.  Follows the suite's lcals/PLANCKIAN.cpp.
#include "Lcals.hpp"

namespace rajaperf {
namespace lcals {

PLANCKIAN::PLANCKIAN(const RunParams& params) : KernelBase(rajaperf::Lcals_PLANCKIAN, params) {
  setDefaultProblemSize(1000000);
  setDefaultReps(50);
  setActualProblemSize(getTargetProblemSize());
  setItsPerRep(getActualProblemSize());
  setKernelsPerRep(1);
  setBytesReadPerRep(3 * sizeof(Real_type) * getActualProblemSize());
  setBytesWrittenPerRep(2 * sizeof(Real_type) * getActualProblemSize());
  setBytesAtomicModifyWrittenPerRep(0);
  setFLOPsPerRep(4 * getActualProblemSize());
  setComplexity(Complexity::N);
  setUsesFeature(Forall);
  setVariantDefined(Base_GB300);
}

void PLANCKIAN::setUp(VariantID vid, size_t) {
  allocAndInitData(m_x, getActualProblemSize(), vid);
  allocAndInitData(m_y, getActualProblemSize(), vid);
  allocAndInitData(m_u, getActualProblemSize(), vid);
  allocAndInitData(m_v, getActualProblemSize(), vid);
  allocAndInitDataConst(m_w, getActualProblemSize(), 0.0, vid);
}

KernelBase::RepBody PLANCKIAN::makeRepBody(size_t tune_idx) {
  const b200_tune tn = getTune(tune_idx);
  const Index_type n = getActualProblemSize();
  return [=](b200_stream_t s) {
    checkB200(b200_lcals_planckian(m_x, m_y, m_u, m_v, m_w, n, &tn, s),
              "b200_lcals_planckian");
  };
}

void PLANCKIAN::updateChecksum(VariantID vid, size_t tune_idx) {
  checksum[vid][tune_idx] += calcChecksum(m_w, getActualProblemSize(), vid);
}

void PLANCKIAN::tearDown(VariantID vid, size_t) {
  deallocData(m_x, vid);
  deallocData(m_y, vid);
  deallocData(m_u, vid);
  deallocData(m_v, vid);
  deallocData(m_w, vid);
}

}  // namespace lcals
}  // namespace rajaperf
