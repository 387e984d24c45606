// Lcals_FIRST_DIFF.  Follows the suite's lcals/FIRST_DIFF.cpp:24-77.
#include "Lcals.hpp"

namespace rajaperf {
namespace lcals {

FIRST_DIFF::FIRST_DIFF(const RunParams& params)
    : KernelBase(rajaperf::Lcals_FIRST_DIFF, params) {
  setDefaultProblemSize(1000000);
  setDefaultReps(2000);
  setActualProblemSize(getTargetProblemSize());
  m_N = getActualProblemSize() + 1;
  setItsPerRep(getActualProblemSize());
  setKernelsPerRep(1);
  setBytesReadPerRep(1 * sizeof(Real_type) * m_N);
  setBytesWrittenPerRep(1 * sizeof(Real_type) * getActualProblemSize());
  setBytesAtomicModifyWrittenPerRep(0);
  setFLOPsPerRep(1 * getActualProblemSize());
  setComplexity(Complexity::N);
  setUsesFeature(Forall);
  setVariantDefined(Base_GB300);
}

void FIRST_DIFF::setUp(VariantID vid, size_t) {
  allocAndInitDataConst(m_x, m_N, 0.0, vid);
  allocAndInitData(m_y, m_N, vid);
  // --host-data: one streaming pass, on the host arrays directly
  hostArray(m_y, m_N, kIn);
  hostArray(m_x, getActualProblemSize(), kOut);
}

KernelBase::RepBody FIRST_DIFF::makeRepBody(size_t tune_idx) {
  const b200_tune tn = getTune(tune_idx);
  const Index_type n = getActualProblemSize();
  return [=](b200_stream_t s) {
    checkB200(b200_lcals_first_diff(m_x, m_y, n, &tn, s), "b200_lcals_first_diff");
  };
}

void FIRST_DIFF::updateChecksum(VariantID vid, size_t tune_idx) {
  checksum[vid][tune_idx] += calcChecksum(m_x, getActualProblemSize(), vid);
}

void FIRST_DIFF::tearDown(VariantID vid, size_t) {
  deallocData(m_x, vid);
  deallocData(m_y, vid);
}

}  // namespace lcals
}  // namespace rajaperf
