// Lcals_DIFF_PREDICT.  Follows the suite's lcals/DIFF_PREDICT.cpp.
#include "Lcals.hpp"

namespace rajaperf {
namespace lcals {

DIFF_PREDICT::DIFF_PREDICT(const RunParams& params)
    : KernelBase(rajaperf::Lcals_DIFF_PREDICT, params) {
  setDefaultProblemSize(1000000);
  setDefaultReps(200);
  setActualProblemSize(getTargetProblemSize());
  setItsPerRep(getActualProblemSize());
  setKernelsPerRep(1);
  setBytesReadPerRep(10 * sizeof(Real_type) * getActualProblemSize());
  setBytesWrittenPerRep(10 * sizeof(Real_type) * getActualProblemSize());
  setBytesAtomicModifyWrittenPerRep(0);
  setFLOPsPerRep(9 * getActualProblemSize());
  setComplexity(Complexity::N);
  setUsesFeature(Forall);
  setVariantDefined(Base_GB300);
}

void DIFF_PREDICT::setUp(VariantID vid, size_t) {
  m_array_length = getActualProblemSize() * 14;
  m_offset = getActualProblemSize();
  allocAndInitDataConst(m_px, m_array_length, 0.0, vid);
  allocAndInitData(m_cx, m_array_length, vid);
}

KernelBase::RepBody DIFF_PREDICT::makeRepBody(size_t tune_idx) {
  const b200_tune tn = getTune(tune_idx);
  const Index_type n = getActualProblemSize();
  return [=](b200_stream_t s) {
    checkB200(b200_lcals_diff_predict(m_px, m_cx, n, &tn, s), "b200_lcals_diff_predict");
  };
}

void DIFF_PREDICT::updateChecksum(VariantID vid, size_t tune_idx) {
  checksum[vid][tune_idx] += calcChecksum(m_px, m_array_length, vid);
}

void DIFF_PREDICT::tearDown(VariantID vid, size_t) {
  deallocData(m_px, vid);
  deallocData(m_cx, vid);
}

}  // namespace lcals
}  // namespace rajaperf
