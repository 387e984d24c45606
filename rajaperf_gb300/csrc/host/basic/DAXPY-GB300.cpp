// Basic_DAXPY: y[i] += a*x[i].  Follows the suite's basic/DAXPY.cpp.
#include "Basic.hpp"

namespace rajaperf {
namespace basic {

DAXPY::DAXPY(const RunParams& params) : KernelBase(rajaperf::Basic_DAXPY, params) {
  setDefaultProblemSize(1000000);
  setDefaultReps(500);
  setActualProblemSize(getTargetProblemSize());
  setItsPerRep(getActualProblemSize());
  setKernelsPerRep(1);
  setBytesReadPerRep(2 * sizeof(Real_type) * getActualProblemSize());
  setBytesWrittenPerRep(1 * sizeof(Real_type) * getActualProblemSize());
  setBytesAtomicModifyWrittenPerRep(0);
  setFLOPsPerRep(2 * getActualProblemSize());
  setComplexity(Complexity::N);
  setUsesFeature(Forall);
  setVariantDefined(Base_GB300);
}

void DAXPY::setUp(VariantID vid, size_t) {
  allocAndInitDataConst(m_y, getActualProblemSize(), 0.0, vid);
  allocAndInitData(m_x, getActualProblemSize(), vid);
  initData(m_a, vid);
}

KernelBase::RepBody DAXPY::makeRepBody(size_t tune_idx) {
  const b200_tune t = getTune(tune_idx);
  const Index_type n = getActualProblemSize();
  return [=](b200_stream_t s) {
    checkB200(b200_basic_daxpy(m_y, m_x, m_a, n, &t, s), "b200_basic_daxpy");
  };
}

void DAXPY::updateChecksum(VariantID vid, size_t tune_idx) {
  checksum[vid][tune_idx] += calcChecksum(m_y, getActualProblemSize(), vid);
}

void DAXPY::tearDown(VariantID vid, size_t) {
  deallocData(m_x, vid);
  deallocData(m_y, vid);
}

}  // namespace basic
}  // namespace rajaperf
