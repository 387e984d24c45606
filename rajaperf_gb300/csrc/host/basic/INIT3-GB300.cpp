// Basic_INIT3.  Follows the suite's basic/INIT3.cpp (sizes, data set-up,
// checksum over the three outputs).
#include "Basic.hpp"

namespace rajaperf {
namespace basic {

INIT3::INIT3(const RunParams& params) : KernelBase(rajaperf::Basic_INIT3, params) {
  setDefaultProblemSize(1000000);
  setDefaultReps(500);
  setActualProblemSize(getTargetProblemSize());
  setItsPerRep(getActualProblemSize());
  setKernelsPerRep(1);
  setBytesReadPerRep(2 * sizeof(Real_type) * getActualProblemSize());
  setBytesWrittenPerRep(3 * sizeof(Real_type) * getActualProblemSize());
  setBytesAtomicModifyWrittenPerRep(0);
  setFLOPsPerRep(1 * getActualProblemSize());
  setComplexity(Complexity::N);
  setUsesFeature(Forall);
  setVariantDefined(Base_GB300);
}

void INIT3::setUp(VariantID vid, size_t) {
  allocAndInitDataConst(m_out1, getActualProblemSize(), 0.0, vid);
  allocAndInitDataConst(m_out2, getActualProblemSize(), 0.0, vid);
  allocAndInitDataConst(m_out3, getActualProblemSize(), 0.0, vid);
  allocAndInitData(m_in1, getActualProblemSize(), vid);
  allocAndInitData(m_in2, getActualProblemSize(), vid);
}

KernelBase::RepBody INIT3::makeRepBody(size_t tune_idx) {
  const b200_tune t = getTune(tune_idx);
  const Index_type n = getActualProblemSize();
  return [=](b200_stream_t s) {
    checkB200(b200_basic_init3(m_out1, m_out2, m_out3, m_in1, m_in2, n, &t, s),
              "b200_basic_init3");
  };
}

void INIT3::updateChecksum(VariantID vid, size_t tune_idx) {
  checksum[vid][tune_idx] += calcChecksum(m_out1, getActualProblemSize(), vid);
  checksum[vid][tune_idx] += calcChecksum(m_out2, getActualProblemSize(), vid);
  checksum[vid][tune_idx] += calcChecksum(m_out3, getActualProblemSize(), vid);
}

void INIT3::tearDown(VariantID vid, size_t) {
  deallocData(m_out1, vid);
  deallocData(m_out2, vid);
  deallocData(m_out3, vid);
  deallocData(m_in1, vid);
  deallocData(m_in2, vid);
}

}  // namespace basic
}  // namespace rajaperf
