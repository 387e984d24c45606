// Stream_MUL: b[i] = alpha*c[i].  Follows the suite's stream/MUL.cpp:21-75.
#include "Stream.hpp"

namespace rajaperf {
namespace stream {

MUL::MUL(const RunParams& params) : KernelBase(rajaperf::Stream_MUL, params) {
  setDefaultProblemSize(1000000);
  setDefaultReps(1800);
  setActualProblemSize(getTargetProblemSize());
  setItsPerRep(getActualProblemSize());
  setKernelsPerRep(1);
  setBytesReadPerRep(1 * sizeof(Real_type) * getActualProblemSize());
  setBytesWrittenPerRep(1 * sizeof(Real_type) * getActualProblemSize());
  setBytesAtomicModifyWrittenPerRep(0);
  setFLOPsPerRep(1 * getActualProblemSize());
  setComplexity(Complexity::N);
  setUsesFeature(Forall);
  setVariantDefined(Base_GB300);
}

void MUL::setUp(VariantID vid, size_t) {
  allocAndInitDataConst(m_b, getActualProblemSize(), 0.0, vid);
  allocAndInitData(m_c, getActualProblemSize(), vid);
  // --host-data: one streaming pass, on the host arrays directly
  hostArray(m_b, getActualProblemSize(), kOut);
  hostArray(m_c, getActualProblemSize(), kIn);
  initData(m_alpha, vid);
}

KernelBase::RepBody MUL::makeRepBody(size_t tune_idx) {
  const b200_tune t = getTune(tune_idx);
  const Index_type n = getActualProblemSize();
  return [=](b200_stream_t s) {
    checkB200(b200_stream_mul(m_b, m_c, m_alpha, n, &t, s), "b200_stream_mul");
  };
}

void MUL::updateChecksum(VariantID vid, size_t tune_idx) {
  checksum[vid][tune_idx] += calcChecksum(m_b, getActualProblemSize(), vid);
}

void MUL::tearDown(VariantID vid, size_t) {
  deallocData(m_b, vid);
  deallocData(m_c, vid);
}

}  // namespace stream
}  // namespace rajaperf
