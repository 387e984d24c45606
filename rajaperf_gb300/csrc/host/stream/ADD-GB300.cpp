// Stream_ADD: c[i] = a[i] + b[i].  Follows the suite's stream/ADD.cpp:21-76.
#include "Stream.hpp"

namespace rajaperf {
namespace stream {

ADD::ADD(const RunParams& params) : KernelBase(rajaperf::Stream_ADD, params) {
  setDefaultProblemSize(1000000);
  setDefaultReps(1000);
  setActualProblemSize(getTargetProblemSize());
  setItsPerRep(getActualProblemSize());
  setKernelsPerRep(1);
  setBytesReadPerRep(2 * sizeof(Real_type) * getActualProblemSize());
  setBytesWrittenPerRep(1 * sizeof(Real_type) * getActualProblemSize());
  setBytesAtomicModifyWrittenPerRep(0);
  setFLOPsPerRep(1 * getActualProblemSize());
  setComplexity(Complexity::N);
  setUsesFeature(Forall);
  setVariantDefined(Base_GB300);
}

void ADD::setUp(VariantID vid, size_t) {
  allocAndInitData(m_a, getActualProblemSize(), vid);
  allocAndInitData(m_b, getActualProblemSize(), vid);
  allocAndInitDataConst(m_c, getActualProblemSize(), 0.0, vid);
  // --host-data: one streaming pass, on the host arrays directly
  hostArray(m_a, getActualProblemSize(), kIn);
  hostArray(m_b, getActualProblemSize(), kIn);
  hostArray(m_c, getActualProblemSize(), kOut);
}

KernelBase::RepBody ADD::makeRepBody(size_t tune_idx) {
  const b200_tune t = getTune(tune_idx);
  const Index_type n = getActualProblemSize();
  return [=](b200_stream_t s) {
    checkB200(b200_stream_add(m_a, m_b, m_c, n, &t, s), "b200_stream_add");
  };
}

void ADD::updateChecksum(VariantID vid, size_t tune_idx) {
  checksum[vid][tune_idx] += calcChecksum(m_c, getActualProblemSize(), vid);
}

void ADD::tearDown(VariantID vid, size_t) {
  deallocData(m_a, vid);
  deallocData(m_b, vid);
  deallocData(m_c, vid);
}

}  // namespace stream
}  // namespace rajaperf
