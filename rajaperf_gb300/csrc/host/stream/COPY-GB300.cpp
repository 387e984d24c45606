// Stream_COPY: c[i] = a[i].  Sizes, bytes and data set-up follow the suite's
// stream/COPY.cpp:21-69; the rep body is one b200_stream_copy call.
#include "Stream.hpp"

namespace rajaperf {
namespace stream {

COPY::COPY(const RunParams& params) : KernelBase(rajaperf::Stream_COPY, params) {
  setDefaultProblemSize(1000000);
  setDefaultReps(1800);
  setActualProblemSize(getTargetProblemSize());
  setItsPerRep(getActualProblemSize());
  setKernelsPerRep(1);
  setBytesReadPerRep(1 * sizeof(Real_type) * getActualProblemSize());
  setBytesWrittenPerRep(1 * sizeof(Real_type) * getActualProblemSize());
  setBytesAtomicModifyWrittenPerRep(0);
  setFLOPsPerRep(0);
  setComplexity(Complexity::N);
  setUsesFeature(Forall);
  setVariantDefined(Base_GB300);
}

void COPY::setUp(VariantID vid, size_t) {
  allocAndInitData(m_a, getActualProblemSize(), vid);
  allocAndInitDataConst(m_c, getActualProblemSize(), 0.0, vid);
  // --host-data: one streaming pass, on the host arrays directly
  hostArray(m_a, getActualProblemSize(), kIn);
  hostArray(m_c, getActualProblemSize(), kOut);
}

KernelBase::RepBody COPY::makeRepBody(size_t tune_idx) {
  const b200_tune t = getTune(tune_idx);
  const Index_type n = getActualProblemSize();
  return [=](b200_stream_t s) {
    checkB200(b200_stream_copy(m_a, m_c, n, &t, s), "b200_stream_copy");
  };
}

void COPY::updateChecksum(VariantID vid, size_t tune_idx) {
  checksum[vid][tune_idx] += calcChecksum(m_c, getActualProblemSize(), vid);
}

void COPY::tearDown(VariantID vid, size_t) {
  deallocData(m_a, vid);
  deallocData(m_c, vid);
}

}  // namespace stream
}  // namespace rajaperf
