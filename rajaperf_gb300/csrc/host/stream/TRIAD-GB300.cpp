// Stream_TRIAD: a[i] = b[i] + alpha*c[i].  Follows the suite's
// stream/TRIAD.cpp:24-84 (checksum scale 0.001*default/actual size).
#include "Stream.hpp"

namespace rajaperf {
namespace stream {

TRIAD::TRIAD(const RunParams& params) : KernelBase(rajaperf::Stream_TRIAD, params) {
  setDefaultProblemSize(1000000);
  setDefaultReps(1000);
  setActualProblemSize(getTargetProblemSize());
  setItsPerRep(getActualProblemSize());
  setKernelsPerRep(1);
  setBytesReadPerRep(2 * sizeof(Real_type) * getActualProblemSize());
  setBytesWrittenPerRep(1 * sizeof(Real_type) * getActualProblemSize());
  setBytesAtomicModifyWrittenPerRep(0);
  setFLOPsPerRep(2 * getActualProblemSize());
  checksum_scale_factor = 0.001 * (static_cast<Checksum_type>(getDefaultProblemSize()) /
                                   getActualProblemSize());
  setComplexity(Complexity::N);
  setUsesFeature(Forall);
  setVariantDefined(Base_GB300);
}

void TRIAD::setUp(VariantID vid, size_t) {
  allocAndInitDataConst(m_a, getActualProblemSize(), 0.0, vid);
  allocAndInitData(m_b, getActualProblemSize(), vid);
  allocAndInitData(m_c, getActualProblemSize(), vid);
  // --host-data: one streaming pass, on the host arrays directly
  hostArray(m_a, getActualProblemSize(), kOut);
  hostArray(m_b, getActualProblemSize(), kIn);
  hostArray(m_c, getActualProblemSize(), kIn);
  initData(m_alpha, vid);
}

KernelBase::RepBody TRIAD::makeRepBody(size_t tune_idx) {
  const b200_tune t = getTune(tune_idx);
  const Index_type n = getActualProblemSize();
  return [=](b200_stream_t s) {
    checkB200(b200_stream_triad(m_a, m_b, m_c, m_alpha, n, &t, s), "b200_stream_triad");
  };
}

void TRIAD::updateChecksum(VariantID vid, size_t tune_idx) {
  checksum[vid][tune_idx] +=
      calcChecksum(m_a, getActualProblemSize(), checksum_scale_factor, vid);
}

void TRIAD::tearDown(VariantID vid, size_t) {
  deallocData(m_a, vid);
  deallocData(m_b, vid);
  deallocData(m_c, vid);
}

}  // namespace stream
}  // namespace rajaperf
