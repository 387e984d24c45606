// Stream_DOT: m_dot += sum a[i]*b[i] per rep.  Follows the suite's
// stream/DOT.cpp:21-81 and DOT-Seq.cpp:34-47.  The per-rep accumulation
// happens on the device (b200_stream_dot adds into m_ddot), so a rep needs
// no host round trip and the rep loop can be captured into a graph.
#include "Stream.hpp"

namespace rajaperf {
namespace stream {

DOT::DOT(const RunParams& params) : KernelBase(rajaperf::Stream_DOT, params) {
  setDefaultProblemSize(1000000);
  setDefaultReps(2000);
  setActualProblemSize(getTargetProblemSize());
  setItsPerRep(getActualProblemSize());
  setKernelsPerRep(1);
  setBytesReadPerRep(1 * sizeof(Real_type) + 2 * sizeof(Real_type) * getActualProblemSize());
  setBytesWrittenPerRep(1 * sizeof(Real_type));
  setBytesAtomicModifyWrittenPerRep(0);
  setFLOPsPerRep(2 * getActualProblemSize());
  setComplexity(Complexity::N);
  setUsesFeature(Forall);
  setUsesFeature(Reduction);
  setVariantDefined(Base_GB300);
}

void DOT::setUp(VariantID vid, size_t tune_idx) {
  allocAndInitData(m_a, getActualProblemSize(), vid);
  allocAndInitData(m_b, getActualProblemSize(), vid);
  m_dot = 0.0;
  m_dot_init = 0.0;
  allocData(m_ddot, 1, vid);
  copyToDevice(m_ddot, &m_dot, sizeof(Real_type));
  // --host-data: one streaming pass over the host arrays; the sum is
  // accumulated in host memory by the kernel
  hostArray(m_a, getActualProblemSize(), kIn);
  hostArray(m_b, getActualProblemSize(), kIn);
  hostArray(m_ddot, 1, kIn | kOut);
  const b200_tune t = getTune(tune_idx);
  m_ws_bytes = b200_reduce_workspace_bytes(getActualProblemSize(), &t);
  m_ws = allocDeviceBytes(m_ws_bytes);
  zeroDeviceBytes(m_ws, m_ws_bytes);
}

KernelBase::RepBody DOT::makeRepBody(size_t tune_idx) {
  const b200_tune t = getTune(tune_idx);
  const Index_type n = getActualProblemSize();
  return [=](b200_stream_t s) {
    checkB200(b200_stream_dot(m_a, m_b, n, m_dot_init, m_ddot, m_ws, m_ws_bytes,
                              &t, s),
              "b200_stream_dot");
  };
}

void DOT::finishRun(size_t) {
  copyToHost(&m_dot, m_ddot, sizeof(Real_type));
}

void DOT::updateChecksum(VariantID vid, size_t tune_idx) {
  checksum[vid][tune_idx] += m_dot;
}

void DOT::tearDown(VariantID vid, size_t) {
  deallocData(m_a, vid);
  deallocData(m_b, vid);
  deallocData(m_ddot, vid);
  deallocDeviceBytes(m_ws);
  m_ws = nullptr;
}

}  // namespace stream
}  // namespace rajaperf
