// Algorithm_REDUCE_SUM.  Follows the suite's algorithm/REDUCE_SUM.cpp:24-76:
// m_sum = sum of x each rep (not accumulated), checksum of m_sum.
#include "Algorithm.hpp"

namespace rajaperf {
namespace algorithm {

REDUCE_SUM::REDUCE_SUM(const RunParams& params)
    : KernelBase(rajaperf::Algorithm_REDUCE_SUM, params) {
  setDefaultProblemSize(1000000);
  setDefaultReps(50);
  setActualProblemSize(getTargetProblemSize());
  setItsPerRep(getActualProblemSize());
  setKernelsPerRep(1);
  setBytesReadPerRep(1 * sizeof(Real_type) * (1 + getActualProblemSize()));
  setBytesWrittenPerRep(1 * sizeof(Real_type));
  setBytesAtomicModifyWrittenPerRep(0);
  setFLOPsPerRep(getActualProblemSize());
  setComplexity(Complexity::N);
  setUsesFeature(Forall);
  setUsesFeature(Reduction);
  setVariantDefined(Base_GB300);
}

void REDUCE_SUM::setUp(VariantID vid, size_t tune_idx) {
  allocAndInitData(m_x, getActualProblemSize(), vid);
  m_sum_init = 0.0;
  m_sum = 0.0;
  allocData(m_dsum, 1, vid);
  copyToDevice(m_dsum, &m_sum, sizeof(Real_type));
  const b200_tune t = getTune(tune_idx);
  m_ws_bytes = b200_reduce_workspace_bytes(getActualProblemSize(), &t);
  m_ws = allocDeviceBytes(m_ws_bytes);
  zeroDeviceBytes(m_ws, m_ws_bytes);
}

KernelBase::RepBody REDUCE_SUM::makeRepBody(size_t tune_idx) {
  const b200_tune tn = getTune(tune_idx);
  const Index_type n = getActualProblemSize();
  return [=](b200_stream_t s) {
    checkB200(b200_algorithm_reduce_sum(m_x, n, m_sum_init, m_dsum, m_ws, m_ws_bytes, &tn, s),
              "b200_algorithm_reduce_sum");
  };
}

void REDUCE_SUM::finishRun(size_t) { copyToHost(&m_sum, m_dsum, sizeof(Real_type)); }

void REDUCE_SUM::updateChecksum(VariantID vid, size_t tune_idx) {
  checksum[vid][tune_idx] += calcChecksumHost(&m_sum, 1, 1.0);
}

void REDUCE_SUM::tearDown(VariantID vid, size_t) {
  deallocData(m_x, vid);
  deallocData(m_dsum, vid);
  deallocDeviceBytes(m_ws);
  m_ws = nullptr;
}

}  // namespace algorithm
}  // namespace rajaperf
