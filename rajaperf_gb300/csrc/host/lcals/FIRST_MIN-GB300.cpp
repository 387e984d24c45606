// Lcals_FIRST_MIN.  Follows the suite's lcals/FIRST_MIN.cpp:24-94: x is 0
// except x[N/2] = -1e10; the checksum is the location found (exact).  In the
// uniform input mode x is uniform in [lo, hi) with one planted minimum lo - 1
// at a seeded index.  The location is written on the device each rep.
#include "Lcals.hpp"

namespace rajaperf {
namespace lcals {

FIRST_MIN::FIRST_MIN(const RunParams& params) : KernelBase(rajaperf::Lcals_FIRST_MIN, params) {
  setDefaultProblemSize(1000000);
  setDefaultReps(100);
  setActualProblemSize(getTargetProblemSize());
  m_N = getActualProblemSize();
  setItsPerRep(getActualProblemSize());
  setKernelsPerRep(1);
  setBytesReadPerRep(1 * sizeof(Index_type) + 1 * sizeof(Real_type) +
                     1 * sizeof(Real_type) * m_N);
  setBytesWrittenPerRep(1 * sizeof(Index_type) + 1 * sizeof(Real_type));
  setBytesAtomicModifyWrittenPerRep(0);
  setFLOPsPerRep(0);
  setComplexity(Complexity::N);
  setUsesFeature(Forall);
  setUsesFeature(Reduction);
  setVariantDefined(Base_GB300);
}

void FIRST_MIN::setUp(VariantID vid, size_t tune_idx) {
  if (run_params.getInitMode() == RunParams::InitUniform) {
    allocAndInitData(m_x, m_N, vid);
    double u = uniformValue(run_params.getSeed(), 0xF1257ULL, 0, 0.0, 1.0);
    Index_type idx = static_cast<Index_type>(u * static_cast<double>(m_N));
    if (idx >= m_N) idx = m_N - 1;
    Real_type v = run_params.getInitLo() - 1.0;
    if (m_N > 0) copyToDevice(m_x + idx, &v, sizeof(Real_type));
  } else {
    allocAndInitDataConst(m_x, m_N, 0.0, vid);
    Real_type v = -1.0e+10;
    if (m_N > 0) copyToDevice(m_x + m_N / 2, &v, sizeof(Real_type));
  }
  m_xmin_init = 0.0;
  if (m_N > 0) copyToHost(&m_xmin_init, m_x, sizeof(Real_type));
  m_initloc = 0;
  m_minloc = -1;
  allocData(m_dminloc, 1, vid);
  copyToDevice(m_dminloc, &m_minloc, sizeof(Index_type));
  // --host-data: one streaming pass over x in host memory; the location is
  // written to host memory by the kernel
  hostArray(m_x, m_N, kIn);
  hostArray(m_dminloc, 1, kOut);
  const b200_tune t = getTune(tune_idx);
  m_ws_bytes = b200_reduce_workspace_bytes(m_N, &t);
  m_ws = allocDeviceBytes(m_ws_bytes);
  zeroDeviceBytes(m_ws, m_ws_bytes);
}

KernelBase::RepBody FIRST_MIN::makeRepBody(size_t tune_idx) {
  const b200_tune tn = getTune(tune_idx);
  return [=](b200_stream_t s) {
    checkB200(b200_lcals_first_min(m_x, m_N, m_xmin_init, m_initloc,
                                   reinterpret_cast<int64_t*>(m_dminloc), nullptr, m_ws,
                                   m_ws_bytes, &tn, s),
              "b200_lcals_first_min");
  };
}

void FIRST_MIN::finishRun(size_t) {
  copyToHost(&m_minloc, m_dminloc, sizeof(Index_type));
}

void FIRST_MIN::updateChecksum(VariantID vid, size_t tune_idx) {
  checksum[vid][tune_idx] += static_cast<long double>(m_minloc);
}

void FIRST_MIN::tearDown(VariantID vid, size_t) {
  deallocData(m_x, vid);
  deallocData(m_dminloc, vid);
  deallocDeviceBytes(m_ws);
  m_ws = nullptr;
}

}  // namespace lcals
}  // namespace rajaperf
