// Algorithm_SCAN.  Follows the suite's algorithm/SCAN.cpp:24-77: x from the
// C library generator (DataUtils.cpp:560-569), exclusive prefix sum into y,
// checksum scale 1e-2*default/actual/actual.
#include "Algorithm.hpp"


namespace rajaperf {
namespace algorithm {

SCAN::SCAN(const RunParams& params) : KernelBase(rajaperf::Algorithm_SCAN, params) {
  setDefaultProblemSize(1000000);
  setDefaultReps(100);
  setActualProblemSize(getTargetProblemSize());
  setItsPerRep(getActualProblemSize());
  setKernelsPerRep(1);
  setBytesReadPerRep(1 * sizeof(Real_type) * getActualProblemSize());
  setBytesWrittenPerRep(1 * sizeof(Real_type) * getActualProblemSize());
  setBytesAtomicModifyWrittenPerRep(0);
  setFLOPsPerRep(1 * getActualProblemSize());
  checksum_scale_factor = 1e-2 * (static_cast<Checksum_type>(getDefaultProblemSize()) /
                                  getActualProblemSize()) /
                          getActualProblemSize();
  setComplexity(Complexity::N);
  setUsesFeature(Scan);
  addTuning("int64", b200_tune{}, false);
  addTuning("int64_graph", b200_tune{}, true);
  setVariantDefined(Base_GB300);
}

void SCAN::setGB300TuningDefinitions(VariantID vid) {
  KernelBase::setGB300TuningDefinitions(vid);
}

bool SCAN::isInt64(size_t tune_idx) const {
  return getVariantTuningName(Base_GB300, tune_idx).rfind("int64", 0) == 0;
}

void SCAN::setUp(VariantID vid, size_t tune_idx) {
  const Index_type n = getActualProblemSize();
  if (isInt64(tune_idx)) {
    allocData(m_xi, n, vid);
    checkB200(b200_init_uniform_i64(m_xi, n, run_params.getSeed(),
                                    static_cast<uint64_t>(detail::getDataInitCount()), 0, 100,
                                    nullptr),
              "b200_init_uniform_i64");
    detail::incDataInitCount();
    allocData(m_yi, n, vid);
    checkB200(b200_init_const_i64(m_yi, n, 0, nullptr), "b200_init_const_i64");
    detail::incDataInitCount();
  } else {
    allocAndInitDataRandValue(m_x, n, vid);
    allocAndInitDataConst(m_y, n, 0.0, vid);
  }
  m_ws_bytes = b200_scan_workspace_bytes(n);
  m_ws = allocDeviceBytes(m_ws_bytes);
  zeroDeviceBytes(m_ws, m_ws_bytes);
  // --host-data: one streaming pass on the host arrays, with the one-CTA-per-
  // tile kernel (plain loads; the persistent kernel's bulk copies stay on
  // device memory)
  if (isInt64(tune_idx)) {
    hostArray(m_xi, n, kIn);
    hostArray(m_yi, n, kOut);
  } else {
    hostArray(m_x, n, kIn);
    hostArray(m_y, n, kOut);
  }
}

KernelBase::RepBody SCAN::makeRepBody(size_t tune_idx) {
  b200_tune tn = getTune(tune_idx);
  if (hostData()) tn.algo = 1;
  const Index_type n = getActualProblemSize();
  if (isInt64(tune_idx)) {
    return [=](b200_stream_t s) {
      checkB200(b200_algorithm_scan_i64(m_xi, m_yi, n, 0, m_ws, m_ws_bytes, &tn, s),
                "b200_algorithm_scan_i64");
    };
  }
  return [=](b200_stream_t s) {
    checkB200(b200_algorithm_scan(m_x, m_y, n, 0.0, m_ws, m_ws_bytes, &tn, s),
              "b200_algorithm_scan");
  };
}

void SCAN::prepareRun(size_t tune_idx) {
  const bool aligned = isInt64(tune_idx)
                           ? (reinterpret_cast<uintptr_t>(m_xi) % 16 == 0 &&
                              reinterpret_cast<uintptr_t>(m_yi) % 16 == 0)
                           : (reinterpret_cast<uintptr_t>(m_x) % 16 == 0 &&
                              reinterpret_cast<uintptr_t>(m_y) % 16 == 0);
  // the ring kernel (algo 0 for int64, 2 for FP64) is the one the stall targets
  b200_tune tn = getTune(tune_idx);
  if (tn.algo == 2 || (tn.algo == 0 && isInt64(tune_idx))) tn.algo = 0;
  else if (tn.algo == 0) tn.algo = 1;
  injectLookbackStall(m_ws, m_ws_bytes, tn, aligned);
}

void SCAN::finishRun(size_t) { checkWorkspace(m_ws, m_ws_bytes, "Algorithm_SCAN"); }

void SCAN::updateChecksum(VariantID vid, size_t tune_idx) {
  const Index_type n = getActualProblemSize();
  if (isInt64(tune_idx)) {
    checksum[vid][tune_idx] +=
        calcChecksumDevice(reinterpret_cast<const Index_type*>(m_yi), n, checksum_scale_factor);
  } else {
    checksum[vid][tune_idx] += calcChecksum(m_y, n, checksum_scale_factor, vid);
  }
}

void SCAN::tearDown(VariantID vid, size_t) {
  if (m_x) deallocData(m_x, vid);
  if (m_y) deallocData(m_y, vid);
  if (m_xi) deallocData(m_xi, vid);
  if (m_yi) deallocData(m_yi, vid);
  deallocDeviceBytes(m_ws);
  m_ws = nullptr;
}

}  // namespace algorithm
}  // namespace rajaperf
