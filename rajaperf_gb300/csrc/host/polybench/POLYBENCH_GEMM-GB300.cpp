// Polybench_GEMM.  Follows the suite's POLYBENCH_GEMM.cpp:24-95: ni = nj =
// sqrt(size) + sqrt(2) - 1, nk = 1.2*ni, alpha = 0.62 (beta = 1.002 is
// overwritten by BODY4, so C = alpha*A*B), checksum over C.
#include "Polybench.hpp"

#include <cmath>

namespace rajaperf {
namespace polybench {

POLYBENCH_GEMM::POLYBENCH_GEMM(const RunParams& params)
    : KernelBase(rajaperf::Polybench_GEMM, params) {
  Index_type ni_default = 1000, nj_default = 1000, nk_default = 1200;
  setDefaultProblemSize(ni_default * nj_default);
  setDefaultReps(4);
  m_ni = static_cast<Index_type>(std::sqrt(getTargetProblemSize()) + std::sqrt(2) - 1);
  m_nj = m_ni;
  m_nk = static_cast<Index_type>(double(nk_default) / ni_default * m_ni);
  m_alpha = 0.62;
  m_beta = 1.002;
  setActualProblemSize(m_ni * m_nj);
  setItsPerRep(m_ni * m_nj);
  setKernelsPerRep(1);
  setBytesReadPerRep(1 * sizeof(Real_type) * m_ni * m_nk + 1 * sizeof(Real_type) * m_nj * m_nk);
  setBytesWrittenPerRep(1 * sizeof(Real_type) * m_ni * m_nj);
  setBytesAtomicModifyWrittenPerRep(0);
  setFLOPsPerRep((1 + 3 * m_nk) * m_ni * m_nj);
  checksum_scale_factor = 0.001 * (static_cast<Checksum_type>(getDefaultProblemSize()) /
                                   getActualProblemSize());
  setComplexity(Complexity::N_to_the_three_halves);
  setUsesFeature(Kernel);
  addTuning("split_fp8", b200_tune{}, false);  // the e4m3 tensor-core engine (default)
  addTuning("split_fp8_graph", b200_tune{}, true);
  b200_tune bf16{};
  bf16.algo = 2;  // the same digits on bf16 tensor cores
  addTuning("split_bf16", bf16, false);
  setVariantDefined(Base_GB300);
}

bool POLYBENCH_GEMM::isSplit(size_t tune_idx) const {
  return getVariantTuningName(Base_GB300, tune_idx).rfind("split", 0) == 0;
}

void POLYBENCH_GEMM::setUp(VariantID vid, size_t tune_idx) {
  allocAndInitData(m_A, m_ni * m_nk, vid);
  allocAndInitData(m_B, m_nk * m_nj, vid);
  allocAndInitDataConst(m_C, m_ni * m_nj, 0.0, vid);
  if (isSplit(tune_idx)) {
    const b200_tune tn = getTune(tune_idx);
    m_ws_bytes = b200_gemm_split_workspace_bytes(m_ni, m_nj, m_nk, &tn);
    m_ws = allocDeviceBytes(m_ws_bytes);
    zeroDeviceBytes(m_ws, m_ws_bytes);
  }
}

KernelBase::RepBody POLYBENCH_GEMM::makeRepBody(size_t tune_idx) {
  const b200_tune tn = getTune(tune_idx);
  if (isSplit(tune_idx)) {
    // C = alpha*A*B (the suite's beta scaling is overwritten by BODY4)
    return [=](b200_stream_t s) {
      checkB200(b200_gemm_split(m_A, m_B, m_C, m_ni, m_nj, m_nk, m_alpha, 0.0, m_ws,
                                m_ws_bytes, &tn, s),
                "b200_gemm_split");
    };
  }
  return [=](b200_stream_t s) {
    checkB200(b200_polybench_gemm(m_A, m_B, m_C, m_ni, m_nj, m_nk, m_alpha, &tn, s),
              "b200_polybench_gemm");
  };
}

void POLYBENCH_GEMM::finishRun(size_t) {
  checkWorkspace(m_ws, m_ws_bytes, "Polybench_GEMM");
}

void POLYBENCH_GEMM::updateChecksum(VariantID vid, size_t tune_idx) {
  checksum[vid][tune_idx] += calcChecksum(m_C, m_ni * m_nj, checksum_scale_factor, vid);
}

void POLYBENCH_GEMM::tearDown(VariantID vid, size_t) {
  deallocData(m_A, vid);
  deallocData(m_B, vid);
  deallocData(m_C, vid);
  deallocDeviceBytes(m_ws);
  m_ws = nullptr;
}

}  // namespace polybench
}  // namespace rajaperf
