// Polybench_3MM.  Follows the suite's POLYBENCH_3MM.cpp:28-117: nk = 1.01*ni,
// nm = 1.2*ni, E = A*B, F = C*D, G = E*F, checksum over G (scale 1e-9).
#include "Polybench.hpp"

#include <algorithm>
#include <cmath>

namespace rajaperf {
namespace polybench {

POLYBENCH_3MM::POLYBENCH_3MM(const RunParams& params)
    : KernelBase(rajaperf::Polybench_3MM, params) {
  Index_type ni_default = 1000, nk_default = 1010, nm_default = 1200;
  setDefaultProblemSize(ni_default * 1000);
  setDefaultReps(2);
  m_ni = static_cast<Index_type>(std::sqrt(getTargetProblemSize()) + std::sqrt(2) - 1);
  m_nj = m_ni;
  m_nk = static_cast<Index_type>(double(nk_default) / ni_default * m_ni);
  m_nl = m_ni;
  m_nm = static_cast<Index_type>(double(nm_default) / ni_default * m_ni);
  setActualProblemSize(std::max(std::max(m_ni * m_nj, m_nj * m_nl), m_ni * m_nl));
  setItsPerRep(m_ni * m_nj + m_nj * m_nl + m_ni * m_nl);
  setKernelsPerRep(3);
  setBytesReadPerRep(1 * sizeof(Real_type) * m_ni * m_nk + 1 * sizeof(Real_type) * m_nj * m_nk +
                     1 * sizeof(Real_type) * m_nj * m_nm + 1 * sizeof(Real_type) * m_nl * m_nm +
                     1 * sizeof(Real_type) * m_ni * m_nj + 1 * sizeof(Real_type) * m_nj * m_nl);
  setBytesWrittenPerRep(1 * sizeof(Real_type) * m_ni * m_nj +
                        1 * sizeof(Real_type) * m_nj * m_nl +
                        1 * sizeof(Real_type) * m_ni * m_nl);
  setBytesAtomicModifyWrittenPerRep(0);
  setFLOPsPerRep(2 * m_ni * m_nj * m_nk + 2 * m_nj * m_nl * m_nm + 2 * m_ni * m_nj * m_nl);
  checksum_scale_factor = 0.000000001 * (static_cast<Checksum_type>(getDefaultProblemSize()) /
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

bool POLYBENCH_3MM::isSplit(size_t tune_idx) const {
  return getVariantTuningName(Base_GB300, tune_idx).rfind("split", 0) == 0;
}

void POLYBENCH_3MM::setUp(VariantID vid, size_t tune_idx) {
  if (isSplit(tune_idx)) {
    const b200_tune tn = getTune(tune_idx);
    m_ws_bytes = std::max(std::max(b200_gemm_split_workspace_bytes(m_ni, m_nj, m_nk, &tn),
                                   b200_gemm_split_workspace_bytes(m_nj, m_nl, m_nm, &tn)),
                          b200_gemm_split_workspace_bytes(m_ni, m_nl, m_nj, &tn));
    m_ws = allocDeviceBytes(m_ws_bytes);
    zeroDeviceBytes(m_ws, m_ws_bytes);
  }
  allocAndInitData(m_A, m_ni * m_nk, vid);
  allocAndInitData(m_B, m_nk * m_nj, vid);
  allocAndInitData(m_C, m_nj * m_nm, vid);
  allocAndInitData(m_D, m_nm * m_nl, vid);
  allocAndInitDataConst(m_E, m_ni * m_nj, 0.0, vid);
  allocAndInitDataConst(m_F, m_nj * m_nl, 0.0, vid);
  allocAndInitDataConst(m_G, m_ni * m_nl, 0.0, vid);
}

KernelBase::RepBody POLYBENCH_3MM::makeRepBody(size_t tune_idx) {
  const b200_tune tn = getTune(tune_idx);
  if (isSplit(tune_idx)) {
    return [=](b200_stream_t s) {
      checkB200(b200_gemm_split(m_A, m_B, m_E, m_ni, m_nj, m_nk, 1.0, 0.0, m_ws, m_ws_bytes,
                                &tn, s), "b200_gemm_split");
      checkB200(b200_gemm_split(m_C, m_D, m_F, m_nj, m_nl, m_nm, 1.0, 0.0, m_ws, m_ws_bytes,
                                &tn, s), "b200_gemm_split");
      checkB200(b200_gemm_split(m_E, m_F, m_G, m_ni, m_nl, m_nj, 1.0, 0.0, m_ws, m_ws_bytes,
                                &tn, s), "b200_gemm_split");
    };
  }
  return [=](b200_stream_t s) {
    checkB200(b200_polybench_3mm(m_A, m_B, m_C, m_D, m_E, m_F, m_G, m_ni, m_nj, m_nk, m_nl,
                                 m_nm, &tn, s),
              "b200_polybench_3mm");
  };
}

void POLYBENCH_3MM::finishRun(size_t) { checkWorkspace(m_ws, m_ws_bytes, "Polybench_3MM"); }

void POLYBENCH_3MM::updateChecksum(VariantID vid, size_t tune_idx) {
  checksum[vid][tune_idx] += calcChecksum(m_G, m_ni * m_nl, checksum_scale_factor, vid);
}

void POLYBENCH_3MM::tearDown(VariantID vid, size_t) {
  for (Real_ptr* p : {&m_A, &m_B, &m_C, &m_D, &m_E, &m_F, &m_G}) deallocData(*p, vid);
  deallocDeviceBytes(m_ws);
  m_ws = nullptr;
}

}  // namespace polybench
}  // namespace rajaperf
