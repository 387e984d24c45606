// Polybench group kernels (suite src/polybench).
#pragma once

#include "common/KernelDecl.hpp"

namespace rajaperf {
namespace polybench {

RAJAPERF_GB300_KERNEL(POLYBENCH_JACOBI_2D,
 public:
  void prepareRun(size_t tune_idx) override;
 private:
  Index_type m_N = 0, m_tsteps = 0;
  Real_ptr m_A = nullptr, m_B = nullptr, m_Ainit = nullptr, m_Binit = nullptr;)

RAJAPERF_GB300_KERNEL(POLYBENCH_HEAT_3D,
 public:
  void prepareRun(size_t tune_idx) override;
 private:
  Index_type m_N = 0, m_tsteps = 0;
  Real_ptr m_A = nullptr, m_B = nullptr, m_Ainit = nullptr, m_Binit = nullptr;)

// FDTD_2D runs one launch per time step (b200_polybench_fdtd_2d_ws, the
// tile-edge snapshots in m_ws); a tuning with algo 1 runs the two-launch form.
RAJAPERF_GB300_KERNEL(POLYBENCH_FDTD_2D,
 private:
  Index_type m_nx = 0, m_ny = 0, m_tsteps = 0;
  Real_ptr m_fict = nullptr, m_ex = nullptr, m_ey = nullptr, m_hz = nullptr;
  void* m_ws = nullptr;
  size_t m_ws_bytes = 0;)

// GEMM and 3MM tunings: "default"/"graph" run the native FP64 kernel;
// "split_fp8"/"split_fp8_graph" run the split-precision tensor-core GEMM
// (b200_gemm_split on e4m3 slices; inner dimensions up to 524288, summed in
// exact chunks of 8192), "split_bf16" the same digits on bf16 tensor cores.
RAJAPERF_GB300_KERNEL(POLYBENCH_GEMM,
 public:
  void finishRun(size_t tune_idx) override;
 private:
  bool isSplit(size_t tune_idx) const;
  Index_type m_ni = 0, m_nj = 0, m_nk = 0;
  Real_type m_alpha = 0.0, m_beta = 0.0;
  Real_ptr m_A = nullptr, m_B = nullptr, m_C = nullptr;
  void* m_ws = nullptr;
  size_t m_ws_bytes = 0;)

RAJAPERF_GB300_KERNEL(POLYBENCH_3MM,
 public:
  void finishRun(size_t tune_idx) override;
 private:
  bool isSplit(size_t tune_idx) const;
  Index_type m_ni = 0, m_nj = 0, m_nk = 0, m_nl = 0, m_nm = 0;
  Real_ptr m_A = nullptr, m_B = nullptr, m_C = nullptr, m_D = nullptr, m_E = nullptr,
           m_F = nullptr, m_G = nullptr;
  void* m_ws = nullptr;
  size_t m_ws_bytes = 0;)

}  // namespace polybench
}  // namespace rajaperf
