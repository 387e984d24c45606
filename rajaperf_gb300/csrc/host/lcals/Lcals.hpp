// LCALS group kernels (suite src/lcals).
#pragma once

#include "common/KernelDecl.hpp"

namespace rajaperf {
namespace lcals {

RAJAPERF_GB300_KERNEL(HYDRO_1D,
 private:
  Real_ptr m_x = nullptr;
  Real_ptr m_y = nullptr;
  Real_ptr m_z = nullptr;
  Real_type m_q = 0.0, m_r = 0.0, m_t = 0.0;
  Index_type m_array_length = 0;)

RAJAPERF_GB300_KERNEL(HYDRO_2D,
 private:
  Real_ptr m_za = nullptr, m_zb = nullptr, m_zm = nullptr, m_zp = nullptr;
  Real_ptr m_zq = nullptr, m_zr = nullptr, m_zu = nullptr, m_zv = nullptr;
  Real_ptr m_zz = nullptr, m_zrout = nullptr, m_zzout = nullptr;
  Real_type m_s = 0.0, m_t = 0.0;
  Index_type m_jn = 0, m_kn = 0, m_array_length = 0;)

RAJAPERF_GB300_KERNEL(EOS,
 private:
  Real_ptr m_x = nullptr, m_y = nullptr, m_z = nullptr, m_u = nullptr;
  Real_type m_q = 0.0, m_r = 0.0, m_t = 0.0;
  Index_type m_array_length = 0;)

RAJAPERF_GB300_KERNEL(FIRST_DIFF,
 private:
  Real_ptr m_x = nullptr, m_y = nullptr;
  Index_type m_N = 0;)

RAJAPERF_GB300_KERNEL(INT_PREDICT,
 private:
  Real_ptr m_px = nullptr;
  Real_type m_px_initval = 0.0;
  Real_type m_dm22 = 0, m_dm23 = 0, m_dm24 = 0, m_dm25 = 0, m_dm26 = 0, m_dm27 = 0,
            m_dm28 = 0, m_c0 = 0;
  Index_type m_array_length = 0, m_offset = 0;)

RAJAPERF_GB300_KERNEL(FIRST_MIN,
 public:
  void finishRun(size_t tune_idx) override;
 private:
  Real_ptr m_x = nullptr;
  Real_type m_xmin_init = 0.0;
  Index_type m_initloc = 0, m_minloc = -1, m_N = 0;
  Index_type* m_dminloc = nullptr;
  void* m_ws = nullptr;
  size_t m_ws_bytes = 0;)

RAJAPERF_GB300_KERNEL(DIFF_PREDICT,
 private:
  Real_ptr m_px = nullptr, m_cx = nullptr;
  Index_type m_array_length = 0, m_offset = 0;)

RAJAPERF_GB300_KERNEL(PLANCKIAN,
 private:
  Real_ptr m_x = nullptr, m_y = nullptr, m_u = nullptr, m_v = nullptr, m_w = nullptr;)

}  // namespace lcals
}  // namespace rajaperf
