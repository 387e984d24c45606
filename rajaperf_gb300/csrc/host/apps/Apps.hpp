// Apps group kernels (suite src/apps).
#pragma once

#include "AppsData.hpp"
#include "common/KernelDecl.hpp"

#include <memory>

namespace rajaperf {
namespace apps {

RAJAPERF_GB300_KERNEL(DEL_DOT_VEC_2D,
 private:
  std::unique_ptr<ADomain> m_domain;
  Index_type m_array_length = 0;
  Real_ptr m_x = nullptr, m_y = nullptr, m_xdot = nullptr, m_ydot = nullptr,
           m_div = nullptr;
  Index_type* m_real_zones = nullptr;
  Real_type m_ptiny = 0.0, m_half = 0.0;)

RAJAPERF_GB300_KERNEL(VOL3D,
 private:
  std::unique_ptr<ADomain> m_domain;
  Index_type m_array_length = 0;
  Real_ptr m_x = nullptr, m_y = nullptr, m_z = nullptr, m_vol = nullptr;
  Real_type m_vnormq = 0.0;)

RAJAPERF_GB300_KERNEL(ENERGY,
 private:
  Real_ptr m_e_new = nullptr, m_e_old = nullptr, m_delvc = nullptr, m_p_new = nullptr,
           m_p_old = nullptr, m_q_new = nullptr, m_q_old = nullptr, m_work = nullptr,
           m_compHalfStep = nullptr, m_pHalfStep = nullptr, m_bvc = nullptr,
           m_pbvc = nullptr, m_ql_old = nullptr, m_qq_old = nullptr, m_vnewc = nullptr;
  Real_type m_rho0 = 0, m_e_cut = 0, m_emin = 0, m_q_cut = 0;)

RAJAPERF_GB300_KERNEL(PRESSURE,
 private:
  Real_ptr m_compression = nullptr, m_bvc = nullptr, m_p_new = nullptr,
           m_e_old = nullptr, m_vnewc = nullptr;
  Real_type m_cls = 0, m_p_cut = 0, m_pmin = 0, m_eosvmax = 0;)

}  // namespace apps
}  // namespace rajaperf
