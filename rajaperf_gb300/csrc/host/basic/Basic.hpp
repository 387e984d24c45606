// Basic group kernels of the batched small-size suite (suite src/basic).
#pragma once

#include "common/KernelDecl.hpp"

namespace rajaperf {
namespace basic {

RAJAPERF_GB300_KERNEL(DAXPY,
 private:
  Real_ptr m_x = nullptr;
  Real_ptr m_y = nullptr;
  Real_type m_a = 0.0;)

RAJAPERF_GB300_KERNEL(INIT3,
 private:
  Real_ptr m_out1 = nullptr;
  Real_ptr m_out2 = nullptr;
  Real_ptr m_out3 = nullptr;
  Real_ptr m_in1 = nullptr;
  Real_ptr m_in2 = nullptr;)

RAJAPERF_GB300_KERNEL(MULADDSUB,
 private:
  Real_ptr m_out1 = nullptr;
  Real_ptr m_out2 = nullptr;
  Real_ptr m_out3 = nullptr;
  Real_ptr m_in1 = nullptr;
  Real_ptr m_in2 = nullptr;)

}  // namespace basic
}  // namespace rajaperf
