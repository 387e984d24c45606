// Basic group kernels of the batched small-size suite (suite src/basic).
#pragma once

#include "common/KernelDecl.hpp"

#include <vector>

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

// INDEXLIST and INDEXLIST_3LOOP: the list of indices with x[i] < 0 and its
// length; both run b200_basic_indexlist (one pass).
RAJAPERF_GB300_KERNEL(INDEXLIST,
 public:
  void prepareRun(size_t tune_idx) override;
  void finishRun(size_t tune_idx) override;
 private:
  Real_ptr m_x = nullptr;
  Int_ptr m_list = nullptr;
  int64_t* m_dlen = nullptr;
  Index_type m_len = -1;
  void* m_ws = nullptr;
  size_t m_ws_bytes = 0;)

RAJAPERF_GB300_KERNEL(INDEXLIST_3LOOP,
 public:
  void prepareRun(size_t tune_idx) override;
  void finishRun(size_t tune_idx) override;
 private:
  Real_ptr m_x = nullptr;
  Int_ptr m_list = nullptr;
  int64_t* m_dlen = nullptr;
  Index_type m_len = -1;
  void* m_ws = nullptr;
  size_t m_ws_bytes = 0;)

RAJAPERF_GB300_KERNEL(MULTI_REDUCE,
 public:
  void finishRun(size_t tune_idx) override;
 private:
  Index_type m_num_bins = 0;
  Index_type* m_bins = nullptr;
  Real_ptr m_data = nullptr;
  Real_ptr m_values_init = nullptr;  // device copies of the suite's vectors
  Real_ptr m_values = nullptr;
  std::vector<Real_type> m_values_final;
  void* m_ws = nullptr;
  size_t m_ws_bytes = 0;)

}  // namespace basic
}  // namespace rajaperf
