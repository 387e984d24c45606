// Algorithm group kernels (suite src/algorithm): SCAN, REDUCE_SUM, MEMSET,
// MEMCPY and HISTOGRAM.
#pragma once

#include "common/KernelDecl.hpp"

#include <vector>

namespace rajaperf {
namespace algorithm {

// SCAN tunings: the FP64 scan of the suite ("default", "graph") and the int64
// form ("int64", "int64_graph"): values uniform in [0, 100) from the seed,
// exact prefix sums.
RAJAPERF_GB300_KERNEL(SCAN,
 public:
  void setGB300TuningDefinitions(VariantID vid) override;
  void prepareRun(size_t tune_idx) override;
  void finishRun(size_t tune_idx) override;
 private:
  bool isInt64(size_t tune_idx) const;
  Real_ptr m_x = nullptr, m_y = nullptr;
  int64_t* m_xi = nullptr;
  int64_t* m_yi = nullptr;
  void* m_ws = nullptr;
  size_t m_ws_bytes = 0;)

RAJAPERF_GB300_KERNEL(REDUCE_SUM,
 public:
  void finishRun(size_t tune_idx) override;
 private:
  Real_ptr m_x = nullptr;
  Real_type m_sum_init = 0.0, m_sum = 0.0;
  Real_ptr m_dsum = nullptr;
  void* m_ws = nullptr;
  size_t m_ws_bytes = 0;)

RAJAPERF_GB300_KERNEL(MEMSET,
 private:
  Real_ptr m_x = nullptr;
  Real_type m_val = 0.0;)

RAJAPERF_GB300_KERNEL(MEMCPY,
 private:
  Real_ptr m_x = nullptr;
  Real_ptr m_y = nullptr;)

RAJAPERF_GB300_KERNEL(HISTOGRAM,
 public:
  void finishRun(size_t tune_idx) override;
 private:
  Index_type m_num_bins = 0;
  Index_type* m_bins = nullptr;
  unsigned long long* m_counts_init = nullptr;  // device copies of the suite's vectors
  unsigned long long* m_counts = nullptr;
  std::vector<unsigned long long> m_counts_final;)

}  // namespace algorithm
}  // namespace rajaperf
