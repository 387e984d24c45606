// Declaration helper for Base_GB300 kernel classes: every kernel overrides
// the same four hooks; kernels that need the untimed before/after-rep-loop
// hooks declare them in their member list.
#pragma once

#include "KernelBase.hpp"

#define RAJAPERF_GB300_KERNEL(NAME, ...)                                   \
  class NAME : public KernelBase {                                         \
   public:                                                                 \
    explicit NAME(const RunParams& params);                                \
    void setUp(VariantID vid, size_t tune_idx) override;                   \
    void updateChecksum(VariantID vid, size_t tune_idx) override;          \
    void tearDown(VariantID vid, size_t tune_idx) override;                \
    RepBody makeRepBody(size_t tune_idx) override;                         \
    __VA_ARGS__                                                            \
  };
