// Stream group kernels (suite src/stream/*.hpp): COPY, MUL, ADD, TRIAD, DOT.
#pragma once

#include "common/KernelBase.hpp"

namespace rajaperf {
namespace stream {

class COPY : public KernelBase {
 public:
  explicit COPY(const RunParams& params);
  void setUp(VariantID vid, size_t tune_idx) override;
  void updateChecksum(VariantID vid, size_t tune_idx) override;
  void tearDown(VariantID vid, size_t tune_idx) override;
  RepBody makeRepBody(size_t tune_idx) override;
 private:
  Real_ptr m_a = nullptr;
  Real_ptr m_c = nullptr;
};

class MUL : public KernelBase {
 public:
  explicit MUL(const RunParams& params);
  void setUp(VariantID vid, size_t tune_idx) override;
  void updateChecksum(VariantID vid, size_t tune_idx) override;
  void tearDown(VariantID vid, size_t tune_idx) override;
  RepBody makeRepBody(size_t tune_idx) override;
 private:
  Real_ptr m_b = nullptr;
  Real_ptr m_c = nullptr;
  Real_type m_alpha = 0.0;
};

class ADD : public KernelBase {
 public:
  explicit ADD(const RunParams& params);
  void setUp(VariantID vid, size_t tune_idx) override;
  void updateChecksum(VariantID vid, size_t tune_idx) override;
  void tearDown(VariantID vid, size_t tune_idx) override;
  RepBody makeRepBody(size_t tune_idx) override;
 private:
  Real_ptr m_a = nullptr;
  Real_ptr m_b = nullptr;
  Real_ptr m_c = nullptr;
};

class TRIAD : public KernelBase {
 public:
  explicit TRIAD(const RunParams& params);
  void setUp(VariantID vid, size_t tune_idx) override;
  void updateChecksum(VariantID vid, size_t tune_idx) override;
  void tearDown(VariantID vid, size_t tune_idx) override;
  RepBody makeRepBody(size_t tune_idx) override;
 private:
  Real_ptr m_a = nullptr;
  Real_ptr m_b = nullptr;
  Real_ptr m_c = nullptr;
  Real_type m_alpha = 0.0;
};

class DOT : public KernelBase {
 public:
  explicit DOT(const RunParams& params);
  void finishRun(size_t tune_idx) override;
  void setUp(VariantID vid, size_t tune_idx) override;
  void updateChecksum(VariantID vid, size_t tune_idx) override;
  void tearDown(VariantID vid, size_t tune_idx) override;
  RepBody makeRepBody(size_t tune_idx) override;
 private:
  Real_ptr m_a = nullptr;
  Real_ptr m_b = nullptr;
  Real_type m_dot = 0.0;
  Real_type m_dot_init = 0.0;
  Real_ptr m_ddot = nullptr;   // device accumulator for m_dot
  void* m_ws = nullptr;        // reduction workspace
  size_t m_ws_bytes = 0;
};

}  // namespace stream
}  // namespace rajaperf
