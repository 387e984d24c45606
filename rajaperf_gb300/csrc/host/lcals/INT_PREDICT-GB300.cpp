// Lcals_INT_PREDICT.  Follows the suite's lcals/INT_PREDICT.cpp:24-93; the
// checksum subtracts the initial value from px[0..N) first (:80-88), done
// here on the host copy.
#include "Lcals.hpp"

#include <vector>

namespace rajaperf {
namespace lcals {

INT_PREDICT::INT_PREDICT(const RunParams& params)
    : KernelBase(rajaperf::Lcals_INT_PREDICT, params) {
  setDefaultProblemSize(1000000);
  setDefaultReps(400);
  setActualProblemSize(getTargetProblemSize());
  setItsPerRep(getActualProblemSize());
  setKernelsPerRep(1);
  setBytesReadPerRep(10 * sizeof(Real_type) * getActualProblemSize());
  setBytesWrittenPerRep(1 * sizeof(Real_type) * getActualProblemSize());
  setBytesAtomicModifyWrittenPerRep(0);
  setFLOPsPerRep(17 * getActualProblemSize());
  setComplexity(Complexity::N);
  setUsesFeature(Forall);
  setVariantDefined(Base_GB300);
}

void INT_PREDICT::setUp(VariantID vid, size_t) {
  m_array_length = getActualProblemSize() * 13;
  m_offset = getActualProblemSize();
  m_px_initval = 1.0;
  allocAndInitDataConst(m_px, m_array_length, m_px_initval, vid);
  initData(m_dm22, vid);
  initData(m_dm23, vid);
  initData(m_dm24, vid);
  initData(m_dm25, vid);
  initData(m_dm26, vid);
  initData(m_dm27, vid);
  initData(m_dm28, vid);
  initData(m_c0, vid);
}

KernelBase::RepBody INT_PREDICT::makeRepBody(size_t tune_idx) {
  const b200_tune tn = getTune(tune_idx);
  const Index_type n = getActualProblemSize();
  return [=](b200_stream_t s) {
    checkB200(b200_lcals_int_predict(m_px, m_dm22, m_dm23, m_dm24, m_dm25, m_dm26, m_dm27,
                                     m_dm28, m_c0, n, &tn, s),
              "b200_lcals_int_predict");
  };
}

void INT_PREDICT::updateChecksum(VariantID vid, size_t tune_idx) {
  const Index_type n = getActualProblemSize();
  std::vector<Real_type> h(n);
  copyToHost(h.data(), m_px, n * sizeof(Real_type));
  for (Index_type i = 0; i < n; ++i) h[i] -= m_px_initval;
  checksum[vid][tune_idx] += calcChecksumHost(h.data(), n, 1.0);
}

void INT_PREDICT::tearDown(VariantID vid, size_t) { deallocData(m_px, vid); }

}  // namespace lcals
}  // namespace rajaperf
