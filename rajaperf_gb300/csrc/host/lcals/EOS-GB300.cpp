// Lcals_EOS.  Follows the suite's lcals/EOS.cpp:24-89.
#include "Lcals.hpp"

namespace rajaperf {
namespace lcals {

EOS::EOS(const RunParams& params) : KernelBase(rajaperf::Lcals_EOS, params) {
  setDefaultProblemSize(1000000);
  setDefaultReps(500);
  setActualProblemSize(getTargetProblemSize());
  m_array_length = getActualProblemSize() + 7;
  setItsPerRep(getActualProblemSize());
  setKernelsPerRep(1);
  setBytesReadPerRep(2 * sizeof(Real_type) * getActualProblemSize() +
                     1 * sizeof(Real_type) * m_array_length);
  setBytesWrittenPerRep(1 * sizeof(Real_type) * getActualProblemSize());
  setBytesAtomicModifyWrittenPerRep(0);
  setFLOPsPerRep(16 * getActualProblemSize());
  checksum_scale_factor = 0.0001 * (static_cast<Checksum_type>(getDefaultProblemSize()) /
                                    getActualProblemSize());
  setComplexity(Complexity::N);
  setUsesFeature(Forall);
  setVariantDefined(Base_GB300);
}

void EOS::setUp(VariantID vid, size_t) {
  allocAndInitDataConst(m_x, m_array_length, 0.0, vid);
  allocAndInitData(m_y, m_array_length, vid);
  allocAndInitData(m_z, m_array_length, vid);
  allocAndInitData(m_u, m_array_length, vid);
  // --host-data: one streaming pass, on the host arrays directly
  hostArray(m_x, getActualProblemSize(), kOut);
  hostArray(m_y, getActualProblemSize(), kIn);
  hostArray(m_z, getActualProblemSize(), kIn);
  hostArray(m_u, m_array_length, kIn);
  initData(m_q, vid);
  initData(m_r, vid);
  initData(m_t, vid);
}

KernelBase::RepBody EOS::makeRepBody(size_t tune_idx) {
  const b200_tune tn = getTune(tune_idx);
  const Index_type n = getActualProblemSize();
  return [=](b200_stream_t s) {
    checkB200(b200_lcals_eos(m_x, m_y, m_z, m_u, m_q, m_r, m_t, n, &tn, s), "b200_lcals_eos");
  };
}

void EOS::updateChecksum(VariantID vid, size_t tune_idx) {
  checksum[vid][tune_idx] +=
      calcChecksum(m_x, getActualProblemSize(), checksum_scale_factor, vid);
}

void EOS::tearDown(VariantID vid, size_t) {
  deallocData(m_x, vid);
  deallocData(m_y, vid);
  deallocData(m_z, vid);
  deallocData(m_u, vid);
}

}  // namespace lcals
}  // namespace rajaperf
