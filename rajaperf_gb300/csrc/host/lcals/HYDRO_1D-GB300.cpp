// Lcals_HYDRO_1D.  Follows the suite's lcals/HYDRO_1D.cpp:24-87.
#include "Lcals.hpp"

namespace rajaperf {
namespace lcals {

HYDRO_1D::HYDRO_1D(const RunParams& params) : KernelBase(rajaperf::Lcals_HYDRO_1D, params) {
  setDefaultProblemSize(1000000);
  setDefaultReps(1000);
  setActualProblemSize(getTargetProblemSize());
  m_array_length = getActualProblemSize() + 12;
  setItsPerRep(getActualProblemSize());
  setKernelsPerRep(1);
  setBytesReadPerRep(1 * sizeof(Real_type) * getActualProblemSize() +
                     1 * sizeof(Real_type) * (getActualProblemSize() + 1));
  setBytesWrittenPerRep(1 * sizeof(Real_type) * getActualProblemSize());
  setBytesAtomicModifyWrittenPerRep(0);
  setFLOPsPerRep(5 * getActualProblemSize());
  checksum_scale_factor = 0.001 * (static_cast<Checksum_type>(getDefaultProblemSize()) /
                                   getActualProblemSize());
  setComplexity(Complexity::N);
  setUsesFeature(Forall);
  setVariantDefined(Base_GB300);
}

void HYDRO_1D::setUp(VariantID vid, size_t) {
  allocAndInitDataConst(m_x, m_array_length, 0.0, vid);
  allocAndInitData(m_y, m_array_length, vid);
  allocAndInitData(m_z, m_array_length, vid);
  initData(m_q, vid);
  initData(m_r, vid);
  initData(m_t, vid);
}

KernelBase::RepBody HYDRO_1D::makeRepBody(size_t tune_idx) {
  const b200_tune tn = getTune(tune_idx);
  const Index_type n = getActualProblemSize();
  return [=](b200_stream_t s) {
    checkB200(b200_lcals_hydro_1d(m_x, m_y, m_z, m_q, m_r, m_t, n, &tn, s),
              "b200_lcals_hydro_1d");
  };
}

void HYDRO_1D::updateChecksum(VariantID vid, size_t tune_idx) {
  checksum[vid][tune_idx] +=
      calcChecksum(m_x, getActualProblemSize(), checksum_scale_factor, vid);
}

void HYDRO_1D::tearDown(VariantID vid, size_t) {
  deallocData(m_x, vid);
  deallocData(m_y, vid);
  deallocData(m_z, vid);
}

}  // namespace lcals
}  // namespace rajaperf
