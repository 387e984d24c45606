// Algorithm_MEMSET (x[i] = val) and Algorithm_MEMCPY (y[i] = x[i]).  Follow
// the suite's algorithm/MEMSET.cpp:22-80 and algorithm/MEMCPY.cpp:22-80.
#include "Algorithm.hpp"

namespace rajaperf {
namespace algorithm {

MEMSET::MEMSET(const RunParams& params) : KernelBase(rajaperf::Algorithm_MEMSET, params) {
  setDefaultProblemSize(1000000);
  setDefaultReps(100);
  setActualProblemSize(getTargetProblemSize());
  setItsPerRep(getActualProblemSize());
  setKernelsPerRep(1);
  setBytesReadPerRep(0);
  setBytesWrittenPerRep(1 * sizeof(Real_type) * getActualProblemSize());
  setBytesAtomicModifyWrittenPerRep(0);
  setFLOPsPerRep(0);
  setComplexity(Complexity::N);
  setUsesFeature(Forall);
  setVariantDefined(Base_GB300);
}

void MEMSET::setUp(VariantID vid, size_t) {
  allocAndInitDataConst(m_x, getActualProblemSize(), -1.234567e89, vid);
  m_val = 0.0;
}

KernelBase::RepBody MEMSET::makeRepBody(size_t tune_idx) {
  const b200_tune tn = getTune(tune_idx);
  const Index_type n = getActualProblemSize();
  return [=](b200_stream_t s) {
    checkB200(b200_algorithm_memset(m_x, m_val, n, &tn, s), "b200_algorithm_memset");
  };
}

void MEMSET::updateChecksum(VariantID vid, size_t tune_idx) {
  checksum[vid][tune_idx] += calcChecksum(m_x, getActualProblemSize(), vid);
}

void MEMSET::tearDown(VariantID vid, size_t) { deallocData(m_x, vid); }

MEMCPY::MEMCPY(const RunParams& params) : KernelBase(rajaperf::Algorithm_MEMCPY, params) {
  setDefaultProblemSize(1000000);
  setDefaultReps(100);
  setActualProblemSize(getTargetProblemSize());
  setItsPerRep(getActualProblemSize());
  setKernelsPerRep(1);
  setBytesReadPerRep(1 * sizeof(Real_type) * getActualProblemSize());
  setBytesWrittenPerRep(1 * sizeof(Real_type) * getActualProblemSize());
  setBytesAtomicModifyWrittenPerRep(0);
  setFLOPsPerRep(0);
  setComplexity(Complexity::N);
  setUsesFeature(Forall);
  setVariantDefined(Base_GB300);
}

void MEMCPY::setUp(VariantID vid, size_t) {
  allocAndInitDataConst(m_x, getActualProblemSize(), 0.0, vid);
  allocAndInitDataConst(m_y, getActualProblemSize(), -1.234567e89, vid);
}

KernelBase::RepBody MEMCPY::makeRepBody(size_t tune_idx) {
  const b200_tune tn = getTune(tune_idx);
  const Index_type n = getActualProblemSize();
  return [=](b200_stream_t s) {
    checkB200(b200_algorithm_memcpy(m_x, m_y, n, &tn, s), "b200_algorithm_memcpy");
  };
}

void MEMCPY::updateChecksum(VariantID vid, size_t tune_idx) {
  checksum[vid][tune_idx] += calcChecksum(m_y, getActualProblemSize(), vid);
}

void MEMCPY::tearDown(VariantID vid, size_t) {
  deallocData(m_x, vid);
  deallocData(m_y, vid);
}

}  // namespace algorithm
}  // namespace rajaperf
