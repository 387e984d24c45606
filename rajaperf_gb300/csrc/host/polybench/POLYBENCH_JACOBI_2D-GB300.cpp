// Polybench_JACOBI_2D.  Follows the suite's POLYBENCH_JACOBI_2D.cpp:26-94:
// N = sqrt(size) + 2 + sqrt(2) - 1, 40 time steps (--polybench_tsteps
// overrides), A/B restored from Ainit/Binit before the timed rep loop
// (POLYBENCH_JACOBI_2D.hpp:30-36), checksum over A and B.
#include "Polybench.hpp"

#include <cmath>

namespace rajaperf {
namespace polybench {

POLYBENCH_JACOBI_2D::POLYBENCH_JACOBI_2D(const RunParams& params)
    : KernelBase(rajaperf::Polybench_JACOBI_2D, params) {
  Index_type N_default = 1002;
  setDefaultProblemSize((N_default - 2) * (N_default - 2));
  setDefaultReps(50);
  m_N = static_cast<Index_type>(std::sqrt(getTargetProblemSize()) + 2 + std::sqrt(2) - 1);
  m_tsteps = params.getPolybenchTsteps() >= 0 ? params.getPolybenchTsteps() : 40;
  setActualProblemSize((m_N - 2) * (m_N - 2));
  setItsPerRep(m_tsteps * (2 * (m_N - 2) * (m_N - 2)));
  setKernelsPerRep(2);
  setBytesReadPerRep((1 * sizeof(Real_type) * (m_N * m_N - 4) +
                      1 * sizeof(Real_type) * (m_N * m_N - 4)) * m_tsteps);
  setBytesWrittenPerRep((1 * sizeof(Real_type) * (m_N - 2) * (m_N - 2) +
                         1 * sizeof(Real_type) * (m_N - 2) * (m_N - 2)) * m_tsteps);
  setBytesAtomicModifyWrittenPerRep(0);
  setFLOPsPerRep(m_tsteps * (5 * (m_N - 2) * (m_N - 2) + 5 * (m_N - 2) * (m_N - 2)));
  checksum_scale_factor = 0.0001 * (static_cast<Checksum_type>(getDefaultProblemSize()) /
                                    getActualProblemSize());
  setComplexity(Complexity::N);
  setUsesFeature(Kernel);
  setVariantDefined(Base_GB300);
}

void POLYBENCH_JACOBI_2D::setUp(VariantID vid, size_t) {
  allocAndInitData(m_Ainit, m_N * m_N, vid);
  allocAndInitData(m_Binit, m_N * m_N, vid);
  allocData(m_A, m_N * m_N, vid);
  allocData(m_B, m_N * m_N, vid);
  // --host-data: all time steps of a rep run on staged copies of A and B
  stageArray(m_A, m_N * m_N, kIn | kOut);
  stageArray(m_B, m_N * m_N, kIn | kOut);
}

void POLYBENCH_JACOBI_2D::prepareRun(size_t) {
  copyDeviceToDevice(m_A, m_Ainit, m_N * m_N * sizeof(Real_type));
  copyDeviceToDevice(m_B, m_Binit, m_N * m_N * sizeof(Real_type));
}

KernelBase::RepBody POLYBENCH_JACOBI_2D::makeRepBody(size_t tune_idx) {
  const b200_tune tn = getTune(tune_idx);
  return [=](b200_stream_t s) {
    checkB200(b200_polybench_jacobi_2d(m_A, m_B, m_N, m_tsteps, &tn, s),
              "b200_polybench_jacobi_2d");
  };
}

void POLYBENCH_JACOBI_2D::updateChecksum(VariantID vid, size_t tune_idx) {
  checksum[vid][tune_idx] += calcChecksum(m_A, m_N * m_N, checksum_scale_factor, vid);
  checksum[vid][tune_idx] += calcChecksum(m_B, m_N * m_N, checksum_scale_factor, vid);
}

void POLYBENCH_JACOBI_2D::tearDown(VariantID vid, size_t) {
  deallocData(m_A, vid);
  deallocData(m_B, vid);
  deallocData(m_Ainit, vid);
  deallocData(m_Binit, vid);
}

}  // namespace polybench
}  // namespace rajaperf
