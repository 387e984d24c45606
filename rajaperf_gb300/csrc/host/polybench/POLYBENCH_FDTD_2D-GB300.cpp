// Polybench_FDTD_2D.  Follows the suite's POLYBENCH_FDTD_2D.cpp:30-116:
// nx = ny = sqrt(size) + 1 + sqrt(2) - 1, 40 time steps (--polybench_tsteps
// overrides), state carried across reps, checksum over hz.
#include "Polybench.hpp"

#include <algorithm>
#include <cmath>

namespace rajaperf {
namespace polybench {

POLYBENCH_FDTD_2D::POLYBENCH_FDTD_2D(const RunParams& params)
    : KernelBase(rajaperf::Polybench_FDTD_2D, params) {
  Index_type nx_default = 1000, ny_default = 1000;
  setDefaultProblemSize(std::max((nx_default - 1) * ny_default, nx_default * (ny_default - 1)));
  setDefaultReps(8);
  m_nx = static_cast<Index_type>(std::sqrt(getTargetProblemSize()) + 1 + std::sqrt(2) - 1);
  m_ny = m_nx;
  m_tsteps = params.getPolybenchTsteps() >= 0 ? params.getPolybenchTsteps() : 40;
  setActualProblemSize(std::max((m_nx - 1) * m_ny, m_nx * (m_ny - 1)));
  setItsPerRep(m_tsteps * (m_ny + (m_nx - 1) * m_ny + m_nx * (m_ny - 1) +
                           (m_nx - 1) * (m_ny - 1)));
  setKernelsPerRep(m_tsteps * 4);
  setBytesReadPerRep((1 * sizeof(Real_type) + 1 * sizeof(Real_type) * (m_nx - 1) * m_ny +
                      1 * sizeof(Real_type) * m_nx * m_ny +
                      1 * sizeof(Real_type) * m_nx * (m_ny - 1) +
                      1 * sizeof(Real_type) * m_nx * m_ny +
                      1 * sizeof(Real_type) * (m_nx - 1) * (m_ny - 1) +
                      1 * sizeof(Real_type) * (m_nx - 1) * m_ny +
                      1 * sizeof(Real_type) * m_nx * (m_ny - 1)) * m_tsteps);
  setBytesWrittenPerRep((1 * sizeof(Real_type) * m_ny +
                         1 * sizeof(Real_type) * (m_nx - 1) * m_ny +
                         1 * sizeof(Real_type) * m_nx * (m_ny - 1) +
                         1 * sizeof(Real_type) * (m_nx - 1) * (m_ny - 1)) * m_tsteps);
  setBytesAtomicModifyWrittenPerRep(0);
  setFLOPsPerRep(m_tsteps * (0 * m_ny + 3 * (m_nx - 1) * m_ny + 3 * m_nx * (m_ny - 1) +
                             5 * (m_nx - 1) * (m_ny - 1)));
  checksum_scale_factor = 0.001 * (static_cast<Checksum_type>(getDefaultProblemSize()) /
                                   getActualProblemSize());
  setComplexity(Complexity::N);
  setUsesFeature(Kernel);
  b200_tune two_launch{};
  two_launch.algo = 1;  // BODY1-3 and BODY4 as two launches per time step
  addTuning("two_launch", two_launch, false);
  setVariantDefined(Base_GB300);
}

void POLYBENCH_FDTD_2D::setUp(VariantID vid, size_t) {
  allocAndInitDataConst(m_hz, m_nx * m_ny, 0.0, vid);
  allocAndInitData(m_ex, m_nx * m_ny, vid);
  allocAndInitData(m_ey, m_nx * m_ny, vid);
  allocAndInitData(m_fict, m_tsteps, vid);
  m_ws_bytes = b200_fdtd_2d_workspace_bytes(m_nx, m_ny);
  m_ws = m_ws_bytes ? allocDeviceBytes(m_ws_bytes) : nullptr;
  // --host-data: all time steps of a rep run on staged copies of the fields
  stageArray(m_ex, m_nx * m_ny, kIn | kOut);
  stageArray(m_ey, m_nx * m_ny, kIn | kOut);
  stageArray(m_hz, m_nx * m_ny, kIn | kOut);
  stageArray(m_fict, m_tsteps, kIn);
}

KernelBase::RepBody POLYBENCH_FDTD_2D::makeRepBody(size_t tune_idx) {
  const b200_tune tn = getTune(tune_idx);
  return [=](b200_stream_t s) {
    checkB200(b200_polybench_fdtd_2d_ws(m_ex, m_ey, m_hz, m_fict, m_nx, m_ny, m_tsteps, m_ws,
                                        m_ws_bytes, &tn, s),
              "b200_polybench_fdtd_2d_ws");
  };
}

void POLYBENCH_FDTD_2D::updateChecksum(VariantID vid, size_t tune_idx) {
  checksum[vid][tune_idx] += calcChecksum(m_hz, m_nx * m_ny, checksum_scale_factor, vid);
}

void POLYBENCH_FDTD_2D::tearDown(VariantID vid, size_t) {
  deallocData(m_fict, vid);
  deallocData(m_ex, vid);
  deallocData(m_ey, vid);
  deallocData(m_hz, vid);
  deallocDeviceBytes(m_ws);
  m_ws = nullptr;
}

}  // namespace polybench
}  // namespace rajaperf
