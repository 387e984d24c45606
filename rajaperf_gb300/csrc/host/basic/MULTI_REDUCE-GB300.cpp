// Basic_MULTI_REDUCE: values[bins[i]] += data[i].  Follows the suite's
// basic/MULTI_REDUCE.cpp:24-153: num_bins and the bin layout from the run
// parameters, data from rand(), values reset to values_init every rep,
// checksum over the final values.
#include "Basic.hpp"

namespace rajaperf {
namespace basic {

MULTI_REDUCE::MULTI_REDUCE(const RunParams& params)
    : KernelBase(rajaperf::Basic_MULTI_REDUCE, params) {
  setDefaultProblemSize(1000000);
  setDefaultReps(50);
  setActualProblemSize(getTargetProblemSize());
  m_num_bins = params.getMultiReduceNumBins();
  setItsPerRep(getActualProblemSize());
  setKernelsPerRep(1);
  setBytesReadPerRep(1 * sizeof(Real_type) * m_num_bins +
                     1 * sizeof(Real_type) * getActualProblemSize() +
                     1 * sizeof(Index_type) * getActualProblemSize());
  setBytesWrittenPerRep(1 * sizeof(Real_type) * m_num_bins);
  setBytesAtomicModifyWrittenPerRep(0);
  setFLOPsPerRep(1 * getActualProblemSize());
  setComplexity(Complexity::N);
  setUsesFeature(Forall);
  setUsesFeature(Atomic);
  setVariantDefined(Base_GB300);
}

void MULTI_REDUCE::setUp(VariantID vid, size_t) {
  const Index_type n = getActualProblemSize();
  allocData(m_bins, n, vid);
  allocAndInitDataRandValue(m_data, n, vid);
  const std::vector<Index_type> bins =
      hostBinAssignment(n, m_num_bins, run_params.getMultiReduceBinAssignmentAlgorithm());
  copyToDevice(m_bins, bins.data(), n * sizeof(Index_type));
  allocData(m_values_init, m_num_bins, vid);
  allocData(m_values, m_num_bins, vid);
  zeroDeviceBytes(m_values_init, m_num_bins * sizeof(Real_type));
  zeroDeviceBytes(m_values, m_num_bins * sizeof(Real_type));
  m_values_final.assign(m_num_bins, 0.0);
  m_ws_bytes = b200_multi_reduce_workspace_bytes(n, m_num_bins);
  m_ws = allocDeviceBytes(m_ws_bytes);
  zeroDeviceBytes(m_ws, m_ws_bytes);
}

KernelBase::RepBody MULTI_REDUCE::makeRepBody(size_t tune_idx) {
  const b200_tune tn = getTune(tune_idx);
  const Index_type n = getActualProblemSize();
  return [=](b200_stream_t s) {
    checkB200(b200_basic_multi_reduce(m_bins, m_data, n, m_num_bins, m_values_init, m_values,
                                      m_ws, m_ws_bytes, &tn, s),
              "b200_basic_multi_reduce");
  };
}

void MULTI_REDUCE::finishRun(size_t) {
  copyToHost(m_values_final.data(), m_values, m_num_bins * sizeof(Real_type));
}

void MULTI_REDUCE::updateChecksum(VariantID vid, size_t tune_idx) {
  checksum[vid][tune_idx] += calcChecksumHost(m_values_final.data(), m_num_bins, 1.0);
}

void MULTI_REDUCE::tearDown(VariantID vid, size_t) {
  deallocData(m_bins, vid);
  deallocData(m_data, vid);
  deallocData(m_values_init, vid);
  deallocData(m_values, vid);
  deallocDeviceBytes(m_ws);
  m_ws = nullptr;
  m_values_final.clear();
}

}  // namespace basic
}  // namespace rajaperf
