// Algorithm_HISTOGRAM: counts[bins[i]] += 1.  Follows the suite's
// algorithm/HISTOGRAM.cpp:24-149: num_bins and the bin layout from the run
// parameters, counts reset to counts_init every rep, checksum over the final
// counts.
#include "Algorithm.hpp"

namespace rajaperf {
namespace algorithm {

HISTOGRAM::HISTOGRAM(const RunParams& params)
    : KernelBase(rajaperf::Algorithm_HISTOGRAM, params) {
  setDefaultProblemSize(1000000);
  setDefaultReps(50);
  setActualProblemSize(getTargetProblemSize());
  m_num_bins = params.getMultiReduceNumBins();
  setItsPerRep(getActualProblemSize());
  setKernelsPerRep(1);
  setBytesReadPerRep(1 * sizeof(unsigned long long) * m_num_bins +
                     1 * sizeof(Index_type) * getActualProblemSize());
  setBytesWrittenPerRep(1 * sizeof(unsigned long long) * m_num_bins);
  setBytesAtomicModifyWrittenPerRep(0);
  setFLOPsPerRep(1 * getActualProblemSize());
  setComplexity(Complexity::N);
  setUsesFeature(Forall);
  setUsesFeature(Atomic);
  setVariantDefined(Base_GB300);
}

void HISTOGRAM::setUp(VariantID vid, size_t) {
  const Index_type n = getActualProblemSize();
  allocData(m_bins, n, vid);
  const std::vector<Index_type> bins =
      hostBinAssignment(n, m_num_bins, run_params.getMultiReduceBinAssignmentAlgorithm());
  copyToDevice(m_bins, bins.data(), n * sizeof(Index_type));
  allocData(m_counts_init, m_num_bins, vid);
  allocData(m_counts, m_num_bins, vid);
  zeroDeviceBytes(m_counts_init, m_num_bins * sizeof(unsigned long long));
  zeroDeviceBytes(m_counts, m_num_bins * sizeof(unsigned long long));
  m_counts_final.assign(m_num_bins, 0ull);
}

KernelBase::RepBody HISTOGRAM::makeRepBody(size_t tune_idx) {
  const b200_tune tn = getTune(tune_idx);
  const Index_type n = getActualProblemSize();
  return [=](b200_stream_t s) {
    checkB200(b200_algorithm_histogram(m_bins, n, m_num_bins, m_counts_init, m_counts, &tn, s),
              "b200_algorithm_histogram");
  };
}

void HISTOGRAM::finishRun(size_t) {
  copyToHost(m_counts_final.data(), m_counts, m_num_bins * sizeof(unsigned long long));
}

void HISTOGRAM::updateChecksum(VariantID vid, size_t tune_idx) {
  checksum[vid][tune_idx] += calcChecksumHost(m_counts_final.data(), m_num_bins, 1.0);
}

void HISTOGRAM::tearDown(VariantID vid, size_t) {
  deallocData(m_bins, vid);
  deallocData(m_counts_init, vid);
  deallocData(m_counts, vid);
  m_counts_final.clear();
}

}  // namespace algorithm
}  // namespace rajaperf
