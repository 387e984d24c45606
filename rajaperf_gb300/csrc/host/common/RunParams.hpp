// Run parameters parsed from the command line.
//
// Mirrors the suite's common/RunParams.hpp:31-408 for the options that shape
// a kernel run (--size/--sizefact, --repfact, --checkrun, --npasses, kernel,
// variant and tuning selection, output directory) and adds the options the
// GB300 path needs: input mode and seed, a Polybench time-step override, a
// per-kernel size map, a tuning-table file and graph batching.
#pragma once

#include "RAJAPerfSuite.hpp"

#include <map>
#include <set>
#include <string>
#include <vector>

namespace rajaperf {

class RunParams {
 public:
  enum InputOpt { InfoRequest, DryRun, CheckRun, PerfRun, BadInput, Undefined };
  enum SizeMeaning { Unset, Factor, Direct };
  // Array contents: the suite's deterministic formulas, or seeded uniform
  // values in [init_lo, init_hi).
  enum InitMode { InitReference, InitUniform };

  RunParams() = default;
  RunParams(int argc, const char* const* argv);

  InputOpt getInputState() const { return input_state; }
  SizeMeaning getSizeMeaning() const { return size_meaning; }
  double getSize() const { return size; }
  double getSizeFactor() const { return size_factor; }
  double getRepFactor() const { return rep_fact; }
  int getCheckRunReps() const { return checkrun_reps; }
  int getNumPasses() const { return npasses; }
  bool showProgress() const { return show_progress; }
  bool getDisableWarmup() const { return disable_warmup; }
  bool graphBatch() const { return graph_batch; }
  int getGraphBatchReps() const { return graph_batch_reps; }

  InitMode getInitMode() const { return init_mode; }
  unsigned long long getSeed() const { return seed; }
  double getInitLo() const { return init_lo; }
  double getInitHi() const { return init_hi; }

  // Limit of the bounded device-side waits (b200_tune.wait_limit_us; 0 =
  // library default) and the test option that makes a lookback wait run out.
  int getWaitLimitUs() const { return wait_limit_us; }
  // --host-data: the kernels' arrays live in pinned host memory (the suite's
  // CudaPinned data space) and every rep moves its data across the host link.
  bool getHostData() const { return host_data; }
  // Reports: npasses combiners of the timing/speedup CSVs (the suite's
  // --npasses-combiners, default Average), the speedup reference variant
  // (--refvar; none by default) and the FOM tolerance (--pass-fail-tol).
  const std::vector<std::string>& getNpassesCombiners() const { return npasses_combiners; }
  const std::string& getReferenceVariant() const { return reference_variant; }
  double getPFTolerance() const { return pf_tolerance; }
  long getInjectLookbackStall() const { return inject_lookback_stall; }

  // -1 when the kernel's own time-step count applies.
  long getPolybenchTsteps() const { return polybench_tsteps; }

  // HISTOGRAM / MULTI_REDUCE bins (RunParams.hpp:107-135 of the suite).
  enum struct BinAssignmentAlgorithm : int { Random, RunsRandomSizes, RunsEvenSizes, Single };
  long getMultiReduceNumBins() const { return multi_reduce_num_bins; }
  // HALO_PACKING halo width and variable count (suite defaults 1 and 3).
  long getHaloWidth() const { return halo_width; }
  long getHaloNumVars() const { return halo_num_vars; }
  BinAssignmentAlgorithm getMultiReduceBinAssignmentAlgorithm() const {
    return multi_reduce_bin_assignment;
  }

  // Per-kernel target size from --size-map, or -1.
  double getKernelSize(KernelID kid) const;

  const std::string& getTuningTableFile() const { return tuning_table_file; }
  const std::string& getAutotuneFile() const { return autotune_file; }
  const std::string& getOutputDirName() const { return outdir; }
  const std::string& getOutputFilePrefix() const { return outfile_prefix; }

  const std::vector<KernelID>& getKernelIDsToRun() const { return run_kernels; }
  const std::set<VariantID>& getVariantIDsToRun() const { return run_variants; }
  const std::vector<std::string>& getTuningInput() const { return tuning_input; }
  const std::vector<std::string>& getExcludeTuningInput() const {
    return exclude_tuning_input;
  }
  const std::string& getErrorMessage() const { return error_message; }

  void print(std::ostream& os) const;
  static std::string usage();

 private:
  void fail(const std::string& msg);

  InputOpt input_state = Undefined;
  SizeMeaning size_meaning = Unset;
  double size = 0.0;
  double size_factor = 1.0;
  double rep_fact = 1.0;
  int checkrun_reps = 1;
  int npasses = 1;
  bool show_progress = false;
  bool disable_warmup = false;
  bool graph_batch = false;
  int graph_batch_reps = -1;

  InitMode init_mode = InitReference;
  unsigned long long seed = 4793ULL;
  double init_lo = 0.5;
  double init_hi = 1.5;
  long polybench_tsteps = -1;
  int wait_limit_us = 0;
  bool host_data = false;
  std::vector<std::string> npasses_combiners;
  std::string reference_variant;
  double pf_tolerance = 0.1;
  long inject_lookback_stall = 0;
  long multi_reduce_num_bins = 10;
  long halo_width = 1;
  long halo_num_vars = 3;
  BinAssignmentAlgorithm multi_reduce_bin_assignment = BinAssignmentAlgorithm::RunsRandomSizes;

  std::map<KernelID, double> size_map;
  std::string tuning_table_file;
  std::string autotune_file;
  std::string outdir = ".";
  std::string outfile_prefix = "RAJAPerf";

  std::vector<KernelID> run_kernels;
  std::set<VariantID> run_variants;
  std::vector<std::string> tuning_input;
  std::vector<std::string> exclude_tuning_input;
  std::string error_message;
};

}  // namespace rajaperf
