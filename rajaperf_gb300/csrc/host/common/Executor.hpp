// Suite executor for the Base_GB300 variant.
//
// Same five steps as the suite's driver (RAJAPerfSuiteDriver.cpp:36-49 and
// common/Executor.hpp:45-51): setupSuite, reportRunSummary, runSuite,
// outputRunData.  runSuite runs every selected kernel x tuning for npasses
// (Executor.cpp:645-724).  outputRunData writes the suite's reports
// (Reports.hpp: timing and speedup CSVs per npasses combiner, checksum
// report, FOM report, kernel details) plus a roofline JSON with achieved
// GB/s and GFLOP/s per kernel and tuning.
//
// Graph batching (--graph-batch): the rep loops of all selected kernels are
// captured together into one CUDA graph and timed against the same work
// issued as individual launches.
#pragma once

#include "Autotuner.hpp"
#include "KernelBase.hpp"
#include "Reports.hpp"
#include "RunParams.hpp"

#include <iosfwd>
#include <memory>
#include <string>
#include <vector>

namespace rajaperf {

struct RunResult {
  std::string kernel;
  std::string variant;
  std::string tuning;
  long double checksum = 0.0L;
  double min_time = 0.0;  // seconds for the whole rep loop, min over passes
  double avg_time = 0.0;
  double max_time = 0.0;
  long long reps = 0;
  long long actual_size = 0;
  long long its_per_rep = 0;
  long long kernels_per_rep = 0;
  long long bytes_per_rep = 0;
  long long flops_per_rep = 0;
  long long h2d_bytes_per_rep = 0;  // --host-data: bytes crossing the host link
  long long d2h_bytes_per_rep = 0;
  int passes = 0;
  std::string error;  // empty when the run succeeded
};

struct GraphBatchResult {
  int kernels = 0;
  long long reps = 0;
  long long launches_per_rep = 0;  // library launches of one rep of the group
  double launch_time = 0.0;        // seconds, individual launches
  double graph_serial_time = 0.0;  // seconds, one graph, all reps in one chain
  double graph_time = 0.0;         // seconds, one graph, one branch per kernel
  std::string error;
};

class Executor {
 public:
  Executor(int argc, const char* const* argv);
  ~Executor();

  const RunParams& getRunParams() const { return run_params; }
  bool ok() const;

  void setupSuite();
  void reportRunSummary(std::ostream& os) const;
  void runSuite();
  void outputRunData();

  const std::vector<RunResult>& results() const { return results_; }
  const GraphBatchResult& graphBatchResult() const { return batch_; }
  const std::vector<AutotuneRecord>& autotuneRecords() const { return autotune_; }

 private:
  void runAutotune();
  void runGraphBatch();
  void collectResults();
  reports::ReportData reportData() const;
  void writeRooflineJSON(const std::string& fname) const;

  RunParams run_params;
  std::vector<std::unique_ptr<KernelBase>> kernels_;
  std::vector<std::vector<size_t>> tunings_;  // per kernel, tuning indices to run
  std::vector<std::string> tuning_names_;     // union, in first-seen order
  std::vector<RunResult> results_;
  std::vector<std::string> errors_;           // per (kernel,tuning) run errors
  GraphBatchResult batch_;
  std::vector<AutotuneRecord> autotune_;
};

}  // namespace rajaperf
