#include "Executor.hpp"

#include "Autotuner.hpp"
#include "GraphRepRunner.hpp"
#include "Reports.hpp"
#include "TuningTable.hpp"

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <stdexcept>
#include <sys/stat.h>

namespace rajaperf {

Executor::Executor(int argc, const char* const* argv) : run_params(argc, argv) {}

Executor::~Executor() = default;

bool Executor::ok() const {
  return run_params.getInputState() != RunParams::BadInput &&
         run_params.getInputState() != RunParams::InfoRequest;
}

// Executor.cpp:246-370: instantiate the selected kernels and resolve which
// tunings run ("default" first, then the kernel's own order).
void Executor::setupSuite() {
  if (!ok()) return;
  if (!run_params.getTuningTableFile().empty()) {
    std::string err;
    if (!TuningTable::instance().load(run_params.getTuningTableFile(), &err)) {
      throw std::runtime_error(err);
    }
  }
  for (KernelID kid : run_params.getKernelIDsToRun()) {
    KernelBase* k = getKernelObject(kid, run_params);
    if (!k) continue;
    std::vector<size_t> tun;
    const auto& names = k->getVariantTuningNames(Base_GB300);
    const auto& want = run_params.getTuningInput();
    const auto& skip = run_params.getExcludeTuningInput();
    for (size_t t = 0; t < names.size(); ++t) {
      bool selected = want.empty() ||
                      std::find(want.begin(), want.end(), names[t]) != want.end();
      if (std::find(skip.begin(), skip.end(), names[t]) != skip.end()) selected = false;
      if (selected) {
        tun.push_back(t);
        if (std::find(tuning_names_.begin(), tuning_names_.end(), names[t]) ==
            tuning_names_.end())
          tuning_names_.push_back(names[t]);
      }
    }
    if (tun.empty()) {
      delete k;
      continue;
    }
    kernels_.emplace_back(k);
    tunings_.push_back(std::move(tun));
  }
}

void Executor::reportRunSummary(std::ostream& os) const {
  if (run_params.getInputState() == RunParams::InfoRequest) {
    os << RunParams::usage();
    return;
  }
  if (run_params.getInputState() == RunParams::BadInput) {
    os << "\nRAJA performance suite (Base_GB300) input error: "
       << run_params.getErrorMessage() << "\n" << RunParams::usage();
    return;
  }
  os << "\nRAJA performance suite, Base_GB300 variant\n";
  run_params.print(os);
  os << "Kernels (" << kernels_.size() << "):\n";
  for (size_t i = 0; i < kernels_.size(); ++i) {
    const KernelBase* k = kernels_[i].get();
    os << "  " << std::left << std::setw(24) << k->getName() << " size "
       << k->getActualProblemSize() << " reps " << k->getRunReps() << " tunings";
    for (size_t t : tunings_[i]) os << " " << k->getVariantTuningName(Base_GB300, t);
    os << "\n";
  }
}

void Executor::runSuite() {
  if (!ok() || run_params.getInputState() == RunParams::DryRun) return;
  checkCuda(cudaFree(nullptr), "cuda context");
  if (!run_params.getAutotuneFile().empty()) runAutotune();
  if (run_params.graphBatch()) {
    runGraphBatch();
    return;
  }
  // Warm-up: one rep of each selected kernel's default tuning, untimed in the
  // report (Executor.cpp:728-823 runs designated warm-up kernels instead).
  if (!run_params.getDisableWarmup()) {
    for (size_t i = 0; i < kernels_.size(); ++i) {
      std::unique_ptr<KernelBase> w(getKernelObject(kernels_[i]->getKernelID(), run_params));
      try {
        w->execute(Base_GB300, tunings_[i].front());
      } catch (const std::exception&) {
        // Errors are reported by the measured runs below.
      }
    }
  }
  errors_.assign(kernels_.size() * tuning_names_.size(), std::string());
  for (int pass = 0; pass < run_params.getNumPasses(); ++pass) {
    for (size_t i = 0; i < kernels_.size(); ++i) {
      KernelBase* k = kernels_[i].get();
      for (size_t t : tunings_[i]) {
        const std::string& tname = k->getVariantTuningName(Base_GB300, t);
        size_t col = std::find(tuning_names_.begin(), tuning_names_.end(), tname) -
                     tuning_names_.begin();
        try {
          k->execute(Base_GB300, t);
          if (run_params.showProgress()) {
            getCout() << "  " << k->getName() << " " << tname << " "
                      << std::setprecision(6) << k->getLastTime() << " s\n";
          }
        } catch (const std::exception& e) {
          errors_[i * tuning_names_.size() + col] = e.what();
          getCout() << "  " << k->getName() << " " << tname << " FAILED: "
                    << e.what() << "\n";
        }
      }
    }
  }
  collectResults();
}

void Executor::collectResults() {
  results_.clear();
  for (size_t i = 0; i < kernels_.size(); ++i) {
    KernelBase* k = kernels_[i].get();
    for (size_t t : tunings_[i]) {
      RunResult r;
      r.kernel = k->getName();
      r.variant = getVariantName(Base_GB300);
      r.tuning = k->getVariantTuningName(Base_GB300, t);
      size_t col = std::find(tuning_names_.begin(), tuning_names_.end(), r.tuning) -
                   tuning_names_.begin();
      r.error = errors_.empty() ? std::string()
                                : errors_[i * tuning_names_.size() + col];
      r.passes = k->getNumExec(Base_GB300, t);
      r.checksum = r.passes > 0 ? k->getChecksum(Base_GB300, t) / r.passes : 0.0L;
      r.min_time = r.passes > 0 ? k->getMinTime(Base_GB300, t) : 0.0;
      r.max_time = r.passes > 0 ? k->getMaxTime(Base_GB300, t) : 0.0;
      r.avg_time = r.passes > 0 ? k->getTotTime(Base_GB300, t) / r.passes : 0.0;
      r.reps = k->getRunReps();
      r.actual_size = k->getActualProblemSize();
      r.its_per_rep = k->getItsPerRep();
      r.kernels_per_rep = k->getKernelsPerRep();
      r.bytes_per_rep = k->getBytesPerRep();
      r.flops_per_rep = k->getFLOPsPerRep();
      r.h2d_bytes_per_rep = k->getH2DBytesPerRep();
      r.d2h_bytes_per_rep = k->getD2HBytesPerRep();
      results_.push_back(r);
    }
  }
}

// Measures launch shapes for the selected kernels (Autotuner.hpp), installs
// the winners ahead of any loaded tuning table and writes them out.
void Executor::runAutotune() {
  autotune_ = autotune(kernels_, tunings_);
  std::vector<TuningTable::Entry> entries;
  for (const AutotuneRecord& r : autotune_)
    entries.push_back(TuningTable::Entry{r.kernel, r.size, r.size, r.best});
  TuningTable::instance().prepend(entries);
  if (!writeAutotuneTable(autotune_, run_params.getAutotuneFile()))
    throw std::runtime_error("cannot write " + run_params.getAutotuneFile());
  if (run_params.showProgress()) {
    for (const AutotuneRecord& r : autotune_) {
      getCout() << "  autotune " << r.kernel << " size " << r.size << ": "
                << TuningTable::format(TuningTable::Entry{r.kernel, r.size, r.size, r.best})
                << " " << r.best_s * 1e6 << " us (default " << r.default_s * 1e6 << ")\n";
    }
  }
}

// The group's rep loops, once as individual library calls and once captured
// into a single CUDA graph.  Every kernel runs its first selected tuning's
// launch shape; checksums are taken after the graph run.
void Executor::runGraphBatch() {
  batch_ = GraphBatchResult{};
  std::vector<KernelBase::RepBody> bodies;
  std::vector<size_t> tune;
  long long reps = run_params.getGraphBatchReps();
  if (reps <= 0) reps = run_params.getInputState() == RunParams::CheckRun
                            ? run_params.getCheckRunReps() : 100;
  try {
    for (size_t i = 0; i < kernels_.size(); ++i) {
      KernelBase* k = kernels_[i].get();
      detail::resetDataInitCount();
      k->setUp(Base_GB300, tunings_[i].front());
      k->prepareRun(tunings_[i].front());
      bodies.push_back(k->makeRepBody(tunings_[i].front()));
      tune.push_back(tunings_[i].front());
    }
    int64_t launches0 = b200_launch_count();
    checkCuda(cudaDeviceSynchronize(), "sync");
    for (const auto& b : bodies) b(nullptr);  // untimed warm-up rep
    checkCuda(cudaDeviceSynchronize(), "sync");
    batch_.launches_per_rep = b200_launch_count() - launches0;

    auto t0 = std::chrono::steady_clock::now();
    for (long long r = 0; r < reps; ++r)
      for (const auto& b : bodies) b(nullptr);
    checkCuda(cudaDeviceSynchronize(), "sync");
    auto t1 = std::chrono::steady_clock::now();
    batch_.launch_time = std::chrono::duration<double>(t1 - t0).count();

    // one chain: every rep of every kernel in launch order
    {
      GraphRepRunner runner(reps);
      runner.capture(reps, [&](b200_stream_t s) {
        for (const auto& b : bodies) b(s);
      });
      checkCuda(cudaDeviceSynchronize(), "sync");
      auto g0 = std::chrono::steady_clock::now();
      runner.launch();
      runner.synchronize();
      auto g1 = std::chrono::steady_clock::now();
      batch_.graph_serial_time = std::chrono::duration<double>(g1 - g0).count();
    }
    // one branch per kernel: the kernels share no data, so only each
    // kernel's own reps stay ordered and the branches run concurrently
    {
      ParallelGraph graph(bodies, reps);
      checkCuda(cudaDeviceSynchronize(), "sync");
      auto g0 = std::chrono::steady_clock::now();
      graph.launch();
      graph.synchronize();
      auto g1 = std::chrono::steady_clock::now();
      batch_.graph_time = std::chrono::duration<double>(g1 - g0).count();
    }
    batch_.kernels = static_cast<int>(kernels_.size());
    batch_.reps = reps;
  } catch (const std::exception& e) {
    batch_.error = e.what();
  }
  for (size_t i = 0; i < kernels_.size() && i < tune.size(); ++i) {
    try {
      kernels_[i]->finishRun(tune[i]);
      kernels_[i]->tearDown(Base_GB300, tune[i]);
    } catch (const std::exception&) {
    }
  }
}

void Executor::outputRunData() {
  if (!ok() || run_params.getInputState() == RunParams::DryRun) return;
  const std::string& dir = run_params.getOutputDirName();
  ::mkdir(dir.c_str(), 0755);
  std::string base = dir + "/" + run_params.getOutputFilePrefix();
  if (run_params.graphBatch()) {
    std::ofstream f(base + "-graph-batch.json");
    f << "{\"kernels\": " << batch_.kernels << ", \"reps\": " << batch_.reps
      << ", \"launches_per_rep\": " << batch_.launches_per_rep
      << ", \"launch_time_s\": " << std::setprecision(9) << batch_.launch_time
      << ", \"graph_time_s\": " << batch_.graph_time
      << ", \"graph_serial_time_s\": " << batch_.graph_serial_time << ", \"error\": \""
      << batch_.error << "\"}\n";
    return;
  }
  const reports::ReportData d = reportData();
  std::vector<std::string> combiners = run_params.getNpassesCombiners();
  if (combiners.empty()) combiners.push_back("Average");  // the suite's default
  for (const std::string& c : combiners) {
    const reports::Combiner m = c == "Minimum"   ? reports::Combiner::Minimum
                                : c == "Maximum" ? reports::Combiner::Maximum
                                                 : reports::Combiner::Average;
    {
      std::ofstream f(base + "-timing-" + c + ".csv");
      reports::writeTimingReport(f, d, m);
    }
    if (d.reference_variant >= 0) {
      std::ofstream f(base + "-speedup-" + c + ".csv");
      reports::writeSpeedupReport(f, d, m);
    }
  }
  {
    std::ofstream f(base + "-checksum.txt");
    reports::writeChecksumReport(f, d);
  }
  if (reports::hasFOMGroups(d)) {
    std::ofstream f(base + "-fom.csv");
    reports::writeFOMReport(f, d);
  }
  {
    std::ofstream f(base + "-kernels.csv");
    reports::writeKernelInfo(f, d);
  }
  writeRooflineJSON(base + "-roofline.json");
}

// The run's results as the report writers' table: one variant (Base_GB300)
// whose columns are the selected tunings in first-seen order.
reports::ReportData Executor::reportData() const {
  reports::ReportData d;
  d.variants.push_back(getVariantName(Base_GB300));
  d.tunings.push_back(tuning_names_);
  d.npasses = run_params.getNumPasses();
  d.pf_tolerance = run_params.getPFTolerance();
  d.reference_variant = run_params.getReferenceVariant().empty() ? -1 : 0;
  for (size_t i = 0; i < kernels_.size(); ++i) {
    const KernelBase* k = kernels_[i].get();
    reports::KernelRow row;
    row.name = k->getName();
    row.problem_size = k->getActualProblemSize();
    row.reps = k->getRunReps();
    row.its_per_rep = k->getItsPerRep();
    row.kernels_per_rep = k->getKernelsPerRep();
    row.bytes_per_rep = k->getBytesPerRep();
    row.flops_per_rep = k->getFLOPsPerRep();
    row.bytes_read_per_rep = k->getBytesReadPerRep();
    row.bytes_written_per_rep = k->getBytesWrittenPerRep();
    row.bytes_atomic_modify_written_per_rep = k->getBytesAtomicModifyWrittenPerRep();
    row.cells.resize(1);
    for (const std::string& tn : tuning_names_) {
      reports::Cell c;
      const size_t t = k->getVariantTuningIndex(Base_GB300, tn);
      c.defined = t != KernelBase::getUnknownTuningIdx();
      c.run = c.defined && k->wasVariantTuningRun(Base_GB300, t);
      if (c.run) {
        c.tot_time = k->getTotTime(Base_GB300, t);
        c.min_time = k->getMinTime(Base_GB300, t);
        c.max_time = k->getMaxTime(Base_GB300, t);
        c.checksum = k->getChecksum(Base_GB300, t);
      }
      row.cells[0].push_back(c);
    }
    d.kernels.push_back(std::move(row));
  }
  return d;
}

// Bandwidth and FLOP rate as scripts/caliper_graph/plot.py:15-31 derives
// them: Bytes/rep / (time / reps) and FLOPs/rep / (time / reps).
void Executor::writeRooflineJSON(const std::string& fname) const {
  std::ofstream f(fname);
  f << "[\n";
  for (size_t i = 0; i < results_.size(); ++i) {
    const RunResult& r = results_[i];
    double per_rep = r.reps > 0 ? r.min_time / r.reps : 0.0;
    double gbs = per_rep > 0 ? r.bytes_per_rep / per_rep / 1e9 : 0.0;
    double gfs = per_rep > 0 ? r.flops_per_rep / per_rep / 1e9 : 0.0;
    f << "  {\"kernel\": \"" << r.kernel << "\", \"tuning\": \"" << r.tuning
      << "\", \"size\": " << r.actual_size << ", \"reps\": " << r.reps
      << ", \"time_per_rep_s\": " << std::setprecision(9) << per_rep
      << ", \"bytes_per_rep\": " << r.bytes_per_rep << ", \"gbs\": " << gbs
      << ", \"gflops\": " << gfs << ", \"checksum\": " << std::setprecision(20)
      << static_cast<double>(r.checksum) << "}" << (i + 1 < results_.size() ? "," : "")
      << "\n";
  }
  f << "]\n";
}

}  // namespace rajaperf
