// C ABI of the host layer (include/rajaperf_gb300.h): runs the Base_GB300
// suite for a command line and returns per kernel/tuning results.
#include "rajaperf_gb300.h"

#include "common/Executor.hpp"

#include <cstring>
#include <exception>
#include <string>

namespace {
thread_local std::string g_error;

void copyName(char* dst, size_t cap, const std::string& s) {
  std::strncpy(dst, s.c_str(), cap - 1);
  dst[cap - 1] = '\0';
}
}  // namespace

extern "C" {

const char* rp_last_error(void) { return g_error.c_str(); }

int rp_run(int argc, const char* const* argv, rp_result* out, int capacity,
           int* count) {
  g_error.clear();
  if (count) *count = 0;
  try {
    rajaperf::Executor ex(argc, argv);
    if (!ex.ok()) {
      g_error = ex.getRunParams().getErrorMessage();
      if (g_error.empty()) g_error = "info request";
      return RP_ERR_INPUT;
    }
    ex.setupSuite();
    ex.runSuite();
    if (!ex.getRunParams().getOutputDirName().empty() &&
        ex.getRunParams().getOutputDirName() != ".")
      ex.outputRunData();
    const auto& res = ex.results();
    int n = 0;
    int status = RP_OK;
    for (const auto& r : res) {
      if (!r.error.empty()) {
        status = RP_ERR_RUN;
        if (g_error.empty()) g_error = r.kernel + " " + r.tuning + ": " + r.error;
      }
      if (n >= capacity || !out) continue;
      rp_result& o = out[n++];
      std::memset(&o, 0, sizeof(o));
      copyName(o.kernel, sizeof(o.kernel), r.kernel);
      copyName(o.variant, sizeof(o.variant), r.variant);
      copyName(o.tuning, sizeof(o.tuning), r.tuning);
      o.checksum = static_cast<double>(r.checksum);
      o.checksum_residual = static_cast<double>(r.checksum - static_cast<long double>(o.checksum));
      o.min_time_s = r.min_time;
      o.avg_time_s = r.avg_time;
      o.max_time_s = r.max_time;
      o.reps = r.reps;
      o.actual_size = r.actual_size;
      o.its_per_rep = r.its_per_rep;
      o.kernels_per_rep = r.kernels_per_rep;
      o.bytes_per_rep = r.bytes_per_rep;
      o.flops_per_rep = r.flops_per_rep;
      o.passes = r.passes;
      o.failed = r.error.empty() ? 0 : 1;
      o.h2d_bytes_per_rep = r.h2d_bytes_per_rep;
      o.d2h_bytes_per_rep = r.d2h_bytes_per_rep;
    }
    if (count) *count = n;
    return status;
  } catch (const std::exception& e) {
    g_error = e.what();
    return RP_ERR_RUN;
  }
}

int rp_graph_batch(int argc, const char* const* argv, rp_batch_result* out) {
  g_error.clear();
  if (!out) return RP_ERR_INPUT;
  std::memset(out, 0, sizeof(*out));
  try {
    rajaperf::Executor ex(argc, argv);
    if (!ex.ok() || !ex.getRunParams().graphBatch()) {
      g_error = ex.ok() ? "command line lacks --graph-batch"
                        : ex.getRunParams().getErrorMessage();
      return RP_ERR_INPUT;
    }
    ex.setupSuite();
    ex.runSuite();
    const auto& b = ex.graphBatchResult();
    out->kernels = b.kernels;
    out->reps = b.reps;
    out->launches_per_rep = b.launches_per_rep;
    out->launch_time_s = b.launch_time;
    out->graph_time_s = b.graph_time;
    out->graph_serial_time_s = b.graph_serial_time;
    if (!b.error.empty()) {
      g_error = b.error;
      return RP_ERR_RUN;
    }
    return RP_OK;
  } catch (const std::exception& e) {
    g_error = e.what();
    return RP_ERR_RUN;
  }
}

}  // extern "C"
