// The suite's run reports, written from a plain table of results.
//
// Layouts follow the suite's Executor so that scripts reading RAJAPerf
// output read these files unchanged (common/Executor.cpp:825-1616 of the
// suite):
//   <prefix>-timing-<Average|Minimum|Maximum>.csv   writeCSVReport, Timing
//   <prefix>-speedup-<combiner>.csv                 writeCSVReport, Speedup
//                                                   (with a reference variant)
//   <prefix>-checksum.txt                           writeChecksumReport
//   <prefix>-fom.csv                                writeFOMReport
//   <prefix>-kernels.csv                            writeKernelInfoSummary
// The writers take a ReportData table and an output stream only (no CUDA, no
// kernel objects), so their layouts are tested without a GPU.
#pragma once

#include <iosfwd>
#include <string>
#include <vector>

namespace rajaperf {
namespace reports {

enum class Combiner { Average, Minimum, Maximum };
const char* combinerName(Combiner c);  // "Average", "Minimum", "Maximum"

// One variant/tuning of one kernel.
struct Cell {
  bool defined = false;  // the kernel has this variant/tuning
  bool run = false;      // it ran (in at least one pass)
  double tot_time = 0.0;  // seconds, summed over passes
  double min_time = 0.0;
  double max_time = 0.0;
  long double checksum = 0.0L;
};

struct KernelRow {
  std::string name;
  long long problem_size = 0, reps = 0, its_per_rep = 0, kernels_per_rep = 0;
  long long bytes_per_rep = 0, flops_per_rep = 0;
  long long bytes_read_per_rep = 0, bytes_written_per_rep = 0,
            bytes_atomic_modify_written_per_rep = 0;
  // cells[v][t]: variant v, tuning t of that variant's column list
  std::vector<std::vector<Cell>> cells;
};

struct ReportData {
  std::vector<std::string> variants;             // in run order
  std::vector<std::vector<std::string>> tunings;  // per variant, column order
  std::vector<KernelRow> kernels;
  int npasses = 1;
  int reference_variant = -1;  // index into variants, -1 = none (no speedup)
  double pf_tolerance = 0.1;   // FOM OVER_TOL threshold (--pass-fail-tol)
};

void writeTimingReport(std::ostream& os, const ReportData& d, Combiner c);
void writeSpeedupReport(std::ostream& os, const ReportData& d, Combiner c);
void writeChecksumReport(std::ostream& os, const ReportData& d);
// FOM groups: each variant whose name contains "Base" starts a group with
// the later variants whose names contain its suffix (Executor.cpp:1618-1647).
void writeFOMReport(std::ostream& os, const ReportData& d);
bool hasFOMGroups(const ReportData& d);
void writeKernelInfo(std::ostream& os, const ReportData& d);

}  // namespace reports
}  // namespace rajaperf
