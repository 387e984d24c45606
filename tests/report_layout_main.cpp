// Writes every suite report for a fixed table of results (two kernels, the
// variants Base_GB300 and RAJA_GB300, a tuning one kernel lacks, a tuning
// that did not run) to stdout, each after a "@@ <name>" marker line.  Built
// and run by tests/test_reports.py, which checks the layouts.
#include "Reports.hpp"

#include <iostream>

using namespace rajaperf::reports;

int main() {
  ReportData d;
  d.variants = {"Base_GB300", "RAJA_GB300"};
  d.tunings = {{"default", "graph", "int64"}, {"default"}};
  d.npasses = 2;
  d.reference_variant = 0;
  d.pf_tolerance = 0.1;
  auto cell = [](bool defined, bool run, double tot, double mn, double mx, long double ck) {
    Cell c;
    c.defined = defined;
    c.run = run;
    c.tot_time = tot;
    c.min_time = mn;
    c.max_time = mx;
    c.checksum = ck;
    return c;
  };
  KernelRow a;
  a.name = "Stream_TRIAD";
  a.problem_size = 1000000;
  a.reps = 1000;
  a.its_per_rep = 1000000;
  a.kernels_per_rep = 1;
  a.bytes_per_rep = 24000000;
  a.flops_per_rep = 2000000;
  a.bytes_read_per_rep = 16000000;
  a.bytes_written_per_rep = 8000000;
  a.cells = {{cell(true, true, 0.5, 0.24, 0.26, 135.91984956172908L),
              cell(true, true, 0.25, 0.12, 0.13, 135.91984956172908L),
              cell(false, false, 0, 0, 0, 0)},
             {cell(true, true, 0.6, 0.29, 0.31, 135.91984956172900L)}};
  KernelRow b;
  b.name = "Algorithm_SCAN";
  b.problem_size = 67108864;
  b.reps = 100;
  b.its_per_rep = 67108864;
  b.kernels_per_rep = 1;
  b.bytes_per_rep = 1073741824;
  b.flops_per_rep = 67108864;
  b.bytes_read_per_rep = 536870912;
  b.bytes_written_per_rep = 536870912;
  b.cells = {{cell(true, true, 2.0, 0.9, 1.1, 4.5L), cell(true, false, 0, 0, 0, 0),
              cell(true, true, 1.0, 0.5, 0.5, 4.25L)},
             {cell(false, false, 0, 0, 0, 0)}};
  d.kernels = {a, b};

  std::cout << "@@ timing-Average\n";
  writeTimingReport(std::cout, d, Combiner::Average);
  std::cout << "@@ timing-Minimum\n";
  writeTimingReport(std::cout, d, Combiner::Minimum);
  std::cout << "@@ speedup-Average\n";
  writeSpeedupReport(std::cout, d, Combiner::Average);
  std::cout << "@@ checksum\n";
  writeChecksumReport(std::cout, d);
  std::cout << "@@ fom\n";
  writeFOMReport(std::cout, d);
  std::cout << "@@ kernels\n";
  writeKernelInfo(std::cout, d);
  return 0;
}
