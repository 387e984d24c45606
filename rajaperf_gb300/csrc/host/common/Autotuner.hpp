// Autotuner: a launch shape per kernel and problem size, chosen by measuring.
//
// For every selected kernel at its actual problem size the autotuner sets
// the kernel up once, then for each candidate shape of the kernel's family
// (block size x items per thread, plus vector width for the Stream map
// kernels, tile length for SCAN) makes that shape the kernel's tuning-table
// answer, captures `reps` reps of the kernel's rep body into a CUDA graph and
// times three replays with CUDA events (the minimum counts).  Graph replay
// keeps host launch overhead out of the comparison, so small sizes are tuned
// for the device time they take inside a captured batch.  Shapes the library
// rejects are skipped.  The library default shape is always a candidate, so
// a winner is never slower than the default in the same measurement.
//
// The winners become table entries covering exactly the tuned size; they are
// installed ahead of any loaded table for the rest of the run and written to
// a file in the tuning-table format (TuningTable.hpp).
#pragma once

#include "KernelBase.hpp"

#include <iosfwd>
#include <memory>
#include <string>
#include <vector>

namespace rajaperf {

struct AutotuneRecord {
  std::string kernel;
  long long size = 0;
  b200_tune best{};
  double best_s = 0.0;     // seconds per rep of the winning shape
  double default_s = 0.0;  // seconds per rep of the library default shape
  int candidates = 0;      // shapes timed (rejected shapes not counted)
};

// Candidate shapes for a kernel; the first is the library default (all zero).
std::vector<b200_tune> autotuneCandidates(KernelID kid);

// Tunes each kernel at its actual size (tunings[i].front() supplies the rep
// body) and returns one record per kernel that has more than one candidate.
std::vector<AutotuneRecord> autotune(const std::vector<std::unique_ptr<KernelBase>>& kernels,
                                     const std::vector<std::vector<size_t>>& tunings);

// Writes the records as tuning-table lines (with the measured times as
// comments); false when the file cannot be written.
bool writeAutotuneTable(const std::vector<AutotuneRecord>& recs, const std::string& path);

}  // namespace rajaperf
