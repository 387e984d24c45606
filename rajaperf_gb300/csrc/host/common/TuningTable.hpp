// Tuning table: launch shapes per kernel and problem-size range.
//
// Text format, one entry per line ('#' starts a comment):
//   <Group_KERNEL> <min_size> <max_size|-1> key=value ...
// keys: block, items, vec, grid, tile_x, tile_y, tile_z, time_block, algo.
// The first entry whose kernel matches and whose [min, max] range contains
// the actual problem size wins.  The autotuner writes this format.
#pragma once

#include "RAJAPerfSuite.hpp"
#include "b200.h"

#include <string>
#include <vector>

namespace rajaperf {

class TuningTable {
 public:
  struct Entry {
    std::string kernel;
    long long min_size;
    long long max_size;  // -1 = unbounded
    b200_tune tune;
  };

  static TuningTable& instance();

  // Loads entries from a file, replacing the current table.  Returns false
  // (with a message) on a parse error.
  bool load(const std::string& path, std::string* error);
  bool parse(const std::string& text, std::string* error);
  void clear() { entries_.clear(); }

  // Returns true and fills `out` when an entry covers (kernel, size).  An
  // override (set by the autotuner while it measures) is consulted first.
  bool lookup(const std::string& kernel, long long size, b200_tune* out) const;

  // Puts entries ahead of the current ones (the autotuner's winners).
  void prepend(const std::vector<Entry>& entries);
  void setOverride(const Entry& e) {
    override_ = e;
    has_override_ = true;
  }
  void clearOverride() { has_override_ = false; }

  const std::vector<Entry>& entries() const { return entries_; }
  static std::string format(const Entry& e);

 private:
  std::vector<Entry> entries_;
  Entry override_{};
  bool has_override_ = false;
};

// Parses "key=value" launch-shape fields into `t`; false on an unknown key.
bool parseTuneField(const std::string& kv, b200_tune* t);

}  // namespace rajaperf
