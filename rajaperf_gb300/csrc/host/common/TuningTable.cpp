#include "TuningTable.hpp"

#include <cstdlib>
#include <fstream>
#include <sstream>

namespace rajaperf {

TuningTable& TuningTable::instance() {
  static TuningTable table;
  return table;
}

bool parseTuneField(const std::string& kv, b200_tune* t) {
  std::size_t eq = kv.find('=');
  if (eq == std::string::npos) return false;
  std::string key = kv.substr(0, eq);
  char* end = nullptr;
  long v = std::strtol(kv.c_str() + eq + 1, &end, 10);
  if (!end || *end != '\0') return false;
  int32_t iv = static_cast<int32_t>(v);
  if (key == "block") t->block_size = iv;
  else if (key == "items") t->items = iv;
  else if (key == "vec") t->vec = iv;
  else if (key == "grid") t->grid_blocks = iv;
  else if (key == "tile_x") t->tile_x = iv;
  else if (key == "tile_y") t->tile_y = iv;
  else if (key == "tile_z") t->tile_z = iv;
  else if (key == "time_block") t->time_block = iv;
  else if (key == "algo") t->algo = iv;
  else return false;
  return true;
}

bool TuningTable::parse(const std::string& text, std::string* error) {
  std::vector<Entry> entries;
  std::istringstream in(text);
  std::string line;
  int lineno = 0;
  while (std::getline(in, line)) {
    ++lineno;
    std::size_t hash = line.find('#');
    if (hash != std::string::npos) line.resize(hash);
    std::istringstream ls(line);
    Entry e{};
    if (!(ls >> e.kernel)) continue;
    if (!(ls >> e.min_size >> e.max_size) ||
        getKernelIDFromName(e.kernel) == NumKernels) {
      if (error) *error = "tuning table line " + std::to_string(lineno) + ": bad entry";
      return false;
    }
    e.kernel = getFullKernelName(getKernelIDFromName(e.kernel));
    std::string kv;
    while (ls >> kv) {
      if (!parseTuneField(kv, &e.tune)) {
        if (error)
          *error = "tuning table line " + std::to_string(lineno) + ": bad field " + kv;
        return false;
      }
    }
    entries.push_back(e);
  }
  entries_ = std::move(entries);
  return true;
}

bool TuningTable::load(const std::string& path, std::string* error) {
  std::ifstream f(path);
  if (!f) {
    if (error) *error = "cannot open tuning table " + path;
    return false;
  }
  std::stringstream ss;
  ss << f.rdbuf();
  return parse(ss.str(), error);
}

bool TuningTable::lookup(const std::string& kernel, long long size,
                         b200_tune* out) const {
  if (has_override_ && override_.kernel == kernel && size >= override_.min_size &&
      (override_.max_size < 0 || size <= override_.max_size)) {
    *out = override_.tune;
    return true;
  }
  for (const Entry& e : entries_) {
    if (e.kernel == kernel && size >= e.min_size &&
        (e.max_size < 0 || size <= e.max_size)) {
      *out = e.tune;
      return true;
    }
  }
  return false;
}

void TuningTable::prepend(const std::vector<Entry>& entries) {
  entries_.insert(entries_.begin(), entries.begin(), entries.end());
}

std::string TuningTable::format(const Entry& e) {
  std::ostringstream os;
  os << e.kernel << " " << e.min_size << " " << e.max_size;
  const b200_tune& t = e.tune;
  if (t.block_size) os << " block=" << t.block_size;
  if (t.items) os << " items=" << t.items;
  if (t.vec) os << " vec=" << t.vec;
  if (t.grid_blocks) os << " grid=" << t.grid_blocks;
  if (t.tile_x) os << " tile_x=" << t.tile_x;
  if (t.tile_y) os << " tile_y=" << t.tile_y;
  if (t.tile_z) os << " tile_z=" << t.tile_z;
  if (t.time_block) os << " time_block=" << t.time_block;
  if (t.algo) os << " algo=" << t.algo;
  return os.str();
}

}  // namespace rajaperf
