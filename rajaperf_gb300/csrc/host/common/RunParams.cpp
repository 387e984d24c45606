// Command-line parsing for RunParams.  Option names and meanings follow the
// suite's RunParams.cpp:296-1269 where they overlap.
#include "RunParams.hpp"

#include <algorithm>
#include <cstdlib>
#include <iostream>
#include <sstream>

namespace rajaperf {

namespace {

bool isOption(const std::string& s) {
  return s.size() > 1 && s[0] == '-' &&
         !(s.size() > 1 && (std::isdigit(static_cast<unsigned char>(s[1])) || s[1] == '.'));
}

bool parseDouble(const std::string& s, double& out) {
  char* end = nullptr;
  out = std::strtod(s.c_str(), &end);
  return end && *end == '\0' && !s.empty();
}

bool parseLong(const std::string& s, long long& out) {
  char* end = nullptr;
  out = std::strtoll(s.c_str(), &end, 10);
  return end && *end == '\0' && !s.empty();
}

}  // namespace

void RunParams::fail(const std::string& msg) {
  input_state = BadInput;
  if (error_message.empty()) error_message = msg;
}

RunParams::RunParams(int argc, const char* const* argv) {
  std::vector<std::string> args(argv + (argc > 0 ? 1 : 0), argv + argc);
  std::vector<std::string> kernel_input, exclude_kernel_input, variant_input;
  bool size_given = false, sizefact_given = false;

  auto takeList = [&](std::size_t& i, std::vector<std::string>& out) {
    while (i + 1 < args.size() && !isOption(args[i + 1])) {
      std::string item = args[++i];
      std::stringstream ss(item);
      std::string tok;
      while (std::getline(ss, tok, ',')) {
        if (!tok.empty()) out.push_back(tok);
      }
    }
  };
  auto takeValue = [&](std::size_t& i, const std::string& opt) -> std::string {
    if (i + 1 >= args.size() || isOption(args[i + 1])) {
      fail("missing value for " + opt);
      return std::string();
    }
    return args[++i];
  };

  for (std::size_t i = 0; i < args.size(); ++i) {
    const std::string& opt = args[i];
    if (opt == "-h" || opt == "--help") {
      input_state = InfoRequest;
    } else if (opt == "--size") {
      double v;
      if (!parseDouble(takeValue(i, opt), v) || v < 0) fail("bad --size");
      size = v;
      size_given = true;
    } else if (opt == "--sizefact") {
      double v;
      if (!parseDouble(takeValue(i, opt), v) || v < 0) fail("bad --sizefact");
      size_factor = v;
      sizefact_given = true;
    } else if (opt == "--repfact") {
      double v;
      if (!parseDouble(takeValue(i, opt), v) || v < 0) fail("bad --repfact");
      rep_fact = v;
    } else if (opt == "--checkrun") {
      input_state = CheckRun;
      if (i + 1 < args.size() && !isOption(args[i + 1])) {
        long long v;
        if (!parseLong(args[++i], v) || v < 1) fail("bad --checkrun");
        checkrun_reps = static_cast<int>(v);
      }
    } else if (opt == "--npasses") {
      long long v;
      if (!parseLong(takeValue(i, opt), v) || v < 1) fail("bad --npasses");
      npasses = static_cast<int>(v);
    } else if (opt == "--dryrun") {
      if (input_state != BadInput) input_state = DryRun;
    } else if (opt == "--show-progress" || opt == "-sp") {
      show_progress = true;
    } else if (opt == "--disable-warmup") {
      disable_warmup = true;
    } else if (opt == "-k" || opt == "--kernels") {
      takeList(i, kernel_input);
    } else if (opt == "-ek" || opt == "--exclude-kernels") {
      takeList(i, exclude_kernel_input);
    } else if (opt == "-v" || opt == "--variants") {
      takeList(i, variant_input);
    } else if (opt == "-t" || opt == "--tunings") {
      takeList(i, tuning_input);
    } else if (opt == "-et" || opt == "--exclude-tunings") {
      takeList(i, exclude_tuning_input);
    } else if (opt == "--init") {
      std::string v = takeValue(i, opt);
      if (v == "reference") init_mode = InitReference;
      else if (v == "uniform") init_mode = InitUniform;
      else fail("bad --init (reference|uniform)");
    } else if (opt == "--seed") {
      long long v;
      if (!parseLong(takeValue(i, opt), v) || v < 0) fail("bad --seed");
      seed = static_cast<unsigned long long>(v);
    } else if (opt == "--init-range") {
      double lo, hi;
      if (!parseDouble(takeValue(i, opt), lo) || !parseDouble(takeValue(i, opt), hi) ||
          !(hi > lo))
        fail("bad --init-range");
      init_lo = lo;
      init_hi = hi;
    } else if (opt == "--polybench_tsteps") {
      long long v;
      if (!parseLong(takeValue(i, opt), v) || v < 0) fail("bad --polybench_tsteps");
      polybench_tsteps = static_cast<long>(v);
    } else if (opt == "--multi_reduce_num_bins") {
      long long v;
      if (!parseLong(takeValue(i, opt), v) || v < 1) fail("bad --multi_reduce_num_bins");
      multi_reduce_num_bins = static_cast<long>(v);
    } else if (opt == "--multi_reduce_bin_assignment_algorithm") {
      std::string v = takeValue(i, opt);
      if (v == "Random") multi_reduce_bin_assignment = BinAssignmentAlgorithm::Random;
      else if (v == "RunsRandomSizes")
        multi_reduce_bin_assignment = BinAssignmentAlgorithm::RunsRandomSizes;
      else if (v == "RunsEvenSizes")
        multi_reduce_bin_assignment = BinAssignmentAlgorithm::RunsEvenSizes;
      else if (v == "Single") multi_reduce_bin_assignment = BinAssignmentAlgorithm::Single;
      else fail("bad --multi_reduce_bin_assignment_algorithm " + v);
    } else if (opt == "--halo_width") {
      long long v;
      if (!parseLong(takeValue(i, opt), v) || v < 1) fail("bad --halo_width");
      halo_width = static_cast<long>(v);
    } else if (opt == "--halo_num_vars") {
      long long v;
      if (!parseLong(takeValue(i, opt), v) || v < 1 || v > 9) fail("bad --halo_num_vars (1-9)");
      halo_num_vars = static_cast<long>(v);
    } else if (opt == "--size-map") {
      std::vector<std::string> items;
      takeList(i, items);
      for (const std::string& it : items) {
        std::size_t eq = it.find('=');
        double v;
        KernelID kid = eq == std::string::npos ? NumKernels
                                               : getKernelIDFromName(it.substr(0, eq));
        if (kid == NumKernels || !parseDouble(it.substr(eq + 1), v) || v < 0) {
          fail("bad --size-map entry " + it);
        } else {
          size_map[kid] = v;
        }
      }
    } else if (opt == "--npasses-combiners") {
      std::vector<std::string> items;
      takeList(i, items);
      for (const std::string& c : items) {
        if (c != "Average" && c != "Minimum" && c != "Maximum")
          fail("bad --npasses-combiners entry " + c + " (Average|Minimum|Maximum)");
        else if (std::find(npasses_combiners.begin(), npasses_combiners.end(), c) ==
                 npasses_combiners.end())
          npasses_combiners.push_back(c);
      }
    } else if (opt == "--refvar" || opt == "-rv") {
      reference_variant = takeValue(i, opt);
    } else if (opt == "--pass-fail-tol" || opt == "-pftol") {
      double v;
      if (!parseDouble(takeValue(i, opt), v) || v < 0) fail("bad --pass-fail-tol");
      pf_tolerance = v;
    } else if (opt == "--host-data") {
      host_data = true;
    } else if (opt == "--wait-limit-us") {
      long long v;
      if (!parseLong(takeValue(i, opt), v) || v < 0 || v > 2000000000LL)
        fail("bad --wait-limit-us");
      wait_limit_us = static_cast<int>(v);
    } else if (opt == "--inject-lookback-stall") {
      long long v;
      if (!parseLong(takeValue(i, opt), v) || v < 1 || v > 1000000LL)
        fail("bad --inject-lookback-stall");
      inject_lookback_stall = static_cast<long>(v);
    } else if (opt == "--tuning-table") {
      tuning_table_file = takeValue(i, opt);
    } else if (opt == "--autotune") {
      autotune_file = takeValue(i, opt);
    } else if (opt == "--graph-batch") {
      graph_batch = true;
      if (i + 1 < args.size() && !isOption(args[i + 1])) {
        long long v;
        if (!parseLong(args[++i], v) || v < 1) fail("bad --graph-batch reps");
        graph_batch_reps = static_cast<int>(v);
      }
    } else if (opt == "-od" || opt == "--outdir") {
      outdir = takeValue(i, opt);
    } else if (opt == "-of" || opt == "--outfile") {
      outfile_prefix = takeValue(i, opt);
    } else {
      fail("unknown option " + opt);
    }
  }

  if (size_given && sizefact_given) fail("--size and --sizefact are exclusive");
  if (size_given) size_meaning = Direct;
  else size_meaning = Factor;

  // Kernel selection: names, short names or group names; default all.
  std::vector<bool> selected(NumKernels, kernel_input.empty());
  for (const std::string& name : kernel_input) {
    GroupID gid = getGroupIDFromName(name);
    KernelID kid = getKernelIDFromName(name);
    if (gid != NumGroups) {
      for (int k = 0; k < NumKernels; ++k)
        if (getGroupOfKernel(static_cast<KernelID>(k)) == gid) selected[k] = true;
    } else if (kid != NumKernels) {
      selected[kid] = true;
    } else {
      fail("unknown kernel or group " + name);
    }
  }
  for (const std::string& name : exclude_kernel_input) {
    GroupID gid = getGroupIDFromName(name);
    KernelID kid = getKernelIDFromName(name);
    if (gid != NumGroups) {
      for (int k = 0; k < NumKernels; ++k)
        if (getGroupOfKernel(static_cast<KernelID>(k)) == gid) selected[k] = false;
    } else if (kid != NumKernels) {
      selected[kid] = false;
    } else {
      fail("unknown kernel or group " + name);
    }
  }
  // Keep the command-line order when kernels are named individually.
  if (!kernel_input.empty()) {
    for (const std::string& name : kernel_input) {
      KernelID kid = getKernelIDFromName(name);
      GroupID gid = getGroupIDFromName(name);
      if (gid != NumGroups) {
        for (int k = 0; k < NumKernels; ++k) {
          KernelID kk = static_cast<KernelID>(k);
          if (getGroupOfKernel(kk) == gid && selected[k] &&
              std::find(run_kernels.begin(), run_kernels.end(), kk) == run_kernels.end())
            run_kernels.push_back(kk);
        }
      } else if (kid != NumKernels && selected[kid] &&
                 std::find(run_kernels.begin(), run_kernels.end(), kid) == run_kernels.end()) {
        run_kernels.push_back(kid);
      }
    }
  } else {
    for (int k = 0; k < NumKernels; ++k)
      if (selected[k]) run_kernels.push_back(static_cast<KernelID>(k));
  }

  if (variant_input.empty()) {
    run_variants.insert(Base_GB300);
  } else {
    for (const std::string& v : variant_input) {
      if (v == getVariantName(Base_GB300)) run_variants.insert(Base_GB300);
      else fail("variant " + v + " is not available in this build");
    }
  }
  if (host_data && (graph_batch || !autotune_file.empty()))
    fail("--host-data runs the suite's rep loops; it does not combine with --graph-batch "
         "or --autotune");
  if (!reference_variant.empty() && reference_variant != getVariantName(Base_GB300))
    fail("reference variant " + reference_variant + " is not available in this build");

  if (input_state == Undefined) input_state = PerfRun;
}

double RunParams::getKernelSize(KernelID kid) const {
  auto it = size_map.find(kid);
  return it == size_map.end() ? -1.0 : it->second;
}

void RunParams::print(std::ostream& os) const {
  os << "size_meaning=" << (size_meaning == Direct ? "direct" : "factor")
     << " size=" << size << " sizefact=" << size_factor
     << " repfact=" << rep_fact << " npasses=" << npasses
     << " init=" << (init_mode == InitUniform ? "uniform" : "reference")
     << " seed=" << seed << "\n";
}

std::string RunParams::usage() {
  return
      "Usage: rajaperf-gb300 [options]\n"
      "  --size N | --sizefact F      problem size (direct) or factor of default\n"
      "  --repfact F                  reps = default reps * F\n"
      "  --checkrun [R]               run R reps (default 1) per kernel\n"
      "  --npasses P                  passes over the kernel list\n"
      "  -k/--kernels NAMES           kernels or groups to run\n"
      "  -ek/--exclude-kernels NAMES  kernels or groups to skip\n"
      "  -v/--variants Base_GB300     variants (only Base_GB300 here)\n"
      "  -t/--tunings NAMES           tunings to run (default: all)\n"
      "  -et/--exclude-tunings NAMES  tunings to skip\n"
      "  --init reference|uniform     array contents (default reference)\n"
      "  --seed S --init-range LO HI  seed and range of the uniform mode\n"
      "  --polybench_tsteps T         override Polybench time steps\n"
      "  --multi_reduce_num_bins B    HISTOGRAM / MULTI_REDUCE bins (10)\n"
      "  --multi_reduce_bin_assignment_algorithm Random|RunsRandomSizes|\n"
      "                               RunsEvenSizes|Single (RunsRandomSizes)\n"
      "  --halo_width W --halo_num_vars V  HALO_PACKING halo (1) and variables (3)\n"
      "  --size-map K=N,...           per-kernel sizes\n"
      "  --tuning-table FILE          tuning table (kernel size-bucket params)\n"
      "  --autotune FILE              measure launch shapes for the selected\n"
      "                               kernels and sizes, use them and write\n"
      "                               them to FILE as a tuning table\n"
      "  --graph-batch [R]            capture every kernel's R-rep loop into\n"
      "                               one CUDA graph and compare with launches\n"
      "  --host-data                  arrays in pinned host memory; every rep\n"
      "                               moves its inputs and outputs across the\n"
      "                               host link (streaming kernels read and write\n"
      "                               host memory directly, iterating ones copy\n"
      "                               their arrays in and out around the rep)\n"
      "  --wait-limit-us U            limit of the kernels' bounded device-side\n"
      "                               waits (0 = library default: 2 s, GEMM 1 s)\n"
      "  --inject-lookback-stall K    test option: before each run of SCAN and\n"
      "                               INDEXLIST(_3LOOP) mark K tile tickets as\n"
      "                               taken, so that the first tile's lookback\n"
      "                               waits for tiles nobody processes until its\n"
      "                               wait limit runs out (the run then fails\n"
      "                               with the device-side timeout)\n"
      "  -od DIR, -of PREFIX          report directory and file prefix\n"
      "  --npasses-combiners C...     timing/speedup reports to write:\n"
      "                               Average Minimum Maximum (Average)\n"
      "  -rv/--refvar VARIANT         write speedup reports against VARIANT\n"
      "  -pftol/--pass-fail-tol T     FOM report OVER_TOL threshold (0.1)\n"
      "  --dryrun, --show-progress, --disable-warmup, -h\n";
}

}  // namespace rajaperf
