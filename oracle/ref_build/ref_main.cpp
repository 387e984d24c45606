// Oracle driver: runs the suite's own Base_Seq variant of one kernel through
// the suite's own KernelBase::execute (common/KernelBase.cpp:359-377) and
// prints one JSON line with the checksum and timing.
//
//   rajaperf_ref <Group_KERNEL> <size> <reps> [suite options ...]
//
// Sizes and reps are passed through the suite's RunParams as
// "--size <size> --checkrun <reps>"; further arguments (e.g.
// "--multi_reduce_num_bins 100") are appended to that command line.
#include "common/RAJAPerfSuite.hpp"
#include "common/KernelBase.hpp"
#include "common/RunParams.hpp"

#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

using namespace rajaperf;

int main(int argc, char** argv) {
  if (argc < 4) {
    std::fprintf(stderr, "usage: %s <Group_KERNEL> <size> <reps>\n", argv[0]);
    return 2;
  }
  std::string kname = argv[1];
  std::vector<std::string> args = {"rajaperf_ref", "--size", argv[2],
                                   "--checkrun", argv[3],
                                   "--disable-warmup",
                                   "-k", kname, "-v", "Base_Seq"};
  for (int a = 4; a < argc; ++a) args.push_back(argv[a]);
  std::vector<char*> cargs;
  for (auto& a : args) cargs.push_back(&a[0]);
  RunParams params(static_cast<int>(cargs.size()), cargs.data());

  KernelID kid = NumKernels;
  for (int k = 0; k < NumKernels; ++k) {
    if (getFullKernelName(static_cast<KernelID>(k)) == kname) {
      kid = static_cast<KernelID>(k);
    }
  }
  if (kid == NumKernels) {
    std::fprintf(stderr, "unknown kernel %s\n", kname.c_str());
    return 2;
  }
  KernelBase* kern = getKernelObject(kid, params);
  if (!kern) {
    std::fprintf(stderr, "kernel %s not built\n", kname.c_str());
    return 2;
  }
  kern->execute(Base_Seq, 0);
  long double ck = kern->getChecksum(Base_Seq, 0);
  std::printf("{\"kernel\": \"%s\", \"variant\": \"Base_Seq\", "
              "\"actual_size\": %lld, \"reps\": %lld, "
              "\"bytes_per_rep\": %lld, \"flops_per_rep\": %lld, "
              "\"checksum\": %.21Lg, \"time_s\": %.9g}\n",
              kname.c_str(),
              static_cast<long long>(kern->getActualProblemSize()),
              static_cast<long long>(kern->getRunReps()),
              static_cast<long long>(kern->getBytesPerRep()),
              static_cast<long long>(kern->getFLOPsPerRep()),
              ck, kern->getMinTime(Base_Seq, 0));
  delete kern;
  return 0;
}
