// Driver of the suite built with the Base_GB300 variant registered as
// INTEGRATION.md describes (integration.py).  Prints one JSON line: for
// Stream_TRIAD and Stream_DOT, whether the variant is defined and its tuning
// names.  With "--run <size> <reps>" it also runs both kernels' Base_Seq and
// Base_GB300 variants through the suite's own KernelBase::execute
// (common/KernelBase.cpp:359-377) and adds their checksums, so that a machine
// with a GPU and the suite's sources can compare them in one executable.
#include "common/KernelBase.hpp"
#include "common/RAJAPerfSuite.hpp"
#include "common/RunParams.hpp"

#include <cstdio>
#include <string>
#include <vector>

using namespace rajaperf;

int main(int argc, char** argv) {
  bool run = argc >= 4 && std::string(argv[1]) == "--run";
  std::vector<std::string> args = {"rajaperf_ref_gb300", "--size", run ? argv[2] : "1000",
                                   "--checkrun", run ? argv[3] : "1", "--disable-warmup",
                                   "-k", "Stream_TRIAD", "Stream_DOT"};
  std::vector<char*> cargs;
  for (auto& a : args) cargs.push_back(&a[0]);
  RunParams params(static_cast<int>(cargs.size()), cargs.data());
  std::printf("{");
  const KernelID kids[2] = {Stream_TRIAD, Stream_DOT};
  for (int n = 0; n < 2; ++n) {
    KernelBase* k = getKernelObject(kids[n], params);
    std::printf("%s\"%s\": {\"gb300_defined\": %s, \"gb300_tunings\": [", n ? ", " : "",
                getFullKernelName(kids[n]).c_str(),
                k->hasVariantDefined(Base_GB300) ? "true" : "false");
    for (size_t t = 0; t < k->getNumVariantTunings(Base_GB300); ++t)
      std::printf("%s\"%s\"", t ? ", " : "", k->getVariantTuningName(Base_GB300, t).c_str());
    std::printf("]");
    if (run) {
      for (VariantID vid : {Base_Seq, Base_GB300}) {
        k->execute(vid, 0);
        std::printf(", \"%s_checksum\": %.17Lg", getVariantName(vid).c_str(),
                    k->getChecksum(vid, 0));
      }
    }
    std::printf("}");
    delete k;
  }
  std::printf("}\n");
  return 0;
}
