// rajaperf-gb300: the suite driver for the Base_GB300 variant, with the same
// five steps as the suite's RAJAPerfSuiteDriver.cpp:22-61.
#include "common/Executor.hpp"

#include <exception>
#include <iostream>

int main(int argc, char** argv) {
  try {
    rajaperf::Executor executor(argc, argv);
    executor.setupSuite();
    executor.reportRunSummary(std::cout);
    if (!executor.ok()) {
      return executor.getRunParams().getInputState() ==
                     rajaperf::RunParams::InfoRequest ? 0 : 1;
    }
    executor.runSuite();
    executor.outputRunData();
    int failed = 0;
    for (const auto& r : executor.results()) {
      std::cout << "  " << r.kernel << " [" << r.tuning << "] checksum "
                << static_cast<double>(r.checksum) << " time/rep "
                << (r.reps ? r.min_time / r.reps : 0.0) << " s"
                << (r.error.empty() ? "" : "  FAILED: " + r.error) << "\n";
      if (!r.error.empty()) ++failed;
    }
    std::cout << "\nDONE!!!...." << std::endl;
    return failed ? 1 : 0;
  } catch (const std::exception& e) {
    std::cerr << "rajaperf-gb300: " << e.what() << std::endl;
    return 1;
  }
}
