// Stand-in for RAJA::Timer: a steady-clock stopwatch whose elapsed() is the
// accumulated start/stop time in seconds, as the suite's KernelBase expects.
#ifndef ORACLE_SHIM_RAJA_TIMER_HPP
#define ORACLE_SHIM_RAJA_TIMER_HPP
#include <chrono>
namespace RAJA {
class Timer {
public:
  using ElapsedType = double;
  void start() { t0 = std::chrono::steady_clock::now(); }
  void stop() {
    auto t1 = std::chrono::steady_clock::now();
    acc += std::chrono::duration<double>(t1 - t0).count();
  }
  ElapsedType elapsed() const { return acc; }
  void reset() { acc = 0.0; }
private:
  std::chrono::steady_clock::time_point t0{};
  double acc = 0.0;
};
}
#endif
