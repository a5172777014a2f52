// Stands in for dune/common/timer.hh: a wall-clock timer (elapsed seconds).
#ifndef GBFEM_SHIM_DG_TIMER_HH
#define GBFEM_SHIM_DG_TIMER_HH
#include <chrono>
namespace Dune {
class Timer {
 public:
  Timer() { reset(); }
  void reset() { t0_ = std::chrono::steady_clock::now(); }
  double elapsed() const { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0_).count(); }

 private:
  std::chrono::steady_clock::time_point t0_;
};
}  // namespace Dune
#endif
