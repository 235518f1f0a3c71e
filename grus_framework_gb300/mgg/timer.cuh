// timer.cuh -- drop-in for the reference's include/timer.cuh: Start() and
// Finish() (elapsed milliseconds since Start, then restart), on the steady
// clock.
#ifndef GRUS_MGG_TIMER_CUH
#define GRUS_MGG_TIMER_CUH

#include <chrono>

class Timer {
  std::chrono::steady_clock::time_point t0_ = std::chrono::steady_clock::now();

 public:
  void Start() { t0_ = std::chrono::steady_clock::now(); }
  float Finish() {
    const auto t1 = std::chrono::steady_clock::now();
    const float ms = std::chrono::duration<float, std::milli>(t1 - t0_).count();
    t0_ = t1;
    return ms;
  }
};

#endif
