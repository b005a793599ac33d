/* ORACLE / TEST INFRASTRUCTURE ONLY. The CUDA samples stopwatch the reference
 * includes (its timings are printed, never used). */
#ifndef CESA_EMU_HELPER_TIMER_H_
#define CESA_EMU_HELPER_TIMER_H_
#include <chrono>

struct StopWatchInterface {
  std::chrono::steady_clock::time_point t0;
  double total_ms = 0.0;
  int laps = 0;
};
inline bool sdkCreateTimer(StopWatchInterface** t) {
  *t = new StopWatchInterface();
  return true;
}
inline bool sdkDeleteTimer(StopWatchInterface** t) {
  delete *t;
  *t = nullptr;
  return true;
}
inline bool sdkStartTimer(StopWatchInterface** t) {
  (*t)->t0 = std::chrono::steady_clock::now();
  return true;
}
inline bool sdkStopTimer(StopWatchInterface** t) {
  (*t)->total_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - (*t)->t0).count();
  (*t)->laps += 1;
  return true;
}
inline float sdkGetTimerValue(StopWatchInterface** t) { return (float)(*t)->total_ms; }
inline float sdkGetAverageTimerValue(StopWatchInterface** t) {
  return (*t)->laps ? (float)((*t)->total_ms / (*t)->laps) : 0.f;
}
#endif
