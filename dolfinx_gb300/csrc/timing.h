// Named wall-clock timings of host work, kept for the life of the process:
// the counterpart of the reference's common::Timer / TimeLogger pair
// (common/Timer.h:38-141, common/TimeLogger.cpp:24-40). Each task name
// accumulates a repetition count and a total in seconds. The host set-up
// stages register under the reference's task names ("Build BoxMesh
// (tetrahedra)", "Reverse Cuthill-McKee ordering", "Build sparsity", ...),
// and the Python Timer registers into the same table through
// dfx_timing_record.
#pragma once

#include <chrono>

namespace dfx
{
// Add one repetition of `seconds` to `task` (thread-safe).
void record_timing(const char* task, double seconds);

// Registers the time from construction to destruction under `task`.
class ScopedTimer
{
public:
  explicit ScopedTimer(const char* task)
      : task_(task), t0_(std::chrono::steady_clock::now())
  {
  }
  ~ScopedTimer()
  {
    const std::chrono::duration<double> dt = std::chrono::steady_clock::now() - t0_;
    record_timing(task_, dt.count());
  }
  ScopedTimer(const ScopedTimer&) = delete;
  ScopedTimer& operator=(const ScopedTimer&) = delete;

private:
  const char* task_;
  std::chrono::steady_clock::time_point t0_;
};
} // namespace dfx
