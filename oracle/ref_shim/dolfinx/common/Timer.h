// Minimal stand-in for dolfinx/common/Timer.h used only when compiling the
// reference's graph/ordering.cpp into oracle/_ref/ (the real header pulls
// in MPI and spdlog, which this machine does not have). Timing is not
// part of what the oracle checks, so the timer does nothing.
#pragma once
#include <string>
namespace dolfinx::common
{
class Timer
{
public:
  explicit Timer(const std::string&) {}
  void stop() {}
  void flush() {}
};
} // namespace dolfinx::common
