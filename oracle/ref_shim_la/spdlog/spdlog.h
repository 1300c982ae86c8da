// No-op stand-in for <spdlog/spdlog.h> (absent here), used only when
// compiling reference sources into oracle/_ref/: diagnostics are not part
// of what the oracle checks.
#pragma once
namespace spdlog
{
template <typename... A> inline void info(A&&...) {}
template <typename... A> inline void debug(A&&...) {}
template <typename... A> inline void warn(A&&...) {}
template <typename... A> inline void error(A&&...) {}
} // namespace spdlog
