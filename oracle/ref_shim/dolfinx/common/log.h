// Minimal stand-in for dolfinx/common/log.h (spdlog is absent here); the
// reference sources compiled into oracle/_ref/ only log diagnostics.
#pragma once
namespace spdlog
{
template <typename... A> inline void info(A&&...) {}
template <typename... A> inline void debug(A&&...) {}
template <typename... A> inline void warn(A&&...) {}
} // namespace spdlog
