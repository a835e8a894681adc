// No-op logging shim for compiling the reference matcher.  Test infrastructure.
#pragma once
namespace spdlog {
template <class... A> inline void info(A&&...) {}
template <class... A> inline void warn(A&&...) {}
template <class... A> inline void debug(A&&...) {}
template <class... A> inline void error(A&&...) {}
}  // namespace spdlog
