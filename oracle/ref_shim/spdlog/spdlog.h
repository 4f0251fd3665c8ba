// Stand-in for gabime/spdlog as used by the reference's hot-path sources.
// TEST INFRASTRUCTURE ONLY (project-written): messages are discarded.
#pragma once
namespace spdlog {
template <typename... A> inline void error(A&&...) {}
template <typename... A> inline void debug(A&&...) {}
template <typename... A> inline void info(A&&...) {}
template <typename... A> inline void warn(A&&...) {}
}  // namespace spdlog
