// Stand-in for the matplotlib-cpp plotting header that the reference's
// Derivatives.cuh includes for its debug plots (it embeds CPython).  The
// plots sit in debug-only code, so the reference harness (oracle/ref_harness.cu)
// compiles against these no-ops instead.
#pragma once
#include <array>
#include <map>
#include <memory>
#include <string>
#include <vector>

namespace matplotlibcpp {
template <typename... A>
inline void figure(A&&...) {}
template <typename... A>
inline void plot(A&&...) {}
template <typename... A>
inline void title(A&&...) {}
template <typename... A>
inline void legend(A&&...) {}
template <typename... A>
inline void show(A&&...) {}
}  // namespace matplotlibcpp
