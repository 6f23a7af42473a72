// Minimal stand-in for scalFMM's FMath as FP2PRCutoff.hpp uses it (harness only).
#pragma once
#include <cmath>
struct FMath {
  template <class T> static T Sqrt(const T v) { return std::sqrt(v); }
};
