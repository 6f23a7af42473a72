// Minimal stand-in for the vector types FP2PRCutoff.hpp names in its
// container specialisations (harness only; never instantiated).
#pragma once
struct InaVecBestTypeDouble {
  static const int VecLength = 1;
};
struct InaVecBestTypeFloat {
  static const int VecLength = 1;
};
