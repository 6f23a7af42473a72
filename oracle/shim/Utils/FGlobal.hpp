// Minimal stand-in for the scalFMM global definitions that
// include/ParticleHandler/FMM/FP2PRCutoff.hpp names (test harness only; the
// harness never instantiates the vectorised container kernels).
#pragma once
#include <cstdint>
using FSize = long long;
#define FRestrict __restrict__
