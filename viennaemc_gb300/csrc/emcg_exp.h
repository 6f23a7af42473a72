// exp(x) in double for the Poisson residual's carrier densities, by Tang's
// table-driven method (P. T. P. Tang, "Table-driven implementation of the
// exponential function in IEEE floating-point arithmetic", ACM Trans. Math.
// Softw. 15(2), 1989):
//   x = (256 m + j) ln2/256 + r,  |r| <= ln2/512,
//   exp(x) = 2^m * 2^(j/256) * (1 + p(r)),
// p the Taylor polynomial of e^r - 1 to r^4 (truncation below
// |r|^5/120 < 4e-17 relative).  k = 256 m + j is rounded by adding 1.5 * 2^52
// (the integer lands in the low bits of the sum); the reduction
// r = x - k ln2/256 takes two fused multiply-adds with ln2/256 split into its
// nearest double and the remainder, so r is accurate to an ulp of r.
// tab[j] = 2^(j/256), j < 256.  |x| >= 700 and NaN go to the library's exp.
// The residual is evaluated in double precision on 16 SMs, and the GPU's
// double-precision rate is a small fraction of its single-precision one: this
// form takes 9 double instructions.
#pragma once

#include <math.h>
#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define EMCG_HD __host__ __device__ __forceinline__
#else
#define EMCG_HD inline
#endif

namespace emcg {

constexpr int kExpTab = 256;

EMCG_HD uint64_t dbits(double x) {
  uint64_t b;
  memcpy(&b, &x, sizeof b);
  return b;
}
EMCG_HD double bitsd(uint64_t b) {
  double x;
  memcpy(&x, &b, sizeof x);
  return x;
}

EMCG_HD double expTab(double x, const double *tab) {
  // |x| < 700 by the high word of |x| (700 = 0x4085E000 00000000); NaN fails
  if ((uint32_t)(dbits(x) >> 32 & 0x7fffffffu) >= 0x4085E000u)
    return exp(x);
  const double kMagic = 6755399441055744.0; // 1.5 * 2^52
  const double t = fma(x, 369.3299304675746, kMagic); // x * 256 / ln 2, rounded
  const int n = (int)(uint32_t)dbits(t);
  const double k = t - kMagic;
  const double r = fma(-k, 9.058776616587108e-20, fma(-k, 0.0027076061740622863, x));
  const int j = n & (kExpTab - 1);
  const int m = (n - j) / kExpTab;
  double q = fma(r, 1.0 / 24, 1.0 / 6);
  q = fma(r, q, 0.5);
  const double p = fma(r * r, q, r);
  const double y = fma(tab[j], p, tab[j]);
  // y * 2^m: y is near 1, the result stays normal
  return bitsd(dbits(y) + ((uint64_t)(int64_t)m << 52));
}

} // namespace emcg
