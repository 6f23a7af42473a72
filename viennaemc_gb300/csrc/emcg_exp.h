// exp(x) in double for the Poisson residual's carrier densities, by Tang's
// table-driven method (P. T. P. Tang, "Table-driven implementation of the
// exponential function in IEEE floating-point arithmetic", ACM Trans. Math.
// Softw. 15(2), 1989):
//   x = (32 m + j) ln2/32 + r,  |r| <= ln2/64,
//   exp(x) = 2^m * 2^(j/32) * (1 + p(r)),
// p the Taylor polynomial of e^r - 1 to r^6 (truncation below
// |r|^7/5040 < 4e-18 relative).  The reduction r = x - k ln2/32 takes two
// fused multiply-adds with ln2/32 split into its nearest double and the
// remainder, so r is accurate to an ulp of r.  tab[j] = 2^(j/32), j < 32.
// |x| >= 700 and NaN go to the library's exp.  The residual is evaluated in
// double precision on 16 SMs; the GPU's double-precision rate is a small
// fraction of its single-precision one, and this form takes about half the
// double instructions of a general-purpose exp.
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

EMCG_HD double expTab(double x, const double *tab) {
  if (!(fabs(x) < 700.0))
    return exp(x);
  const double k = rint(x * 46.16624130844683); // 32 / ln 2
  const double r = fma(-k, 7.247021293269686e-19, fma(-k, 0.02166084939249829, x));
  const int n = (int)k;
  const int j = n & 31;
  const int m = (n - j) / 32;
  double q = fma(r, 1.0 / 720, 1.0 / 120);
  q = fma(r, q, 1.0 / 24);
  q = fma(r, q, 1.0 / 6);
  q = fma(r, q, 0.5);
  const double p = fma(r * r, q, r);
  double y = fma(tab[j], p, tab[j]);
  uint64_t b;
  memcpy(&b, &y, sizeof b);
  b += (uint64_t)(int64_t)m << 52; // y * 2^m: y is near 1, the result stays normal
  memcpy(&y, &b, sizeof b);
  return y;
}

} // namespace emcg
