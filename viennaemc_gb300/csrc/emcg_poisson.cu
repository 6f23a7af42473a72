// Grid Poisson solver of the device engine: double-precision Newton / defect
// correction around geometric multigrid V-cycles (see emcg_poisson.cuh).
#include <algorithm>
#include <array>
#include <atomic>
#include <map>
#include <cmath>
#include <cstring>
#include <vector>

#include <cooperative_groups.h>

#include "emcg_common.cuh"
#include "emcg_exp.h"
#include "emcg_host.h"
#include "emcg_poisson.cuh"

namespace emcg {

namespace cg = cooperative_groups;

namespace {

constexpr int kBlock = 256;
constexpr double kMaxNewtonStep = 2.0; // thermal voltages per iteration

__device__ __forceinline__ void atomicMaxPos(double *addr, double v) {
  // non-negative doubles order like their bit patterns
  atomicMax(reinterpret_cast<unsigned long long *>(addr), (unsigned long long)__double_as_longlong(v));
}

__device__ __forceinline__ double blockMax(double v) {
  __shared__ double sh[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
    v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0)
    sh[w] = v;
  __syncthreads();
  if (w == 0) {
    v = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
      v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  }
  return v; // valid in thread 0
}

// Gauss-Seidel update s / (diagonal): the float smoother divides with the
// fast approximate division (its error is far below the float multigrid's own
// 1e-7), the double one exactly
__device__ __forceinline__ float mgDiv(float s, float den) { return __fdividef(s, den); }
__device__ __forceinline__ double mgDiv(double s, double den) { return s / den; }

__global__ void resetBCKernel(double *pot, const uint8_t *mask, const double *val, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && mask[i])
    pot[i] = val[i];
}

// x is finite (neither an infinity nor a NaN), by its exponent bits: no
// double-precision instruction
__device__ __forceinline__ bool finiteBits(double x) {
  return (__double2hiint(x) & 0x7ff00000) != 0x7ff00000;
}

// max of two non-negative doubles (+0 to +inf; a NaN ranks above all) by
// their bit patterns, which order like the values: integer instructions only
__device__ __forceinline__ unsigned long long bitsMax(unsigned long long a, unsigned long long b) {
  return a > b ? a : b;
}
__device__ __forceinline__ double dmaxPos(double a, double b) {
  return __longlong_as_double(
      (long long)bitsMax((unsigned long long)__double_as_longlong(a),
                         (unsigned long long)__double_as_longlong(b)));
}

// F(phi) at node i = (x, y) of the reference equation (the SOR fixed point
// of emcSORSolver.hpp:131-197 times the FV area), with p = exp(-phi) and n
// (the concentration, or exp(phi) at equilibrium).  Both solve paths call this
// one function, so they see the same values to the last bit.  Written for the
// GPU's narrow double-precision pipes: the table exp, the stencil as three
// fused multiply-adds, and the gate terms only where a gate contact is (their
// sums are zero elsewhere, and adding zero changes nothing).
struct NodeF {
  double F, p, n;
};
__device__ __forceinline__ NodeF nodeResidual(const double *__restrict__ pot,
                                              const double *__restrict__ conc,
                                              const double *__restrict__ C,
                                              const double *__restrict__ gSum,
                                              const double *__restrict__ gV, int i, int x, int y,
                                              int nx, int ny, double hF0, double hF1, double c2,
                                              double hP, const double *tab) {
  const double phi = pot[i];
  const double w = x > 0 ? pot[i - 1] : pot[i + 1];
  const double e = x < nx - 1 ? pot[i + 1] : pot[i - 1];
  const double s = y > 0 ? pot[i - nx] : pot[i + nx];
  const double nn = y < ny - 1 ? pot[i + nx] : pot[i - nx];
  const double gs = gSum[i], gv = gV[i];
  NodeF r;
  r.p = expTab(-phi, tab);
  r.n = conc ? conc[i] : expTab(phi, tab);
  double F = hF0 * (w + e);
  F = fma(hF1, s + nn, F);
  F = fma(c2, phi, F); // c2 = -2 (hF0 + hF1)
  F = fma(hP, (r.p - r.n) + C[i], F);
  if (((__double_as_longlong(gs) | __double_as_longlong(gv)) << 1) != 0)
    F += gv - gs * phi;
  r.F = F;
  return r;
}

// F(phi) of the reference equation, the Jacobian's reaction density and the
// FV-scaled right-hand side of the correction equation on level 0.
template <class MT>
__global__ void nonlinResidualKernel(const double *__restrict__ pot, const double *__restrict__ conc,
                                     const double *__restrict__ C, const uint8_t *__restrict__ fixed,
                                     const double *__restrict__ gSum, const double *__restrict__ gV,
                                     int nx, int ny, double hF0, double hF1, double hP,
                                     MT *__restrict__ rhs, MT *__restrict__ rho, MT *__restrict__ d,
                                     double *__restrict__ stats, int withScale) {
  __shared__ double tab[kExpTab]; // 2^(j/256) for expTab
  for (int k = threadIdx.x; k < kExpTab; k += blockDim.x)
    tab[k] = exp2(k * (1.0 / kExpTab));
  __syncthreads();
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  MT aF = 0;
  double sc = 0.;
  if (i < nx * ny) {
    d[i] = MT(0);
    if (fixed[i]) {
      rhs[i] = MT(0);
      rho[i] = MT(0);
    } else {
      int x = i % nx, y = i / nx;
      const NodeF q = nodeResidual(pot, conc, C, gSum, gV, i, x, y, nx, ny, hF0, hF1,
                                   -2.0 * (hF0 + hF1), hP, tab);
      const double F = q.F, p = q.p, n = q.n;
      int bd = (x == 0 || x == nx - 1) + (y == 0 || y == ny - 1);
      // the FV scale (1, 1/2, 1/4) and the maxima in the multigrid's type:
      // exact scalings, and the maximum needs no more than float accuracy
      const MT fF = (MT)F;
      rhs[i] = fF * (bd == 0 ? MT(1) : (bd == 1 ? MT(0.5) : MT(0.25)));
      rho[i] = (MT)(conc ? p : p + n);
      aF = fabs(fF);
      if (withScale)
        sc = hP * (fabs(C[i]) + n + p);
      // a NaN would vanish in the maxima (fmax drops it): a non-finite
      // residual or scale term counts as an infinite residual, which ends
      // the solve as not converged
      if (!finiteBits(F) || !finiteBits(sc) || !isfinite(fF))
        aF = INFINITY;
    }
  }
  double m1 = blockMax((double)aF);
  __syncthreads();
  double m2 = withScale ? blockMax(sc) : 0.;
  if (threadIdx.x == 0) {
    atomicMaxPos(&stats[0], m1);
    if (withScale)
      atomicMaxPos(&stats[1], m2);
  }
}

// 2^(j/256), j < 256, for expTab: the same values as the multi-launch
// residual kernel forms in its shared memory
__global__ void expTableKernel(double *tab) {
  const int k = threadIdx.x;
  if (k < kExpTab)
    tab[k] = exp2(k * (1.0 / kExpTab));
}

template <class MT>
__global__ void updatePotKernel(double *__restrict__ pot, const MT *__restrict__ d,
                                const uint8_t *__restrict__ fixed, int n, double *stats) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  MT a = 0;
  if (i < n && !fixed[i]) {
    // clamped in the correction's own type (the bound is exact in float)
    MT v = d[i];
    // the clamp would turn a NaN correction into -kMaxNewtonStep (fmax drops
    // NaN): a non-finite correction is passed on, so that the next residual
    // reports it
    if (isfinite(v))
      v = fmin(MT(kMaxNewtonStep), fmax(MT(-kMaxNewtonStep), v));
    pot[i] += (double)v;
    a = isfinite(v) ? fabs(v) : MT(INFINITY);
  }
  double m = blockMax((double)a);
  if (threadIdx.x == 0)
    atomicMaxPos(&stats[2], m);
}

template <class MT> struct LevelK {
  int nx, ny;
  const MT *cw, *ce, *cs, *cn, *area, *diag0;
  const uint8_t *fixed;
  MT *d, *r, *rho;
};

template <class MT>
__device__ __forceinline__ MT applyRow(const LevelK<MT> &L, int i, int x, int y, MT di) {
  MT s = (L.diag0[i] + L.area[i] * L.rho[i]) * di;
  if (x > 0)
    s -= L.cw[i] * L.d[i - 1];
  if (x < L.nx - 1)
    s -= L.ce[i] * L.d[i + 1];
  if (y > 0)
    s -= L.cs[i] * L.d[i - L.nx];
  if (y < L.ny - 1)
    s -= L.cn[i] * L.d[i + L.nx];
  return s;
}

template <class MT> __global__ void smoothKernel(LevelK<MT> L, int color) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  // thread t handles the t-th node of the colour
  int half = (L.nx + 1) / 2;
  int y = t / half;
  if (y >= L.ny)
    return;
  int x = 2 * (t - y * half) + ((y + color) & 1);
  if (x >= L.nx)
    return;
  int i = y * L.nx + x;
  if (L.fixed[i])
    return;
  MT s = L.r[i];
  if (x > 0)
    s += L.cw[i] * L.d[i - 1];
  if (x < L.nx - 1)
    s += L.ce[i] * L.d[i + 1];
  if (y > 0)
    s += L.cs[i] * L.d[i - L.nx];
  if (y < L.ny - 1)
    s += L.cn[i] * L.d[i + L.nx];
  L.d[i] = mgDiv(s, L.diag0[i] + L.area[i] * L.rho[i]);
}

// coarse rhs = P^T (fine residual); coarse reaction by injection; coarse d = 0
template <class MT>
__global__ void restrictKernel(LevelK<MT> F, LevelK<MT> Cc, const int *rxIdx, const float *rxW,
                               const int *ryIdx, const float *ryW, const int *mapX,
                               const int *mapY) {
  int I = blockIdx.x * blockDim.x + threadIdx.x;
  if (I >= Cc.nx * Cc.ny)
    return;
  int X = I % Cc.nx, Y = I / Cc.nx;
  Cc.d[I] = MT(0);
  Cc.rho[I] = F.rho[mapY[Y] * F.nx + mapX[X]];
  if (Cc.fixed[I]) {
    Cc.r[I] = MT(0);
    return;
  }
  MT acc = MT(0);
  for (int b = 0; b < 3; b++) {
    MT wy = (MT)ryW[3 * Y + b];
    if (wy == MT(0))
      continue;
    int y = ryIdx[3 * Y + b];
    for (int a = 0; a < 3; a++) {
      MT wx = (MT)rxW[3 * X + a];
      if (wx == MT(0))
        continue;
      int x = rxIdx[3 * X + a];
      int i = y * F.nx + x;
      if (F.fixed[i])
        continue;
      acc += wx * wy * (F.r[i] - applyRow(F, i, x, y, F.d[i]));
    }
  }
  Cc.r[I] = acc;
}

template <class MT>
__global__ void prolongKernel(LevelK<MT> F, LevelK<MT> Cc, const int *pxIdx, const float *pxW,
                              const int *pyIdx, const float *pyW) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= F.nx * F.ny || F.fixed[i])
    return;
  int x = i % F.nx, y = i / F.nx;
  int X0 = pxIdx[x], Y0 = pyIdx[y];
  MT wx = (MT)pxW[x], wy = (MT)pyW[y];
  MT v = wx * wy * Cc.d[Y0 * Cc.nx + X0];
  if (wx < MT(1))
    v += (MT(1) - wx) * wy * Cc.d[Y0 * Cc.nx + X0 + 1];
  if (wy < MT(1)) {
    v += wx * (MT(1) - wy) * Cc.d[(Y0 + 1) * Cc.nx + X0];
    if (wx < MT(1))
      v += (MT(1) - wx) * (MT(1) - wy) * Cc.d[(Y0 + 1) * Cc.nx + X0 + 1];
  }
  F.d[i] += v;
}

// coarsest level: red-black sweeps inside one block
template <class MT> __global__ void coarseSolveKernel(LevelK<MT> L, int sweeps) {
  const int n = L.nx * L.ny;
  for (int it = 0; it < sweeps; it++) {
    for (int color = 0; color < 2; color++) {
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        int x = i % L.nx, y = i / L.nx;
        if (((x + y) & 1) != color || L.fixed[i])
          continue;
        MT s = L.r[i];
        if (x > 0)
          s += L.cw[i] * L.d[i - 1];
        if (x < L.nx - 1)
          s += L.ce[i] * L.d[i + 1];
        if (y > 0)
          s += L.cs[i] * L.d[i - L.nx];
        if (y < L.ny - 1)
          s += L.cn[i] * L.d[i + L.nx];
        L.d[i] = mgDiv(s, L.diag0[i] + L.area[i] * L.rho[i]);
      }
      __syncthreads();
    }
  }
}

template <class MT> LevelK<MT> levelK(const MGLevel &l);
template <> LevelK<float> levelK<float>(const MGLevel &l) {
  return {l.nx, l.ny, l.cw, l.ce, l.cs, l.cn, l.area, l.diag0, l.fixed, l.d, l.r, l.rho};
}
template <> LevelK<double> levelK<double>(const MGLevel &l) {
  return {l.nx, l.ny, l.dcw, l.dce, l.dcs, l.dcn, l.darea, l.ddiag0, l.fixed, l.dd, l.dr, l.drho};
}

// ---------------------------------------------------------------------------
// The whole solve in one launch of one thread-block cluster.
//
// Device-engine grids hold at most a few 1e5 nodes and stay on chip, so the
// multi-launch solve is bound by launch and host-synchronisation latency (one
// V-cycle is ~90 dependent phases), not by bandwidth.  Here one cluster of up to
// 16 CTAs runs the Newton / defect-correction loop, every V-cycle and the
// convergence test, with everything a phase touches in shared memory:
//  - rows of each level are split over the CTAs in bands, aligned between
//    levels where the sizes allow (a CTA's coarse rows lie under its fine
//    rows); the correction d, right-hand side r, reaction rho and residual of
//    every level live in the owning CTA, neighbours' rows are read through
//    distributed shared memory; the double potential stays in global memory,
//    read and written only by the residual and update phases;
//  - the static coefficients are a per-node class index into a small table of
//    the level's distinct coefficient tuples; they and the transfer tables are
//    staged once per launch;
//  - levels with at most kSmallNodes nodes live whole in CTA 0, which runs the
//    coarse part of every V-cycle alone with block barriers (warp barriers on
//    levels of at most kWarpNodes, which warp 0 works alone), the coarsest
//    grid in the registers of one warp;
//  - rows in a CTA's own shared memory are addressed from the kernel's
//    shared-memory base, so their loads and stores are shared-memory
//    instructions rather than generic ones; the sweeps keep each thread's nodes
//    in registers (cSweepsHeld);
//  - phases over distributed levels are separated by cluster barriers
//    (release / acquire).
// Every phase evaluates the expressions of the corresponding multi-launch
// kernel on the same values, so both paths give the same potential.
// ---------------------------------------------------------------------------
constexpr int kClusterThreads = 512;
constexpr int kMaxCluster = 16;
constexpr int kSmallNodes = 4096;
// levels below the finest of at most this many nodes (all held by CTA 0) are
// worked by warp 0 alone, its phases ending in __syncwarp instead of a
// barrier of the whole CTA.  Measured on the 201 x 101 resistor: 64 nodes
// (8x5 and coarser) -0.3 %, 128 nodes +5 %, 512 nodes +31 % against none:
// one warp walks a larger level's nodes one after another.
constexpr int kWarpNodes = 64;
constexpr size_t kClusterSmemMax = 227 * 1024;

// q = t / d for 0 <= t and t * d < 2^32, by one wide multiply (m = ceil(2^32 / d))
struct FastDiv {
  unsigned long long m;
  __host__ void set(unsigned d) { m = ((1ull << 32) + d - 1) / d; }
  __device__ __forceinline__ int div(int t) const {
    return (int)(((unsigned long long)(unsigned)t * m) >> 32);
  }
};

template <class MT> struct CLevel {
  int nx, ny, small, rowsPer; // small: all rows in CTA 0; else rowsPer rows per CTA
  int nCls, ncx, ncy, warp;   // ncx, ncy: next level's size (0 on the coarsest);
                              // warp: worked by warp 0 of CTA 0 alone
  FastDiv byNx, byHalf, byRows; // nx, (nx + 1) / 2 and rowsPer
  // byte offsets in dynamic shared memory: this CTA's rows of d, r, rho, the
  // residual and the class index, the class table (8 MT per class) and the
  // transfer tables to the next level (prolongation index / weight per fine x
  // and y, restriction 3 per coarse index, injection map)
  unsigned offD, offR, offRho, offRes, offCls, offTab;
  unsigned offPxI, offPxW, offPyI, offPyW, offRxI, offRxW, offRyI, offRyW, offMapX, offMapY;
  const uint8_t *cls; // global sources staged at launch
  const MT *tab;
  const int *rxIdx, *ryIdx, *pxIdx, *pyIdx, *mapX, *mapY;
  const float *rxW, *ryW, *pxW, *pyW;
};

template <class MT> struct CMG {
  int nLev, pre, post, coarseSweeps, firstSmall, vcycles;
  double twoCycleRel;
  unsigned offRed;
  CLevel<MT> L[16];
};

struct CCtx {
  char *const *base; // generic address of each rank's dynamic shared memory
  char *smem;        // this CTA's dynamic shared memory
  int rank;
};

template <class MT> struct Coef {
  MT cw, ce, cs, cn, area, diag0, fixed, pad;
};

template <class MT> __device__ __forceinline__ Coef<MT> loadCoef(const MT *K);
template <> __device__ __forceinline__ Coef<float> loadCoef<float>(const float *K) {
  const float4 a = reinterpret_cast<const float4 *>(K)[0];
  const float4 b = reinterpret_cast<const float4 *>(K)[1];
  return {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
}
template <> __device__ __forceinline__ Coef<double> loadCoef<double>(const double *K) {
  const double2 a = reinterpret_cast<const double2 *>(K)[0];
  const double2 b = reinterpret_cast<const double2 *>(K)[1];
  const double2 e = reinterpret_cast<const double2 *>(K)[2];
  const double2 f = reinterpret_cast<const double2 *>(K)[3];
  return {a.x, a.y, b.x, b.y, e.x, e.y, f.x, f.y};
}

// rows [r0, r1) of level L held by this CTA
template <class MT>
__device__ __forceinline__ void cOwnRows(const CCtx &c, const CLevel<MT> &L, int &r0, int &r1) {
  if (L.small) {
    r0 = 0;
    r1 = c.rank == 0 ? L.ny : 0;
  } else {
    r0 = min(L.ny, c.rank * L.rowsPer);
    r1 = min(L.ny, r0 + L.rowsPer);
  }
}

// row y of an array of level L, wherever it lives
template <class T, class MT>
__device__ __forceinline__ T *cRow(const CCtx &c, const CLevel<MT> &L, unsigned off, int y) {
  if (L.small)
    return reinterpret_cast<T *>((c.rank == 0 ? c.smem : c.base[0]) + off) + (size_t)y * L.nx;
  const int owner = L.byRows.div(y);
  return reinterpret_cast<T *>((owner == c.rank ? c.smem : c.base[owner]) + off) +
         (size_t)(y - owner * L.rowsPer) * L.nx;
}

// row r0 + ly of level L, for this CTA's rows and their neighbours
template <class T, class MT>
__device__ __forceinline__ T *cRowNear(const CCtx &c, const CLevel<MT> &L, unsigned off, int ly) {
  if (L.small || (ly >= 0 && ly < L.rowsPer))
    return reinterpret_cast<T *>(c.smem + off) + (size_t)ly * L.nx;
  if (ly < 0)
    return reinterpret_cast<T *>(c.base[c.rank - 1] + off) + (size_t)(L.rowsPer - 1) * L.nx;
  return reinterpret_cast<T *>(c.base[c.rank + 1] + off);
}

template <class T> __device__ __forceinline__ const T *cTab(const CCtx &c, unsigned off) {
  return reinterpret_cast<const T *>(c.smem + off);
}

template <class MT>
__device__ __forceinline__ Coef<MT> cCoef(const CCtx &c, const CLevel<MT> &L, uint8_t k) {
  return loadCoef<MT>(reinterpret_cast<const MT *>(c.smem + L.offTab) + 8 * k);
}

// end of a phase over level L: cluster barrier for a distributed level, block
// barrier for one held by CTA 0, warp barrier for one worked by warp 0
template <class MT> __device__ __forceinline__ void cSync(const CLevel<MT> &L) {
  if (L.warp)
    __syncwarp();
  else if (L.small)
    __syncthreads();
  else
    cg::this_cluster().sync();
}

// threads that take no part in a phase over level L (warp-level levels: all
// but warp 0), and the stride of the threads that do
template <class MT> __device__ __forceinline__ bool cIdle(const CLevel<MT> &L) {
  return L.warp && threadIdx.x >= 32;
}
template <class MT> __device__ __forceinline__ int cStride(const CLevel<MT> &L) {
  return L.warp ? 32 : (int)blockDim.x;
}

// row accessors of a phase; kS: the row is in this CTA's shared memory (its
// own rows, or any row of a level held whole by CTA 0 in a phase that runs
// there), so the accesses compile to shared-memory loads and stores rather
// than generic ones
template <bool kS, class T, class MT>
__device__ __forceinline__ T *cRowT(const CCtx &c, const CLevel<MT> &L, unsigned off, int y) {
  if (kS)
    return reinterpret_cast<T *>(c.smem + off) + (size_t)y * L.nx;
  return cRow<T>(c, L, off, y);
}
template <bool kS, class T, class MT>
__device__ __forceinline__ T *cRowNearT(const CCtx &c, const CLevel<MT> &L, unsigned off, int ly) {
  if (kS)
    return reinterpret_cast<T *>(c.smem + off) + (size_t)ly * L.nx;
  return cRowNear<T>(c, L, off, ly);
}

template <bool kS, class MT>
__device__ __forceinline__ void cSmoothT(const CCtx &c, const CLevel<MT> &L, int color) {
  int r0, r1;
  cOwnRows(c, L, r0, r1);
  const int half = (L.nx + 1) / 2, cnt = half * (r1 - r0), stride = cStride(L);
  for (int t = threadIdx.x; t < cnt; t += stride) {
    const int ly = L.byHalf.div(t), y = r0 + ly;
    const int x = 2 * (t - ly * half) + ((y + color) & 1);
    if (x >= L.nx)
      continue;
    // row ly is this CTA's own; its neighbours are too, but at a band edge
    const Coef<MT> K = cCoef(c, L, cRowNearT<true, uint8_t>(c, L, L.offCls, ly)[x]);
    if (K.fixed != MT(0))
      continue;
    MT *d = cRowNearT<true, MT>(c, L, L.offD, ly);
    MT s = cRowNearT<true, MT>(c, L, L.offR, ly)[x];
    if (x > 0)
      s += K.cw * d[x - 1];
    if (x < L.nx - 1)
      s += K.ce * d[x + 1];
    if (y > 0)
      s += K.cs * (kS || ly > 0 ? cRowNearT<true, MT>(c, L, L.offD, ly - 1)[x]
                                : cRowNearT<false, MT>(c, L, L.offD, ly - 1)[x]);
    if (y < L.ny - 1)
      s += K.cn * (kS || ly + 1 < L.rowsPer ? cRowNearT<true, MT>(c, L, L.offD, ly + 1)[x]
                                            : cRowNearT<false, MT>(c, L, L.offD, ly + 1)[x]);
    d[x] = mgDiv(s, K.diag0 + K.area * cRowNearT<true, MT>(c, L, L.offRho, ly)[x]);
  }
}
template <class MT> __device__ void cSmooth(const CCtx &c, const CLevel<MT> &Lr, int color) {
  const CLevel<MT> L = Lr; // a private copy: stores to shared memory cannot alias it
  if (cIdle(L))
    return;
  if (L.small)
    cSmoothT<true>(c, L, color);
  else
    cSmoothT<false>(c, L, color);
  cSync(L);
}

// Several red-black sweeps over level L with each thread's nodes held in
// registers: a thread keeps the same nodes over the sweeps, so their position,
// class, right-hand side and diagonal are read once, and a half sweep reads
// only the neighbours' corrections.  The arithmetic is cSmoothT's.
//
// kSweepNodes: nodes of one colour per thread.  Six, for the 2,814-node bands
// of a 401 x 201 grid, spilled registers: 0.5 % faster there, 1.4 % slower on
// 201 x 101.
constexpr int kSweepNodes = 3;
template <bool kS, int K, class MT>
__device__ __forceinline__ void cHalfSweep(const CCtx &c, const CLevel<MT> &L, int r0,
                                           const int (&pos)[2][kSweepNodes],
                                           const int (&cl)[2][kSweepNodes],
                                           const MT (&rr)[2][kSweepNodes],
                                           const MT (&den)[2][kSweepNodes]) {
#pragma unroll
  for (int j = 0; j < kSweepNodes; j++) {
    if (pos[K][j] < 0)
      continue;
    const int ly = pos[K][j] >> 16, x = pos[K][j] & 0xffff, y = r0 + ly;
    const Coef<MT> C = cCoef(c, L, cl[K][j]);
    MT *d = cRowNearT<true, MT>(c, L, L.offD, ly);
    MT s = rr[K][j];
    if (x > 0)
      s += C.cw * d[x - 1];
    if (x < L.nx - 1)
      s += C.ce * d[x + 1];
    if (y > 0)
      s += C.cs * (kS || ly > 0 ? cRowNearT<true, MT>(c, L, L.offD, ly - 1)[x]
                                : cRowNearT<false, MT>(c, L, L.offD, ly - 1)[x]);
    if (y < L.ny - 1)
      s += C.cn * (kS || ly + 1 < L.rowsPer ? cRowNearT<true, MT>(c, L, L.offD, ly + 1)[x]
                                            : cRowNearT<false, MT>(c, L, L.offD, ly + 1)[x]);
    d[x] = mgDiv(s, den[K][j]);
  }
  cSync(L);
}

// residual r - A d at the held nodes of colour K (cResidualT's arithmetic;
// the Dirichlet nodes' zeros are written once, at the start of the launch)
template <bool kS, int K, class MT>
__device__ __forceinline__ void cResidualHeld(const CCtx &c, const CLevel<MT> &L, int r0,
                                              const int (&pos)[2][kSweepNodes],
                                              const int (&cl)[2][kSweepNodes],
                                              const MT (&rr)[2][kSweepNodes],
                                              const MT (&den)[2][kSweepNodes]) {
#pragma unroll
  for (int j = 0; j < kSweepNodes; j++) {
    if (pos[K][j] < 0)
      continue;
    const int ly = pos[K][j] >> 16, x = pos[K][j] & 0xffff, y = r0 + ly;
    const Coef<MT> C = cCoef(c, L, cl[K][j]);
    const MT *d = cRowNearT<true, MT>(c, L, L.offD, ly);
    MT a = den[K][j] * d[x];
    if (x > 0)
      a -= C.cw * d[x - 1];
    if (x < L.nx - 1)
      a -= C.ce * d[x + 1];
    if (y > 0)
      a -= C.cs * (kS || ly > 0 ? cRowNearT<true, MT>(c, L, L.offD, ly - 1)[x]
                                : cRowNearT<false, MT>(c, L, L.offD, ly - 1)[x]);
    if (y < L.ny - 1)
      a -= C.cn * (kS || ly + 1 < L.rowsPer ? cRowNearT<true, MT>(c, L, L.offD, ly + 1)[x]
                                            : cRowNearT<false, MT>(c, L, L.offD, ly + 1)[x]);
    cRowNearT<true, MT>(c, L, L.offRes, ly)[x] = rr[K][j] - a;
  }
}

template <bool kS, class MT>
__device__ __forceinline__ void cSweepsHeld(const CCtx &c, const CLevel<MT> &L, int r0, int r1,
                                            int sweeps, int first, bool residual) {
  const int half = (L.nx + 1) / 2, cnt = half * (r1 - r0), stride = cStride(L);
  int pos[2][kSweepNodes], cl[2][kSweepNodes];
  MT rr[2][kSweepNodes], den[2][kSweepNodes];
#pragma unroll
  for (int k = 0; k < 2; k++) {
#pragma unroll
    for (int j = 0; j < kSweepNodes; j++) {
      pos[k][j] = -1;
      cl[k][j] = 0;
      rr[k][j] = MT(0);
      den[k][j] = MT(1);
      const int t = threadIdx.x + j * stride;
      if (t >= cnt)
        continue;
      const int ly = L.byHalf.div(t), y = r0 + ly;
      const int x = 2 * (t - ly * half) + ((y + k) & 1);
      if (x >= L.nx)
        continue;
      const int q = cRowNearT<true, uint8_t>(c, L, L.offCls, ly)[x];
      const Coef<MT> K = cCoef(c, L, q);
      if (K.fixed != MT(0))
        continue;
      pos[k][j] = (ly << 16) | x;
      cl[k][j] = q;
      rr[k][j] = cRowNearT<true, MT>(c, L, L.offR, ly)[x];
      den[k][j] = K.diag0 + K.area * cRowNearT<true, MT>(c, L, L.offRho, ly)[x];
    }
  }
  for (int s = 0; s < sweeps; s++) {
    if (first == 0) {
      cHalfSweep<kS, 0>(c, L, r0, pos, cl, rr, den);
      cHalfSweep<kS, 1>(c, L, r0, pos, cl, rr, den);
    } else {
      cHalfSweep<kS, 1>(c, L, r0, pos, cl, rr, den);
      cHalfSweep<kS, 0>(c, L, r0, pos, cl, rr, den);
    }
  }
  if (residual) {
    cResidualHeld<kS, 0>(c, L, r0, pos, cl, rr, den);
    cResidualHeld<kS, 1>(c, L, r0, pos, cl, rr, den);
    cSync(L);
  }
}

// `sweeps` red-black sweeps over level L, colour `first` first, then (residual)
// the residual of the correction equation; every CTA passes the same
// 2 * sweeps (+ 1) barriers whichever form its rows take
template <class MT>
__device__ void cSmoothSweeps(const CCtx &c, const CLevel<MT> &Lr, int sweeps, int first,
                              bool residual = false) {
  const CLevel<MT> L = Lr;
  if (cIdle(L))
    return;
  int r0, r1;
  cOwnRows(c, L, r0, r1);
  const int cnt = (L.nx + 1) / 2 * (r1 - r0);
  if (cnt <= kSweepNodes * cStride(L) && L.nx <= 0xffff && r1 - r0 <= 0x7fff) {
    if (L.small)
      cSweepsHeld<true>(c, L, r0, r1, sweeps, first, residual);
    else
      cSweepsHeld<false>(c, L, r0, r1, sweeps, first, residual);
    return;
  }
  for (int s = 0; s < sweeps; s++) {
    cSmooth(c, L, first);
    cSmooth(c, L, 1 - first);
  }
  if (residual)
    cResidual(c, L);
}

// residual r - A d of the correction equation at this CTA's nodes of level F
// (0 at Dirichlet nodes), as restrictKernel evaluates it
template <bool kS, class MT>
__device__ __forceinline__ void cResidualT(const CCtx &c, const CLevel<MT> &F) {
  int r0, r1;
  cOwnRows(c, F, r0, r1);
  const int cnt = F.nx * (r1 - r0), stride = cStride(F);
  for (int t = threadIdx.x; t < cnt; t += stride) {
    const int ly = F.byNx.div(t), y = r0 + ly, x = t - ly * F.nx;
    const Coef<MT> K = cCoef(c, F, cRowNearT<true, uint8_t>(c, F, F.offCls, ly)[x]);
    MT res = MT(0);
    if (K.fixed == MT(0)) {
      const MT *d = cRowNearT<true, MT>(c, F, F.offD, ly);
      MT a = (K.diag0 + K.area * cRowNearT<true, MT>(c, F, F.offRho, ly)[x]) * d[x];
      if (x > 0)
        a -= K.cw * d[x - 1];
      if (x < F.nx - 1)
        a -= K.ce * d[x + 1];
      if (y > 0)
        a -= K.cs * (kS || ly > 0 ? cRowNearT<true, MT>(c, F, F.offD, ly - 1)[x]
                                  : cRowNearT<false, MT>(c, F, F.offD, ly - 1)[x]);
      if (y < F.ny - 1)
        a -= K.cn * (kS || ly + 1 < F.rowsPer ? cRowNearT<true, MT>(c, F, F.offD, ly + 1)[x]
                                              : cRowNearT<false, MT>(c, F, F.offD, ly + 1)[x]);
      res = cRowNearT<true, MT>(c, F, F.offR, ly)[x] - a;
    }
    cRowNearT<true, MT>(c, F, F.offRes, ly)[x] = res;
  }
}
template <class MT> __device__ void cResidual(const CCtx &c, const CLevel<MT> &Fr) {
  const CLevel<MT> F = Fr;
  if (cIdle(F))
    return;
  if (F.small)
    cResidualT<true>(c, F);
  else
    cResidualT<false>(c, F);
  cSync(F);
}

// coarse rows whose injection row mapY[Y] this CTA holds: [Y0, Y1)
template <class MT>
__device__ __forceinline__ void cRestrictRows(const CCtx &c, const CLevel<MT> &F,
                                              const CLevel<MT> &Cc, int &Y0, int &Y1) {
  int r0, r1;
  cOwnRows(c, F, r0, r1);
  if (r0 >= r1) {
    Y0 = Y1 = 0;
    return;
  }
  if (F.ny <= 3) { // not coarsened along y: identity map
    Y0 = r0;
    Y1 = r1;
    return;
  }
  Y0 = (r0 + 1) / 2;
  Y1 = r1 == F.ny ? Cc.ny : min(Cc.ny, (r1 + 1) / 2);
}

// coarse right-hand side P^T (fine residual), reaction by injection, d = 0
template <bool kS, class MT>
__device__ __forceinline__ void cRestrictT(const CCtx &c, const CLevel<MT> &F,
                                        const CLevel<MT> &Cc) {
  int Y0, Y1;
  cRestrictRows(c, F, Cc, Y0, Y1);
  const int cnt = Cc.nx * (Y1 - Y0), stride = cStride(F);
  for (int t = threadIdx.x; t < cnt; t += stride) {
    const int q = Cc.byNx.div(t), Y = Y0 + q, X = t - q * Cc.nx;
    cRowT<kS, MT>(c, Cc, Cc.offD, Y)[X] = MT(0);
    cRowT<kS, MT>(c, Cc, Cc.offRho, Y)[X] =
        cRowT<kS, MT>(c, F, F.offRho, cTab<int>(c, F.offMapY)[Y])[cTab<int>(c, F.offMapX)[X]];
    const Coef<MT> KC = cCoef(c, Cc, cRowT<kS, uint8_t>(c, Cc, Cc.offCls, Y)[X]);
    MT acc = MT(0);
    if (KC.fixed == MT(0)) {
      MT wxs[3];
      int xs[3];
#pragma unroll
      for (int k = 0; k < 3; k++) {
        wxs[k] = (MT)cTab<float>(c, F.offRxW)[3 * X + k];
        xs[k] = cTab<int>(c, F.offRxI)[3 * X + k];
      }
#pragma unroll
      for (int b = 0; b < 3; b++) {
        const MT wy = (MT)cTab<float>(c, F.offRyW)[3 * Y + b];
        if (wy == MT(0))
          continue;
        const MT *res = cRowT<kS, MT>(c, F, F.offRes, cTab<int>(c, F.offRyI)[3 * Y + b]);
#pragma unroll
        for (int a = 0; a < 3; a++) {
          if (wxs[a] == MT(0))
            continue;
          acc += wxs[a] * wy * res[xs[a]];
        }
      }
    }
    cRowT<kS, MT>(c, Cc, Cc.offR, Y)[X] = acc;
  }
}
template <class MT>
__device__ void cRestrict(const CCtx &c, const CLevel<MT> &Fr, const CLevel<MT> &Cr) {
  const CLevel<MT> F = Fr, Cc = Cr;
  if (cIdle(F))
    return;
  if (F.small)
    cRestrictT<true>(c, F, Cc);
  else
    cRestrictT<false>(c, F, Cc);
  cSync(F);
}

template <bool kS, class MT>
__device__ __forceinline__ void cProlongT(const CCtx &c, const CLevel<MT> &F,
                                        const CLevel<MT> &Cc) {
  int r0, r1;
  cOwnRows(c, F, r0, r1);
  const int cnt = F.nx * (r1 - r0), stride = cStride(F);
  for (int t = threadIdx.x; t < cnt; t += stride) {
    const int ly = F.byNx.div(t), y = r0 + ly, x = t - ly * F.nx;
    if (cCoef(c, F, cRowNearT<true, uint8_t>(c, F, F.offCls, ly)[x]).fixed != MT(0))
      continue;
    const int X0 = cTab<int>(c, F.offPxI)[x], Y0 = cTab<int>(c, F.offPyI)[y];
    const MT wx = (MT)cTab<float>(c, F.offPxW)[x], wy = (MT)cTab<float>(c, F.offPyW)[y];
    const MT *c0 = cRowT<kS, MT>(c, Cc, Cc.offD, Y0);
    MT v = wx * wy * c0[X0];
    if (wx < MT(1))
      v += (MT(1) - wx) * wy * c0[X0 + 1];
    if (wy < MT(1)) {
      const MT *c1 = cRowT<kS, MT>(c, Cc, Cc.offD, Y0 + 1);
      v += wx * (MT(1) - wy) * c1[X0];
      if (wx < MT(1))
        v += (MT(1) - wx) * (MT(1) - wy) * c1[X0 + 1];
    }
    cRowNearT<true, MT>(c, F, F.offD, ly)[x] += v;
  }
}
template <class MT>
__device__ void cProlong(const CCtx &c, const CLevel<MT> &Fr, const CLevel<MT> &Cr) {
  const CLevel<MT> F = Fr, Cc = Cr;
  if (cIdle(F))
    return;
  if (F.small)
    cProlongT<true>(c, F, Cc);
  else
    cProlongT<false>(c, F, Cc);
  cSync(F);
}

// coarsest level (held by CTA 0): red-black sweeps, in the registers of warp 0
// when it has at most 32 nodes, else by the threads of the level (warp 0 or the
// block) with their barriers
template <class MT> __device__ void cCoarse(const CCtx &c, const CLevel<MT> &L, int sweeps) {
  if (cIdle(L))
    return;
  const int n = L.nx * L.ny;
  if (n <= 32) {
    if (threadIdx.x < 32) {
      const int i = threadIdx.x, x = i % L.nx, y = i / L.nx;
      const bool live = i < n;
      const Coef<MT> K = cCoef(c, L, live ? cRowT<true, uint8_t>(c, L, L.offCls, y)[x] : 0);
      MT *dp = live ? cRowT<true, MT>(c, L, L.offD, y) + x : nullptr;
      const MT r = live ? cRowT<true, MT>(c, L, L.offR, y)[x] : MT(0);
      const MT den = live ? K.diag0 + K.area * cRowT<true, MT>(c, L, L.offRho, y)[x] : MT(1);
      const bool upd = live && K.fixed == MT(0);
      MT d = live ? *dp : MT(0);
      for (int it = 0; it < sweeps; it++) {
        for (int color = 0; color < 2; color++) {
          const MT dw = __shfl_sync(0xffffffffu, d, (i + 31) & 31);
          const MT de = __shfl_sync(0xffffffffu, d, (i + 1) & 31);
          const MT ds = __shfl_sync(0xffffffffu, d, (i - L.nx + 32) & 31);
          const MT dn = __shfl_sync(0xffffffffu, d, (i + L.nx) & 31);
          if (upd && ((x + y) & 1) == color) {
            MT s = r;
            if (x > 0)
              s += K.cw * dw;
            if (x < L.nx - 1)
              s += K.ce * de;
            if (y > 0)
              s += K.cs * ds;
            if (y < L.ny - 1)
              s += K.cn * dn;
            d = mgDiv(s, den);
          }
        }
      }
      if (live)
        *dp = d;
    }
    cSync(L);
    return;
  }
  const int stride = cStride(L);
  for (int it = 0; it < sweeps; it++) {
    for (int color = 0; color < 2; color++) {
      for (int i = threadIdx.x; i < n; i += stride) {
        const int x = i % L.nx, y = i / L.nx;
        const Coef<MT> K = cCoef(c, L, cRowT<true, uint8_t>(c, L, L.offCls, y)[x]);
        if (((x + y) & 1) != color || K.fixed != MT(0))
          continue;
        MT *d = cRowT<true, MT>(c, L, L.offD, y);
        MT s = cRowT<true, MT>(c, L, L.offR, y)[x];
        if (x > 0)
          s += K.cw * d[x - 1];
        if (x < L.nx - 1)
          s += K.ce * d[x + 1];
        if (y > 0)
          s += K.cs * cRowT<true, MT>(c, L, L.offD, y - 1)[x];
        if (y < L.ny - 1)
          s += K.cn * cRowT<true, MT>(c, L, L.offD, y + 1)[x];
        d[x] = mgDiv(s, K.diag0 + K.area * cRowT<true, MT>(c, L, L.offRho, y)[x]);
      }
      cSync(L);
    }
  }
}

// max over the block, then over the cluster (every thread of every CTA gets it);
// each CTA's two block maxima sit at byte offset offRed of its shared memory
__device__ __forceinline__ void cClusterMax2(const CCtx &c, unsigned offRed, double &a,
                                             double &b, double *sh) {
  // non-negative values: maxima of their bit patterns (integer instructions;
  // the double-precision pipes are narrow)
  unsigned long long ua = (unsigned long long)__double_as_longlong(a) & ~(1ull << 63);
  unsigned long long ub = (unsigned long long)__double_as_longlong(b) & ~(1ull << 63);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    ua = bitsMax(ua, __shfl_xor_sync(0xffffffffu, ua, o));
    ub = bitsMax(ub, __shfl_xor_sync(0xffffffffu, ub, o));
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nW = (int)(blockDim.x >> 5);
  unsigned long long *shu = reinterpret_cast<unsigned long long *>(sh);
  if (lane == 0) {
    shu[2 * w] = ua;
    shu[2 * w + 1] = ub;
  }
  __syncthreads();
  if (w == 0) {
    ua = lane < nW ? shu[2 * lane] : 0ull;
    ub = lane < nW ? shu[2 * lane + 1] : 0ull;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      ua = bitsMax(ua, __shfl_xor_sync(0xffffffffu, ua, o));
      ub = bitsMax(ub, __shfl_xor_sync(0xffffffffu, ub, o));
    }
    if (lane == 0) {
      unsigned long long *red = reinterpret_cast<unsigned long long *>(c.smem + offRed);
      red[0] = ua;
      red[1] = ub;
    }
  }
  cg::this_cluster().sync();
  // every warp: lane r reads rank r's maxima, then the warp reduces them
  const int ranks = (int)cg::this_cluster().num_blocks();
  ua = 0ull;
  ub = 0ull;
  for (int r = lane; r < ranks; r += 32) {
    const unsigned long long *o =
        reinterpret_cast<const unsigned long long *>(c.base[r] + offRed);
    ua = bitsMax(ua, o[0]);
    ub = bitsMax(ub, o[1]);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    ua = bitsMax(ua, __shfl_xor_sync(0xffffffffu, ua, o));
    ub = bitsMax(ub, __shfl_xor_sync(0xffffffffu, ub, o));
  }
  a = __longlong_as_double((long long)ua);
  b = __longlong_as_double((long long)ub);
}

// out[0] = final relative residual, out[1] = Newton steps done, out[2] = 1 if the
// update rule stopped the solve
template <class MT>
__global__ void __launch_bounds__(kClusterThreads, 1)
    poissonClusterKernel(CMG<MT> Mp, double *__restrict__ pot, const double *__restrict__ conc,
                         const double *__restrict__ C, const double *__restrict__ gSum,
                         const double *__restrict__ gV, double hF0, double hF1, double hP,
                         double rtol, int maxCycles, double updTol,
                         const double *__restrict__ expG, double *__restrict__ out) {
  extern __shared__ __align__(16) char smem[];
  __shared__ char *sBase[kMaxCluster];
  __shared__ double sh[2 * (kClusterThreads / 32)];
  // the level descriptors, read by every phase, from shared memory rather than
  // the parameter bank
  __shared__ __align__(16) int sM[sizeof(CMG<MT>) / sizeof(int)];
  __shared__ __align__(16) double sExp[kExpTab]; // 2^(j/256) for expTab
  // Staging.  Every table goes by asynchronous copies, all in flight at once
  // (a plain copy loop per table waited for each table's loads in turn: 20 us
  // per launch), in two groups: the exp table and level 0's coefficient
  // classes, which the first residual needs, and then the rest, which lands
  // while the first residual runs (it is first needed by the V-cycle).
  const unsigned sBaseAddr = (unsigned)__cvta_generic_to_shared(smem);
  {
    const unsigned a = (unsigned)__cvta_generic_to_shared(sExp);
    for (int k = threadIdx.x; k < kExpTab / 2; k += blockDim.x)
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(a + 16u * k),
                   "l"(expG + 2 * k)
                   : "memory");
  }
  for (int k = threadIdx.x; k < (int)(sizeof(CMG<MT>) / sizeof(int)); k += blockDim.x)
    sM[k] = reinterpret_cast<const int *>(&Mp)[k];
  __syncthreads();
  const CMG<MT> &M = *reinterpret_cast<const CMG<MT> *>(sM);
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank(), ranks = (int)cluster.num_blocks();
  if (threadIdx.x < ranks)
    sBase[threadIdx.x] = static_cast<char *>(cluster.map_shared_rank((void *)smem, threadIdx.x));
  auto stage = [&](unsigned off, const void *src, int n) {
    const int *sp = static_cast<const int *>(src);
    for (int k = threadIdx.x; k < n; k += blockDim.x)
      asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(sBaseAddr + off + 4u * k),
                   "l"(sp + k)
                   : "memory");
  };
  int clsEnd[16]; // prefix sums of this CTA's class bytes per level
  {
    int nCls = 0;
    for (int l = 0; l < M.nLev; l++) {
      const CLevel<MT> &L = M.L[l];
      int r0, r1;
      cOwnRows(CCtx{sBase, smem, rank}, L, r0, r1);
      nCls += L.nx * (r1 - r0);
      clsEnd[l] = nCls;
    }
  }
  stage(M.L[0].offTab, M.L[0].tab, 8 * M.L[0].nCls * (int)(sizeof(MT) / 4));
  asm volatile("cp.async.commit_group;" ::: "memory");
  for (int l = 0; l < M.nLev; l++) {
    const CLevel<MT> &L = M.L[l];
    if (l > 0)
      stage(L.offTab, L.tab, 8 * L.nCls * (int)(sizeof(MT) / 4));
    if (L.ncx > 0) {
      stage(L.offPxI, L.pxIdx, L.nx);
      stage(L.offPxW, L.pxW, L.nx);
      stage(L.offPyI, L.pyIdx, L.ny);
      stage(L.offPyW, L.pyW, L.ny);
      stage(L.offRxI, L.rxIdx, 3 * L.ncx);
      stage(L.offRxW, L.rxW, 3 * L.ncx);
      stage(L.offRyI, L.ryIdx, 3 * L.ncy);
      stage(L.offRyW, L.ryW, 3 * L.ncy);
      stage(L.offMapX, L.mapX, L.ncx);
      stage(L.offMapY, L.mapY, L.ncy);
    }
  }
  asm volatile("cp.async.commit_group;" ::: "memory");
  // this CTA's class bytes of the levels [clsEnd[l0 - 1], clsEnd[l1 - 1]), four
  // bytes per thread and pass: the loads first, then the stores
  auto copyCls = [&](int l0, int l1) {
    const int begin = l0 > 0 ? clsEnd[l0 - 1] : 0, end = clsEnd[l1 - 1];
    for (int t0 = begin + (int)threadIdx.x; t0 < end; t0 += 4 * blockDim.x) {
      uint8_t v[4];
      uint8_t *dst[4];
#pragma unroll
      for (int j = 0; j < 4; j++) {
        const int t = t0 + j * (int)blockDim.x;
        dst[j] = nullptr;
        if (t < end) {
          int l = l0;
          while (t >= clsEnd[l])
            l++;
          const CLevel<MT> &L = M.L[l];
          const int k = t - (l > 0 ? clsEnd[l - 1] : 0);
          const int r0 = L.small ? 0 : min(L.ny, rank * L.rowsPer);
          v[j] = L.cls[(size_t)r0 * L.nx + k];
          dst[j] = reinterpret_cast<uint8_t *>(smem + L.offCls) + k;
        }
      }
#pragma unroll
      for (int j = 0; j < 4; j++)
        if (dst[j])
          *dst[j] = v[j];
    }
  };
  copyCls(0, 1);
  asm volatile("cp.async.wait_group 1;" ::: "memory"); // the exp table and level 0's classes
  __syncthreads();
  // (no cluster barrier yet: the first access to another CTA's shared memory
  // comes after the cluster barrier of the first residual's maxima)
  CCtx c{sBase, smem, rank};
  const CLevel<MT> &L0 = M.L[0];
  const int nx = L0.nx, ny = L0.ny;
  int p0, p1;
  cOwnRows(c, L0, p0, p1);
  const int nOwn = nx * (p1 - p0);
  double rel = INFINITY, scale = 0.;
  int it = 0;
  bool stopped = false;
  const double c2 = -2.0 * (hF0 + hF1);
  for (;; it++) {
    // F(phi), Jacobian reaction and FV-scaled right-hand side (nonlinResidualKernel);
    // the scale of the relative residual from the first iteration's state
    MT aFm = 0;
    double sc = 0.;
    for (int t = threadIdx.x; t < nOwn; t += blockDim.x) {
      const int ly = L0.byNx.div(t), y = p0 + ly, x = t - ly * nx, i = y * nx + x;
      MT *d0 = cRowNearT<true, MT>(c, L0, L0.offD, ly);
      MT *r0 = cRowNearT<true, MT>(c, L0, L0.offR, ly);
      MT *rho0 = cRowNearT<true, MT>(c, L0, L0.offRho, ly);
      d0[x] = MT(0);
      if (cCoef(c, L0, cRowNearT<true, uint8_t>(c, L0, L0.offCls, ly)[x]).fixed != MT(0)) {
        r0[x] = MT(0);
        rho0[x] = MT(0);
        continue;
      }
      const NodeF q =
          nodeResidual(pot, conc, C, gSum, gV, i, x, y, nx, ny, hF0, hF1, c2, hP, sExp);
      const double F = q.F, p = q.p, n = q.n;
      const int bd = (x == 0 || x == nx - 1) + (y == 0 || y == ny - 1);
      const MT fF = (MT)F;
      r0[x] = fF * (bd == 0 ? MT(1) : (bd == 1 ? MT(0.5) : MT(0.25)));
      rho0[x] = (MT)(conc ? p : p + n);
      aFm = fmax(aFm, fabs(fF));
      if (it == 0)
        sc = dmaxPos(sc, hP * (fabs(C[i]) + n + p));
      // a NaN would vanish in the maxima: non-finite values count as an
      // infinite residual, which ends the solve as not converged
      if (!finiteBits(F) || !finiteBits(p) || !finiteBits(n) || !isfinite(fF))
        aFm = MT(INFINITY);
    }
    if (it == 0) {
      // the rest of the staging: the class bytes of the other levels, zero
      // residuals (Dirichlet nodes keep them), the asynchronous copies; the
      // barriers of the maxima below make them visible
      copyCls(1, M.nLev);
      for (int l = 0; l + 1 < M.nLev; l++) {
        const CLevel<MT> &L = M.L[l];
        int r0, r1;
        cOwnRows(c, L, r0, r1);
        MT *res = reinterpret_cast<MT *>(smem + L.offRes);
        for (int k = threadIdx.x; k < L.nx * (r1 - r0); k += blockDim.x)
          res[k] = MT(0);
      }
      asm volatile("cp.async.wait_group 0;" ::: "memory");
    }
    double aF = (double)aFm;
    // its cluster barrier also orders the writes above; the maxima are next
    // written after the V-cycle's barriers, when every CTA has read them
    cClusterMax2(c, M.offRed, aF, sc, sh);
    if (it == 0)
      scale = sc;
    rel = scale > 0 ? aF / scale : aF;
    if (rel <= rtol || it == maxCycles || !isfinite(rel))
      break;
    // under the update-size rule a Newton step needs only a rough correction
    const int nv = updTol <= 0. && rel < M.twoCycleRel ? M.vcycles : 1;
    for (int vc = 0; vc < nv; vc++) {
      // one V-cycle: the distributed levels down ...
      const int Ls = M.firstSmall;
      for (int l = 0; l < Ls; l++) {
        cSmoothSweeps(c, M.L[l], M.pre, 0, true);
        cRestrict(c, M.L[l], M.L[l + 1]);
      }
      // ... the levels held by CTA 0 ...
      if (rank == 0) {
        for (int l = Ls; l + 1 < M.nLev; l++) {
          cSmoothSweeps(c, M.L[l], M.pre, 0, true);
          cRestrict(c, M.L[l], M.L[l + 1]);
        }
        cCoarse(c, M.L[M.nLev - 1], M.coarseSweeps);
        for (int l = M.nLev - 2; l >= Ls; l--) {
          // the CTA reads what warp 0 wrote on the level below
          if (M.L[l + 1].warp && !M.L[l].warp)
            __syncthreads();
          cProlong(c, M.L[l], M.L[l + 1]);
          cSmoothSweeps(c, M.L[l], M.post, 1);
        }
      }
      cluster.sync();
      // ... and the distributed levels up
      for (int l = Ls - 1; l >= 0; l--) {
        cProlong(c, M.L[l], M.L[l + 1]);
        cSmoothSweeps(c, M.L[l], M.post, 1);
      }
    }
    // clamped Newton update of this CTA's rows (updatePotKernel); the cluster
    // barrier makes the new values visible to the neighbours' next residual
    MT updM = 0;
    for (int t = threadIdx.x; t < nOwn; t += blockDim.x) {
      const int ly = L0.byNx.div(t), x = t - ly * nx;
      if (cCoef(c, L0, cRowNearT<true, uint8_t>(c, L0, L0.offCls, ly)[x]).fixed != MT(0))
        continue;
      MT v = cRowNearT<true, MT>(c, L0, L0.offD, ly)[x];
      if (isfinite(v)) // a non-finite correction is passed on to the next residual
        v = fmin(MT(kMaxNewtonStep), fmax(MT(-kMaxNewtonStep), v));
      pot[(size_t)(p0 + ly) * nx + x] += (double)v;
      updM = isfinite(v) ? fmax(updM, fabs(v)) : MT(INFINITY);
    }
    double upd = (double)updM;
    if (updTol > 0.) {
      // the maxima of this rule use their own slot (offRed + 16)
      double none = 0.;
      cClusterMax2(c, M.offRed + 16, upd, none, sh);
      if (upd < updTol) {
        it++;
        stopped = true;
        break;
      }
    }
    cluster.sync();
  }
  if (rank == 0 && threadIdx.x == 0) {
    out[0] = rel;
    out[1] = (double)it;
    out[2] = stopped ? 1. : 0.;
  }
  cluster.sync(); // no CTA leaves while another may still read its shared memory
}

// Level layout of the cluster solve for CL CTAs; *bytes = dynamic shared memory,
// 0 if some level has too many coefficient classes.  evenRows: a distributed
// level followed by another gets an even number of rows per CTA, so that a
// CTA's coarse rows lie under its fine rows; without it the bands of two
// levels may be a row apart, and a restriction or prolongation then reaches a
// neighbour's row through distributed shared memory (the same arithmetic, a
// row less per CTA and level: the 401 x 201 grid fits in 12 CTAs).
template <class MT>
CMG<MT> clusterDesc(const PoissonMG &P, int CL, size_t *bytes, bool evenRows = true) {
  CMG<MT> M;
  std::memset(&M, 0, sizeof(M));
  M.nLev = (int)P.L.size();
  M.pre = P.pre;
  M.post = P.post;
  M.coarseSweeps = P.coarseSweeps;
  M.vcycles = P.vcyclesPerNewton;
  M.twoCycleRel = P.twoCycleRel;
  M.firstSmall = M.nLev - 1;
  *bytes = 0;
  for (int l = 0; l < M.nLev; l++) {
    if (P.L[l].nCls <= 0)
      return M;
    const bool small = CL == 1 || P.L[l].nx * P.L[l].ny <= kSmallNodes || l == M.nLev - 1;
    if (small && l < M.firstSmall)
      M.firstSmall = l;
  }
  for (int l = 0; l < M.nLev; l++) {
    CLevel<MT> &c = M.L[l];
    c.nx = P.L[l].nx;
    c.ny = P.L[l].ny;
    c.small = l >= M.firstSmall ? 1 : 0;
    c.warp = l >= 1 && c.small && c.nx * c.ny <= kWarpNodes ? 1 : 0;
  }
  // bands: level 0 split evenly (rounded to even rows when a distributed
  // level follows), each next distributed level on half the rows of the level
  // above where that covers it, else split evenly
  const int B = M.firstSmall - 1;
  for (int l = 0; l <= B; l++) {
    CLevel<MT> &c = M.L[l];
    const int even = (c.ny + CL - 1) / CL;
    int rows = even;
    if (l > 0 && M.L[l - 1].ny > 3 && M.L[l - 1].rowsPer / 2 * CL >= c.ny)
      rows = M.L[l - 1].rowsPer / 2;
    if (evenRows && l < B && (rows & 1))
      rows++;
    c.rowsPer = rows;
  }
  size_t off = 0;
  auto take = [&](size_t b) {
    const size_t o = off;
    off += (b + 15) & ~size_t(15);
    return (unsigned)o;
  };
  for (int l = 0; l < M.nLev; l++) {
    const MGLevel &v = P.L[l];
    CLevel<MT> &c = M.L[l];
    if (c.small)
      c.rowsPer = c.ny;
    c.byNx.set(c.nx);
    c.byHalf.set((c.nx + 1) / 2);
    c.byRows.set(c.rowsPer);
    const size_t cells = (size_t)c.rowsPer * c.nx;
    c.offD = take(cells * sizeof(MT));
    c.offR = take(cells * sizeof(MT));
    c.offRho = take(cells * sizeof(MT));
    c.offRes = l + 1 < M.nLev ? take(cells * sizeof(MT)) : 0;
    c.offCls = take(cells);
    c.nCls = v.nCls;
    c.offTab = take((size_t)8 * v.nCls * sizeof(MT));
    c.cls = v.cls;
    c.tab = static_cast<const MT *>(v.clsTab);
    if (l + 1 < M.nLev) {
      c.ncx = P.L[l + 1].nx;
      c.ncy = P.L[l + 1].ny;
      c.offPxI = take(4 * (size_t)c.nx);
      c.offPxW = take(4 * (size_t)c.nx);
      c.offPyI = take(4 * (size_t)c.ny);
      c.offPyW = take(4 * (size_t)c.ny);
      c.offRxI = take(12 * (size_t)c.ncx);
      c.offRxW = take(12 * (size_t)c.ncx);
      c.offRyI = take(12 * (size_t)c.ncy);
      c.offRyW = take(12 * (size_t)c.ncy);
      c.offMapX = take(4 * (size_t)c.ncx);
      c.offMapY = take(4 * (size_t)c.ncy);
    }
    c.rxIdx = v.rxIdx;
    c.ryIdx = v.ryIdx;
    c.pxIdx = v.pxIdx;
    c.pyIdx = v.pyIdx;
    c.mapX = v.mapX;
    c.mapY = v.mapY;
    c.rxW = v.rxW;
    c.ryW = v.ryW;
    c.pxW = v.pxW;
    c.pyW = v.pyW;
  }
  M.offRed = take(4 * sizeof(double)); // two slots of two maxima
  *bytes = off;
  return M;
}

template <class MT> cudaLaunchConfig_t clusterConfig(int CL, size_t bytes, cudaStream_t st,
                                                     cudaLaunchAttribute *at) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(CL, 1, 1);
  cfg.blockDim = dim3(kClusterThreads, 1, 1);
  cfg.dynamicSmemBytes = bytes;
  cfg.stream = st;
  at->id = cudaLaunchAttributeClusterDimension;
  at->val.clusterDim.x = CL;
  at->val.clusterDim.y = 1;
  at->val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cfg;
}

// Largest cluster (16, 14, 12, 10, 8, 4, 2 or 1 CTAs, at most P.clusterCap
// when that is set) whose layout fits in shared memory and of which the
// device can hold `concurrent` at once (solves of engines stepped side by
// side); none: the multi-launch path serves the grid.  On GB300 with one
// 512-thread CTA per SM, 16 or 14 CTAs give 7 resident clusters, 12 give 8,
// 10 give 13 and 8 give 15.
template <class MT> void clusterPlan(PoissonMG &P, int concurrent) {
  P.clusterSize = 0;
  P.clusterSmem = 0;
  const int n = P.S.nx * P.S.ny;
  auto k = poissonClusterKernel<MT>;
  // the kernel may take all the dynamic shared memory a block can have: the
  // attribute is one per kernel, shared by every hierarchy (engines of other
  // grid sizes), so it is set to the device's limit, not to one layout's size
  cudaFuncAttributes fa;
  int dev = 0, optin = 0;
  if (cudaFuncGetAttributes(&fa, k) != cudaSuccess || cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) !=
          cudaSuccess ||
      optin <= (int)fa.sharedSizeBytes ||
      cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           optin - (int)fa.sharedSizeBytes) != cudaSuccess) {
    cudaGetLastError();
    return;
  }
  const size_t maxDyn = (size_t)(optin - (int)fa.sharedSizeBytes);
  const bool bigOk =
      cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess;
  if (!bigOk)
    cudaGetLastError();
  const int cands[] = {16, 14, 12, 10, 8, 4, 2, 1};
  for (int CL : cands) {
    if (P.clusterCap > 0 && CL > P.clusterCap)
      continue;
    if (CL > 1 && n <= kSmallNodes)
      continue;
    if (CL > 8 && !bigOk)
      continue;
    // the static part: the level descriptors, the exp table and the reduction slots
    auto fits = [&](size_t b) {
      return b != 0 && b <= maxDyn &&
             b + sizeof(CMG<MT>) + kExpTab * sizeof(double) + 1024 <= kClusterSmemMax;
    };
    size_t bytes = 0;
    bool even = true;
    clusterDesc<MT>(P, CL, &bytes, true);
    if (!fits(bytes)) {
      even = false;
      clusterDesc<MT>(P, CL, &bytes, false);
      if (!fits(bytes))
        continue;
    }
    cudaLaunchAttribute at;
    cudaLaunchConfig_t cfg = clusterConfig<MT>(CL, bytes, nullptr, &at);
    int nc = 0;
    if (cudaOccupancyMaxActiveClusters(&nc, k, &cfg) != cudaSuccess) {
      cudaGetLastError();
      continue;
    }
    if (nc < std::max(1, concurrent))
      continue;
    P.clusterSize = CL;
    P.clusterSmem = bytes;
    P.clusterEven = even;
    return;
  }
}

} // namespace

int32_t poissonPlanCluster(PoissonMG &P, int concurrent) {
  if (P.L.empty())
    return EMCG_OK;
  if (P.fp32)
    clusterPlan<float>(P, concurrent);
  else
    clusterPlan<double>(P, concurrent);
  // a cap or a concurrency that nothing meets: plan for one solve at a time
  if (P.clusterSize == 0 && concurrent > 1) {
    if (P.fp32)
      clusterPlan<float>(P, 1);
    else
      clusterPlan<double>(P, 1);
  }
  return cudaGetLastError() == cudaSuccess ? EMCG_OK : EMCG_ERR_CUDA;
}

namespace {

template <class MT> void vcycle(PoissonMG &P, int l, cudaStream_t st) {
  MGLevel &lv = P.L[l];
  LevelK<MT> K = levelK<MT>(lv);
  const int n = lv.nx * lv.ny;
  if (l + 1 == (int)P.L.size()) {
    coarseSolveKernel<MT><<<1, 256, 0, st>>>(K, P.coarseSweeps);
    return;
  }
  const int half = ((lv.nx + 1) / 2) * lv.ny;
  const int gs = (half + kBlock - 1) / kBlock;
  for (int s = 0; s < P.pre; s++) {
    smoothKernel<MT><<<gs, kBlock, 0, st>>>(K, 0);
    smoothKernel<MT><<<gs, kBlock, 0, st>>>(K, 1);
  }
  MGLevel &cl = P.L[l + 1];
  LevelK<MT> Kc = levelK<MT>(cl);
  const int nc = cl.nx * cl.ny;
  restrictKernel<MT><<<(nc + kBlock - 1) / kBlock, kBlock, 0, st>>>(
      K, Kc, lv.rxIdx, lv.rxW, lv.ryIdx, lv.ryW, lv.mapX, lv.mapY);
  vcycle<MT>(P, l + 1, st);
  prolongKernel<MT><<<(n + kBlock - 1) / kBlock, kBlock, 0, st>>>(K, Kc, lv.pxIdx, lv.pxW,
                                                                  lv.pyIdx, lv.pyW);
  for (int s = 0; s < P.post; s++) {
    smoothKernel<MT><<<gs, kBlock, 0, st>>>(K, 1);
    smoothKernel<MT><<<gs, kBlock, 0, st>>>(K, 0);
  }
}

// 1-D coarsening: coarse node I sits on fine node min(2I, n-1)
void coarsen1d(int n, std::vector<int> &map) {
  map.clear();
  if (n <= 3) {
    for (int i = 0; i < n; i++)
      map.push_back(i);
    return;
  }
  int nc = (n - 1 + 1) / 2 + 1;
  for (int I = 0; I < nc; I++)
    map.push_back(std::min(2 * I, n - 1));
}

// transfer weights between fine coordinates xf and coarse xc (= xf[map])
void transfer1d(const std::vector<double> &xf, const std::vector<int> &map,
                std::vector<int> &pIdx, std::vector<float> &pW, std::vector<int> &rIdx,
                std::vector<float> &rW) {
  const int nf = (int)xf.size(), nc = (int)map.size();
  pIdx.assign(nf, 0);
  pW.assign(nf, 1.f);
  int I = 0;
  for (int i = 0; i < nf; i++) {
    while (I + 1 < nc && map[I + 1] <= i)
      I++;
    pIdx[i] = I;
    if (map[I] == i || I + 1 >= nc)
      pW[i] = 1.f;
    else
      pW[i] = (float)((xf[map[I + 1]] - xf[i]) / (xf[map[I + 1]] - xf[map[I]]));
  }
  rIdx.assign(3 * nc, 0);
  rW.assign(3 * nc, 0.f);
  std::vector<int> cnt(nc, 0);
  for (int i = 0; i < nf; i++) {
    int J = pIdx[i];
    float w = pW[i];
    if (w > 0.f && cnt[J] < 3) {
      rIdx[3 * J + cnt[J]] = i;
      rW[3 * J + cnt[J]] = w;
      cnt[J]++;
    }
    if (w < 1.f && J + 1 < nc && cnt[J + 1] < 3) {
      rIdx[3 * (J + 1) + cnt[J + 1]] = i;
      rW[3 * (J + 1) + cnt[J + 1]] = 1.f - w;
      cnt[J + 1]++;
    }
  }
}

template <class V> int32_t upload(V **dst, const std::vector<V> &src, cudaStream_t st) {
  EMCG_CUDA(cudaMalloc(dst, sizeof(V) * std::max<size_t>(src.size(), 1)));
  if (!src.empty())
    EMCG_CUDA(cudaMemcpyAsync(*dst, src.data(), sizeof(V) * src.size(), cudaMemcpyHostToDevice, st));
  return EMCG_OK;
}

// Distinct coefficient tuples of a level (a uniform grid has a handful:
// interior, edges, corners, contacts, gates) and each node's class.
template <class MT>
int32_t coefficientClasses(MGLevel &L, const std::vector<double> &cw,
                           const std::vector<double> &ce, const std::vector<double> &cs,
                           const std::vector<double> &cn, const std::vector<double> &ar,
                           const std::vector<double> &dg, const std::vector<uint8_t> &fixed,
                           cudaStream_t st) {
  const size_t m = cw.size();
  std::vector<uint8_t> cls(m);
  std::vector<MT> tab;
  std::map<std::array<MT, 7>, int> ids;
  for (size_t k = 0; k < m && L.nCls >= 0; k++) {
    std::array<MT, 7> t = {(MT)cw[k], (MT)ce[k], (MT)cs[k], (MT)cn[k],
                           (MT)ar[k], (MT)dg[k], (MT)(fixed[k] ? 1 : 0)};
    auto it = ids.find(t);
    if (it == ids.end()) {
      if (ids.size() == 255) {
        L.nCls = -1;
        break;
      }
      it = ids.emplace(t, (int)ids.size()).first;
      tab.insert(tab.end(), t.begin(), t.end());
      tab.push_back(MT(0));
    }
    cls[k] = (uint8_t)it->second;
  }
  if (L.nCls < 0) {
    L.nCls = 0;
    return EMCG_OK;
  }
  L.nCls = (int)ids.size();
  EMCG_TRY(upload(&L.cls, cls, st));
  MT *t = nullptr;
  EMCG_TRY(upload(&t, tab, st));
  L.clsTab = t;
  return EMCG_OK;
}

} // namespace

int32_t poissonCreate(PoissonMG &P, const PoissonSetup &S, bool fp32, int smooth,
                      cudaStream_t st) {
  P.S = S;
  P.fp32 = fp32;
  if (smooth > 0)
    P.pre = P.post = smooth;
  const int nx = S.nx, ny = S.ny;
  P.hF[0] = S.h[1] / S.h[0];
  P.hF[1] = S.h[0] / S.h[1];
  P.hP = 1.;
  P.hP = P.hP * S.h[0];
  P.hP = P.hP * S.h[1];
  EMCG_TRY(upload(&P.C, S.C, st));
  EMCG_TRY(upload(&P.gSum, S.gSum, st));
  EMCG_TRY(upload(&P.gVeq, S.gVeq, st));
  EMCG_TRY(upload(&P.gVne, S.gVne, st));
  EMCG_TRY(upload(&P.resetMask, S.resetMask, st));
  EMCG_TRY(upload(&P.resetEq, S.resetEq, st));
  EMCG_TRY(upload(&P.resetNe, S.resetNe, st));
  EMCG_CUDA(cudaMalloc(&P.stats, 3 * sizeof(double)));
  EMCG_CUDA(cudaMalloc(&P.expTab, kExpTab * sizeof(double)));
  expTableKernel<<<1, kExpTab, 0, st>>>(P.expTab);
  EMCG_CUDA(cudaGetLastError());
  // level hierarchy (host)
  std::vector<double> X(nx), Y(ny);
  for (int i = 0; i < nx; i++)
    X[i] = i * S.h[0];
  for (int j = 0; j < ny; j++)
    Y[j] = j * S.h[1];
  std::vector<uint8_t> fixed = S.fixed;
  std::vector<double> gx = S.gDensX, gy = S.gDensY;
  int lx = nx, ly = ny;
  for (int lev = 0; lev < 16; lev++) {
    MGLevel L;
    std::memset(&L, 0, sizeof(L));
    L.nx = lx;
    L.ny = ly;
    const int m = lx * ly;
    std::vector<double> cw(m), ce(m), cs(m), cn(m), ar(m), dg(m);
    for (int j = 0; j < ly; j++)
      for (int i = 0; i < lx; i++) {
        int k = j * lx + i;
        double dxw = i > 0 ? X[i] - X[i - 1] : 0, dxe = i < lx - 1 ? X[i + 1] - X[i] : 0;
        double dys = j > 0 ? Y[j] - Y[j - 1] : 0, dyn = j < ly - 1 ? Y[j + 1] - Y[j] : 0;
        double lxd = 0.5 * (dxw + dxe), lyd = 0.5 * (dys + dyn);
        cw[k] = i > 0 ? lyd / dxw : 0;
        ce[k] = i < lx - 1 ? lyd / dxe : 0;
        cs[k] = j > 0 ? lxd / dys : 0;
        cn[k] = j < ly - 1 ? lxd / dyn : 0;
        ar[k] = lxd * lyd;
        dg[k] = cw[k] + ce[k] + cs[k] + cn[k] + gx[k] * lyd + gy[k] * lxd;
      }
    if (fp32) {
      auto f = [](const std::vector<double> &v) { return std::vector<float>(v.begin(), v.end()); };
      EMCG_TRY(upload(&L.cw, f(cw), st));
      EMCG_TRY(upload(&L.ce, f(ce), st));
      EMCG_TRY(upload(&L.cs, f(cs), st));
      EMCG_TRY(upload(&L.cn, f(cn), st));
      EMCG_TRY(upload(&L.area, f(ar), st));
      EMCG_TRY(upload(&L.diag0, f(dg), st));
      EMCG_CUDA(cudaMalloc(&L.d, sizeof(float) * m));
      EMCG_CUDA(cudaMalloc(&L.r, sizeof(float) * m));
      EMCG_CUDA(cudaMalloc(&L.rho, sizeof(float) * m));
    } else {
      EMCG_TRY(upload(&L.dcw, cw, st));
      EMCG_TRY(upload(&L.dce, ce, st));
      EMCG_TRY(upload(&L.dcs, cs, st));
      EMCG_TRY(upload(&L.dcn, cn, st));
      EMCG_TRY(upload(&L.darea, ar, st));
      EMCG_TRY(upload(&L.ddiag0, dg, st));
      EMCG_CUDA(cudaMalloc(&L.dd, sizeof(double) * m));
      EMCG_CUDA(cudaMalloc(&L.dr, sizeof(double) * m));
      EMCG_CUDA(cudaMalloc(&L.drho, sizeof(double) * m));
    }
    EMCG_TRY(upload(&L.fixed, fixed, st));
    EMCG_TRY(fp32 ? coefficientClasses<float>(L, cw, ce, cs, cn, ar, dg, fixed, st)
                  : coefficientClasses<double>(L, cw, ce, cs, cn, ar, dg, fixed, st));
    std::vector<int> mx, my;
    coarsen1d(lx, mx);
    coarsen1d(ly, my);
    bool last = (int)mx.size() == lx && (int)my.size() == ly;
    if (!last) {
      std::vector<int> pxI, pyI, rxI, ryI;
      std::vector<float> pxW, pyW, rxW, ryW;
      transfer1d(X, mx, pxI, pxW, rxI, rxW);
      transfer1d(Y, my, pyI, pyW, ryI, ryW);
      EMCG_TRY(upload(&L.pxIdx, pxI, st));
      EMCG_TRY(upload(&L.pyIdx, pyI, st));
      EMCG_TRY(upload(&L.pxW, pxW, st));
      EMCG_TRY(upload(&L.pyW, pyW, st));
      EMCG_TRY(upload(&L.rxIdx, rxI, st));
      EMCG_TRY(upload(&L.ryIdx, ryI, st));
      EMCG_TRY(upload(&L.rxW, rxW, st));
      EMCG_TRY(upload(&L.ryW, ryW, st));
      EMCG_TRY(upload(&L.mapX, mx, st));
      EMCG_TRY(upload(&L.mapY, my, st));
    }
    P.L.push_back(L);
    if (last)
      break;
    // next level's static data by injection
    std::vector<double> Xc(mx.size()), Yc(my.size());
    for (size_t I = 0; I < mx.size(); I++)
      Xc[I] = X[mx[I]];
    for (size_t J = 0; J < my.size(); J++)
      Yc[J] = Y[my[J]];
    const int ncx = (int)mx.size(), ncy = (int)my.size();
    std::vector<uint8_t> fc(ncx * ncy);
    std::vector<double> gxc(ncx * ncy), gyc(ncx * ncy);
    for (int J = 0; J < ncy; J++)
      for (int I = 0; I < ncx; I++) {
        int k = my[J] * lx + mx[I];
        fc[J * ncx + I] = fixed[k];
        gxc[J * ncx + I] = gx[k];
        gyc[J * ncx + I] = gy[k];
      }
    X = Xc;
    Y = Yc;
    fixed = fc;
    gx = gxc;
    gy = gyc;
    lx = ncx;
    ly = ncy;
  }
  EMCG_CUDA(cudaStreamSynchronize(st));
  return poissonPlanCluster(P, 1);
}

void poissonFree(PoissonMG &P) {
  for (auto &L : P.L) {
    void *ps[] = {L.cw,  L.ce,    L.cs,    L.cn,    L.area,  L.diag0, L.dcw,   L.dce,
                  L.dcs, L.dcn,   L.darea, L.ddiag0, L.fixed, L.d,     L.r,     L.rho,
                  L.dd,  L.dr,    L.drho,  L.rxIdx, L.ryIdx, L.rxW,   L.ryW,   L.pxIdx,
                  L.pyIdx, L.pxW, L.pyW,   L.mapX,  L.mapY, L.cls, L.clsTab};
    for (void *p : ps)
      cudaFree(p);
  }
  P.L.clear();
  void *ps[] = {P.C,       P.gSum,    P.gVeq,  P.gVne,  P.resetMask,
                P.resetEq, P.resetNe, P.stats, P.expTab};
  for (void *p : ps)
    cudaFree(p);
  if (P.hStats)
    cudaFreeHost(P.hStats);
  P.hStats = nullptr;
}

// the single-launch cluster solve, enqueued on st
// out: where the kernel writes [relative residual, Newton steps, stopped by
// the update rule] (device memory, or mapped page-locked host memory)
template <class MT>
static int32_t clusterLaunch(PoissonMG &P, double *pot, const double *conc, double rtol,
                             int maxCycles, cudaStream_t st, double *out) {
  size_t bytes = 0;
  const CMG<MT> M = clusterDesc<MT>(P, P.clusterSize, &bytes, P.clusterEven);
  cudaLaunchAttribute at;
  cudaLaunchConfig_t cfg = clusterConfig<MT>(P.clusterSize, bytes, st, &at);
  EMCG_CUDA(cudaLaunchKernelEx(&cfg, poissonClusterKernel<MT>, M, pot, conc, P.C, P.gSum,
                               conc ? P.gVne : P.gVeq, P.hF[0], P.hF[1], P.hP, rtol, maxCycles,
                               P.updTol, (const double *)P.expTab, out));
  return EMCG_OK;
}

// the outcome of a solve from its statistics
static int32_t solveOutcome(double rel, int it, bool updStop, double rtol, double *relRes,
                            int *cycles) {
  if (relRes)
    *relRes = rel;
  if (cycles)
    *cycles = it;
  if (!std::isfinite(rel)) {
    setError("Poisson: non-finite residual after %d Newton steps (NaN or Inf in the potential, "
             "the concentration or a correction)", it);
    return EMCG_ERR_NONCONVERGED;
  }
  if (!updStop && !(rel <= rtol)) {
    setError("Poisson: relative residual %.3e after %d Newton steps (target %.1e)", rel, it, rtol);
    return EMCG_ERR_NONCONVERGED;
  }
  return EMCG_OK;
}

template <class MT>
static int32_t solveT(PoissonMG &P, double *pot, const double *conc, bool resetBC, double rtol,
                      int maxCycles, cudaStream_t st, double *relRes, int *cycles) {
  const int nx = P.S.nx, ny = P.S.ny, n = nx * ny;
  const int grid = (n + kBlock - 1) / kBlock;
  if (resetBC) {
    resetBCKernel<<<grid, kBlock, 0, st>>>(pot, P.resetMask, conc ? P.resetNe : P.resetEq, n);
    EMCG_CUDA(cudaGetLastError());
  }
  MGLevel &L0 = P.L[0];
  LevelK<MT> K0 = levelK<MT>(L0);
  double stats[3] = {0, 0, 0};
  double rel = INFINITY;
  int it = 0;
  bool updStop = false;
  const bool cluster = P.useCluster && P.clusterSize > 0;
  if (cluster) {
    EMCG_TRY(clusterLaunch<MT>(P, pot, conc, rtol, maxCycles, st, P.stats));
    EMCG_CUDA(cudaMemcpyAsync(stats, P.stats, 3 * sizeof(double), cudaMemcpyDeviceToHost, st));
    EMCG_CUDA(cudaStreamSynchronize(st));
    rel = stats[0];
    it = (int)stats[1];
    updStop = stats[2] != 0.;
  }
  double scale = 0.;
  for (; !cluster && it <= maxCycles; it++) {
    EMCG_CUDA(cudaMemsetAsync(P.stats, 0, 3 * sizeof(double), st));
    nonlinResidualKernel<MT><<<grid, kBlock, 0, st>>>(
        pot, conc, P.C, L0.fixed, P.gSum, conc ? P.gVne : P.gVeq, nx, ny, P.hF[0], P.hF[1], P.hP,
        K0.r, K0.rho, K0.d, P.stats, it == 0);
    EMCG_CUDA(cudaGetLastError());
    EMCG_CUDA(cudaMemcpyAsync(stats, P.stats, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
    EMCG_CUDA(cudaStreamSynchronize(st));
    if (it == 0)
      scale = stats[1];
    rel = scale > 0 ? stats[0] / scale : stats[0];
    if (rel <= rtol || it == maxCycles || !std::isfinite(rel))
      break;
    // under the update-size rule a Newton step needs only a rough correction
    const int nv = P.updTol <= 0. && rel < P.twoCycleRel ? P.vcyclesPerNewton : 1;
    for (int k = 0; k < nv; k++)
      vcycle<MT>(P, 0, st);
    updatePotKernel<MT><<<grid, kBlock, 0, st>>>(pot, K0.d, L0.fixed, n, P.stats);
    EMCG_CUDA(cudaGetLastError());
    if (P.updTol > 0.) {
      EMCG_CUDA(cudaMemcpyAsync(&stats[2], P.stats + 2, sizeof(double), cudaMemcpyDeviceToHost,
                                st));
      EMCG_CUDA(cudaStreamSynchronize(st));
      if (stats[2] < P.updTol) {
        it++;
        updStop = true;
        break;
      }
    }
  }
  return solveOutcome(rel, it, updStop, rtol, relRes, cycles);
}

int32_t poissonSolve(PoissonMG &P, double *pot, const double *conc, bool resetBC, double rtol,
                     int maxCycles, cudaStream_t st, double *relRes, int *cycles) {
  return P.fp32 ? solveT<float>(P, pot, conc, resetBC, rtol, maxCycles, st, relRes, cycles)
                : solveT<double>(P, pot, conc, resetBC, rtol, maxCycles, st, relRes, cycles);
}

int32_t poissonEnqueue(PoissonMG &P, double *pot, const double *conc, bool resetBC, double rtol,
                       int maxCycles, cudaStream_t st, bool *queued, double *relRes,
                       int *cycles) {
  *queued = false;
  if (!(P.useCluster && P.clusterSize > 0))
    return poissonSolve(P, pot, conc, resetBC, rtol, maxCycles, st, relRes, cycles);
  if (!P.hStats) {
    EMCG_CUDA(cudaHostAlloc(&P.hStats, 3 * sizeof(double), cudaHostAllocMapped));
    EMCG_CUDA(cudaHostGetDevicePointer(&P.hStatsDev, P.hStats, 0));
  }
  if (resetBC) {
    const int n = P.S.nx * P.S.ny;
    resetBCKernel<<<(n + kBlock - 1) / kBlock, kBlock, 0, st>>>(
        pot, P.resetMask, conc ? P.resetNe : P.resetEq, n);
    EMCG_CUDA(cudaGetLastError());
  }
  // the kernel writes its statistics straight into the page-locked block: no
  // copy follows it on the stream
  EMCG_TRY(P.fp32 ? clusterLaunch<float>(P, pot, conc, rtol, maxCycles, st, P.hStatsDev)
                  : clusterLaunch<double>(P, pot, conc, rtol, maxCycles, st, P.hStatsDev));
  *queued = true;
  return EMCG_OK;
}

int32_t poissonFinish(PoissonMG &P, double rtol, double *relRes, int *cycles) {
  EMCG_CHECK_ARG(P.hStats, "no enqueued Poisson solve");
  return solveOutcome(P.hStats[0], (int)P.hStats[1], P.hStats[2] != 0., rtol, relRes, cycles);
}

} // namespace emcg

// ===========================================================================
// Poisson solve that allocates nothing (emcg_poisson_solve_noalloc).
//
// Some callers cannot allocate device memory at the moment they solve: a host
// whose memory pool owns the whole GPU, a caller inside a region where the CUDA
// allocator must not be entered, or an embedder that must not grow the
// process's device footprint after start-up.  For them the solver's working set
// -- fine-grid inputs, the multigrid hierarchy, transfer tables and residual
// statistics -- lives in one file-scope device array of fixed size, reserved
// when this library's device code is loaded.  It is rebuilt from the caller's
// description by kernels on every call; the host side uses only stack memory.
// Host code cannot pass the array's name to a kernel as an address: the first
// call on each device asks the runtime for the address (cudaGetSymbolAddress,
// with that device current) and keeps it.  The array is shared by all calls,
// so calls whose work can overlap on a device race with one another.
// ===========================================================================
namespace emcg {
namespace {

constexpr int kNAMaxNodes = 1 << 17;           // fine-grid nodes, e.g. 401 x 201 or 362 x 362
constexpr int kNAMaxDim = 8192;                // nodes per dimension
constexpr int kNAMaxLevels = 16;               // as the allocating hierarchy
constexpr int kNAMaxContacts = 64;
constexpr int kNAMaxDevices = 64;
constexpr int kNAVcyclesPerNewton = 3; // as PoissonMG's defaults
constexpr double kNATwoCycleRel = 1e30;
constexpr int kNALevelNodes = 2 * kNAMaxNodes; // nodes of all levels together
constexpr int kNA1D = 16 * kNAMaxDim;          // 1-D transfer entries of all levels

// byte offsets inside the scratch array
constexpr size_t kOffDoping = 0;                       // double [N]  doping (upload)
constexpr size_t kOffC = kOffDoping + 8ull * kNAMaxNodes;   // double [N]  C = doping / ni
constexpr size_t kOffGSum = kOffC + 8ull * kNAMaxNodes;     // double [N]  gate sums
constexpr size_t kOffGVeq = kOffGSum + 8ull * kNAMaxNodes;
constexpr size_t kOffGVne = kOffGVeq + 8ull * kNAMaxNodes;
constexpr size_t kOffGDx = kOffGVne + 8ull * kNAMaxNodes;   // double [N]  Robin densities
constexpr size_t kOffGDy = kOffGDx + 8ull * kNAMaxNodes;
constexpr size_t kOffResEq = kOffGDy + 8ull * kNAMaxNodes;  // double [N]  resetBC values
constexpr size_t kOffResNe = kOffResEq + 8ull * kNAMaxNodes;
constexpr size_t kOffStats = kOffResNe + 8ull * kNAMaxNodes; // double [4] residual maxima
constexpr size_t kOffLevelF = kOffStats + 256;               // float [9 x all levels]
constexpr size_t kOffTransF = kOffLevelF + 4ull * 9 * kNALevelNodes; // float [1-D]
constexpr size_t kOffTransI = kOffTransF + 4ull * kNA1D;             // int   [1-D]
constexpr size_t kOffBnd = kOffTransI + 4ull * kNA1D;                // int   [2 (ny + nx)]
constexpr size_t kOffCtype = kOffBnd + 4ull * 4 * kNAMaxDim;         // int   [contacts]
constexpr size_t kOffResMask = kOffCtype + 4ull * kNAMaxContacts;    // u8    [N]
constexpr size_t kOffFixed = kOffResMask + kNAMaxNodes;              // u8    [all levels]
constexpr size_t kNABytes = (kOffFixed + kNALevelNodes + 255) & ~size_t(255); // about 21 MB

struct NALevels {
  int n;
  int nx[kNAMaxLevels], ny[kNAMaxLevels];
  double h0, h1; // normalised fine spacing
};

struct NAContacts {
  double gF[kNAMaxContacts], barrier[kNAMaxContacts], volt[kNAMaxContacts];
};

// fine index of node I of level l along one dimension (coarse node I sits on
// node min(2I, n - 1) of the level below while that level has more than 3)
__device__ __forceinline__ int naFineIndex(const NALevels &lv, int l, int I, bool ydim) {
  for (int k = l; k > 0; k--) {
    int nf = ydim ? lv.ny[k - 1] : lv.nx[k - 1];
    if (nf > 3)
      I = min(2 * I, nf - 1);
  }
  return I;
}
__device__ __forceinline__ double naCoord(const NALevels &lv, int l, int I, bool ydim) {
  return naFineIndex(lv, l, I, ydim) * (ydim ? lv.h1 : lv.h0);
}

// Fine-grid data of the reference equation
// (include/PoissonSolver/emcSORSolver.hpp:25-36, 330-368): the same values
// emcg_device_create prepares on the host for the allocating solver.
__global__ void naFineSetupKernel(int nx, int ny, double Ni, double hF0, double hF1, double h0,
                                  double h1, NAContacts ct, const double *doping,
                                  const int32_t *bnd, const int32_t *ctype, double *C,
                                  double *gSum, double *gVeq, double *gVne, double *gDx,
                                  double *gDy, uint8_t *resMask, double *resEq, double *resNe,
                                  uint8_t *fixed) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nx * ny)
    return;
  const int x = i % nx, y = i / nx;
  // boundary b's contact at a node: XMIN/XMAX indexed by y, YMIN/YMAX by x
  auto contact = [&](int b) { return b == 0 ? bnd[y] : b == 1 ? bnd[ny + y]
                                     : b == 2 ? bnd[2 * ny + x] : bnd[2 * ny + nx + x]; };
  const double c = doping[i] / Ni;
  C[i] = c;
  // reservoir nodes: the first boundary holding the node decides
  // (emcSurface::getBoundaryPos, include/emcSurface.hpp)
  int fb = x == 0 ? 0 : (x == nx - 1 ? 1 : (y == 0 ? 2 : (y == ny - 1 ? 3 : -1)));
  int fc = fb < 0 ? -1 : contact(fb);
  fixed[i] = fc >= 0 && ctype[fc] == EMCG_CONTACT_OHMIC;
  // gate Robin terms of every side the node lies on
  const double hF[2] = {hF0, hF1}, h[2] = {h0, h1};
  double gs = 0, ge = 0, gn = 0, dx = 0, dy = 0;
  for (int k = 0; k < 2; k++) {
    int co = k == 0 ? x : y, mx = k == 0 ? nx - 1 : ny - 1;
    for (int side = 0; side < 2; side++) {
      if (co != (side == 0 ? 0 : mx))
        continue;
      int cc = contact(2 * k + side);
      if (cc < 0 || ctype[cc] != EMCG_CONTACT_GATE)
        continue;
      double G = __dmul_rn(__dmul_rn(ct.gF[cc], hF[k]), h[k]);
      gs = __dadd_rn(gs, G);
      ge = __dadd_rn(ge, __dmul_rn(G, ct.barrier[cc]));
      gn = __dadd_rn(gn, __dmul_rn(G, __dadd_rn(ct.barrier[cc], ct.volt[cc])));
      if (k == 0)
        dx = __dadd_rn(dx, 0.5 * ct.gF[cc]);
      else
        dy = __dadd_rn(dy, 0.5 * ct.gF[cc]);
    }
  }
  gSum[i] = gs;
  gVeq[i] = ge;
  gVne[i] = gn;
  gDx[i] = dx;
  gDy[i] = dy;
  // resetBC: every boundary coordinate of an ohmic contact, later boundaries
  // (XMIN, XMAX, YMIN, YMAX order) overriding earlier ones at corners
  uint8_t m = 0;
  double re = 0, rn = 0;
  for (int b = 0; b < 4; b++) {
    bool on = b == 0 ? x == 0 : b == 1 ? x == nx - 1 : b == 2 ? y == 0 : y == ny - 1;
    int cc = on ? contact(b) : -1;
    if (cc < 0 || ctype[cc] != EMCG_CONTACT_OHMIC)
      continue;
    double bi = asinh(0.5 * c);
    m = 1;
    re = bi;
    rn = __dadd_rn(ct.volt[cc], bi);
  }
  resMask[i] = m;
  resEq[i] = re;
  resNe[i] = rn;
}

// finite-volume coefficients and Dirichlet mask of level l, by injection of
// the fine data (the construction poissonCreate runs on the host)
__global__ void naLevelSetupKernel(NALevels lv, int l, const double *gDx, const double *gDy,
                                   const uint8_t *fixed0, int nx0, float *cw, float *ce, float *cs,
                                   float *cn, float *area, float *diag0, uint8_t *fixed) {
  const int lx = lv.nx[l], ly = lv.ny[l];
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= lx * ly)
    return;
  const int i = k % lx, j = k / lx;
  const double Xi = naCoord(lv, l, i, false), Yj = naCoord(lv, l, j, true);
  const double dxw = i > 0 ? Xi - naCoord(lv, l, i - 1, false) : 0;
  const double dxe = i < lx - 1 ? naCoord(lv, l, i + 1, false) - Xi : 0;
  const double dys = j > 0 ? Yj - naCoord(lv, l, j - 1, true) : 0;
  const double dyn = j < ly - 1 ? naCoord(lv, l, j + 1, true) - Yj : 0;
  const double lxd = 0.5 * (dxw + dxe), lyd = 0.5 * (dys + dyn);
  const double w = i > 0 ? lyd / dxw : 0, e = i < lx - 1 ? lyd / dxe : 0;
  const double s = j > 0 ? lxd / dys : 0, n = j < ly - 1 ? lxd / dyn : 0;
  const int f = naFineIndex(lv, l, j, true) * nx0 + naFineIndex(lv, l, i, false);
  double d = __dadd_rn(__dadd_rn(__dadd_rn(w, e), s), n);
  d = __dadd_rn(__dadd_rn(d, __dmul_rn(gDx[f], lyd)), __dmul_rn(gDy[f], lxd));
  cw[k] = (float)w;
  ce[k] = (float)e;
  cs[k] = (float)s;
  cn[k] = (float)n;
  area[k] = (float)(lxd * lyd);
  diag0[k] = (float)d;
  if (l > 0)
    fixed[k] = fixed0[f];
}

// 1-D transfer between level l (nf nodes) and level l + 1 (nc nodes) along one
// dimension: prolongation's lower coarse node and weight per fine node,
// restriction's (up to 3) fine nodes and weights per coarse node in ascending
// fine order, and the coarse -> fine injection map
__global__ void naTransferKernel(NALevels lv, int l, bool ydim, int *pIdx, float *pW, int *rIdx,
                                 float *rW, int *map) {
  const int nf = ydim ? lv.ny[l] : lv.nx[l];
  const int nc = ydim ? lv.ny[l + 1] : lv.nx[l + 1];
  auto cmap = [&](int J) { return nf > 3 ? min(2 * J, nf - 1) : J; };
  auto X = [&](int i) { return naCoord(lv, l, i, ydim); };
  auto lower = [&](int i, int &I, float &w) {
    I = min(nf > 3 ? i / 2 : i, nc - 1);
    while (I + 1 < nc && cmap(I + 1) <= i)
      I++;
    while (I > 0 && cmap(I) > i)
      I--;
    if (cmap(I) == i || I + 1 >= nc)
      w = 1.f;
    else
      w = (float)((X(cmap(I + 1)) - X(i)) / (X(cmap(I + 1)) - X(cmap(I))));
  };
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < nf) {
    int I;
    float w;
    lower(t, I, w);
    pIdx[t] = I;
    pW[t] = w;
  }
  if (t < nc) {
    map[t] = cmap(t);
    for (int q = 0; q < 3; q++) {
      rIdx[3 * t + q] = 0;
      rW[3 * t + q] = 0.f;
    }
    int cnt = 0;
    const int lo = t > 0 ? cmap(t - 1) : 0, hi = t + 1 < nc ? cmap(t + 1) : nf - 1;
    for (int i = lo; i <= hi && cnt < 3; i++) {
      int I;
      float w;
      lower(i, I, w);
      if (I == t && w > 0.f) {
        rIdx[3 * t + cnt] = i;
        rW[3 * t + cnt] = w;
        cnt++;
      } else if (I + 1 == t && w < 1.f) {
        rIdx[3 * t + cnt] = i;
        rW[3 * t + cnt] = 1.f - w;
        cnt++;
      }
    }
  }
}

// the allocating solver's V-cycle (float multigrid), over a fixed level array
void naVcycle(const MGLevel *lev, int nLev, int l, int pre, int post, int coarseSweeps,
              cudaStream_t st) {
  const MGLevel &lv = lev[l];
  LevelK<float> K = levelK<float>(lv);
  const int n = lv.nx * lv.ny;
  if (l + 1 == nLev) {
    coarseSolveKernel<float><<<1, 256, 0, st>>>(K, coarseSweeps);
    return;
  }
  const int half = ((lv.nx + 1) / 2) * lv.ny;
  const int gs = (half + kBlock - 1) / kBlock;
  for (int s = 0; s < pre; s++) {
    smoothKernel<float><<<gs, kBlock, 0, st>>>(K, 0);
    smoothKernel<float><<<gs, kBlock, 0, st>>>(K, 1);
  }
  const MGLevel &cl = lev[l + 1];
  LevelK<float> Kc = levelK<float>(cl);
  const int nc = cl.nx * cl.ny;
  restrictKernel<float><<<(nc + kBlock - 1) / kBlock, kBlock, 0, st>>>(
      K, Kc, lv.rxIdx, lv.rxW, lv.ryIdx, lv.ryW, lv.mapX, lv.mapY);
  naVcycle(lev, nLev, l + 1, pre, post, coarseSweeps, st);
  prolongKernel<float><<<(n + kBlock - 1) / kBlock, kBlock, 0, st>>>(K, Kc, lv.pxIdx, lv.pxW,
                                                                     lv.pyIdx, lv.pyW);
  for (int s = 0; s < post; s++) {
    smoothKernel<float><<<gs, kBlock, 0, st>>>(K, 1);
    smoothKernel<float><<<gs, kBlock, 0, st>>>(K, 0);
  }
}

} // namespace

// the array and its per-device address
static __device__ __align__(256) unsigned char g_poissonScratch[kNABytes];
static std::atomic<void *> g_poissonScratchAddr[kNAMaxDevices];

static int32_t poissonScratchAddress(unsigned char **out) {
  int dev = -1;
  EMCG_CUDA(cudaGetDevice(&dev));
  EMCG_CHECK_ARG(dev >= 0 && dev < kNAMaxDevices, "device %d is beyond the %d devices supported",
                 dev, kNAMaxDevices);
  void *p = g_poissonScratchAddr[dev].load(std::memory_order_acquire);
  if (!p) {
    cudaError_t e = cudaGetSymbolAddress(&p, g_poissonScratch);
    if (e != cudaSuccess || !p) {
      setError("cudaGetSymbolAddress of the Poisson scratch array failed on device %d: %s", dev,
               cudaGetErrorString(e));
      return EMCG_ERR_CUDA;
    }
    g_poissonScratchAddr[dev].store(p, std::memory_order_release);
  }
  *out = static_cast<unsigned char *>(p);
  return EMCG_OK;
}

} // namespace emcg

extern "C" int32_t emcg_poisson_solve_noalloc(const emcg_device_desc *dv, double *d_pot,
                                              const double *d_conc, int32_t reset_bc,
                                              int32_t smooth, double rtol, int32_t max_cycles,
                                              void *cuda_stream, double *rel_residual,
                                              int32_t *cycles) {
  using namespace emcg;
  EMCG_CHECK_ARG(dv && d_pot, "device description and potential are required");
  const int nx = dv->nx, ny = dv->ny;
  EMCG_CHECK_ARG(nx >= 3 && ny >= 3, "grid must have at least 3 x 3 nodes (got %d x %d)", nx, ny);
  EMCG_CHECK_ARG(nx <= kNAMaxDim && ny <= kNAMaxDim && (int64_t)nx * ny <= kNAMaxNodes,
                 "grid %d x %d exceeds the no-allocation Poisson limit of %d nodes and %d per "
                 "dimension",
                 nx, ny, kNAMaxNodes, kNAMaxDim);
  EMCG_CHECK_ARG(dv->n_contacts >= 0 && dv->n_contacts <= kNAMaxContacts,
                 "%d contacts exceed the no-allocation Poisson limit of %d", dv->n_contacts,
                 kNAMaxContacts);
  EMCG_CHECK_ARG(dv->doping && dv->boundary_contact[0] && dv->boundary_contact[1] &&
                     dv->boundary_contact[2] && dv->boundary_contact[3],
                 "doping and boundary contact arrays are required");
  EMCG_CHECK_ARG(dv->n_contacts == 0 ||
                     (dv->contact_type && dv->contact_voltage && dv->contact_param),
                 "contact arrays are required");
  EMCG_CHECK_ARG(dv->hx > 0 && dv->hy > 0 && dv->temperature > 0 && dv->ni > 0 && dv->eps_r > 0,
                 "spacing, temperature, ni and eps_r must be positive");
  EMCG_CHECK_ARG(rtol > 0 && max_cycles >= 0 && smooth >= 0, "bad Poisson settings");
  for (int c = 0; c < dv->n_contacts; c++)
    EMCG_CHECK_ARG(dv->contact_type[c] == EMCG_CONTACT_OHMIC ||
                       dv->contact_type[c] == EMCG_CONTACT_GATE,
                   "contact %d: only ohmic and gate contacts are supported", c);
  for (int b = 0; b < 4; b++)
    for (int k = 0; k < (b < 2 ? ny : nx); k++)
      EMCG_CHECK_ARG(dv->boundary_contact[b][k] >= -1 &&
                         dv->boundary_contact[b][k] < dv->n_contacts,
                     "boundary %d, node %d: contact index %d out of range", b, k,
                     dv->boundary_contact[b][k]);
  // level shapes and their scratch footprint, checked before anything is written
  NALevels lv;
  lv.n = 0;
  size_t nodes = 0, oneD = 0;
  for (int l = 0, lx = nx, ly = ny; l < kNAMaxLevels; l++) {
    lv.nx[l] = lx;
    lv.ny[l] = ly;
    lv.n = l + 1;
    nodes += (size_t)lx * ly;
    const int cx = lx > 3 ? lx / 2 + 1 : lx, cy = ly > 3 ? ly / 2 + 1 : ly;
    if (cx == lx && cy == ly)
      break;
    oneD += (size_t)lx + ly + 4 * (size_t)cx + 4 * (size_t)cy;
    lx = cx;
    ly = cy;
  }
  EMCG_CHECK_ARG(nodes <= (size_t)kNALevelNodes && oneD <= (size_t)kNA1D,
                 "grid %d x %d: multigrid hierarchy exceeds the no-allocation scratch", nx, ny);
  cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
  unsigned char *S = nullptr;
  EMCG_TRY(poissonScratchAddress(&S));
  const int n = nx * ny;
  // normalisation (include/emcDevice.hpp:87, emcSORSolver.hpp:330-368)
  const double Vt = kKB / kQ * dv->temperature;
  const double Ld = std::sqrt(kEPS0 * dv->eps_r * Vt / kQ / dv->ni);
  lv.h0 = dv->hx / Ld;
  lv.h1 = dv->hy / Ld;
  NAContacts ct;
  for (int c = 0; c < dv->n_contacts; c++) {
    ct.volt[c] = dv->contact_voltage[c] / Vt;
    ct.gF[c] = ct.barrier[c] = 0;
    if (dv->contact_type[c] == EMCG_CONTACT_GATE) {
      const double gamma = dv->contact_param[3 * c + 0] / dv->eps_r;
      const double tox = dv->contact_param[3 * c + 1] / Ld;
      ct.gF[c] = 2 * gamma / tox;
      ct.barrier[c] = dv->contact_param[3 * c + 2] / Vt;
    }
  }
  double *doping = (double *)(S + kOffDoping), *C = (double *)(S + kOffC);
  double *gSum = (double *)(S + kOffGSum), *gVeq = (double *)(S + kOffGVeq);
  double *gVne = (double *)(S + kOffGVne), *gDx = (double *)(S + kOffGDx);
  double *gDy = (double *)(S + kOffGDy), *resEq = (double *)(S + kOffResEq);
  double *resNe = (double *)(S + kOffResNe), *stats = (double *)(S + kOffStats);
  float *levF = (float *)(S + kOffLevelF), *trF = (float *)(S + kOffTransF);
  int *trI = (int *)(S + kOffTransI);
  int32_t *bnd = (int32_t *)(S + kOffBnd), *ctype = (int32_t *)(S + kOffCtype);
  uint8_t *resMask = S + kOffResMask, *fixedAll = S + kOffFixed;
  EMCG_CUDA(cudaMemcpyAsync(doping, dv->doping, sizeof(double) * n, cudaMemcpyHostToDevice, st));
  const int32_t *bsrc[4] = {dv->boundary_contact[0], dv->boundary_contact[1],
                            dv->boundary_contact[2], dv->boundary_contact[3]};
  const size_t boff[4] = {0, (size_t)ny, 2 * (size_t)ny, 2 * (size_t)ny + nx};
  for (int b = 0; b < 4; b++)
    EMCG_CUDA(cudaMemcpyAsync(bnd + boff[b], bsrc[b], sizeof(int32_t) * (b < 2 ? ny : nx),
                              cudaMemcpyHostToDevice, st));
  if (dv->n_contacts)
    EMCG_CUDA(cudaMemcpyAsync(ctype, dv->contact_type, sizeof(int32_t) * dv->n_contacts,
                              cudaMemcpyHostToDevice, st));
  const double hF0 = lv.h1 / lv.h0, hF1 = lv.h0 / lv.h1;
  double hP = 1.;
  hP = hP * lv.h0;
  hP = hP * lv.h1;
  naFineSetupKernel<<<(n + kBlock - 1) / kBlock, kBlock, 0, st>>>(
      nx, ny, dv->ni, hF0, hF1, lv.h0, lv.h1, ct, doping, bnd, ctype, C, gSum, gVeq, gVne, gDx,
      gDy, resMask, resEq, resNe, fixedAll);
  EMCG_CUDA(cudaGetLastError());
  // carve the levels out of the scratch and build them
  MGLevel lev[kNAMaxLevels];
  size_t fo = 0, uo = 0, to = 0;
  for (int l = 0; l < lv.n; l++) {
    MGLevel &M = lev[l];
    std::memset(&M, 0, sizeof(M));
    M.nx = lv.nx[l];
    M.ny = lv.ny[l];
    const size_t m = (size_t)M.nx * M.ny;
    float **arr[9] = {&M.cw, &M.ce, &M.cs, &M.cn, &M.area, &M.diag0, &M.d, &M.r, &M.rho};
    for (int a = 0; a < 9; a++) {
      *arr[a] = levF + fo;
      fo += m;
    }
    M.fixed = fixedAll + uo;
    uo += m;
    naLevelSetupKernel<<<(int)((m + kBlock - 1) / kBlock), kBlock, 0, st>>>(
        lv, l, gDx, gDy, fixedAll, nx, M.cw, M.ce, M.cs, M.cn, M.area, M.diag0, M.fixed);
    EMCG_CUDA(cudaGetLastError());
    if (l + 1 < lv.n) {
      const int nfx = M.nx, nfy = M.ny, ncx = lv.nx[l + 1], ncy = lv.ny[l + 1];
      M.pxIdx = trI + to;
      M.pxW = trF + to;
      to += nfx;
      M.pyIdx = trI + to;
      M.pyW = trF + to;
      to += nfy;
      M.rxIdx = trI + to;
      M.rxW = trF + to;
      to += 3 * (size_t)ncx;
      M.ryIdx = trI + to;
      M.ryW = trF + to;
      to += 3 * (size_t)ncy;
      M.mapX = trI + to;
      to += ncx;
      M.mapY = trI + to;
      to += ncy;
      naTransferKernel<<<(nfx + kBlock - 1) / kBlock, kBlock, 0, st>>>(lv, l, false, M.pxIdx,
                                                                       M.pxW, M.rxIdx, M.rxW,
                                                                       M.mapX);
      naTransferKernel<<<(nfy + kBlock - 1) / kBlock, kBlock, 0, st>>>(lv, l, true, M.pyIdx,
                                                                       M.pyW, M.ryIdx, M.ryW,
                                                                       M.mapY);
      EMCG_CUDA(cudaGetLastError());
    }
  }
  // Newton / defect correction: the loop of the allocating solver (float MG)
  const int grid = (n + kBlock - 1) / kBlock;
  if (reset_bc) {
    resetBCKernel<<<grid, kBlock, 0, st>>>(d_pot, resMask, d_conc ? resNe : resEq, n);
    EMCG_CUDA(cudaGetLastError());
  }
  const int pre = smooth > 0 ? smooth : 3, post = pre, coarseSweeps = 16;
  LevelK<float> K0 = levelK<float>(lev[0]);
  double h_stats[2] = {0, 0};
  double rel = INFINITY;
  int it = 0;
  double scale = 0.;
  for (; it <= max_cycles; it++) {
    // the residual maxima accumulate by atomic max and must start at zero
    EMCG_CUDA(cudaMemsetAsync(stats, 0, 4 * sizeof(double), st));
    nonlinResidualKernel<float><<<grid, kBlock, 0, st>>>(
        d_pot, d_conc, C, lev[0].fixed, gSum, d_conc ? gVne : gVeq, nx, ny, hF0, hF1, hP, K0.r,
        K0.rho, K0.d, stats, it == 0);
    EMCG_CUDA(cudaGetLastError());
    EMCG_CUDA(cudaMemcpyAsync(h_stats, stats, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
    EMCG_CUDA(cudaStreamSynchronize(st));
    if (it == 0)
      scale = h_stats[1];
    rel = scale > 0 ? h_stats[0] / scale : h_stats[0];
    if (rel <= rtol || it == max_cycles || !std::isfinite(rel))
      break;
    const int nv = rel < kNATwoCycleRel ? kNAVcyclesPerNewton : 1;
    for (int k = 0; k < nv; k++)
      naVcycle(lev, lv.n, 0, pre, post, coarseSweeps, st);
    updatePotKernel<float><<<grid, kBlock, 0, st>>>(d_pot, K0.d, lev[0].fixed, n, stats);
    EMCG_CUDA(cudaGetLastError());
  }
  if (rel_residual)
    *rel_residual = rel;
  if (cycles)
    *cycles = it;
  if (!std::isfinite(rel)) {
    setError("Poisson: non-finite residual after %d Newton steps (NaN or Inf in the potential, "
             "the concentration or a correction)", it);
    return EMCG_ERR_NONCONVERGED;
  }
  if (!(rel <= rtol)) {
    setError("Poisson: relative residual %.3e after %d Newton steps (target %.1e)", rel, it, rtol);
    return EMCG_ERR_NONCONVERGED;
  }
  return EMCG_OK;
}
