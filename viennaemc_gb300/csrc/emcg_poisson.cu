// Grid Poisson solver of the device engine: double-precision Newton / defect
// correction around geometric multigrid V-cycles (see emcg_poisson.cuh).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "emcg_host.h"
#include "emcg_poisson.cuh"

namespace emcg {

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

__global__ void resetBCKernel(double *pot, const uint8_t *mask, const double *val, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && mask[i])
    pot[i] = val[i];
}

// F(phi) of the reference equation, the Jacobian's reaction density and the
// FV-scaled right-hand side of the correction equation on level 0.
template <class MT>
__global__ void nonlinResidualKernel(const double *__restrict__ pot, const double *__restrict__ conc,
                                     const double *__restrict__ C, const uint8_t *__restrict__ fixed,
                                     const double *__restrict__ gSum, const double *__restrict__ gV,
                                     int nx, int ny, double hF0, double hF1, double hP,
                                     MT *__restrict__ rhs, MT *__restrict__ rho, MT *__restrict__ d,
                                     double *__restrict__ stats) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  double aF = 0., sc = 0.;
  if (i < nx * ny) {
    d[i] = MT(0);
    if (fixed[i]) {
      rhs[i] = MT(0);
      rho[i] = MT(0);
    } else {
      int x = i % nx, y = i / nx;
      double phi = pot[i];
      double p = exp(-phi);
      double n = conc ? conc[i] : exp(phi);
      double w = x > 0 ? pot[i - 1] : pot[i + 1];
      double e = x < nx - 1 ? pot[i + 1] : pot[i - 1];
      double s = y > 0 ? pot[i - nx] : pot[i + nx];
      double nn = y < ny - 1 ? pot[i + nx] : pot[i - nx];
      double F = hF0 * (w + e - 2 * phi) + hF1 * (s + nn - 2 * phi) + hP * (p - n + C[i]) +
                 (gV[i] - gSum[i] * phi);
      int bd = (x == 0 || x == nx - 1) + (y == 0 || y == ny - 1);
      double scale = bd == 0 ? 1.0 : (bd == 1 ? 0.5 : 0.25);
      rhs[i] = (MT)(F * scale);
      rho[i] = (MT)(conc ? p : p + n);
      aF = fabs(F);
      sc = hP * (fabs(C[i]) + n + p);
    }
  }
  double m1 = blockMax(aF);
  __syncthreads();
  double m2 = blockMax(sc);
  if (threadIdx.x == 0) {
    atomicMaxPos(&stats[0], m1);
    atomicMaxPos(&stats[1], m2);
  }
}

template <class MT>
__global__ void updatePotKernel(double *__restrict__ pot, const MT *__restrict__ d,
                                const uint8_t *__restrict__ fixed, int n, double *stats) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  double a = 0.;
  if (i < n && !fixed[i]) {
    double v = (double)d[i];
    v = fmin(kMaxNewtonStep, fmax(-kMaxNewtonStep, v));
    pot[i] += v;
    a = fabs(v);
  }
  double m = blockMax(a);
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
  L.d[i] = s / (L.diag0[i] + L.area[i] * L.rho[i]);
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
        L.d[i] = s / (L.diag0[i] + L.area[i] * L.rho[i]);
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
  return EMCG_OK;
}

void poissonFree(PoissonMG &P) {
  for (auto &L : P.L) {
    void *ps[] = {L.cw,  L.ce,    L.cs,    L.cn,    L.area,  L.diag0, L.dcw,   L.dce,
                  L.dcs, L.dcn,   L.darea, L.ddiag0, L.fixed, L.d,     L.r,     L.rho,
                  L.dd,  L.dr,    L.drho,  L.rxIdx, L.ryIdx, L.rxW,   L.ryW,   L.pxIdx,
                  L.pyIdx, L.pxW, L.pyW,   L.mapX,  L.mapY};
    for (void *p : ps)
      cudaFree(p);
  }
  P.L.clear();
  void *ps[] = {P.C, P.gSum, P.gVeq, P.gVne, P.resetMask, P.resetEq, P.resetNe, P.stats};
  for (void *p : ps)
    cudaFree(p);
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
  for (; it <= maxCycles; it++) {
    EMCG_CUDA(cudaMemsetAsync(P.stats, 0, 3 * sizeof(double), st));
    nonlinResidualKernel<MT><<<grid, kBlock, 0, st>>>(
        pot, conc, P.C, L0.fixed, P.gSum, conc ? P.gVne : P.gVeq, nx, ny, P.hF[0], P.hF[1], P.hP,
        K0.r, K0.rho, K0.d, P.stats);
    EMCG_CUDA(cudaGetLastError());
    EMCG_CUDA(cudaMemcpyAsync(stats, P.stats, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
    EMCG_CUDA(cudaStreamSynchronize(st));
    rel = stats[1] > 0 ? stats[0] / stats[1] : stats[0];
    if (rel <= rtol || it == maxCycles)
      break;
    vcycle<MT>(P, 0, st);
    updatePotKernel<MT><<<grid, kBlock, 0, st>>>(pot, K0.d, L0.fixed, n, P.stats);
    EMCG_CUDA(cudaGetLastError());
  }
  if (relRes)
    *relRes = rel;
  if (cycles)
    *cycles = it;
  if (!(rel <= rtol)) {
    setError("Poisson: relative residual %.3e after %d V-cycles (target %.1e)", rel, it, rtol);
    return EMCG_ERR_NONCONVERGED;
  }
  return EMCG_OK;
}

int32_t poissonSolve(PoissonMG &P, double *pot, const double *conc, bool resetBC, double rtol,
                     int maxCycles, cudaStream_t st, double *relRes, int *cycles) {
  return P.fp32 ? solveT<float>(P, pot, conc, resetBC, rtol, maxCycles, st, relRes, cycles)
                : solveT<double>(P, pot, conc, resetBC, rtol, maxCycles, st, relRes, cycles);
}

} // namespace emcg
