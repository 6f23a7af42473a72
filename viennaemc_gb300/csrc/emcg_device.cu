// Device (2-D) engine: the per-step pipeline of emcSimulation::performEMCStep
// (include/emcSimulation.hpp:164-193): Poisson -> E field -> drift/scatter
// with boundaries -> ohmic contacts (remove / inject) -> charge assignment
// and carrier concentration.  Particles live in double-buffered SoA arrays;
// removals are stable compactions so that the particle order -- and with it
// the random-number attribution of the reference -- is preserved.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "emcg_common.cuh"
#include "emcg_host.h"
#include "emcg_model.h"
#include "emcg_poisson.cuh"
#include "emcg_rates.cuh"

namespace emcg {

constexpr int kMaxScatterPerStepDev = 1 << 16;
constexpr int kCB = 1024; // compaction block

// ---------------------------------------------------------------------------
// kernel-side device description
// ---------------------------------------------------------------------------
struct DevK {
  int nx, ny;
  double hx, hy, invhx, invhy, maxX, maxY;
  double Vt, Ni, cellVol;
  const int32_t *region;      // doping region per node
  const int32_t *nodeContact; // getContactIdx (first boundary), -1 if none
  const uint8_t *nodeOhmic;   // isOhmicContact (first boundary)
  const int32_t *nodeRes;     // reservoir contact index (ohmic / Schottky)
  const int32_t *bnd[4];      // contact index along each boundary
};

template <class T> __device__ __forceinline__ int roundIdx(T v, double h, double invh);
template <> __device__ __forceinline__ int roundIdx<double>(double v, double h, double) {
  return (int)round(v / h);
}
template <> __device__ __forceinline__ int roundIdx<float>(float v, double, double invh) {
  return (int)rintf(v * (float)invh);
}
__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

template <class T> __device__ __forceinline__ T floorDiv(T v, double h, double invh, int &m);
template <> __device__ __forceinline__ double floorDiv<double>(double v, double h, double, int &m) {
  double q = v / h;
  double f = floor(q);
  m = (int)f;
  return q - f;
}
template <> __device__ __forceinline__ float floorDiv<float>(float v, double, double invh, int &m) {
  float q = v * (float)invh;
  float f = floorf(q);
  m = (int)f;
  return q - f;
}

template <class T>
__device__ __forceinline__ T gridAt(const DevK &G, const T *E, int x, int y) {
  return (x < 0 || y < 0 || x >= G.nx || y >= G.ny) ? T(0) : E[y * G.nx + x];
}

// NGP (include/PMSchemes/emcNGPScheme.hpp:46-57), CIC with the reference's
// weights (include/PMSchemes/emcCICScheme.hpp:126-143), NEC
// (include/PMSchemes/emcNECScheme.hpp:102-113: the element's two edges along
// each direction) or NEC-VWD (examples/mosfet2D/NECSchemeVWD.hpp,
// interpolateForce: nearest column, the edge below only on the last column).
// Corners outside the grid read 0 (a particle exactly on the far boundary).
template <class T, int SCHEME>
__device__ __forceinline__ void interpForce(const DevK &G, const T *Ex, const T *Ey, T x, T y,
                                            T charge, T F[2]) {
  if (SCHEME == EMCG_PM_NEC || SCHEME == EMCG_PM_NEC_VWD) {
    int mx, my;
    if (SCHEME == EMCG_PM_NEC)
      floorDiv<T>(x, G.hx, G.invhx, mx);
    else
      mx = roundIdx<T>(x, G.hx, G.invhx);
    floorDiv<T>(y, G.hy, G.invhy, my);
    F[0] = charge * (gridAt(G, Ex, mx, my) + gridAt(G, Ex, mx, my + 1)) / T(2);
    if (SCHEME == EMCG_PM_NEC_VWD && mx == G.nx - 1)
      F[1] = charge * gridAt(G, Ey, mx, my);
    else
      F[1] = charge * (gridAt(G, Ey, mx, my) + gridAt(G, Ey, mx + 1, my)) / T(2);
  } else if (SCHEME == EMCG_PM_NGP) {
    int cx = clampi(roundIdx<T>(x, G.hx, G.invhx), 0, G.nx - 1);
    int cy = clampi(roundIdx<T>(y, G.hy, G.invhy), 0, G.ny - 1);
    F[0] = charge * Ex[cy * G.nx + cx];
    F[1] = charge * Ey[cy * G.nx + cx];
  } else {
    int mx, my;
    T wX = floorDiv<T>(x, G.hx, G.invhx, mx);
    T wY = floorDiv<T>(y, G.hy, G.invhy, my);
    const T *E[2] = {Ex, Ey};
#pragma unroll
    for (int k = 0; k < 2; k++)
      F[k] = charge * (gridAt(G, E[k], mx, my) * wX * wY +
                       gridAt(G, E[k], mx + 1, my) * (T(1) - wX) * wY +
                       gridAt(G, E[k], mx, my + 1) * wX * (T(1) - wY) +
                       gridAt(G, E[k], mx + 1, my + 1) * (T(1) - wY) * (T(1) - wY));
  }
}

// emcMomentumDependentSurfaceScatterMechanism::solveForTheta
// (include/SurfaceScatterMechanisms/emcMomentumDependentSurfaceScatterMechanism.hpp:
// 38-66): the reference's fixed-point iteration as it stands, at most 10000
// steps, stopping once a step moves theta by at most 1e-10 (it often runs to
// the cap; the capped result is insensitive to rounding, ~1e-15 relative).
template <class T> __device__ __noinline__ T solveForTheta(T r, T height, T speed) {
  const T c = (T(2) * height * speed) * (T(2) * height * speed);
  const T e = m_exp(-c);
  T x = m_sqrt(r * (T(1) / (T(1) - e) - T(1) / c));
  T error = T(1);
  for (int it = 0; error > T(1e-10) && it < 10000; it++) {
    T si, co;
    m_sincos(x, &si, &co);
    const T ecos = m_exp(-c * (co * co));
    const T esin = m_exp(-c * (si * si));
    const T x1 = x - (((e - ecos) / c + si * si - r * (T(1) - (T(1) - e) / c)) *
                      (T(2) * esin * c * si * co * (ecos - T(1))) / (e * (c - T(1)) - T(1)));
    error = fabs(x1 - x);
    x = x1;
  }
  return x;
}

// emcScatterHandler::scatterParticleAtBoundary (include/emcScatterHandler.hpp:
// 172-191) with the surface mechanism of boundary b
// (emcSurfaceScatterMechanism::scatterParticle, :38-44): diffuse with the
// mechanism's probability (calculateAndAssignKAndPos, :128-148: |k| kept, k at
// polar angle theta from the inward normal), else specular; either way the
// position goes back into the device and k is turned inwards where it points
// out (scatterParticleSpecularly, :75-86).  The energy is not updated.
template <class T, class Src>
__device__ __forceinline__ void surfaceScatter(const ModelK<T> &M, const DevK &G, int b,
                                               T pos[2], T k[3], Src &rng) {
  const int kind = M.surfKind[b], perp = b >> 1;
  const T par = M.surfParam[b];
  const T pDiff = kind == EMCG_SURFACE_CONSTANT
                      ? T(1) - par // emcConstantSurfaceScatterMechanism.hpp:33
                      : T(1) - m_exp(-((T(2) * par * k[perp]) * (T(2) * par * k[perp])));
  if (rng.u01() < pDiff) {
    T theta;
    if (kind == EMCG_SURFACE_CONSTANT)
      theta = asin(m_sqrt(rng.u01()));
    else
      theta = solveForTheta(rng.u01(), par, m_sqrt(k[0] * k[0] + k[1] * k[1] + k[2] * k[2]));
    const T phi = T(2) * T(3.14159265358979323846) * rng.u01(); // constants::pi
    const T speed = m_sqrt(k[0] * k[0] + k[1] * k[1] + k[2] * k[2]);
    T st, ct, sp, cp;
    m_sincos(theta, &st, &ct);
    m_sincos(phi, &sp, &cp);
    k[perp] = speed * ct * ((b & 1) ? T(-1) : T(1));
    k[(perp + 1) % 3] = speed * st * cp;
    k[(perp + 2) % 3] = speed * st * sp;
  }
  const T mx[2] = {(T)G.maxX, (T)G.maxY};
#pragma unroll
  for (int i = 0; i < 2; i++) {
    if (pos[i] < T(0)) {
      pos[i] *= T(-1);
      if (k[i] < T(0))
        k[i] *= T(-1);
    } else if (pos[i] > mx[i]) {
      pos[i] = T(2) * mx[i] - pos[i];
      if (k[i] > T(0))
        k[i] *= T(-1);
    }
  }
}

// the first boundary (XMIN, XMAX, YMIN, YMAX) holding node (x, y)
// (emcSurface::getBoundaryPos, include/emcSurface.hpp:338-349)
__device__ __forceinline__ int boundaryOf(const DevK &G, int x, int y) {
  return x == 0 ? 0 : x == G.nx - 1 ? 1 : y == 0 ? 2 : 3;
}

// free flight under force F, then the boundary treatment of
// include/emcParticleDrift.hpp:41-66 (removal at ohmic contacts, a surface
// mechanism or specular reflection elsewhere) and the region update of
// include/ParticleHandler/emcAbstractParticleHandler.hpp:238-249.  kSurf: the
// instance for models with surface mechanisms (the others keep the plain
// reflection and their register allocation).
template <class T, bool kSurf, class Src>
__device__ __forceinline__ bool devDrift(const ModelK<T> &M, const DevK &G, int valley, int sub,
                                         const T F[2], T dt, T k[3], T &E, T pos[2],
                                         int &region, Src &rng) {
  const ValleyK<T> &V = M.v[valley];
  T fE[3];
  toEcs(V.rot[sub], F[0], F[1], T(0), fE);
  T fv[3] = {fE[0] * V.cF[0], fE[1] * V.cF[1], fE[2] * V.cF[2]};
  T kN[3];
  drift<T, 2>(V, sub, fv, dt, k, E, pos, kN);
  const T mx[2] = {(T)G.maxX, (T)G.maxY};
  if (pos[0] < T(0) || pos[0] > mx[0] || pos[1] < T(0) || pos[1] > mx[1]) {
    T pb[2];
#pragma unroll
    for (int i = 0; i < 2; i++) {
      T a = (mx[i] < pos[i]) ? mx[i] : pos[i];
      pb[i] = (T(0) < a) ? a : T(0);
    }
    int cx = clampi(roundIdx<T>(pb[0], G.hx, G.invhx), 0, G.nx - 1);
    int cy = clampi(roundIdx<T>(pb[1], G.hy, G.invhy), 0, G.ny - 1);
    if (G.nodeOhmic[cy * G.nx + cx]) {
      pos[0] = pb[0];
      pos[1] = pb[1];
      return true;
    }
    const int b = boundaryOf(G, cx, cy);
    if (kSurf && M.surfKind[b] != EMCG_SURFACE_SPECULAR) {
      surfaceScatter(M, G, b, pos, k, rng);
    } else {
#pragma unroll
      for (int i = 0; i < 2; i++) {
        if (pos[i] < T(0)) {
          pos[i] = -pos[i];
          k[i] = -k[i];
        } else if (pos[i] > mx[i]) {
          pos[i] = T(2) * mx[i] - pos[i];
          k[i] = -k[i];
        }
      }
    }
  }
  int cx = clampi(roundIdx<T>(pos[0], G.hx, G.invhx), 0, G.nx - 1);
  int cy = clampi(roundIdx<T>(pos[1], G.hy, G.invhy), 0, G.ny - 1);
  region = G.region[cy * G.nx + cx];
  return false;
}

__device__ __forceinline__ void recordErr(int *err, int code) {
  if (code)
    atomicCAS(err, 0, code);
}

// driftScatterParticles for one particle
// (include/ParticleHandler/emcBasicParticleHandler.hpp:93-139)
template <class T, int SCHEME, bool kSurf, class Src>
__device__ __forceinline__ int devParticleStep(const ModelK<T> &M, const DevK &G, const T *Ex,
                                               const T *Ey, T charge, T dt, T k[3], T pos[2],
                                               T &E, T &tau, T &gtau, int &valley, int &sub,
                                               int &region, Src &rng, bool &removed) {
  int err = 0;
  T F[2];
  interpForce<T, SCHEME>(G, Ex, Ey, pos[0], pos[1], charge, F);
  if (tau >= dt) {
    removed = devDrift<T, kSurf>(M, G, valley, sub, F, dt, k, E, pos, region, rng);
  } else {
    removed = devDrift<T, kSurf>(M, G, valley, sub, F, tau, k, E, pos, region, rng);
    T tRem = dt - tau;
    int guard = 0;
    while (tRem > T(0) && !removed) {
      if (++guard > kMaxScatterPerStepDev) {
        err = EMCG_ERR_TIMEOUT;
        break;
      }
      int e = scatterParticle(M, k, E, valley, sub, region, rng);
      if (e) {
        err = e;
        break;
      }
      T nt = -m_log(rng.ulog()) * tauOf(M, valley, region);
      tau += nt;
      interpForce<T, SCHEME>(G, Ex, Ey, pos[0], pos[1], charge, F);
      removed = devDrift<T, kSurf>(M, G, valley, sub, F, nt < tRem ? nt : tRem, k, E, pos,
                                       region, rng);
      tRem -= nt;
    }
  }
  tau -= dt;
  gtau -= dt;
  if (gtau <= T(0) && !removed) { // emcBasicParticleHandler.hpp:131-138
    if (M.grain)
      grainScatter(M, k, rng);
    gtau = -m_log(rng.ulog()) * M.grainTau;
  }
  return err;
}

// the float instance is capped at 64 registers, 4 blocks of 256 per SM (72
// registers gave 3; a one-step launch needs the warps to hide its loads)
template <class T, int SCHEME, bool REPLAY, bool kSurf>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 4 : 1)
    devMoveKernel(StateK<T> st, const ModelK<T> *__restrict__ models, DevK G,
                  const T *__restrict__ Ex, const T *__restrict__ Ey, T charge, T dt,
                  const int64_t *__restrict__ nPtr, uint32_t step, uint32_t key0, uint32_t key1,
                  uint32_t stream, uint8_t *__restrict__ drop, int32_t *__restrict__ netto,
                  const uint64_t *__restrict__ rw, const int64_t *__restrict__ roff,
                  int *__restrict__ err) {
  const int64_t n = *nPtr;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  const ModelK<T> &M = models[0];
  T k[3] = {st.kx[i], st.ky[i], st.kz[i]};
  T pos[2] = {st.px[i], st.py[i]};
  T E = st.E[i], tau = st.tau[i], gtau = st.gtau[i];
  uint32_t mt = st.meta[i];
  int valley = mt & 0xff, sub = (mt >> 8) & 0xff, region = mt >> 16;
  bool removed = false;
  int e;
  if constexpr (REPLAY) {
    ReplaySrc src{rw, roff[i], roff[i + 1], 0};
    e = devParticleStep<T, SCHEME, kSurf>(M, G, Ex, Ey, charge, dt, k, pos, E, tau, gtau, valley,
                                          sub, region, src, removed);
    if (!e && (src.bad || src.pos != src.end))
      e = EMCG_ERR_REPLAY;
  } else {
    PhiloxSrc<T> src;
    src.init((uint32_t)i, step, stream, key0, key1);
    e = devParticleStep<T, SCHEME, kSurf>(M, G, Ex, Ey, charge, dt, k, pos, E, tau, gtau, valley,
                                          sub, region, src, removed);
  }
  recordErr(err, e);
  st.kx[i] = k[0];
  st.ky[i] = k[1];
  st.kz[i] = k[2];
  st.px[i] = pos[0];
  st.py[i] = pos[1];
  st.E[i] = E;
  st.tau[i] = tau;
  st.gtau[i] = gtau;
  st.meta[i] = packMeta(valley, sub, region);
  drop[i] = removed ? 1 : 0;
  if (removed) {
    int cx = clampi(roundIdx<T>(pos[0], G.hx, G.invhx), 0, G.nx - 1);
    int cy = clampi(roundIdx<T>(pos[1], G.hy, G.invhy), 0, G.ny - 1);
    int c = G.nodeContact[cy * G.nx + cx];
    if (c >= 0)
      atomicAdd(&netto[c], 1);
  }
}

// ---- stable compaction ------------------------------------------------------
__device__ __forceinline__ int blockExclusiveScan(int v, int *total) {
  __shared__ int warpSums[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o)
      x += y;
  }
  if (lane == 31)
    warpSums[w] = x;
  __syncthreads();
  if (w == 0) {
    int s = lane < (int)(blockDim.x >> 5) ? warpSums[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o)
        s += y;
    }
    warpSums[lane] = s; // inclusive over warps
  }
  __syncthreads();
  int off = (w > 0 ? warpSums[w - 1] : 0) + x - v;
  *total = warpSums[(blockDim.x >> 5) - 1];
  __syncthreads();
  return off;
}

__global__ void compactCountKernel(const uint8_t *__restrict__ drop, const int64_t *__restrict__ nPtr,
                                   int32_t *__restrict__ blockCount) {
  const int64_t n = *nPtr;
  const int64_t i = (int64_t)blockIdx.x * kCB + threadIdx.x;
  int keep = (i < n && !drop[i]) ? 1 : 0;
  int tot;
  blockExclusiveScan(keep, &tot);
  if (threadIdx.x == 0)
    blockCount[blockIdx.x] = tot;
}

// exclusive scan of nb block counts (one block); total -> *nOut
__global__ void scanBlocksKernel(int32_t *__restrict__ counts, int nb, int64_t *__restrict__ nOut) {
  int64_t carry = 0;
  for (int base = 0; base < nb; base += blockDim.x) {
    int i = base + threadIdx.x;
    int v = i < nb ? counts[i] : 0;
    int tot;
    int ex = blockExclusiveScan(v, &tot);
    if (i < nb)
      counts[i] = (int32_t)(carry + ex);
    carry += tot;
  }
  if (threadIdx.x == 0)
    *nOut = carry;
}

template <class T>
__global__ void compactScatterKernel(StateK<T> src, StateK<T> dst, const uint8_t *__restrict__ drop,
                                     const int64_t *__restrict__ nPtr,
                                     const int32_t *__restrict__ blockOff) {
  const int64_t n = *nPtr;
  const int64_t i = (int64_t)blockIdx.x * kCB + threadIdx.x;
  int keep = (i < n && !drop[i]) ? 1 : 0;
  int tot;
  int r = blockExclusiveScan(keep, &tot);
  if (!keep)
    return;
  int64_t j = blockOff[blockIdx.x] + r;
  dst.kx[j] = src.kx[i];
  dst.ky[j] = src.ky[i];
  dst.kz[j] = src.kz[i];
  dst.px[j] = src.px[i];
  dst.py[j] = src.py[i];
  dst.pz[j] = src.pz[i];
  dst.E[j] = src.E[i];
  dst.tau[j] = src.tau[i];
  dst.gtau[j] = src.gtau[i];
  dst.meta[j] = src.meta[i];
}

// ---- contacts (include/ParticleHandler/emcBasicParticleHandler.hpp:158-192) --
// list of the particles sitting at reservoir nodes, in index order
template <class T>
__global__ void reservoirListKernel(StateK<T> st, DevK G, const int64_t *__restrict__ nPtr,
                                    const uint8_t *__restrict__ skip,
                                    int32_t *__restrict__ list, int32_t *__restrict__ listNode,
                                    int32_t *__restrict__ listCount) {
  const int64_t n = *nPtr;
  const int64_t i = (int64_t)blockIdx.x * kCB + threadIdx.x;
  int node = -1;
  if (i < n && !(skip && skip[i])) { // skip: removed by the move, not yet compacted
    int cx = clampi(roundIdx<T>(st.px[i], G.hx, G.invhx), 0, G.nx - 1);
    int cy = clampi(roundIdx<T>(st.py[i], G.hy, G.invhy), 0, G.ny - 1);
    int g = cy * G.nx + cx;
    if (G.nodeRes[g] >= 0)
      node = g;
  }
  int tot;
  int r = blockExclusiveScan(node >= 0 ? 1 : 0, &tot);
  if (node >= 0) {
    list[(int64_t)blockIdx.x * kCB + r] = (int32_t)i;
    listNode[(int64_t)blockIdx.x * kCB + r] = node;
  }
  if (threadIdx.x == 0)
    listCount[blockIdx.x] = tot;
}

// the per-block reservoir lists, concatenated in block order: all reservoir
// particles in index order (off = exclusive scan of the block counts)
__global__ void gatherListKernel(const int32_t *__restrict__ list,
                                 const int32_t *__restrict__ listNode,
                                 const int32_t *__restrict__ off, int nb,
                                 const int64_t *__restrict__ total, int32_t *__restrict__ gList,
                                 int32_t *__restrict__ gNode) {
  const int b = blockIdx.x;
  const int o = off[b];
  const int cnt = (b + 1 < nb ? off[b + 1] : (int)*total) - o;
  for (int j = threadIdx.x; j < cnt; j += blockDim.x) {
    gList[o + j] = list[(int64_t)b * kCB + j];
    gNode[o + j] = listNode[(int64_t)b * kCB + j];
  }
}

// Ranking of the particles on reservoir nodes (emcBasicParticleHandler::
// handleOhmicContacts, :158-192): the r-th particle at a node (r from 0, in
// particle order) stays while r * carriers is below the expected number there,
// the rest are marked for removal.  The gathered list (particle order) is cut
// into kRankChunks chunks; a warp per (node, chunk) counts the node's entries
// in its chunk (contactCountKernel), then ranks them from the counts of the
// earlier chunks (contactRankKernel), so no warp walks the whole list.
constexpr int kRankChunks = 16;

__device__ __forceinline__ void rankChunk(int R, int c, int &j0, int &j1) {
  const int len = (R + kRankChunks - 1) / kRankChunks;
  j0 = min(R, c * len);
  j1 = min(R, j0 + len);
}

__global__ void contactCountKernel(const int32_t *__restrict__ gNode,
                                   const int64_t *__restrict__ total,
                                   const int32_t *__restrict__ resNodes, int nRes,
                                   int32_t *__restrict__ chunkCount) {
  const int w = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (w >= nRes * kRankChunks)
    return;
  const int r = w / kRankChunks, c = w - r * kRankChunks;
  const int g = resNodes[r];
  int j0, j1;
  rankChunk((int)*total, c, j0, j1);
  int cnt = 0;
  for (int base = j0; base < j1; base += 32) {
    const int j = base + lane;
    cnt += __popc(__ballot_sync(0xffffffffu, j < j1 && gNode[j] == g));
  }
  if (lane == 0)
    chunkCount[w] = cnt;
}

__global__ void contactRankKernel(const int32_t *__restrict__ gList,
                                  const int32_t *__restrict__ gNode,
                                  const int64_t *__restrict__ total,
                                  const int32_t *__restrict__ resNodes, int nRes,
                                  const double *__restrict__ expNr, double nrC,
                                  const int32_t *__restrict__ nodeContact,
                                  const int32_t *__restrict__ chunkCount,
                                  uint8_t *__restrict__ drop, int32_t *__restrict__ kept,
                                  int32_t *__restrict__ remInj) {
  const int w = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (w >= nRes * kRankChunks)
    return;
  const int r = w / kRankChunks, c = w - r * kRankChunks;
  const int g = resNodes[r];
  const double e = expNr[g];
  int j0, j1;
  rankChunk((int)*total, c, j0, j1);
  int seen = 0; // the node's entries in the earlier chunks
  for (int q = 0; q < c; q++)
    seen += chunkCount[r * kRankChunks + q];
  int nKept = 0, nDrop = 0;
  for (int base = j0; base < j1; base += 32) {
    const int j = base + lane;
    const bool mine = j < j1 && gNode[j] == g;
    const unsigned m = __ballot_sync(0xffffffffu, mine);
    if (mine) {
      const int rk = seen + __popc(m & ((1u << lane) - 1u));
      if ((double)rk * nrC < e)
        nKept++;
      else {
        drop[gList[j]] = 1;
        nDrop++;
      }
    }
    seen += __popc(m);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    nKept += __shfl_xor_sync(0xffffffffu, nKept, o);
    nDrop += __shfl_xor_sync(0xffffffffu, nDrop, o);
  }
  if (lane == 0) {
    if (nKept)
      atomicAdd(&kept[g], nKept);
    if (nDrop)
      atomicAdd(&remInj[nodeContact[g]], -nDrop);
  }
}

// particles to inject per reservoir node (emcAbstractParticleHandler.hpp:200-216)
__global__ void injectCountKernel(const int32_t *__restrict__ resNodes, int nRes,
                                  const double *__restrict__ expNr, const int32_t *__restrict__ kept,
                                  double nrC, int32_t *__restrict__ injCount) {
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nRes)
    return;
  int g = resNodes[r];
  double diff = expNr[g] - (double)kept[g] * nrC;
  int c = 0;
  while (diff > 0 && c < (1 << 20)) {
    c++;
    diff -= nrC;
  }
  injCount[r] = c;
}

// emcElectron::generateInjectedParticle + initParticlePos (2-D)
template <class T, class Src>
__device__ __forceinline__ void initParticle2D(const ModelK<T> &M, const DevK &G, int cx, int cy,
                                               int region, bool tauRegionIsValley, Src &rng,
                                               T k[3], T pos[2], T &E, T &tau, T &gtau,
                                               int &valley, int &sub) {
  const int c[2] = {cx, cy};
  const int ext[2] = {G.nx, G.ny};
  const double h[2] = {G.hx, G.hy};
#pragma unroll
  for (int d = 0; d < 2; d++) {
    if (c[d] == ext[d] - 1)
      pos[d] = ((T)c[d] - rng.u01() * T(0.5)) * (T)h[d];
    else if (c[d] == 0)
      pos[d] = rng.u01() * T(0.5) * (T)h[d];
    else
      pos[d] = ((T)c[d] + rng.u01() - T(0.5)) * (T)h[d];
  }
  valley = (int)m_floor((T)M.nV * rng.ulog());
  const ValleyK<T> &V = M.v[valley];
  sub = (int)m_floor((T)V.deg * rng.ulog());
  E = T(-1.5) * (T)G.Vt * m_log(rng.ulog());
  randomDirection(V.cK * m_sqrt(gammaOf(V, E)), rng, k);
#pragma unroll
  for (int d = 0; d < 2; d++)
    if ((c[d] == 0 && k[d] < T(0)) || (c[d] == ext[d] - 1 && k[d] > T(0)))
      k[d] *= T(-1);
  tau = -m_log(rng.ulog()) * tauOf(M, valley, tauRegionIsValley ? valley : region);
  gtau = -m_log(rng.ulog()) * M.grainTau;
}

template <class T, bool REPLAY>
__global__ void injectKernel(StateK<T> st, const ModelK<T> *__restrict__ models, DevK G,
                             const int32_t *__restrict__ resNodes, int nRes,
                             const int32_t *__restrict__ injBase, const int64_t *__restrict__ injTotal,
                             int64_t *__restrict__ nPtr, int64_t capacity, uint32_t step,
                             uint32_t key0, uint32_t key1, uint32_t stream, bool tauRegionIsValley,
                             int32_t *__restrict__ remInj, const uint64_t *__restrict__ rw,
                             const int64_t *__restrict__ roff, int *__restrict__ err) {
  const int64_t total = *injTotal;
  const int64_t n = *nPtr;
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= total)
    return;
  if (n + total > capacity) {
    if (j == 0)
      recordErr(err, EMCG_ERR_CAPACITY);
    return;
  }
  int lo = 0, hi = nRes - 1; // last r with injBase[r] <= j
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (injBase[mid] <= j)
      lo = mid;
    else
      hi = mid - 1;
  }
  const int g = resNodes[lo];
  const int cx = g % G.nx, cy = g / G.nx;
  const int region = G.region[g];
  T k[3], pos[2], E, tau, gtau;
  int valley, sub;
  const ModelK<T> &M = models[0];
  if constexpr (REPLAY) {
    ReplaySrc src{rw, roff[j], roff[j + 1], 0};
    initParticle2D(M, G, cx, cy, region, tauRegionIsValley, src, k, pos, E, tau, gtau, valley, sub);
    if (src.bad || src.pos != src.end)
      recordErr(err, EMCG_ERR_REPLAY);
  } else {
    PhiloxSrc<T> src;
    src.init((uint32_t)j, step, stream | 0x80000000u, key0, key1);
    initParticle2D(M, G, cx, cy, region, tauRegionIsValley, src, k, pos, E, tau, gtau, valley, sub);
  }
  const int64_t d = n + j;
  st.kx[d] = k[0];
  st.ky[d] = k[1];
  st.kz[d] = k[2];
  st.px[d] = pos[0];
  st.py[d] = pos[1];
  st.pz[d] = T(0);
  st.E[d] = E;
  st.tau[d] = tau;
  st.gtau[d] = gtau;
  st.meta[d] = packMeta(valley, sub, region);
  atomicAdd(&remInj[G.nodeContact[g]], 1);
}

__global__ void addCountKernel(int64_t *nPtr, const int64_t *add, int64_t capacity) {
  if (*nPtr + *add <= capacity)
    *nPtr += *add;
}

// initial particles at given nodes (counts decided on the host)
template <class T>
__global__ void devInitKernel(StateK<T> st, const ModelK<T> *__restrict__ models, DevK G,
                              const int32_t *__restrict__ nodeOf, int64_t n, uint32_t key0,
                              uint32_t key1, uint32_t stream, bool tauRegionIsValley) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  const int g = nodeOf[i];
  const int region = G.region[g];
  T k[3], pos[2], E, tau, gtau;
  int valley, sub;
  PhiloxSrc<T> src;
  src.init((uint32_t)i, 0xFFFFFFFFu, stream, key0, key1);
  initParticle2D(models[0], G, g % G.nx, g / G.nx, region, tauRegionIsValley, src, k, pos, E,
                 tau, gtau, valley, sub);
  st.kx[i] = k[0];
  st.ky[i] = k[1];
  st.kz[i] = k[2];
  st.px[i] = pos[0];
  st.py[i] = pos[1];
  st.pz[i] = T(0);
  st.E[i] = E;
  st.tau[i] = tau;
  st.gtau[i] = gtau;
  st.meta[i] = packMeta(valley, sub, region);
}

// ---- particle -> mesh ------------------------------------------------------
// Deposition in fixed point.  Each particle adds its corner weights to the
// nodes as integers, so the node sums do not depend on the order in which the
// atomics run: the assigned charge is the same bit for bit on every run
// (double-precision atomics add in a different order each run, and the last
// bits of the charge, and so of the potential, change).  The double engine's
// weights are 128-bit fixed point at 2^fixBits, the largest scale for which
// the capacity's worth of particles at one node stays below 2^126: a weight
// keeps every bit above 2^-fixBits, so even a corner weight of 1e-14 keeps its
// double precision, and the sums equal the double sums of the reference to
// about one rounding.  The float engine forms its weights in float and adds
// them as 64-bit integers at 2^fixBitsF (capacity's worth below 2^62), finer
// than the float positions' own rounding.  The weights are the reference
// schemes':
//   NGP  the whole particle to round(pos / h) (emcNGPScheme.hpp:21-66);
//   CIC  w = pos / h - floor to the lower node (emcCICScheme.hpp:30-66);
//   NEC  a quarter to each corner of the element (emcNECScheme.hpp:24-33).
// Sorting the particles by cell to combine a warp's weights before the
// atomics was built and measured: since the particles stay in the reference's
// order (its contact rule and the replay depend on it), the sort is four more
// passes a step, and the resistor's step took 0.651 ms against 0.620 ms.

// w >= 0 as the 128-bit integer w 2^k (bits below 2^-k dropped)
__device__ __forceinline__ void toFix128(double w, int k, unsigned long long &lo,
                                        unsigned long long &hi) {
  lo = hi = 0;
  if (!(w > 0.))
    return;
  int ex;
  const double f = frexp(w, &ex);                              // w = f 2^ex, f in [0.5, 1)
  const unsigned long long m = (unsigned long long)ldexp(f, 53); // w = m 2^(ex - 53)
  const int sh = ex - 53 + k;
  if (sh >= 64) {
    hi = m << (sh - 64);
  } else if (sh > 0) {
    lo = m << sh;
    hi = m >> (64 - sh);
  } else if (sh > -64) {
    lo = m >> (-sh);
  }
}

// 128-bit add of (lo, hi) to a node's two words: the carry of the low word
// goes to the high word, so the pair sums exactly in any order
__device__ __forceinline__ void fixAdd(const DevK &G, unsigned long long *fix, int x, int y,
                                       unsigned long long lo, unsigned long long hi) {
  if (x < 0 || y < 0 || x >= G.nx || y >= G.ny || (lo == 0 && hi == 0))
    return; // the far-boundary corner of a particle exactly on maxPos
  unsigned long long *p = fix + 2 * ((size_t)y * G.nx + x);
  const unsigned long long old = atomicAdd(p, lo);
  hi += (old + lo < old) ? 1ull : 0ull;
  if (hi)
    atomicAdd(p + 1, hi);
}

template <class T, int SCHEME>
__global__ void assignKernel(StateK<T> st, DevK G, const int64_t *__restrict__ nPtr, double nrC,
                             int fixBits, unsigned long long *__restrict__ fix) {
  const int64_t n = *nPtr;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  int mx, my;
  if constexpr (sizeof(T) == 4) {
    const float s = ldexpf((float)nrC, fixBits);
    unsigned long long v[4];
    if (SCHEME == EMCG_PM_NGP) {
      mx = roundIdx<float>(st.px[i], G.hx, G.invhx);
      my = roundIdx<float>(st.py[i], G.hy, G.invhy);
      fixAdd(G, fix, mx, my, __float2ull_rn(s), 0ull);
      return;
    } else if (SCHEME == EMCG_PM_CIC) {
      const float wX = floorDiv<float>(st.px[i], G.hx, G.invhx, mx);
      const float wY = floorDiv<float>(st.py[i], G.hy, G.invhy, my);
      v[0] = __float2ull_rn(wX * wY * s);
      v[1] = __float2ull_rn((1.f - wX) * wY * s);
      v[2] = __float2ull_rn(wX * (1.f - wY) * s);
      v[3] = __float2ull_rn((1.f - wX) * (1.f - wY) * s);
    } else {
      floorDiv<float>(st.px[i], G.hx, G.invhx, mx);
      floorDiv<float>(st.py[i], G.hy, G.invhy, my);
      v[0] = v[1] = v[2] = v[3] = __float2ull_rn(0.25f * s);
    }
    fixAdd(G, fix, mx, my, v[0], 0ull);
    fixAdd(G, fix, mx + 1, my, v[1], 0ull);
    fixAdd(G, fix, mx, my + 1, v[2], 0ull);
    fixAdd(G, fix, mx + 1, my + 1, v[3], 0ull);
  } else {
    double w[4];
    if (SCHEME == EMCG_PM_NGP) {
      mx = roundIdx<T>(st.px[i], G.hx, G.invhx);
      my = roundIdx<T>(st.py[i], G.hy, G.invhy);
      unsigned long long lo, hi;
      toFix128(nrC, fixBits, lo, hi);
      fixAdd(G, fix, mx, my, lo, hi);
      return;
    } else if (SCHEME == EMCG_PM_CIC) {
      const double wX = (double)floorDiv<T>(st.px[i], G.hx, G.invhx, mx);
      const double wY = (double)floorDiv<T>(st.py[i], G.hy, G.invhy, my);
      w[0] = wX * wY * nrC;
      w[1] = (1 - wX) * wY * nrC;
      w[2] = wX * (1 - wY) * nrC;
      w[3] = (1 - wX) * (1 - wY) * nrC;
    } else {
      floorDiv<T>(st.px[i], G.hx, G.invhx, mx);
      floorDiv<T>(st.py[i], G.hy, G.invhy, my);
      w[0] = w[1] = w[2] = w[3] = 0.25 * nrC;
    }
    const int cx[4] = {mx, mx + 1, mx, mx + 1}, cy[4] = {my, my, my + 1, my + 1};
#pragma unroll
    for (int c = 0; c < 4; c++) {
      unsigned long long lo, hi;
      toFix128(w[c], fixBits, lo, hi);
      fixAdd(G, fix, cx[c], cy[c], lo, hi);
    }
  }
}

// the fixed-point sums as particle counts, and the concentration
// (include/emcSimulationResults.hpp:98-116)
__global__ void concKernel(DevK G, const unsigned long long *__restrict__ fix, int fixBits,
                           double *__restrict__ nr, double *__restrict__ conc) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= G.nx * G.ny)
    return;
  nr[i] = ldexp((double)fix[2 * i + 1], 64 - fixBits) + ldexp((double)fix[2 * i], -fixBits);
  int x = i % G.nx, y = i / G.nx;
  double c = nr[i] / G.Ni * (1. / G.cellVol);
  if (x == 0 || x == G.nx - 1)
    c *= 2;
  if (y == 0 || y == G.ny - 1)
    c *= 2;
  conc[i] = c;
}

// The E field of the PM scheme.  NGP, CIC: at the grid points
// (include/PMSchemes/emcEFieldCalculation.hpp:13-30).  NEC: forward differences
// on the edges (calcEFieldAtEdgeMidPts, :35-52).  Both then take the boundary
// values of :58-81 (0 normal to an artificial boundary, else the neighbour).
// NEC-VWD (examples/mosfet2D/NECSchemeVWD.hpp, calcEField): forward
// differences, 0 on the last edge, no boundary pass.
template <class T>
__global__ void efieldKernel(DevK G, const double *__restrict__ pot, T *__restrict__ Ex,
                             T *__restrict__ Ey, int scheme) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= G.nx * G.ny)
    return;
  const int nx = G.nx, ny = G.ny, x = i % nx, y = i / nx;
  const bool edges = scheme == EMCG_PM_NEC || scheme == EMCG_PM_NEC_VWD;
  auto ex = [&](int xi) {
    int j = y * nx + xi;
    return edges ? (pot[j] - pot[j + 1]) * G.Vt / G.hx
                 : (pot[j - 1] - pot[j + 1]) * G.Vt / (2 * G.hx);
  };
  auto ey = [&](int yi) {
    int j = yi * nx + x;
    return edges ? (pot[j] - pot[j + nx]) * G.Vt / G.hy
                 : (pot[j - nx] - pot[j + nx]) * G.Vt / (2 * G.hy);
  };
  if (scheme == EMCG_PM_NEC_VWD) {
    Ex[i] = (T)(x != nx - 1 ? ex(x) : 0.);
    Ey[i] = (T)(y != ny - 1 ? ey(y) : 0.);
    return;
  }
  double vx, vy;
  if (x != 0 && x != nx - 1)
    vx = ex(x);
  else if (x == 0)
    vx = G.bnd[0][y] == -1 ? 0. : ex(1);
  else
    vx = G.bnd[1][y] == -1 ? 0. : ex(nx - 2);
  if (y != 0 && y != ny - 1)
    vy = ey(y);
  else if (y == 0)
    vy = G.bnd[2][x] == -1 ? 0. : ey(1);
  else
    vy = G.bnd[3][x] == -1 ? 0. : ey(ny - 2);
  Ex[i] = (T)vx;
  Ey[i] = (T)vy;
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct DeviceImpl {
  int precision = EMCG_FP64;
  bool surfaces = false; // the model has a surface mechanism (devMoveKernel's kSurf)
  size_t tsz = 8;
  emcg_device_config cfg;
  int nx = 0, ny = 0, nContacts = 0;
  double hx = 0, hy = 0, maxX = 0, maxY = 0, width = 0, T = 300, Ni = 0, epsR = 0, Vt = 0;
  double cellVol = 0;
  std::vector<double> doping;
  std::vector<int32_t> region, bnd[4], ctype;
  std::vector<double> cvolt, cpar;
  std::vector<int32_t> nodeContactH, nodeResH, resNodesH;
  std::vector<uint8_t> nodeOhmicH;
  std::vector<double> expNrH;
  // device
  void *dModel = nullptr, *dTables = nullptr;
  RateLayout rates;            // table layout (rate-table rebuild)
  RateScratch rateScratch;     // device scratch of rebuilds
  int32_t *dRegion = nullptr, *dNodeContact = nullptr, *dNodeRes = nullptr, *dBnd[4] = {};
  uint8_t *dNodeOhmic = nullptr;
  double *dPot = nullptr, *dNr = nullptr, *dConc = nullptr, *dExp = nullptr;
  void *dEx = nullptr, *dEy = nullptr;
  void *dState[2][9] = {};
  uint32_t *dMeta[2] = {};
  int cur = 0;
  int64_t capacity = 0;
  int64_t *dN = nullptr; // [0] particle count, [1] scratch count, [2] injection total,
                         // [3] reservoir particles
  uint8_t *dDrop = nullptr;
  int32_t *dBlock = nullptr;  // per compaction block counts / offsets
  int32_t *dList = nullptr, *dListNode = nullptr, *dListCount = nullptr;
  int32_t *dKept = nullptr;
  int32_t *dChunkCount = nullptr; // [reservoir node][kRankChunks] (contact ranking)
  int32_t *dGList = nullptr, *dGNode = nullptr; // reservoir particles in index order
  int32_t *dResNodes = nullptr, *dInjCount = nullptr;
  int32_t *dNetto = nullptr, *dRemInj = nullptr;
  // deposition: 128-bit fixed-point node sums (low, high word) at 2^fixBits
  // (double engine) or 2^fixBitsF (float engine, low word only)
  unsigned long long *dNodeFix = nullptr;
  int fixBits = 0, fixBitsF = 0;
  int *dErr = nullptr;
  int64_t injBound = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[4] = {};
  PoissonMG mg;
  bool bcReset = true; // the next non-equilibrium solve resets the contact values
  // replay
  uint64_t *dWords[2] = {};
  int64_t *dOff[2] = {};
  int64_t wordsCap[2] = {0, 0}, offCap[2] = {0, 0};
  bool replay[2] = {false, false};
  double stepMs = 0, poissonMs = 0;
  int64_t poissonCycles = 0, poissonSolves = 0; // V-cycles and solves of the last step call
  int nBlocks() const { return (int)((capacity + kCB - 1) / kCB); }
};

static DevK devK(const DeviceImpl *d) {
  DevK G;
  G.nx = d->nx;
  G.ny = d->ny;
  G.hx = d->hx;
  G.hy = d->hy;
  G.invhx = 1.0 / d->hx;
  G.invhy = 1.0 / d->hy;
  G.maxX = d->maxX;
  G.maxY = d->maxY;
  G.Vt = d->Vt;
  G.Ni = d->Ni;
  G.cellVol = d->cellVol;
  G.region = d->dRegion;
  G.nodeContact = d->dNodeContact;
  G.nodeOhmic = d->dNodeOhmic;
  G.nodeRes = d->dNodeRes;
  for (int b = 0; b < 4; b++)
    G.bnd[b] = d->dBnd[b];
  return G;
}

template <class T> static StateK<T> devState(DeviceImpl *d, int which) {
  StateK<T> s;
  T **f[9] = {&s.kx, &s.ky, &s.kz, &s.px, &s.py, &s.pz, &s.E, &s.tau, &s.gtau};
  for (int i = 0; i < 9; i++)
    *f[i] = (T *)d->dState[which][i];
  s.meta = d->dMeta[which];
  return s;
}

static int32_t readErr(DeviceImpl *d) {
  int e = 0;
  EMCG_CUDA(cudaMemcpyAsync(&e, d->dErr, sizeof(int), cudaMemcpyDeviceToHost, d->stream));
  EMCG_CUDA(cudaStreamSynchronize(d->stream));
  if (e) {
    EMCG_CUDA(cudaMemsetAsync(d->dErr, 0, sizeof(int), d->stream));
    setError("device kernel reported: %s", statusName(e));
    return e;
  }
  return EMCG_OK;
}

static int32_t devOf(emcg_handle *h, DeviceImpl **out) {
  EMCG_CHECK_ARG(h && h->kind == 2 && h->dev, "handle is not a device engine");
  *out = h->dev;
  return EMCG_OK;
}

int32_t deviceUpdateRates(emcg_handle *h, const double *raw, bool onDevice) {
  DeviceImpl *d;
  EMCG_TRY(devOf(h, &d));
  if (d->precision == EMCG_FP64)
    return launchRateUpdate<double>(d->dModel, d->dTables, d->rates, raw, onDevice,
                                    d->rateScratch, d->dErr, d->stream);
  return launchRateUpdate<float>(d->dModel, d->dTables, d->rates, raw, onDevice,
                                 d->rateScratch, d->dErr, d->stream);
}

int32_t deviceGetRates(emcg_handle *h, double *tables, double *tau) {
  DeviceImpl *d;
  EMCG_TRY(devOf(h, &d));
  EMCG_TRY(d->precision == EMCG_FP64
               ? readRateTables<double>(d->dModel, d->dTables, d->rates, tables, tau, d->stream)
               : readRateTables<float>(d->dModel, d->dTables, d->rates, tables, tau, d->stream));
  return readErr(d);
}

int32_t destroyDevice(emcg_handle *h) {
  DeviceImpl *d = h ? h->dev : nullptr;
  if (!d)
    return EMCG_OK;
  if (d->stream)
    cudaStreamSynchronize(d->stream);
  poissonFree(d->mg);
  void *ps[] = {d->dModel, d->dTables, d->dRegion, d->dNodeContact, d->dNodeRes, d->dNodeOhmic,
                d->dPot, d->dNr, d->dConc, d->dExp, d->dEx, d->dEy, d->dN, d->dDrop, d->dBlock,
                d->dList, d->dListNode, d->dListCount, d->dGList, d->dGNode, d->dKept,
                d->dChunkCount, d->dResNodes,
                d->dInjCount, d->dNetto, d->dRemInj, d->dErr, d->dNodeFix};
  freeRateScratch(d->rateScratch);
  for (void *p : ps)
    cudaFree(p);
  for (int b = 0; b < 4; b++)
    cudaFree(d->dBnd[b]);
  for (int w = 0; w < 2; w++) {
    for (void *p : d->dState[w])
      cudaFree(p);
    cudaFree(d->dMeta[w]);
    cudaFree(d->dWords[w]);
    cudaFree(d->dOff[w]);
  }
  for (auto &e : d->ev)
    if (e)
      cudaEventDestroy(e);
  if (d->stream)
    cudaStreamDestroy(d->stream);
  delete d;
  h->dev = nullptr;
  return EMCG_OK;
}

// surface queries (include/emcSurface.hpp) on the host description
static int firstBoundary(const DeviceImpl *d, int x, int y) {
  if (x == 0)
    return 0;
  if (x == d->nx - 1)
    return 1;
  if (y == 0)
    return 2;
  if (y == d->ny - 1)
    return 3;
  return -1;
}
static int contactAt(const DeviceImpl *d, int b, int x, int y) {
  return b < 2 ? d->bnd[b][y] : d->bnd[b][x];
}

template <class V> static int32_t up(V **dst, const V *src, size_t n, cudaStream_t st) {
  EMCG_CUDA(cudaMalloc(dst, sizeof(V) * std::max<size_t>(n, 1)));
  if (n)
    EMCG_CUDA(cudaMemcpyAsync(*dst, src, sizeof(V) * n, cudaMemcpyHostToDevice, st));
  return EMCG_OK;
}

template <class T> static int32_t createModel(DeviceImpl *d, const emcg_model_desc &m) {
  ModelK<T> K;
  std::vector<T> tab;
  EMCG_TRY(buildModelK<T>(m, K, tab));
  d->rates = rateLayoutOf(m);
  d->surfaces = false;
  for (int b = 0; b < 4; b++)
    d->surfaces = d->surfaces || m.surface_kind[b] != EMCG_SURFACE_SPECULAR;
  EMCG_TRY(up((T **)&d->dTables, tab.data(), tab.size(), d->stream));
  K.tables = (const T *)d->dTables;
  EMCG_TRY(up((ModelK<T> **)&d->dModel, &K, 1, d->stream));
  const size_t n = (size_t)d->nx * d->ny;
  EMCG_CUDA(cudaMalloc(&d->dEx, n * sizeof(T)));
  EMCG_CUDA(cudaMalloc(&d->dEy, n * sizeof(T)));
  EMCG_CUDA(cudaMemsetAsync(d->dEx, 0, n * sizeof(T), d->stream));
  EMCG_CUDA(cudaMemsetAsync(d->dEy, 0, n * sizeof(T), d->stream));
  return EMCG_OK;
}

} // namespace emcg

using namespace emcg;

extern "C" int32_t emcg_device_create(const emcg_model_desc *model, const emcg_device_desc *dv,
                                      const emcg_device_config *cfg, int32_t precision,
                                      emcg_handle **out) {
  EMCG_CHECK_ARG(out, "out is NULL");
  *out = nullptr;
  EMCG_CHECK_ARG(model && dv && cfg, "NULL descriptor");
  EMCG_CHECK_ARG(precision == EMCG_FP64 || precision == EMCG_FP32, "bad precision");
  EMCG_CHECK_ARG(dv->nx >= 3 && dv->ny >= 3 && (int64_t)dv->nx * dv->ny < (1 << 26),
                 "grid must be at least 3 x 3 nodes");
  EMCG_CHECK_ARG(dv->hx > 0 && dv->hy > 0 && dv->width > 0 && dv->temperature > 0 &&
                     dv->ni > 0 && dv->eps_r > 0,
                 "bad device geometry or material");
  EMCG_CHECK_ARG(dv->doping && dv->region, "doping/region arrays are NULL");
  EMCG_CHECK_ARG(dv->n_contacts >= 0 && dv->n_contacts <= 64, "n_contacts out of [0, 64]");
  EMCG_CHECK_ARG(dv->n_contacts == 0 || (dv->contact_type && dv->contact_voltage &&
                                         dv->contact_param),
                 "contact arrays are NULL");
  for (int b = 0; b < 4; b++)
    EMCG_CHECK_ARG(dv->boundary_contact[b], "boundary_contact[%d] is NULL", b);
  EMCG_CHECK_ARG(cfg->pm_scheme >= EMCG_PM_NGP && cfg->pm_scheme <= EMCG_PM_NEC_VWD,
                 "bad PM scheme %d", cfg->pm_scheme);
  EMCG_CHECK_ARG(cfg->capacity > 0 && cfg->capacity < (int64_t(1) << 31), "bad capacity");
  EMCG_CHECK_ARG(cfg->dt > 0 && cfg->carriers_per_particle > 0, "bad dt / carriers");
  EMCG_CHECK_ARG(cfg->poisson_max_cycles >= 1 && cfg->poisson_rtol > 0, "bad Poisson settings");
  const int nx = dv->nx, ny = dv->ny, n = nx * ny;
  for (int i = 0; i < n; i++)
    EMCG_CHECK_ARG(dv->region[i] >= 0 && dv->region[i] < EMCG_MAX_REGIONS,
                   "node %d: doping region %d out of [0,%d)", i, dv->region[i], EMCG_MAX_REGIONS);
  for (int b = 0; b < 4; b++) {
    int len = b < 2 ? ny : nx;
    for (int c = 0; c < len; c++)
      EMCG_CHECK_ARG(dv->boundary_contact[b][c] >= -1 &&
                         dv->boundary_contact[b][c] < dv->n_contacts,
                     "boundary %d: bad contact index", b);
  }
  for (int c = 0; c < dv->n_contacts; c++) {
    EMCG_CHECK_ARG(dv->contact_type[c] >= 0 && dv->contact_type[c] <= 2, "bad contact type");
    // a Schottky reservoir needs the degenerate 2-D carrier statistics that the
    // reference enables with setDegeneracyBeta (emcSORSolver.hpp:299-308)
    EMCG_CHECK_ARG(dv->contact_type[c] != EMCG_CONTACT_SCHOTTKY,
                   "contact %d: Schottky contacts are not supported", c);
  }
  DeviceImpl *d = new DeviceImpl();
  auto fail = [&](int32_t s) {
    emcg_handle tmp;
    tmp.kind = 2;
    tmp.dev = d;
    destroyDevice(&tmp);
    return s;
  };
  d->precision = precision;
  d->tsz = precision == EMCG_FP64 ? 8 : 4;
  d->cfg = *cfg;
  d->nx = nx;
  d->ny = ny;
  d->hx = dv->hx;
  d->hy = dv->hy;
  d->maxX = dv->max_x > 0 ? dv->max_x : dv->hx * (nx - 1);
  d->maxY = dv->max_y > 0 ? dv->max_y : dv->hy * (ny - 1);
  d->width = dv->width;
  d->T = dv->temperature;
  d->Ni = dv->ni;
  d->epsR = dv->eps_r;
  d->Vt = kKB / kQ * d->T; // include/emcDevice.hpp:87
  {                        // include/emcDevice.hpp:333-343
    double v = 1.;
    v = v * d->hx;
    v = v * d->hy;
    d->cellVol = v * d->width;
  }
  d->nContacts = dv->n_contacts;
  d->doping.assign(dv->doping, dv->doping + n);
  d->region.assign(dv->region, dv->region + n);
  for (int b = 0; b < 4; b++)
    d->bnd[b].assign(dv->boundary_contact[b], dv->boundary_contact[b] + (b < 2 ? ny : nx));
  d->ctype.assign(dv->contact_type, dv->contact_type + d->nContacts);
  d->cvolt.assign(dv->contact_voltage, dv->contact_voltage + d->nContacts);
  d->cpar.assign(dv->contact_param, dv->contact_param + 3 * d->nContacts);
  // node tables (first-boundary rule of emcSurface::getBoundaryPos)
  d->nodeContactH.assign(n, -1);
  d->nodeResH.assign(n, -1);
  d->nodeOhmicH.assign(n, 0);
  d->expNrH.assign(n, 0.);
  for (int y = 0; y < ny; y++)
    for (int x = 0; x < nx; x++) {
      int g = y * nx + x, b = firstBoundary(d, x, y);
      if (b < 0)
        continue;
      int c = contactAt(d, b, x, y);
      d->nodeContactH[g] = c;
      if (c >= 0 && d->ctype[c] == EMCG_CONTACT_OHMIC)
        d->nodeOhmicH[g] = 1;
      if (c >= 0 && (d->ctype[c] == EMCG_CONTACT_OHMIC || d->ctype[c] == EMCG_CONTACT_SCHOTTKY)) {
        d->nodeResH[g] = c;
        d->resNodesH.push_back(g);
        double e = d->cellVol * d->doping[g]; // include/ParticleType/emcElectron.hpp:63-73
        if (x == 0 || x == nx - 1)
          e *= 0.5;
        if (y == 0 || y == ny - 1)
          e *= 0.5;
        if (cfg->round_expected) // examples/mosfet2D/electronVWD.hpp:46-56
          e = std::round(e);
        d->expNrH[g] = e;
        d->injBound += (int64_t)std::ceil(std::max(e, 0.) / cfg->carriers_per_particle) + 1;
      }
    }
  d->capacity = cfg->capacity;
  if (cudaStreamCreateWithFlags(&d->stream, cudaStreamNonBlocking) != cudaSuccess) {
    setError("cudaStreamCreate failed");
    return fail(EMCG_ERR_CUDA);
  }
  for (auto &e : d->ev)
    if (cudaEventCreate(&e) != cudaSuccess)
      return fail(EMCG_ERR_CUDA);
  int32_t s = precision == EMCG_FP64 ? createModel<double>(d, *model)
                                     : createModel<float>(d, *model);
  if (s)
    return fail(s);
  cudaStream_t st = d->stream;
  if ((s = up(&d->dRegion, d->region.data(), n, st)) || (s = up(&d->dNodeContact, d->nodeContactH.data(), n, st)) ||
      (s = up(&d->dNodeRes, d->nodeResH.data(), n, st)) || (s = up(&d->dNodeOhmic, d->nodeOhmicH.data(), n, st)) ||
      (s = up(&d->dExp, d->expNrH.data(), n, st)) ||
      (s = up(&d->dResNodes, d->resNodesH.data(), d->resNodesH.size(), st)))
    return fail(s);
  for (int b = 0; b < 4; b++)
    if ((s = up(&d->dBnd[b], d->bnd[b].data(), d->bnd[b].size(), st)))
      return fail(s);
  const size_t cap = (size_t)d->capacity;
  const int nb = d->nBlocks();
  bool ok = true;
  for (int w = 0; w < 2 && ok; w++) {
    for (int f = 0; f < 9 && ok; f++)
      ok = cudaMalloc(&d->dState[w][f], cap * d->tsz) == cudaSuccess;
    ok = ok && cudaMalloc(&d->dMeta[w], cap * sizeof(uint32_t)) == cudaSuccess;
  }
  ok = ok && cudaMalloc(&d->dPot, n * sizeof(double)) == cudaSuccess &&
       cudaMalloc(&d->dNr, n * sizeof(double)) == cudaSuccess &&
       cudaMalloc(&d->dConc, n * sizeof(double)) == cudaSuccess &&
       cudaMalloc(&d->dN, 4 * sizeof(int64_t)) == cudaSuccess &&
       cudaMalloc(&d->dDrop, cap) == cudaSuccess &&
       cudaMalloc(&d->dBlock, (nb + 1) * sizeof(int32_t)) == cudaSuccess &&
       cudaMalloc(&d->dList, cap * sizeof(int32_t)) == cudaSuccess &&
       cudaMalloc(&d->dListNode, cap * sizeof(int32_t)) == cudaSuccess &&
       cudaMalloc(&d->dListCount, (nb + 1) * sizeof(int32_t)) == cudaSuccess &&
       cudaMalloc(&d->dGList, cap * sizeof(int32_t)) == cudaSuccess &&
       cudaMalloc(&d->dGNode, cap * sizeof(int32_t)) == cudaSuccess &&
       cudaMalloc(&d->dKept, n * sizeof(int32_t)) == cudaSuccess &&
       cudaMalloc(&d->dChunkCount, (d->resNodesH.size() + 1) * kRankChunks * sizeof(int32_t)) ==
           cudaSuccess &&
       cudaMalloc(&d->dInjCount, (d->resNodesH.size() + 1) * sizeof(int32_t)) == cudaSuccess &&
       cudaMalloc(&d->dNetto, (d->nContacts + 1) * sizeof(int32_t)) == cudaSuccess &&
       cudaMalloc(&d->dRemInj, (d->nContacts + 1) * sizeof(int32_t)) == cudaSuccess &&
       cudaMalloc(&d->dNodeFix, 2 * n * sizeof(unsigned long long)) == cudaSuccess &&
       cudaMalloc(&d->dErr, sizeof(int)) == cudaSuccess;
  if (!ok) {
    setError("CUDA allocation of the device engine failed (capacity %lld)", (long long)cap);
    return fail(EMCG_ERR_CUDA);
  }
  cudaMemsetAsync(d->dN, 0, 4 * sizeof(int64_t), st);
  cudaMemsetAsync(d->dErr, 0, sizeof(int), st);
  // fixed-point scale of the deposition: 2^k with capacity x carriers x 2^k
  // at most 2^126, so that no node sum can overflow 128 bits
  d->fixBits = (int)std::floor(
      126. - std::log2(std::max(1., (double)cap * std::max(d->cfg.carriers_per_particle, 1.))));
  d->fixBitsF = d->fixBits - 64;
  cudaMemsetAsync(d->dNr, 0, n * sizeof(double), st);
  cudaMemsetAsync(d->dConc, 0, n * sizeof(double), st);
  // initial potential asinh(C / 2) (include/emcSimulationResults.hpp:208-213)
  {
    std::vector<double> pot(n);
    for (int i = 0; i < n; i++)
      pot[i] = std::asinh(0.5 * (d->doping[i] / d->Ni));
    cudaMemcpyAsync(d->dPot, pot.data(), n * sizeof(double), cudaMemcpyHostToDevice, st);
    cudaStreamSynchronize(st);
  }
  // Poisson setup (include/PoissonSolver/emcSORSolver.hpp:25-36, 330-368)
  PoissonSetup S;
  S.nx = nx;
  S.ny = ny;
  const double L = std::sqrt(kEPS0 * d->epsR * d->Vt / kQ / d->Ni);
  S.h[0] = d->hx / L;
  S.h[1] = d->hy / L;
  S.fixed.assign(n, 0);
  S.C.resize(n);
  S.gSum.assign(n, 0.);
  S.gVeq.assign(n, 0.);
  S.gVne.assign(n, 0.);
  S.gDensX.assign(n, 0.);
  S.gDensY.assign(n, 0.);
  S.resetMask.assign(n, 0);
  S.resetEq.assign(n, 0.);
  S.resetNe.assign(n, 0.);
  const double hF[2] = {S.h[1] / S.h[0], S.h[0] / S.h[1]};
  for (int i = 0; i < n; i++) {
    S.C[i] = d->doping[i] / d->Ni;
    S.fixed[i] = d->nodeResH[i] >= 0;
  }
  for (int y = 0; y < ny; y++)
    for (int x = 0; x < nx; x++) {
      int g = y * nx + x;
      for (int k = 0; k < 2; k++) {
        int co = k == 0 ? x : y, mx = k == 0 ? nx - 1 : ny - 1;
        for (int side = 0; side < 2; side++) {
          if (co != (side == 0 ? 0 : mx))
            continue;
          int b = 2 * k + side;
          int c = contactAt(d, b, x, y);
          if (c < 0 || d->ctype[c] != EMCG_CONTACT_GATE)
            continue;
          double gamma = d->cpar[3 * c + 0] / d->epsR;
          double tox = d->cpar[3 * c + 1] / L;
          double gF = 2 * gamma / tox;
          double G = gF * hF[k] * S.h[k];
          double barrier = d->cpar[3 * c + 2] / d->Vt;
          S.gSum[g] += G;
          S.gVeq[g] += G * barrier;
          S.gVne[g] += G * (barrier + d->cvolt[c] / d->Vt);
          (k == 0 ? S.gDensX : S.gDensY)[g] += 0.5 * gF;
        }
      }
    }
  for (int b = 0; b < 4; b++) { // resetBC: every boundary coordinate of an ohmic contact
    int len = b < 2 ? ny : nx;
    for (int c0 = 0; c0 < len; c0++) {
      int c = d->bnd[b][c0];
      if (c < 0 || d->ctype[c] != EMCG_CONTACT_OHMIC)
        continue;
      int x = b < 2 ? (b == 0 ? 0 : nx - 1) : c0;
      int y = b < 2 ? c0 : (b == 2 ? 0 : ny - 1);
      int g = y * nx + x;
      double bi = std::asinh(0.5 * S.C[g]);
      S.resetMask[g] = 1;
      S.resetEq[g] = bi;
      S.resetNe[g] = d->cvolt[c] / d->Vt + bi;
    }
  }
  if ((s = poissonCreate(d->mg, S, cfg->poisson_fp32 != 0, cfg->poisson_smooth, st)))
    return fail(s);
  d->mg.updTol = cfg->poisson_update_tol > 0 ? cfg->poisson_update_tol / d->Vt : 0.;
  emcg_handle *h = new emcg_handle();
  h->kind = 2;
  h->dev = d;
  *out = h;
  return EMCG_OK;
}

namespace emcg {

template <class T> static int32_t efieldT(DeviceImpl *d) {
  const int n = d->nx * d->ny;
  efieldKernel<T><<<(n + 255) / 256, 256, 0, d->stream>>>(devK(d), d->dPot, (T *)d->dEx,
                                                          (T *)d->dEy, d->cfg.pm_scheme);
  EMCG_CUDA(cudaGetLastError());
  return EMCG_OK;
}

static int32_t compact(DeviceImpl *d) {
  const int nb = d->nBlocks();
  compactCountKernel<<<nb, kCB, 0, d->stream>>>(d->dDrop, d->dN, d->dBlock);
  scanBlocksKernel<<<1, 1024, 0, d->stream>>>(d->dBlock, nb, d->dN + 1);
  if (d->precision == EMCG_FP64)
    compactScatterKernel<double><<<nb, kCB, 0, d->stream>>>(
        devState<double>(d, d->cur), devState<double>(d, 1 - d->cur), d->dDrop, d->dN, d->dBlock);
  else
    compactScatterKernel<float><<<nb, kCB, 0, d->stream>>>(
        devState<float>(d, d->cur), devState<float>(d, 1 - d->cur), d->dDrop, d->dN, d->dBlock);
  EMCG_CUDA(cudaGetLastError());
  EMCG_CUDA(cudaMemcpyAsync(d->dN, d->dN + 1, sizeof(int64_t), cudaMemcpyDeviceToDevice, d->stream));
  d->cur = 1 - d->cur;
  return EMCG_OK;
}

// compactAfter = false: the removed particles stay marked in dDrop for the
// contact handling's single compaction (device step)
template <class T> static int32_t moveT(DeviceImpl *d, uint32_t step, bool compactAfter = true) {
  const int nb = (int)((d->capacity + 255) / 256);
  const emcg_device_config &c = d->cfg;
  uint32_t k0 = (uint32_t)c.seed, k1 = (uint32_t)(c.seed >> 32);
  StateK<T> st = devState<T>(d, d->cur);
  const ModelK<T> *M = (const ModelK<T> *)d->dModel;
  const T *Ex = (const T *)d->dEx, *Ey = (const T *)d->dEy;
  DevK G = devK(d);
  bool rep = d->replay[0];
  if (rep && sizeof(T) != 8) {
    setError("replay needs the FP64 engine");
    return EMCG_ERR_ARG;
  }
#define EMCG_MOVE(SCH, REP)                                                                      \
  (d->surfaces ? devMoveKernel<T, SCH, REP, true> : devMoveKernel<T, SCH, REP, false>)           \
      <<<nb, 256, 0, d->stream>>>(st, M, G, Ex, Ey, (T)c.charge, (T)c.dt, d->dN, step, k0, k1,    \
                                  c.stream, d->dDrop, d->dNetto, d->dWords[0], d->dOff[0],        \
                                  d->dErr)
  if (rep) {
    if constexpr (sizeof(T) == 8) {
      if (c.pm_scheme == EMCG_PM_NGP)
        EMCG_MOVE(EMCG_PM_NGP, true);
      else if (c.pm_scheme == EMCG_PM_CIC)
        EMCG_MOVE(EMCG_PM_CIC, true);
      else if (c.pm_scheme == EMCG_PM_NEC)
        EMCG_MOVE(EMCG_PM_NEC, true);
      else
        EMCG_MOVE(EMCG_PM_NEC_VWD, true);
    }
  } else if (c.pm_scheme == EMCG_PM_NGP) {
    EMCG_MOVE(EMCG_PM_NGP, false);
  } else if (c.pm_scheme == EMCG_PM_CIC) {
    EMCG_MOVE(EMCG_PM_CIC, false);
  } else if (c.pm_scheme == EMCG_PM_NEC) {
    EMCG_MOVE(EMCG_PM_NEC, false);
  } else {
    EMCG_MOVE(EMCG_PM_NEC_VWD, false);
  }
#undef EMCG_MOVE
  EMCG_CUDA(cudaGetLastError());
  d->replay[0] = false;
  return compactAfter ? compact(d) : EMCG_OK;
}

// movedDrops: the move's removals are still marked in dDrop (moveT without its
// compaction); the reservoir list skips them and one compaction removes both.
// The ranks are those of the compacted order, since compaction is stable.
template <class T> static int32_t contactsT(DeviceImpl *d, uint32_t step, bool movedDrops = false) {
  const int nb = d->nBlocks();
  const int n = d->nx * d->ny;
  cudaStream_t st = d->stream;
  DevK G = devK(d);
  const int nRes = (int)d->resNodesH.size();
  if (!movedDrops)
    EMCG_CUDA(cudaMemsetAsync(d->dDrop, 0, d->capacity, st));
  EMCG_CUDA(cudaMemsetAsync(d->dKept, 0, n * sizeof(int32_t), st));
  reservoirListKernel<T><<<nb, kCB, 0, st>>>(devState<T>(d, d->cur), G, d->dN,
                                             movedDrops ? d->dDrop : nullptr, d->dList,
                                             d->dListNode, d->dListCount);
  scanBlocksKernel<<<1, 1024, 0, st>>>(d->dListCount, nb, d->dN + 3);
  gatherListKernel<<<nb, 256, 0, st>>>(d->dList, d->dListNode, d->dListCount, nb, d->dN + 3,
                                       d->dGList, d->dGNode);
  if (nRes > 0) {
    const unsigned rb = (unsigned)(((int64_t)nRes * kRankChunks * 32 + 255) / 256);
    contactCountKernel<<<rb, 256, 0, st>>>(d->dGNode, d->dN + 3, d->dResNodes, nRes,
                                           d->dChunkCount);
    contactRankKernel<<<rb, 256, 0, st>>>(d->dGList, d->dGNode, d->dN + 3, d->dResNodes, nRes,
                                          d->dExp, d->cfg.carriers_per_particle,
                                          d->dNodeContact, d->dChunkCount, d->dDrop, d->dKept,
                                          d->dRemInj);
  }
  EMCG_CUDA(cudaGetLastError());
  EMCG_TRY(compact(d));
  if (nRes == 0)
    return EMCG_OK;
  injectCountKernel<<<(nRes + 255) / 256, 256, 0, st>>>(d->dResNodes, nRes, d->dExp, d->dKept,
                                                        d->cfg.carriers_per_particle, d->dInjCount);
  scanBlocksKernel<<<1, 1024, 0, st>>>(d->dInjCount, nRes, d->dN + 2);
  const emcg_device_config &c = d->cfg;
  uint32_t k0 = (uint32_t)c.seed, k1 = (uint32_t)(c.seed >> 32);
  const int ib = (int)((d->injBound + 255) / 256);
  bool rep = d->replay[1];
  if (rep) {
    if constexpr (sizeof(T) == 8)
      injectKernel<T, true><<<ib, 256, 0, st>>>(
          devState<T>(d, d->cur), (const ModelK<T> *)d->dModel, G, d->dResNodes, nRes,
          d->dInjCount, d->dN + 2, d->dN, d->capacity, step, k0, k1, c.stream,
          c.tau_region_is_valley != 0, d->dRemInj, d->dWords[1], d->dOff[1], d->dErr);
  } else {
    injectKernel<T, false><<<ib, 256, 0, st>>>(
        devState<T>(d, d->cur), (const ModelK<T> *)d->dModel, G, d->dResNodes, nRes,
        d->dInjCount, d->dN + 2, d->dN, d->capacity, step, k0, k1, c.stream,
        c.tau_region_is_valley != 0, d->dRemInj, nullptr, nullptr, d->dErr);
  }
  addCountKernel<<<1, 1, 0, st>>>(d->dN, d->dN + 2, d->capacity);
  EMCG_CUDA(cudaGetLastError());
  d->replay[1] = false;
  return EMCG_OK;
}

template <class T> static int32_t assignT(DeviceImpl *d) {
  const int n = d->nx * d->ny;
  const int nb = (int)((d->capacity + 255) / 256);
  const int fb = sizeof(T) == 4 ? d->fixBitsF : d->fixBits;
  const double nrC = d->cfg.carriers_per_particle;
  const StateK<T> st = devState<T>(d, d->cur);
  EMCG_CUDA(cudaMemsetAsync(d->dNodeFix, 0, 2 * n * sizeof(unsigned long long), d->stream));
  if (d->cfg.pm_scheme == EMCG_PM_NGP)
    assignKernel<T, EMCG_PM_NGP><<<nb, 256, 0, d->stream>>>(st, devK(d), d->dN, nrC, fb,
                                                           d->dNodeFix);
  else if (d->cfg.pm_scheme == EMCG_PM_CIC)
    assignKernel<T, EMCG_PM_CIC><<<nb, 256, 0, d->stream>>>(st, devK(d), d->dN, nrC, fb,
                                                           d->dNodeFix);
  else
    assignKernel<T, EMCG_PM_NEC><<<nb, 256, 0, d->stream>>>(st, devK(d), d->dN, nrC, fb,
                                                           d->dNodeFix);
  concKernel<<<(n + 255) / 256, 256, 0, d->stream>>>(devK(d), d->dNodeFix, fb, d->dNr, d->dConc);
  EMCG_CUDA(cudaGetLastError());
  return EMCG_OK;
}

static int32_t poissonRun(DeviceImpl *d, bool eq, bool reset, double *rel, int *cycles) {
  EMCG_CUDA(cudaEventRecord(d->ev[2], d->stream));
  int32_t s = poissonSolve(d->mg, d->dPot, eq ? nullptr : d->dConc, reset, d->cfg.poisson_rtol,
                           d->cfg.poisson_max_cycles, d->stream, rel, cycles);
  EMCG_CUDA(cudaEventRecord(d->ev[3], d->stream));
  EMCG_CUDA(cudaEventSynchronize(d->ev[3]));
  float ms = 0;
  cudaEventElapsedTime(&ms, d->ev[2], d->ev[3]);
  d->poissonMs = ms;
  return s;
}

} // namespace emcg

extern "C" int32_t emcg_device_set_grid(emcg_handle *h, int32_t which, const double *v) {
  DeviceImpl *d;
  EMCG_TRY(devOf(h, &d));
  EMCG_CHECK_ARG(v, "values are NULL");
  const int n = d->nx * d->ny;
  double *dst = which == EMCG_GRID_POTENTIAL ? d->dPot
                : which == EMCG_GRID_NRPART  ? d->dNr
                : which == EMCG_GRID_CONC    ? d->dConc
                                             : nullptr;
  if (which == EMCG_GRID_EX || which == EMCG_GRID_EY) {
    void *e = which == EMCG_GRID_EX ? d->dEx : d->dEy;
    if (d->precision == EMCG_FP64) {
      EMCG_CUDA(cudaMemcpy(e, v, n * sizeof(double), cudaMemcpyHostToDevice));
    } else {
      std::vector<float> f(v, v + n);
      EMCG_CUDA(cudaMemcpy(e, f.data(), n * sizeof(float), cudaMemcpyHostToDevice));
    }
    return EMCG_OK;
  }
  EMCG_CHECK_ARG(dst, "unknown grid %d", which);
  EMCG_CUDA(cudaMemcpy(dst, v, n * sizeof(double), cudaMemcpyHostToDevice));
  return EMCG_OK;
}

extern "C" int32_t emcg_device_get_grid(emcg_handle *h, int32_t which, double *v) {
  DeviceImpl *d;
  EMCG_TRY(devOf(h, &d));
  EMCG_CHECK_ARG(v, "values are NULL");
  EMCG_CUDA(cudaStreamSynchronize(d->stream));
  const int n = d->nx * d->ny;
  if (which == EMCG_GRID_EX || which == EMCG_GRID_EY) {
    void *e = which == EMCG_GRID_EX ? d->dEx : d->dEy;
    if (d->precision == EMCG_FP64) {
      EMCG_CUDA(cudaMemcpy(v, e, n * sizeof(double), cudaMemcpyDeviceToHost));
    } else {
      std::vector<float> f(n);
      EMCG_CUDA(cudaMemcpy(f.data(), e, n * sizeof(float), cudaMemcpyDeviceToHost));
      for (int i = 0; i < n; i++)
        v[i] = f[i];
    }
    return EMCG_OK;
  }
  double *src = which == EMCG_GRID_POTENTIAL ? d->dPot
                : which == EMCG_GRID_NRPART  ? d->dNr
                : which == EMCG_GRID_CONC    ? d->dConc
                                             : nullptr;
  EMCG_CHECK_ARG(src, "unknown grid %d", which);
  EMCG_CUDA(cudaMemcpy(v, src, n * sizeof(double), cudaMemcpyDeviceToHost));
  return EMCG_OK;
}

extern "C" int32_t emcg_device_poisson(emcg_handle *h, int32_t equilibrium, int32_t reset_bc,
                                       double *rel, int32_t *cycles) {
  DeviceImpl *d;
  EMCG_TRY(devOf(h, &d));
  int cyc = 0;
  int32_t s = poissonRun(d, equilibrium != 0, reset_bc != 0, rel, &cyc);
  if (cycles)
    *cycles = cyc;
  if (!equilibrium && reset_bc)
    d->bcReset = false;
  return s;
}

namespace emcg {
// scatterParticleAtBoundary (include/emcScatterHandler.hpp:172-191) at boundary
// b for n independent particles: the model's surface mechanism there, else the
// plain reflection (known-answer tests of the reference)
template <class T>
__global__ void surfaceKatKernel(const ModelK<T> *__restrict__ models, DevK G, int b, int64_t n,
                                 double *__restrict__ k, double *__restrict__ pos, uint32_t step,
                                 uint32_t key0, uint32_t key1, uint32_t stream) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  const ModelK<T> &M = models[0];
  T kk[3] = {(T)k[i], (T)k[n + i], (T)k[2 * n + i]}, p[2] = {(T)pos[i], (T)pos[n + i]};
  PhiloxSrc<T> rng;
  rng.init((uint32_t)i, step, stream, key0, key1);
  if (M.surfKind[b] != EMCG_SURFACE_SPECULAR) {
    surfaceScatter(M, G, b, p, kk, rng);
  } else {
    const T mx[2] = {(T)G.maxX, (T)G.maxY};
#pragma unroll
    for (int j = 0; j < 2; j++) {
      if (p[j] < T(0)) {
        p[j] = -p[j];
        kk[j] = -kk[j];
      } else if (p[j] > mx[j]) {
        p[j] = T(2) * mx[j] - p[j];
        kk[j] = -kk[j];
      }
    }
  }
  for (int j = 0; j < 3; j++)
    k[j * n + i] = (double)kk[j];
  pos[i] = (double)p[0];
  pos[n + i] = (double)p[1];
}
} // namespace emcg

extern "C" int32_t emcg_device_surface_kat(emcg_handle *h, int32_t boundary, int64_t n,
                                           double *k, double *pos, uint32_t step) {
  DeviceImpl *d;
  EMCG_TRY(devOf(h, &d));
  EMCG_CHECK_ARG(boundary >= 0 && boundary < 4 && n >= 0 && k && pos, "bad surface arguments");
  if (n == 0)
    return EMCG_OK;
  double *buf = nullptr;
  EMCG_CUDA(cudaMalloc(&buf, 5 * n * sizeof(double)));
  EMCG_CUDA(cudaMemcpy(buf, k, 3 * n * sizeof(double), cudaMemcpyHostToDevice));
  EMCG_CUDA(cudaMemcpy(buf + 3 * n, pos, 2 * n * sizeof(double), cudaMemcpyHostToDevice));
  const uint32_t k0 = (uint32_t)d->cfg.seed, k1 = (uint32_t)(d->cfg.seed >> 32);
  const int blocks = (int)((n + 127) / 128);
  if (d->precision == EMCG_FP64)
    surfaceKatKernel<double><<<blocks, 128, 0, d->stream>>>(
        (const ModelK<double> *)d->dModel, devK(d), boundary, n, buf, buf + 3 * n, step, k0, k1,
        d->cfg.stream);
  else
    surfaceKatKernel<float><<<blocks, 128, 0, d->stream>>>(
        (const ModelK<float> *)d->dModel, devK(d), boundary, n, buf, buf + 3 * n, step, k0, k1,
        d->cfg.stream);
  int32_t st = EMCG_OK;
  if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(d->stream) != cudaSuccess ||
      cudaMemcpy(k, buf, 3 * n * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemcpy(pos, buf + 3 * n, 2 * n * sizeof(double), cudaMemcpyDeviceToHost) !=
          cudaSuccess) {
    setError("surface known-answer kernel failed");
    st = EMCG_ERR_CUDA;
  }
  cudaFree(buf);
  return st;
}

extern "C" int32_t emcg_device_efield(emcg_handle *h) {
  DeviceImpl *d;
  EMCG_TRY(devOf(h, &d));
  EMCG_TRY(d->precision == EMCG_FP64 ? efieldT<double>(d) : efieldT<float>(d));
  EMCG_CUDA(cudaStreamSynchronize(d->stream));
  return EMCG_OK;
}

extern "C" int32_t emcg_device_move(emcg_handle *h, uint32_t step, int32_t *netto) {
  DeviceImpl *d;
  EMCG_TRY(devOf(h, &d));
  EMCG_CUDA(cudaMemsetAsync(d->dNetto, 0, (d->nContacts + 1) * sizeof(int32_t), d->stream));
  EMCG_TRY(d->precision == EMCG_FP64 ? moveT<double>(d, step) : moveT<float>(d, step));
  if (netto)
    EMCG_CUDA(cudaMemcpyAsync(netto, d->dNetto, d->nContacts * sizeof(int32_t),
                              cudaMemcpyDeviceToHost, d->stream));
  EMCG_CUDA(cudaStreamSynchronize(d->stream));
  return readErr(d);
}

extern "C" int32_t emcg_device_contacts(emcg_handle *h, uint32_t step, int32_t *rem_inj) {
  DeviceImpl *d;
  EMCG_TRY(devOf(h, &d));
  EMCG_CUDA(cudaMemsetAsync(d->dRemInj, 0, (d->nContacts + 1) * sizeof(int32_t), d->stream));
  EMCG_TRY(d->precision == EMCG_FP64 ? contactsT<double>(d, step) : contactsT<float>(d, step));
  if (rem_inj)
    EMCG_CUDA(cudaMemcpyAsync(rem_inj, d->dRemInj, d->nContacts * sizeof(int32_t),
                              cudaMemcpyDeviceToHost, d->stream));
  EMCG_CUDA(cudaStreamSynchronize(d->stream));
  return readErr(d);
}

extern "C" int32_t emcg_device_assign(emcg_handle *h) {
  DeviceImpl *d;
  EMCG_TRY(devOf(h, &d));
  EMCG_TRY(d->precision == EMCG_FP64 ? assignT<double>(d) : assignT<float>(d));
  EMCG_CUDA(cudaStreamSynchronize(d->stream));
  return EMCG_OK;
}

extern "C" int32_t emcg_device_step(emcg_handle *h, int32_t n_steps, uint32_t step0,
                                    int32_t *netto) {
  DeviceImpl *d;
  EMCG_TRY(devOf(h, &d));
  EMCG_CHECK_ARG(n_steps >= 0, "n_steps must be >= 0");
  const int nc = d->nContacts;
  std::vector<int32_t> hn(2 * (nc + 1));
  double stepMs = 0, poisMs = 0;
  d->poissonCycles = d->poissonSolves = 0;
  for (int s = 0; s < n_steps; s++) {
    EMCG_CUDA(cudaEventRecord(d->ev[0], d->stream));
    // the cluster solve is only enqueued: the step's particle kernels follow
    // it on the stream at once, and its outcome is read at the end of the step
    double rel = 0.;
    int cyc = 0;
    bool queued = false;
    EMCG_CUDA(cudaEventRecord(d->ev[2], d->stream));
    int32_t ps = poissonEnqueue(d->mg, d->dPot, d->dConc, d->bcReset, d->cfg.poisson_rtol,
                                d->cfg.poisson_max_cycles, d->stream, &queued, &rel, &cyc);
    EMCG_CUDA(cudaEventRecord(d->ev[3], d->stream));
    d->bcReset = false;
    if (ps)
      return ps;
    EMCG_TRY(d->precision == EMCG_FP64 ? efieldT<double>(d) : efieldT<float>(d));
    EMCG_CUDA(cudaMemsetAsync(d->dNetto, 0, (nc + 1) * sizeof(int32_t), d->stream));
    EMCG_CUDA(cudaMemsetAsync(d->dRemInj, 0, (nc + 1) * sizeof(int32_t), d->stream));
    // one compaction per step, after the contacts (the move's removals wait marked)
    EMCG_TRY(d->precision == EMCG_FP64 ? moveT<double>(d, step0 + s, false)
                                       : moveT<float>(d, step0 + s, false));
    EMCG_TRY(d->precision == EMCG_FP64 ? contactsT<double>(d, step0 + s, true)
                                       : contactsT<float>(d, step0 + s, true));
    EMCG_TRY(d->precision == EMCG_FP64 ? assignT<double>(d) : assignT<float>(d));
    EMCG_CUDA(cudaEventRecord(d->ev[1], d->stream));
    if (netto) {
      EMCG_CUDA(cudaMemcpyAsync(hn.data(), d->dNetto, nc * sizeof(int32_t), cudaMemcpyDeviceToHost,
                                d->stream));
      EMCG_CUDA(cudaMemcpyAsync(hn.data() + nc + 1, d->dRemInj, nc * sizeof(int32_t),
                                cudaMemcpyDeviceToHost, d->stream));
    }
    EMCG_CUDA(cudaEventSynchronize(d->ev[1]));
    float ms = 0;
    cudaEventElapsedTime(&ms, d->ev[0], d->ev[1]);
    stepMs += ms;
    cudaEventElapsedTime(&ms, d->ev[2], d->ev[3]);
    d->poissonMs = ms;
    poisMs += ms;
    if (queued)
      ps = poissonFinish(d->mg, d->cfg.poisson_rtol, &rel, &cyc);
    d->poissonCycles += cyc;
    d->poissonSolves++;
    if (ps)
      return ps;
    EMCG_TRY(readErr(d));
    if (netto)
      for (int c = 0; c < nc; c++)
        netto[(int64_t)s * nc + c] = hn[c] - hn[nc + 1 + c];
  }
  d->stepMs = stepMs;
  d->poissonMs = poisMs;
  return EMCG_OK;
}

extern "C" int32_t emcg_device_step_many(emcg_handle **hs, int32_t n, int32_t n_steps,
                                         uint32_t step0, int32_t **netto) {
  EMCG_CHECK_ARG(hs && n >= 0 && n_steps >= 0, "bad batch arguments");
  for (int i = 0; i < n; i++) {
    DeviceImpl *d;
    EMCG_TRY(devOf(hs[i], &d));
    for (int j = 0; j < i; j++)
      EMCG_CHECK_ARG(hs[j] != hs[i], "handle %d appears twice in the batch", i);
  }
  int dev = 0;
  EMCG_CUDA(cudaGetDevice(&dev));
  // Each engine's Poisson solve is one thread-block cluster of one CTA per SM.
  // A batch plans the clusters so that all n fit on the device at once (16
  // CTAs: 7 resident clusters on GB300; 12: 8), and restores each engine's
  // own plan afterwards.  The cluster size does not change the result.  The
  // plan for a batch size is kept until the batch size or the engine's bound
  // changes (planning queries the runtime for every candidate size).
  struct Plan {
    int size;
    size_t smem;
    bool even;
  };
  std::vector<Plan> ownPlan(n);
  for (int i = 0; i < n; i++) {
    PoissonMG &P = hs[i]->dev->mg;
    ownPlan[i] = {P.clusterSize, P.clusterSmem, P.clusterEven};
  }
  int32_t planStatus = EMCG_OK;
  for (int i = 0; i < n && planStatus == EMCG_OK && n > 1; i++) {
    PoissonMG &P = hs[i]->dev->mg;
    if (!P.useCluster || P.clusterSize == 0)
      continue;
    if (P.batchFor != n || P.batchCap != P.clusterCap) {
      planStatus = poissonPlanCluster(P, n);
      P.batchFor = n;
      P.batchCap = P.clusterCap;
      P.batchSize = P.clusterSize;
      P.batchSmem = P.clusterSmem;
      P.batchEven = P.clusterEven;
    }
    P.clusterSize = P.batchSize;
    P.clusterSmem = P.batchSmem;
    P.clusterEven = P.batchEven;
  }
  auto restore = [&]() {
    for (int i = 0; i < n; i++) {
      PoissonMG &P = hs[i]->dev->mg;
      P.clusterSize = ownPlan[i].size;
      P.clusterSmem = ownPlan[i].smem;
      P.clusterEven = ownPlan[i].even;
    }
  };
  if (planStatus != EMCG_OK) {
    restore();
    for (int i = 0; i < n; i++)
      hs[i]->dev->mg.batchFor = 0;
    return planStatus;
  }
  // one host thread per engine: each drives its own stream, so the engines'
  // kernels (one Poisson cluster each, the particle kernels) run side by side
  std::vector<int32_t> status(n, EMCG_OK);
  std::vector<std::string> message(n);
  std::vector<std::thread> workers;
  workers.reserve(n);
  for (int i = 0; i < n; i++)
    workers.emplace_back([&, i]() {
      if (cudaSetDevice(dev) != cudaSuccess) {
        status[i] = EMCG_ERR_CUDA;
        message[i] = "cudaSetDevice failed in a batch worker";
        return;
      }
      status[i] = emcg_device_step(hs[i], n_steps, step0, netto ? netto[i] : nullptr);
      if (status[i] != EMCG_OK)
        message[i] = emcg_last_error();
    });
  for (auto &w : workers)
    w.join();
  restore();
  for (int i = 0; i < n; i++)
    if (status[i] != EMCG_OK) {
      setError("engine %d of the batch: %s", i, message[i].c_str());
      return status[i];
    }
  return EMCG_OK;
}

extern "C" int32_t emcg_device_poisson_mode(emcg_handle *h, int32_t mode, int32_t *cluster_size) {
  DeviceImpl *d;
  EMCG_TRY(devOf(h, &d));
  EMCG_CHECK_ARG(mode >= -1 && mode <= 1, "mode must be -1 (query), 0 or 1");
  if (mode >= 0)
    d->mg.useCluster = mode == 1;
  if (cluster_size)
    *cluster_size = d->mg.useCluster ? d->mg.clusterSize : 0;
  return EMCG_OK;
}

extern "C" int32_t emcg_device_set_poisson_cluster(emcg_handle *h, int32_t max_ctas,
                                                   int32_t *cluster_size) {
  DeviceImpl *d;
  EMCG_TRY(devOf(h, &d));
  EMCG_CHECK_ARG(max_ctas >= 0 && max_ctas <= 16, "max_ctas must be 0 (no bound) to 16");
  d->mg.clusterCap = max_ctas;
  d->mg.batchFor = 0; // a batch plans again under the new bound
  EMCG_TRY(poissonPlanCluster(d->mg, 1));
  if (cluster_size)
    *cluster_size = d->mg.useCluster ? d->mg.clusterSize : 0;
  return EMCG_OK;
}

extern "C" int32_t emcg_device_set_poisson(emcg_handle *h, double rtol, int32_t max_cycles,
                                           double update_tol) {
  DeviceImpl *d;
  EMCG_TRY(devOf(h, &d));
  if (rtol >= 0) {
    EMCG_CHECK_ARG(rtol > 0, "rtol must be positive");
    d->cfg.poisson_rtol = rtol;
  }
  if (max_cycles >= 0)
    d->cfg.poisson_max_cycles = max_cycles;
  if (update_tol >= 0) {
    d->cfg.poisson_update_tol = update_tol;
    d->mg.updTol = update_tol > 0 ? update_tol / d->Vt : 0.;
  }
  return EMCG_OK;
}

extern "C" int32_t emcg_device_poisson_counts(emcg_handle *h, int64_t *cycles, int64_t *solves) {
  DeviceImpl *d;
  EMCG_TRY(devOf(h, &d));
  if (cycles)
    *cycles = d->poissonCycles;
  if (solves)
    *solves = d->poissonSolves;
  return EMCG_OK;
}

extern "C" int32_t emcg_device_timing(emcg_handle *h, double *step_ms, double *poisson_ms) {
  DeviceImpl *d;
  EMCG_TRY(devOf(h, &d));
  if (step_ms)
    *step_ms = d->stepMs;
  if (poisson_ms)
    *poisson_ms = d->poissonMs;
  return EMCG_OK;
}

// host Philox / canonical map for the initial counts (same stream as the oracle)
static void philoxHost(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1,
                       uint32_t o[4]) {
  for (int r = 0; r < 10; r++) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0, n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
    c0 = n0;
    c1 = (uint32_t)p1;
    c2 = n2;
    c3 = (uint32_t)p0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  o[0] = c0;
  o[1] = c1;
  o[2] = c2;
  o[3] = c3;
}

extern "C" int32_t emcg_device_init(emcg_handle *h, int32_t potential_based, int32_t round_counts) {
  DeviceImpl *d;
  EMCG_TRY(devOf(h, &d));
  const int nx = d->nx, ny = d->ny, n = nx * ny;
  std::vector<double> pot(n);
  if (potential_based)
    EMCG_CUDA(cudaMemcpy(pot.data(), d->dPot, n * sizeof(double), cudaMemcpyDeviceToHost));
  const emcg_device_config &c = d->cfg;
  uint32_t k0 = (uint32_t)c.seed, k1 = (uint32_t)(c.seed >> 32);
  std::vector<int32_t> nodeOf;
  for (int y = 0; y < ny; y++)
    for (int x = 0; x < nx; x++) {
      int g = y * nx + x;
      double e = potential_based ? std::exp(pot[g]) * d->Ni : d->doping[g];
      if (x == 0 || x == nx - 1)
        e *= 0.5;
      if (y == 0 || y == ny - 1)
        e *= 0.5;
      double nr = round_counts ? std::round(e * d->cellVol) : e * d->cellVol;
      while (nr >= 1) {
        nodeOf.push_back(g);
        nr -= c.carriers_per_particle;
      }
      uint32_t o[4];
      philoxHost((uint32_t)nodeOf.size(), 0xFFFFFFFEu, 0, c.stream, k0, k1, o);
      uint64_t w = (uint64_t)o[0] | ((uint64_t)o[1] << 32);
      double u = (double)w / 18446744073709551616.0;
      if (u >= 1.0)
        u = std::nextafter(1.0, 0.0);
      if (u < nr)
        nodeOf.push_back(g);
    }
  const int64_t np = (int64_t)nodeOf.size();
  EMCG_CHECK_ARG(np <= d->capacity, "%lld initial particles exceed capacity %lld", (long long)np,
                 (long long)d->capacity);
  int32_t *dNode = nullptr;
  EMCG_CUDA(cudaMalloc(&dNode, sizeof(int32_t) * std::max<int64_t>(np, 1)));
  EMCG_CUDA(cudaMemcpy(dNode, nodeOf.data(), sizeof(int32_t) * np, cudaMemcpyHostToDevice));
  const int nb = (int)((np + 255) / 256);
  if (np) {
    if (d->precision == EMCG_FP64)
      devInitKernel<double><<<nb, 256, 0, d->stream>>>(devState<double>(d, d->cur),
                                                       (const ModelK<double> *)d->dModel, devK(d),
                                                       dNode, np, k0, k1, c.stream,
                                                       c.tau_region_is_valley != 0);
    else
      devInitKernel<float><<<nb, 256, 0, d->stream>>>(devState<float>(d, d->cur),
                                                      (const ModelK<float> *)d->dModel, devK(d),
                                                      dNode, np, k0, k1, c.stream,
                                                      c.tau_region_is_valley != 0);
    EMCG_CUDA(cudaGetLastError());
  }
  EMCG_CUDA(cudaMemcpyAsync(d->dN, &np, sizeof(int64_t), cudaMemcpyHostToDevice, d->stream));
  EMCG_CUDA(cudaStreamSynchronize(d->stream));
  cudaFree(dNode);
  return EMCG_OK;
}

extern "C" int32_t emcg_device_set_replay(emcg_handle *h, int32_t phase, const uint64_t *words,
                                          int64_t nwords, const int64_t *offsets,
                                          int64_t n_offsets) {
  DeviceImpl *d;
  EMCG_TRY(devOf(h, &d));
  EMCG_CHECK_ARG(phase == 0 || phase == 1, "phase must be 0 (move) or 1 (inject)");
  if (!words) {
    d->replay[phase] = false;
    return EMCG_OK;
  }
  EMCG_CHECK_ARG(d->precision == EMCG_FP64, "replay needs the FP64 engine");
  EMCG_CHECK_ARG(offsets && n_offsets >= 1 && nwords >= 0, "bad replay arguments");
  for (int64_t i = 0; i + 1 < n_offsets; i++)
    EMCG_CHECK_ARG(offsets[i] >= 0 && offsets[i] <= offsets[i + 1] && offsets[i + 1] <= nwords,
                   "replay offsets not monotone within [0, nwords]");
  if (phase == 0) {
    int64_t n = 0;
    EMCG_CUDA(cudaMemcpy(&n, d->dN, sizeof(int64_t), cudaMemcpyDeviceToHost));
    EMCG_CHECK_ARG(n_offsets == n + 1, "move replay needs n+1 = %lld offsets", (long long)(n + 1));
  }
  if (nwords > d->wordsCap[phase]) {
    cudaFree(d->dWords[phase]);
    d->dWords[phase] = nullptr;
    EMCG_CUDA(cudaMalloc(&d->dWords[phase], sizeof(uint64_t) * std::max<int64_t>(nwords, 1)));
    d->wordsCap[phase] = nwords;
  }
  if (n_offsets > d->offCap[phase]) {
    cudaFree(d->dOff[phase]);
    d->dOff[phase] = nullptr;
    EMCG_CUDA(cudaMalloc(&d->dOff[phase], sizeof(int64_t) * n_offsets));
    d->offCap[phase] = n_offsets;
  }
  if (nwords)
    EMCG_CUDA(cudaMemcpy(d->dWords[phase], words, sizeof(uint64_t) * nwords, cudaMemcpyHostToDevice));
  EMCG_CUDA(cudaMemcpy(d->dOff[phase], offsets, sizeof(int64_t) * n_offsets, cudaMemcpyHostToDevice));
  d->replay[phase] = true;
  return EMCG_OK;
}

// ---- particle state of a device engine (used by emcg_set_state & co.) -------
namespace emcg {

template <class T> static int32_t devSetStateT(DeviceImpl *d, const emcg_state *s) {
  const int64_t n = s->n;
  const double *src[9] = {s->kx, s->ky, s->kz, s->px, s->py, s->pz, s->energy, s->tau, s->grain_tau};
  std::vector<T> tmp((size_t)std::max<int64_t>(n, 1));
  for (int f = 0; f < 9; f++) {
    for (int64_t i = 0; i < n; i++)
      tmp[i] = src[f] ? (T)src[f][i] : T(0);
    if (n)
      EMCG_CUDA(cudaMemcpy(d->dState[d->cur][f], tmp.data(), n * sizeof(T), cudaMemcpyHostToDevice));
  }
  std::vector<uint32_t> meta((size_t)std::max<int64_t>(n, 1));
  for (int64_t i = 0; i < n; i++) {
    EMCG_CHECK_ARG(s->valley[i] >= 0 && s->valley[i] < EMCG_MAX_VALLEYS && s->sub[i] >= 0 &&
                       s->sub[i] < EMCG_MAX_DEG && s->region[i] >= 0 &&
                       s->region[i] < EMCG_MAX_REGIONS,
                   "particle %lld: valley/sub/region out of range", (long long)i);
    meta[i] = packMeta(s->valley[i], s->sub[i], s->region[i]);
  }
  if (n)
    EMCG_CUDA(cudaMemcpy(d->dMeta[d->cur], meta.data(), n * sizeof(uint32_t), cudaMemcpyHostToDevice));
  EMCG_CUDA(cudaMemcpy(d->dN, &n, sizeof(int64_t), cudaMemcpyHostToDevice));
  return EMCG_OK;
}

int32_t deviceSetState(emcg_handle *h, const emcg_state *s) {
  DeviceImpl *d;
  EMCG_TRY(devOf(h, &d));
  EMCG_CHECK_ARG(s && s->n >= 0 && s->n <= d->capacity, "state size exceeds capacity");
  EMCG_CHECK_ARG(s->valley && s->sub && s->region, "state index arrays are NULL");
  EMCG_CUDA(cudaStreamSynchronize(d->stream));
  return d->precision == EMCG_FP64 ? devSetStateT<double>(d, s) : devSetStateT<float>(d, s);
}

int64_t deviceNumParticles(emcg_handle *h) {
  DeviceImpl *d;
  if (devOf(h, &d))
    return -1;
  int64_t n = 0;
  if (cudaStreamSynchronize(d->stream) != cudaSuccess ||
      cudaMemcpy(&n, d->dN, sizeof(int64_t), cudaMemcpyDeviceToHost) != cudaSuccess)
    return -1;
  return n;
}

template <class T> static int32_t devGetStateT(DeviceImpl *d, emcg_state *s, int64_t n) {
  double *dst[9] = {s->kx, s->ky, s->kz, s->px, s->py, s->pz, s->energy, s->tau, s->grain_tau};
  std::vector<T> tmp((size_t)std::max<int64_t>(n, 1));
  for (int f = 0; f < 9; f++) {
    if (!dst[f])
      continue;
    if (n)
      EMCG_CUDA(cudaMemcpy(tmp.data(), d->dState[d->cur][f], n * sizeof(T), cudaMemcpyDeviceToHost));
    for (int64_t i = 0; i < n; i++)
      dst[f][i] = (double)tmp[i];
  }
  std::vector<uint32_t> meta((size_t)std::max<int64_t>(n, 1));
  if (n)
    EMCG_CUDA(cudaMemcpy(meta.data(), d->dMeta[d->cur], n * sizeof(uint32_t), cudaMemcpyDeviceToHost));
  for (int64_t i = 0; i < n; i++) {
    if (s->valley)
      s->valley[i] = meta[i] & 0xff;
    if (s->sub)
      s->sub[i] = (meta[i] >> 8) & 0xff;
    if (s->region)
      s->region[i] = meta[i] >> 16;
  }
  s->n = n;
  return EMCG_OK;
}

int32_t deviceGetState(emcg_handle *h, emcg_state *s) {
  DeviceImpl *d;
  EMCG_TRY(devOf(h, &d));
  EMCG_CHECK_ARG(s, "state is NULL");
  int64_t n = deviceNumParticles(h);
  EMCG_CHECK_ARG(n >= 0, "cannot read the particle count");
  return d->precision == EMCG_FP64 ? devGetStateT<double>(d, s, n) : devGetStateT<float>(d, s, n);
}

} // namespace emcg
