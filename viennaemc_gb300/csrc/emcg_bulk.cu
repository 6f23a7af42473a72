// Bulk engine: ensembles of electrons in a periodic box under a constant
// field (examples/bulkSimulation/basicBulkParticleHandler.hpp).  Many
// time steps run inside one launch with the particle state held in
// registers; per-step ensemble observables are reduced warp -> block ->
// device with double accumulators.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "emcg_common.cuh"
#include "emcg_host.h"
#include "emcg_model.h"
#include "emcg_p2p.cuh"
#include "emcg_rates.cuh"

namespace emcg {

constexpr int kMaxScatterPerStep = 1 << 16; // bound on the per-step scatter loop

// ---------------------------------------------------------------------------
// device code
// ---------------------------------------------------------------------------
// free flight + periodic wrap (basicBulkParticleHandler.hpp:600-613)
template <class T>
__device__ __forceinline__ void driftBulk(const ValleyK<T> &V, int sub, const T fv[3], T dt,
                                          T k[3], T &E, T pos[3], T kN[3], const T box[3]) {
  drift<T, 3>(V, sub, fv, dt, k, E, pos, kN);
#pragma unroll
  for (int i = 0; i < 3; i++) {
    T c = pos[i];
    if (c < T(0))
      pos[i] = c + box[i];
    else if (c > box[i])
      pos[i] = c - box[i];
  }
}

// One particle, one time step (basicBulkParticleHandler.hpp:195-220).
template <class T, class Src>
__device__ __forceinline__ int bulkParticleStep(const ModelK<T> &M, const EnsK<T> &EK, T k[3],
                                                T pos[3], T &E, T &tau, T &gtau, int &valley,
                                                int &sub, int region, T kN[3], Src &rng) {
  const T dt = EK.dt;
  int err = 0;
  driftBulk(M.v[valley], sub, EK.fv[valley][sub], dt < tau ? dt : tau, k, E, pos, kN, EK.box);
  T tRem = dt - tau;
  int guard = 0;
  while (tRem > T(0)) {
    if (++guard > kMaxScatterPerStep) {
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
    driftBulk(M.v[valley], sub, EK.fv[valley][sub], nt < tRem ? nt : tRem, k, E, pos, kN,
              EK.box);
    tRem -= nt;
  }
  tau -= dt;
  gtau -= dt;
  if (gtau <= T(0)) { // basicBulkParticleHandler.hpp:215-219
    if (M.grain) {
      grainScatter(M, k, rng);
      toEcs(M.v[valley].rot[sub], k[0], k[1], k[2], kN);
    }
    gtau = -m_log(rng.ulog()) * M.grainTau;
  }
  return err;
}

// One particle, one time step with its own force F (FMMBulkParticleHandler::
// moveParticles, examples/bulkSimulationFMM/FMMBulkParticleHandler.hpp:233-277):
// the same free flights and scattering as bulkParticleStep, the force rotated
// into the frame of the current subvalley for each free flight.
template <class T, class Src>
__device__ __forceinline__ int bulkParticleStepF(const ModelK<T> &M, const EnsK<T> &EK,
                                                 const T F[3], T k[3], T pos[3], T &E, T &tau,
                                                 T &gtau, int &valley, int &sub, int region,
                                                 T kN[3], Src &rng) {
  const T dt = EK.dt;
  int err = 0;
  auto fvOf = [&](T fv[3]) {
    const ValleyK<T> &V = M.v[valley];
    toEcs(V.rot[sub], F[0], F[1], F[2], fv);
#pragma unroll
    for (int i = 0; i < 3; i++)
      fv[i] *= V.cF[i];
  };
  T fv[3];
  fvOf(fv);
  driftBulk(M.v[valley], sub, fv, dt < tau ? dt : tau, k, E, pos, kN, EK.box);
  T tRem = dt - tau;
  int guard = 0;
  while (tRem > T(0)) {
    if (++guard > kMaxScatterPerStep) {
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
    fvOf(fv);
    driftBulk(M.v[valley], sub, fv, nt < tRem ? nt : tRem, k, E, pos, kN, EK.box);
    tRem -= nt;
  }
  tau -= dt;
  gtau -= dt;
  if (gtau <= T(0)) { // basicBulkParticleHandler.hpp:215-219
    if (M.grain) {
      grainScatter(M, k, rng);
      toEcs(M.v[valley].rot[sub], k[0], k[1], k[2], kN);
    }
    gtau = -m_log(rng.ulog()) * M.grainTau;
  }
  return err;
}

template <class T> __device__ __forceinline__ T warpSum(T x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
    x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

__device__ __forceinline__ void recordError(int *err, int code) {
  if (code)
    atomicCAS(err, 0, code);
}

// Advance all tiles by nSteps time steps.  obs layout:
// [ens][step][nVmax][3] of {sum E, sum v.dir, count} (doubles).
// MINB: minimum resident blocks of 256 threads per SM requested from the
// compiler (register cap); 1 leaves the allocation unconstrained.
template <class T, bool REPLAY, int MINB>
__global__ void __launch_bounds__(256, MINB) bulkStepKernel(StateK<T> st, const ModelK<T> *__restrict__ models,
                               const EnsK<T> *__restrict__ ens, const Tile *__restrict__ tiles,
                               int nSteps, uint32_t step0, int chunk, int nVmax,
                               double *__restrict__ obs, const uint64_t *__restrict__ rw,
                               const int64_t *__restrict__ roff, int *__restrict__ err) {
  extern __shared__ __align__(16) unsigned char smemRaw[];
  T *sbuf = reinterpret_cast<T *>(smemRaw); // [chunk][nWarps][Q]
  const Tile tl = tiles[blockIdx.x];
  const EnsK<T> &EK = ens[tl.ens];
  const ModelK<T> &M = models[EK.model];
  const int nV = EK.nV;
  const int Q = nVmax * 3;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nWarps = blockDim.x >> 5;
  const int64_t gi = tl.begin + threadIdx.x;
  const bool active = gi < tl.end;
  const uint32_t pid = (uint32_t)(gi - EK.begin);

  T k[3] = {0, 0, 0}, pos[3] = {0, 0, 0}, kN[3] = {0, 0, 0}, E = 0, tau = 0, gtau = 0;
  int valley = 0, sub = 0, region = 0;
  if (active) {
    k[0] = st.kx[gi];
    k[1] = st.ky[gi];
    k[2] = st.kz[gi];
    pos[0] = st.px[gi];
    pos[1] = st.py[gi];
    pos[2] = st.pz[gi];
    E = st.E[gi];
    tau = st.tau[gi];
    gtau = st.gtau[gi];
    uint32_t mt = st.meta[gi];
    valley = mt & 0xff;
    sub = (mt >> 8) & 0xff;
    region = mt >> 16;
  }
  int myErr = 0;
  double *obsE = obs + (size_t)tl.ens * nSteps * Q;
  for (int s = 0; s < nSteps; s++) {
    if (active && !myErr) {
      if constexpr (REPLAY) {
        ReplaySrc src{rw, roff[pid], roff[pid + 1], 0};
        myErr = bulkParticleStep(M, EK, k, pos, E, tau, gtau, valley, sub, region, kN, src);
        if (!myErr && (src.bad || src.pos != src.end))
          myErr = EMCG_ERR_REPLAY;
      } else {
        PhiloxSrc<T> src;
        src.init(pid, step0 + (uint32_t)s, EK.stream, EK.key0, EK.key1, EK.floatDraws);
        myErr = bulkParticleStep(M, EK, k, pos, E, tau, gtau, valley, sub, region, kN, src);
      }
    }
    // drift velocity v.dir = cX (g . k_ecs) / sqrt(1 + 4 alpha gamma)
    // (emcNonParabolicAnistropValley.hpp:126-136 projected on the field)
    T vd = T(0);
    if (active) {
      const ValleyK<T> &V = M.v[valley];
      const T *g = EK.g[valley][sub];
      T npf = m_sqrt(T(1) + T(4) * V.alpha * gammaOf(V, E));
      vd = m_div(V.cX * (g[0] * kN[0] + g[1] * kN[1] + g[2] * kN[2]), npf);
    }
    T *row = sbuf + ((s % chunk) * nWarps + warp) * Q;
    for (int v = 0; v < nV; v++) {
      bool in = active && valley == v;
      T e = warpSum(in ? E : T(0));
      T d = warpSum(in ? vd : T(0));
      unsigned c = __popc(__ballot_sync(0xffffffffu, in));
      if (lane == 0) {
        row[v * 3 + 0] = e;
        row[v * 3 + 1] = d;
        row[v * 3 + 2] = (T)c;
      }
    }
    if ((s + 1) % chunk == 0 || s == nSteps - 1) {
      __syncthreads();
      const int inChunk = s % chunk + 1, sBase = s - s % chunk;
      const int nQ = nV * 3;
      for (int idx = threadIdx.x; idx < inChunk * nQ; idx += blockDim.x) {
        int cs = idx / nQ, q = idx - cs * nQ;
        double acc = 0.;
        for (int w = 0; w < nWarps; w++)
          acc += (double)sbuf[(cs * nWarps + w) * Q + q];
        atomicAdd(&obsE[(size_t)(sBase + cs) * Q + q], acc);
      }
      __syncthreads();
    }
  }
  if (active) {
    st.kx[gi] = k[0];
    st.ky[gi] = k[1];
    st.kz[gi] = k[2];
    st.px[gi] = pos[0];
    st.py[gi] = pos[1];
    st.pz[gi] = pos[2];
    st.E[gi] = E;
    st.tau[gi] = tau;
    st.gtau[gi] = gtau;
    st.meta[gi] = packMeta(valley, sub, region);
  }
  recordError(err, myErr);
}


// ---------------------------------------------------------------------------
// Particle-particle Coulomb steps (FMMBulkParticleHandler,
// examples/bulkSimulationFMM).  Per step: the sources of each ensemble -- its
// particles and its fixed charges -- are gathered, the Coulomb sums over them
// are formed for its particles (emcg_p2p.cuh, in place of executeFMM), and
// every particle moves one step with force = charge x field + coulFactor x sum
// (getForceAtParticle, :433-440).
// ---------------------------------------------------------------------------
template <class T>
__global__ void coulombGatherKernel(StateK<T> st, int64_t begin, int64_t n, double q,
                                    const double *__restrict__ fixed, int64_t nf,
                                    double *__restrict__ src) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, m = n + nf;
  if (i >= m)
    return;
  if (i < n) {
    src[i] = (double)st.px[begin + i];
    src[m + i] = (double)st.py[begin + i];
    src[2 * m + i] = (double)st.pz[begin + i];
    src[3 * m + i] = q;
  } else {
    const int64_t j = i - n;
    for (int v = 0; v < 4; v++)
      src[v * m + i] = fixed[v * nf + j];
  }
}

// One step of every particle with its own force; obs: [ens][Q] sums of this step.
template <class T>
__global__ void __launch_bounds__(256)
    bulkForceStepKernel(StateK<T> st, const ModelK<T> *__restrict__ models,
                        const EnsK<T> *__restrict__ ens, const Tile *__restrict__ tiles,
                        uint32_t step, int nVmax, const double *__restrict__ coulF,
                        int64_t stride, T coulFactor, double *__restrict__ obs,
                        int *__restrict__ err) {
  const Tile tl = tiles[blockIdx.x];
  const EnsK<T> &EK = ens[tl.ens];
  const ModelK<T> &M = models[EK.model];
  const int nV = EK.nV, Q = nVmax * 3, lane = threadIdx.x & 31;
  const int64_t gi = tl.begin + threadIdx.x;
  const bool active = gi < tl.end;
  const uint32_t pid = (uint32_t)(gi - EK.begin);
  T k[3] = {0, 0, 0}, pos[3] = {0, 0, 0}, kN[3] = {0, 0, 0}, E = 0, tau = 0, gtau = 0;
  int valley = 0, sub = 0, region = 0, myErr = 0;
  if (active) {
    k[0] = st.kx[gi];
    k[1] = st.ky[gi];
    k[2] = st.kz[gi];
    pos[0] = st.px[gi];
    pos[1] = st.py[gi];
    pos[2] = st.pz[gi];
    E = st.E[gi];
    tau = st.tau[gi];
    gtau = st.gtau[gi];
    const uint32_t mt = st.meta[gi];
    valley = mt & 0xff;
    sub = (mt >> 8) & 0xff;
    region = mt >> 16;
    T F[3];
#pragma unroll
    for (int v = 0; v < 3; v++)
      F[v] = EK.F[v] + coulFactor * (T)coulF[v * stride + gi];
    PhiloxSrc<T> rng;
    rng.init(pid, step, EK.stream, EK.key0, EK.key1, EK.floatDraws);
    myErr = bulkParticleStepF(M, EK, F, k, pos, E, tau, gtau, valley, sub, region, kN, rng);
  }
  T vd = T(0);
  if (active) {
    const ValleyK<T> &V = M.v[valley];
    const T *g = EK.g[valley][sub];
    const T npf = m_sqrt(T(1) + T(4) * V.alpha * gammaOf(V, E));
    vd = m_div(V.cX * (g[0] * kN[0] + g[1] * kN[1] + g[2] * kN[2]), npf);
  }
  for (int v = 0; v < nV; v++) {
    const bool in = active && valley == v;
    const T e = warpSum(in ? E : T(0)), d = warpSum(in ? vd : T(0));
    const unsigned c = __popc(__ballot_sync(0xffffffffu, in));
    if (lane == 0 && c) {
      double *o = obs + (size_t)tl.ens * Q + v * 3;
      atomicAdd(o + 0, (double)e);
      atomicAdd(o + 1, (double)d);
      atomicAdd(o + 2, (double)c);
    }
  }
  if (active) {
    st.kx[gi] = k[0];
    st.ky[gi] = k[1];
    st.kz[gi] = k[2];
    st.px[gi] = pos[0];
    st.py[gi] = pos[1];
    st.pz[gi] = pos[2];
    st.E[gi] = E;
    st.tau[gi] = tau;
    st.gtau[gi] = gtau;
    st.meta[gi] = packMeta(valley, sub, region);
  }
  recordError(err, myErr);
}

// ---------------------------------------------------------------------------
// Queued variant (Philox only).  The block's particles live in shared memory
// for the whole launch.  Each step:
//   A (owner)  free flight to min(tau, dt); a particle with an event inside
//              the step appends its index to the block's queue;
//   B (block)  the first warps process every queued event (selection, final
//              state, new free flight, remaining drift) for the whole block;
//   C (owner)  tau -= dt, grain timer, observables (merged with the next A).
// The scatter path thus runs once per 32 queued particles instead of once
// per warp holding one, and no particle state stays in registers across the
// barriers.  Random numbers: the event of particle pid in step s uses counter
// (pid, s, call, stream) as in the lockstep kernel; the grain free-flight
// redraw uses calls from 0x40000000 so that it does not depend on how many
// words the event consumed.
template <class T> struct BlockState {
  T *k0, *k1, *k2, *p0, *p1, *p2, *E, *tau, *gtau, *n0, *n1, *n2;
  uint32_t *meta;
  int32_t *queue;
};

template <class T>
__device__ __forceinline__ BlockState<T> blockState(unsigned char *base, int cap) {
  BlockState<T> b;
  T *t = reinterpret_cast<T *>(base);
  T **f[12] = {&b.k0, &b.k1, &b.k2, &b.p0, &b.p1, &b.p2, &b.E, &b.tau, &b.gtau, &b.n0, &b.n1, &b.n2};
  for (int i = 0; i < 12; i++)
    *f[i] = t + (size_t)i * cap;
  b.meta = reinterpret_cast<uint32_t *>(t + (size_t)12 * cap);
  b.queue = reinterpret_cast<int32_t *>(b.meta + cap);
  return b;
}

template <class T>
__host__ __device__ constexpr size_t blockStateBytes(int cap) {
  return (size_t)cap * (12 * sizeof(T) + sizeof(uint32_t) + sizeof(int32_t));
}

template <class T, int MINB>
__global__ void __launch_bounds__(256, MINB)
    bulkStepQueuedKernel(StateK<T> st, const ModelK<T> *__restrict__ models,
                         const EnsK<T> *__restrict__ ens, const Tile *__restrict__ tiles,
                         int nSteps, uint32_t step0, int chunk, int nVmax,
                         double *__restrict__ obs, int *__restrict__ err) {
  extern __shared__ __align__(16) unsigned char smemRaw[];
  const int nWarps = blockDim.x >> 5;
  const int Q = nVmax * 3;
  T *sbuf = reinterpret_cast<T *>(smemRaw); // [chunk][nWarps][Q]
  unsigned char *base = smemRaw + (((size_t)chunk * nWarps * Q * sizeof(T) + 15) & ~size_t(15));
  const BlockState<T> B = blockState<T>(base, blockDim.x);
  __shared__ int qCount[2];
  const Tile tl = tiles[blockIdx.x];
  const EnsK<T> &EK = ens[tl.ens];
  const ModelK<T> &M = models[EK.model];
  const int nV = EK.nV;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, me = threadIdx.x;
  const int64_t gi = tl.begin + me;
  const bool active = gi < tl.end;
  const T dt = EK.dt;
  if (me < 2)
    qCount[me] = 0;
  if (active) {
    B.k0[me] = st.kx[gi];
    B.k1[me] = st.ky[gi];
    B.k2[me] = st.kz[gi];
    B.p0[me] = st.px[gi];
    B.p1[me] = st.py[gi];
    B.p2[me] = st.pz[gi];
    B.E[me] = st.E[gi];
    B.tau[me] = st.tau[gi];
    B.gtau[me] = st.gtau[gi];
    B.meta[me] = st.meta[gi];
  }
  __syncthreads();
  // phase A of the first step
  if (active) {
    T k[3] = {B.k0[me], B.k1[me], B.k2[me]}, pos[3] = {B.p0[me], B.p1[me], B.p2[me]};
    T E = B.E[me], tau = B.tau[me], kN[3];
    uint32_t mt = B.meta[me];
    int valley = mt & 0xff, sub = (mt >> 8) & 0xff;
    driftBulk(M.v[valley], sub, EK.fv[valley][sub], dt < tau ? dt : tau, k, E, pos, kN, EK.box);
    B.k0[me] = k[0];
    B.k1[me] = k[1];
    B.k2[me] = k[2];
    B.p0[me] = pos[0];
    B.p1[me] = pos[1];
    B.p2[me] = pos[2];
    B.E[me] = E;
    B.n0[me] = kN[0];
    B.n1[me] = kN[1];
    B.n2[me] = kN[2];
    if (dt - tau > T(0))
      B.queue[atomicAdd(&qCount[0], 1)] = me;
  }
  __syncthreads();
  double *obsE = obs + (size_t)tl.ens * nSteps * Q;
  for (int s = 0; s < nSteps; s++) {
    const uint32_t step = step0 + (uint32_t)s;
    // phase B: queued events of step s
    const int nq = qCount[s & 1];
    if (me == 0)
      qCount[(s + 1) & 1] = 0;
    for (int j = me; j < nq; j += blockDim.x) {
      const int p = B.queue[j];
      T k[3] = {B.k0[p], B.k1[p], B.k2[p]}, pos[3] = {B.p0[p], B.p1[p], B.p2[p]};
      T E = B.E[p], tau = B.tau[p], kN[3];
      uint32_t mt = B.meta[p];
      int valley = mt & 0xff, sub = (mt >> 8) & 0xff, region = mt >> 16;
      T tRem = dt - tau;
      PhiloxSrc<T> rng;
      rng.init((uint32_t)(tl.begin + p - EK.begin), step, EK.stream, EK.key0, EK.key1,
               EK.floatDraws);
      int guard = 0, e = 0;
      while (tRem > T(0)) {
        if (++guard > kMaxScatterPerStep) {
          e = EMCG_ERR_TIMEOUT;
          break;
        }
        e = scatterParticle(M, k, E, valley, sub, region, rng);
        if (e)
          break;
        T nt = -m_log(rng.ulog()) * tauOf(M, valley, region);
        tau += nt;
        driftBulk(M.v[valley], sub, EK.fv[valley][sub], nt < tRem ? nt : tRem, k, E, pos, kN,
                  EK.box);
        tRem -= nt;
      }
      recordError(err, e);
      B.k0[p] = k[0];
      B.k1[p] = k[1];
      B.k2[p] = k[2];
      B.p0[p] = pos[0];
      B.p1[p] = pos[1];
      B.p2[p] = pos[2];
      B.E[p] = E;
      B.tau[p] = tau;
      B.n0[p] = kN[0];
      B.n1[p] = kN[1];
      B.n2[p] = kN[2];
      B.meta[p] = packMeta(valley, sub, region);
    }
    __syncthreads();
    // phase C of step s (+ phase A of step s + 1)
    T E = T(0), vd = T(0);
    int valley = 0;
    if (active) {
      T tau = B.tau[me] - dt, gtau = B.gtau[me] - dt;
      E = B.E[me];
      uint32_t mt = B.meta[me];
      valley = mt & 0xff;
      int sub = (mt >> 8) & 0xff;
      if (gtau <= T(0)) {
        PhiloxSrc<T> rng;
        rng.init((uint32_t)(gi - EK.begin), step, EK.stream, EK.key0, EK.key1, EK.floatDraws);
        rng.c2 = 0x40000000u;
        if (M.grain) { // the step's new k and its ellipse-frame copy for the sums
          T k[3] = {B.k0[me], B.k1[me], B.k2[me]}, kN[3];
          grainScatter(M, k, rng);
          toEcs(M.v[valley].rot[sub], k[0], k[1], k[2], kN);
          B.k0[me] = k[0];
          B.k1[me] = k[1];
          B.k2[me] = k[2];
          B.n0[me] = kN[0];
          B.n1[me] = kN[1];
          B.n2[me] = kN[2];
        }
        gtau = -m_log(rng.ulog()) * M.grainTau;
      }
      B.gtau[me] = gtau;
      const ValleyK<T> &V = M.v[valley];
      const T *g = EK.g[valley][sub];
      T npf = m_sqrt(T(1) + T(4) * V.alpha * gammaOf(V, E));
      vd = m_div(V.cX * (g[0] * B.n0[me] + g[1] * B.n1[me] + g[2] * B.n2[me]), npf);
      if (s + 1 < nSteps) { // phase A of the next step
        T k[3] = {B.k0[me], B.k1[me], B.k2[me]}, pos[3] = {B.p0[me], B.p1[me], B.p2[me]};
        T E2 = E, kN[3];
        driftBulk(V, sub, EK.fv[valley][sub], dt < tau ? dt : tau, k, E2, pos, kN, EK.box);
        B.k0[me] = k[0];
        B.k1[me] = k[1];
        B.k2[me] = k[2];
        B.p0[me] = pos[0];
        B.p1[me] = pos[1];
        B.p2[me] = pos[2];
        B.E[me] = E2;
        B.n0[me] = kN[0];
        B.n1[me] = kN[1];
        B.n2[me] = kN[2];
        if (dt - tau > T(0))
          B.queue[atomicAdd(&qCount[(s + 1) & 1], 1)] = me;
      }
      B.tau[me] = tau;
    }
    T *row = sbuf + ((s % chunk) * nWarps + warp) * Q;
    for (int v = 0; v < nV; v++) {
      bool in = active && valley == v;
      T e = warpSum(in ? E : T(0));
      T d = warpSum(in ? vd : T(0));
      unsigned c = __popc(__ballot_sync(0xffffffffu, in));
      if (lane == 0) {
        row[v * 3 + 0] = e;
        row[v * 3 + 1] = d;
        row[v * 3 + 2] = (T)c;
      }
    }
    __syncthreads();
    if ((s + 1) % chunk == 0 || s == nSteps - 1) {
      const int inChunk = s % chunk + 1, sBase = s - s % chunk;
      const int nQ = nV * 3;
      for (int idx = me; idx < inChunk * nQ; idx += blockDim.x) {
        int cs = idx / nQ, qq = idx - cs * nQ;
        double acc = 0.;
        for (int w = 0; w < nWarps; w++)
          acc += (double)sbuf[(cs * nWarps + w) * Q + qq];
        atomicAdd(&obsE[(size_t)(sBase + cs) * Q + qq], acc);
      }
      __syncthreads();
    }
  }
  if (active) {
    st.kx[gi] = B.k0[me];
    st.ky[gi] = B.k1[me];
    st.kz[gi] = B.k2[me];
    st.px[gi] = B.p0[me];
    st.py[gi] = B.p1[me];
    st.pz[gi] = B.p2[me];
    st.E[gi] = B.E[me];
    st.tau[gi] = B.tau[me];
    st.gtau[gi] = B.gtau[me];
    st.meta[gi] = B.meta[me];
  }
}

// Initial particles (include/ParticleType/emcElectron.hpp:75-90,
// include/emcParticleInitialization.hpp:14-51), Philox counter
// (i, 0xFFFFFFFF, call, stream).  coords == nullptr: uniform in the box.
template <class T>
__global__ void bulkInitKernel(StateK<T> st, const ModelK<T> *__restrict__ models, int model,
                               int64_t begin, int64_t n, const int64_t *__restrict__ coords,
                               int64_t e0, int64_t e1, int64_t e2, double h0, double h1,
                               double h2, double Vt, double b0, double b1, double b2,
                               uint32_t key0, uint32_t key1, uint32_t stream) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  const ModelK<T> &M = models[model];
  PhiloxSrc<T> rng;
  rng.init((uint32_t)i, 0xFFFFFFFFu, stream, key0, key1);
  T pos[3];
  int64_t c[3] = {0, 0, 0};
  const int64_t ext[3] = {e0, e1, e2};
  const double h[3] = {h0, h1, h2};
  if (coords) {
    c[0] = coords[3 * i];
    c[1] = coords[3 * i + 1];
    c[2] = coords[3 * i + 2];
#pragma unroll
    for (int d = 0; d < 3; d++) {
      if (c[d] == ext[d] - 1)
        pos[d] = ((T)c[d] - rng.u01() * T(0.5)) * (T)h[d];
      else if (c[d] == 0)
        pos[d] = rng.u01() * T(0.5) * (T)h[d];
      else
        pos[d] = ((T)c[d] + rng.u01() - T(0.5)) * (T)h[d];
    }
  } else {
    pos[0] = rng.u01() * (T)b0;
    pos[1] = rng.u01() * (T)b1;
    pos[2] = rng.u01() * (T)b2;
  }
  int valley = (int)m_floor((T)M.nV * rng.ulog());
  const ValleyK<T> &V = M.v[valley];
  int sub = (int)m_floor((T)V.deg * rng.ulog());
  T E = T(-1.5) * (T)Vt * m_log(rng.ulog());
  T k[3];
  randomDirection(V.cK * m_sqrt(gammaOf(V, E)), rng, k);
  if (coords) {
#pragma unroll
    for (int d = 0; d < 3; d++)
      if ((c[d] == 0 && k[d] < T(0)) || (c[d] == ext[d] - 1 && k[d] > T(0)))
        k[d] *= T(-1);
  }
  T tau = -m_log(rng.ulog()) * tauOf(M, valley, 0);
  T gtau = -m_log(rng.ulog()) * M.grainTau;
  int64_t g = begin + i;
  st.kx[g] = k[0];
  st.ky[g] = k[1];
  st.kz[g] = k[2];
  st.px[g] = pos[0];
  st.py[g] = pos[1];
  st.pz[g] = pos[2];
  st.E[g] = E;
  st.tau[g] = tau;
  st.gtau[g] = gtau;
  st.meta[g] = packMeta(valley, sub, 0);
}

// ---------------------------------------------------------------------------
// Warp-asynchronous variant (float, Philox).  In the lockstep kernel nearly
// every warp holds a particle with an event in a given step, so the warp runs
// the scatter path with a few lanes active.  Here each lane runs its own
// particle and the warp works in passes.  In a drift pass every lane that can
// go on flies freely to whichever comes first, the end of its current step
// (then the end-of-step bookkeeping and its observables) or its next event
// (then it waits); all of them run the drift together.  Once kEventBatch
// lanes wait at events (one, by measurement), or no lane can go on, a scatter
// pass scatters the waiting lanes together.  The physics and the random numbers are those of
// the lockstep kernel: the same free flights, the Philox counter (pid, step,
// call) restarted at each step, the grain timer at each step end.
// Observables: a lane writes its per-step values into its own column of a
// small per-warp window; once every lane of the warp has passed a step, the
// warp folds that row into the block's float step sums (shared memory), which
// go to the device's double sums at the end of the launch.  A lane runs at
// most a window's length of steps ahead of the slowest lane of its warp.  The
// constants below were chosen by measurement on 2^20 and 2^22 electrons.
// ---------------------------------------------------------------------------
// window length with several valleys (the window also keeps each step's
// valley), and with one valley: 24 steps of E and v.dir per lane still let 4
// blocks of 256 threads share an SM at 500 steps per launch (+2.2 % on 2^20
// electrons, +1.4 % on the sweep against 20)
constexpr int kAsyncWindow = 20;
constexpr int kAsyncWindowOne = 24;
// lanes of a warp that wait at an event before the warp scatters them together.
// With six free flights per pass and the 24-step window one is best: the warp
// scatters as soon as a lane waits.  Measured on 2^20 electrons (ms per
// launch, 20 steps / 500 steps) and the 64-ensemble sweep (500 steps, 3
// flights per pass): 1 lane 0.3029 / 5.514 / 82.60, 2 0.3035 / 5.529, 3
// 0.3049 / 5.527 / 83.03, 4 0.3052 / 5.520, 5 0.3076 / 5.531, 6 0.3100 /
// 5.543, 7 0.3116 / 5.565 / 83.08 (7 was best with one or five flights per
// pass and shorter windows)
constexpr int kEventBatch = 1;
// free flights a lane may take in one drift pass, by default (set per handle:
// emcg_set_pass_actions).  Measured on 2^20 electrons, 2000 steps, 20-step
// window: 3 gave 8.90e10, 4 9.00e10, 5 9.06e10, 6 9.02e10, 8 8.70e10, 20
// 6.79e10; with the 24-step one-valley window 4 gave 9.11e10, 5 9.30e10, 6
// 9.34e10, 7 9.28e10.  On the 64-ensemble sweep 5 was 3.6 % slower than 3, so
// the autotuner tries 3 and 6.
constexpr int kPassActions = 6;
// the default for launches shorter than kShortLaunchSteps: measured on 2^20
// electrons, one 20-step launch, L2 flushed (ms; 64 / 128 / 256 threads): 4
// 0.3155 / 0.3159 / 0.3171, 5 0.3116 / 0.3108 / 0.3149, 6 0.3133 / 0.3128 /
// 0.3170, 8 0.3256 / 0.3236 / 0.3278
constexpr int kPassActionsShort = 5;
// fixed-point scales of a warp's step sums: energy 2^-20 eV, velocity
// 0.25 m/s per unit; below kFixMax per lane, 32 lanes stay within int32
constexpr float kFixE = 1048576.f;
constexpr float kFixD = 4.f;
constexpr float kFixMax = 67108864.f;

// the windows of a block: Q = 3 (one valley) holds E and v.dir per slot,
// more valleys also the slot's valley
__host__ __device__ constexpr size_t asyncWindowBytes(int nWarps, int Q) {
  return Q == 3 ? (size_t)nWarps * kAsyncWindowOne * 32 * (2 * sizeof(float))
                : (size_t)nWarps * kAsyncWindow * 32 * (2 * sizeof(float) + 1);
}
__host__ __device__ constexpr size_t asyncSmemBytes(int nWarps, int nSteps, int Q) {
  return (size_t)nSteps * Q * sizeof(float) + asyncWindowBytes(nWarps, Q);
}
// steps per launch whose block sums fit beside the windows in 64 KB
inline int asyncMaxSteps(int nWarps, int Q) {
  const long rest = 65536 - (long)asyncWindowBytes(nWarps, Q);
  return (int)std::max(1L, rest / (long)(Q * sizeof(float)));
}


// drift() (include/emcParticleDrift.hpp:11-36) with k held in the ellipse
// frame of the particle's subvalley: the frame changes only at scattering, so
// k goes to the device frame and back there, not at every free flight.  The
// displacement is summed in the ellipse frame too (dP) and added to the
// position by flushPos.  |k| is the same in both frames (R orthonormal).
// Returns hbar / (mc (1 + 2 alpha E)) at the new energy: the velocity factor
// of the ellipse-frame k (emcNonParabolicAnistropValley.hpp:185-204, with
// sqrt(1 + 4 alpha gamma) = 1 + 2 alpha E).  With g = hbar^2 k^2 / (mc q) and
// s = sqrt(1 + 2 alpha g), E = g / (1 + s) (:109-113) and 1 + 2 alpha E = s, so
// one reciprocal square root serves the energy and the velocity factor.  dP
// sums (k_old + k_new) c without the Herring-Vogt factors, which flushPos
// applies: they are constant until the valley changes.
__device__ __forceinline__ float driftEcs(const ValleyK<float> &V, const float fv[3], float dt,
                                          float kE[3], float &E, float dP[3]) {
  float kO[3];
#pragma unroll
  for (int i = 0; i < 3; i++) {
    kO[i] = kE[i];
    kE[i] = kO[i] + fv[i] * dt;
  }
  const float g = V.cE * (kE[0] * kE[0] + kE[1] * kE[1] + kE[2] * kE[2]);
  const float t = fmaf(2.f * V.alpha, g, 1.f);
  const float rs = rsqrtf(t);
  E = m_div(g, 1.f + t * rs);
  const float vf = V.cX * rs;
  const float c = vf * (0.5f * dt);
#pragma unroll
  for (int i = 0; i < 3; i++)
    dP[i] = fmaf(kE[i] + kO[i], c, dP[i]);
  return vf;
}

// The summed displacement into the device frame and the periodic box
// (basicBulkParticleHandler.hpp:600-613); the sum covers one free flight or
// less, far below a box length.
__device__ __forceinline__ void flushPos(const float *R, const float vogt[3], float dP[3],
                                         float pos[3], const float box[3]) {
  float dd[3];
  toDev(R, dP[0] * vogt[0], dP[1] * vogt[1], dP[2] * vogt[2], dd);
#pragma unroll
  for (int i = 0; i < 3; i++) {
    float c = pos[i] + dd[i];
    if (c < 0.f || c > box[i])
      c -= box[i] * floorf(c / box[i]);
    pos[i] = c;
    dP[i] = 0.f;
  }
}

// kGrain: an instance for batches with a grain mechanism; the other keeps the
// grain branch out of the register allocation of the step loop (64 registers
// at 4 blocks per SM: the branch spilled 64 B there)
template <int MINB, bool kOne, bool kGrain>
__global__ void __launch_bounds__(256, MINB)
    bulkStepAsyncKernel(StateK<float> st, StateK<float> src, int srcEns,
                        const ModelK<float> *__restrict__ models,
                        const EnsK<float> *__restrict__ ens, const Tile *__restrict__ tiles,
                        int nSteps, uint32_t step0, int chunk, int nVmax, int passActions,
                        double *__restrict__ obs, int *__restrict__ err) {
  using T = float;
  extern __shared__ __align__(16) unsigned char smemRaw[];
  const int Q = nVmax * 3;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nWarps = blockDim.x >> 5;
  float *bins = reinterpret_cast<float *>(smemRaw); // [nSteps][Q] block sums
  constexpr int W = kOne ? kAsyncWindowOne : kAsyncWindow;
  float *winE = bins + (size_t)nSteps * Q + (size_t)warp * W * 64; // [W][32]
  float *winD = winE + W * 32;                                    // [W][32]
  uint8_t *winVal = reinterpret_cast<uint8_t *>(bins + (size_t)nSteps * Q +
                                                (size_t)nWarps * W * 64) +
                    warp * W * 32; // [W][32], several valleys only
  for (int i = threadIdx.x; i < nSteps * Q; i += blockDim.x)
    bins[i] = 0.f;
  __syncthreads();
  const Tile tl = tiles[blockIdx.x];
  const EnsK<T> &EK = ens[tl.ens];
  const ModelK<T> &M = models[EK.model];
  const int nV = kOne ? 1 : EK.nV;
  const int64_t gi = tl.begin + threadIdx.x;
  bool active = gi < tl.end;
  const uint32_t pid = (uint32_t)(gi - EK.begin);
  const T dt = EK.dt;

  // kE: k in the ellipse frame of the subvalley; dP: displacement in that
  // frame not yet added to pos
  T kE[3] = {0, 0, 0}, pos[3] = {0, 0, 0}, dP[3] = {0, 0, 0}, E = 0, tau = 0, gtau = 0;
  int valley = 0, sub = 0, region = 0;
  int myErr = 0;
  if (active) {
    // the start state: ensemble srcEns's page-locked host arrays (read over
    // the host link, the upload fused into the launch), else the device state
    const StateK<float> ld = tl.ens == srcEns ? src : st;
    const uint32_t mt = ld.meta[gi];
    valley = mt & 0xff;
    sub = (mt >> 8) & 0xff;
    region = mt >> 16;
    if (valley >= nV || sub >= EMCG_MAX_DEG || region >= EMCG_MAX_REGIONS) {
      active = false; // an unchecked host state: neither stepped nor stored
      myErr = EMCG_ERR_ARG;
    } else {
      pos[0] = ld.px[gi];
      pos[1] = ld.py[gi];
      pos[2] = ld.pz[gi];
      E = ld.E[gi];
      tau = ld.tau[gi];
      gtau = ld.gtau[gi];
      toEcs(M.v[valley].rot[sub], ld.kx[gi], ld.ky[gi], ld.kz[gi], kE);
    }
  }
  bool live = active;    // false once the particle has failed
  int s = live ? 0 : nSteps; // the step the particle is in
  T tIn = 0;             // time already spent inside step s
  int nEv = 0;           // events in step s (bounded)
  PhiloxSrc<T> rng;
  rng.init(pid, step0, EK.stream, EK.key0, EK.key1);
  int flushed = 0;  // steps folded into the block sums
  float accE = 0.f, accD = 0.f, accC = 0.f; // one valley: sums of a step of the 32-step group
  int ws = 0;        // window slot of step s (s mod W)
  bool pend = false; // drifted to an event inside step s, not yet scattered
  while (true) {
    const int sMin = __reduce_min_sync(0xffffffffu, s);
    for (; flushed < sMin; flushed++) {
      const int slot = (flushed % W) * 32 + lane;
      for (int v = 0; v < nV; v++) {
        const bool in = live && (nV == 1 || winVal[slot] == v);
        const T ev = in ? winE[slot] : T(0), dv = in ? winD[slot] : T(0);
        // the warp's sums in fixed point, exact and one instruction each
        // (redux.sync); a step with a value out of range sums in float
        const T fe = ev * kFixE, fd = dv * kFixD;
        T e, d;
        if (__all_sync(0xffffffffu, fabsf(fe) < kFixMax && fabsf(fd) < kFixMax)) {
          e = (T)(int)__reduce_add_sync(0xffffffffu, (unsigned)__float2int_rn(fe)) *
              (T(1) / kFixE);
          d = (T)(int)__reduce_add_sync(0xffffffffu, (unsigned)__float2int_rn(fd)) *
              (T(1) / kFixD);
        } else {
          e = warpSum(ev);
          d = warpSum(dv);
        }
        const unsigned c = __popc(__ballot_sync(0xffffffffu, in));
        if (nV == 1) {
          // one valley: lane (step mod 32) keeps the step's sums, and the
          // warp adds 32 steps to the block sums in one go
          if (lane == (flushed & 31)) {
            accE = e;
            accD = d;
            accC = (float)c;
          }
          if ((flushed & 31) == 31) {
            float *b = bins + (size_t)((flushed & ~31) + lane) * Q;
            atomicAdd(b + 0, accE);
            atomicAdd(b + 1, accD);
            atomicAdd(b + 2, accC);
          }
        } else if (lane == 0) {
          float *b = bins + (size_t)flushed * Q + v * 3;
          atomicAdd(b + 0, e);
          atomicAdd(b + 1, d);
          atomicAdd(b + 2, (float)c);
        }
      }
    }
    if (sMin >= nSteps)
      break;
    const int limit = min(nSteps, flushed + W);
    // a lane whose free flight ended at an event waits (pend) until enough
    // lanes of its warp wait too, or no lane can go on: then they scatter
    // together, so the scatter path runs for several lanes at once
    const bool can = !pend && s < limit;
    const unsigned pendMask = __ballot_sync(0xffffffffu, pend);
    const unsigned canMask = __ballot_sync(0xffffffffu, can);
    if (pendMask && (__popc(pendMask) >= kEventBatch || !canMask)) {
      if (pend) { // scattering (device frame), new free flight
        pend = false;
        T k[3];
        const T *R = M.v[valley].rot[sub];
        toDev(R, kE[0], kE[1], kE[2], k);
        flushPos(R, M.v[valley].vogt, dP, pos, EK.box);
        const int e = scatterParticle(M, k, E, valley, sub, region, rng);
        if (e) {
          myErr = e;
          live = false;
          s = nSteps;
        } else {
          tau = -m_log(rng.ulog()) * tauOf(M, valley, region);
        }
        toEcs(M.v[valley].rot[sub], k[0], k[1], k[2], kE);
      }
    } else {
      // up to passActions free flights per lane and pass: each ends either at
      // the end of step s (bulkParticleStep without an event) or at the next
      // event inside it; both drift first, so the warp's lanes drift together
      // the subvalley's force and field direction, read once per pass
      const int vd = kOne ? 0 : valley;
      T fvl[3], gl[3];
#pragma unroll
      for (int i = 0; i < 3; i++) {
        fvl[i] = EK.fv[vd][sub][i];
        gl[i] = EK.g[vd][sub][i];
      }
#pragma unroll 1
      for (int act = 0; act < passActions && !pend && s < limit; act++) {
        const T rem = dt - tIn;
        const bool ev = tau < rem;
        if (ev && ++nEv > kMaxScatterPerStep) {
          myErr = EMCG_ERR_TIMEOUT;
          live = false;
          s = nSteps;
        } else {
          const T vf = driftEcs(M.v[vd], fvl, ev ? tau : rem, kE, E, dP);
          if (ev) {
            tIn += tau;
            pend = true;
          } else { // end of step s: its observables, then step s + 1
            tau -= rem;
            gtau -= dt;
            if (gtau <= T(0)) { // basicBulkParticleHandler.hpp:215-219
              if (kGrain && M.grain) { // in the device frame; the subvalley (and dP's frame) stay
                const T *R = M.v[vd].rot[sub];
                T k[3];
                toDev(R, kE[0], kE[1], kE[2], k);
                grainScatter(M, k, rng);
                toEcs(R, k[0], k[1], k[2], kE);
              }
              gtau = -m_log(rng.ulog()) * M.grainTau;
            }
            const int slot = ws * 32 + lane;
            winE[slot] = E;
            winD[slot] = vf * (gl[0] * kE[0] + gl[1] * kE[1] + gl[2] * kE[2]);
            if (nV > 1)
              winVal[slot] = (uint8_t)valley;
            s++;
            tIn = T(0);
            nEv = 0;
            ws = ws + 1 == W ? 0 : ws + 1;
            rng.restart(step0 + (uint32_t)s);
          }
        }
      }
    }
  }
  if (nV == 1 && lane < (flushed & 31)) { // the last, partial group of steps
    float *b = bins + (size_t)((flushed & ~31) + lane) * Q;
    atomicAdd(b + 0, accE);
    atomicAdd(b + 1, accD);
    atomicAdd(b + 2, accC);
  }
  __syncthreads();
  double *obsE = obs + (size_t)tl.ens * nSteps * Q;
  for (int i = threadIdx.x; i < nSteps * Q; i += blockDim.x)
    if (bins[i] != 0.f)
      atomicAdd(&obsE[i], (double)bins[i]);
  if (active) {
    T k[3];
    const T *R = M.v[valley].rot[sub];
    toDev(R, kE[0], kE[1], kE[2], k);
    flushPos(R, M.v[valley].vogt, dP, pos, EK.box);
    st.kx[gi] = k[0];
    st.ky[gi] = k[1];
    st.kz[gi] = k[2];
    st.px[gi] = pos[0];
    st.py[gi] = pos[1];
    st.pz[gi] = pos[2];
    st.E[gi] = E;
    st.tau[gi] = tau;
    st.gtau[gi] = gtau;
    st.meta[gi] = packMeta(valley, sub, region);
  }
  recordError(err, myErr);
}

// dynamic shared memory above the default 48 KB needs the kernel's opt-in
template <int MINB> int32_t asyncSmemOptIn(size_t bytes) {
  if (bytes <= 48 * 1024)
    return EMCG_OK;
  for (auto k : {bulkStepAsyncKernel<MINB, false, false>, bulkStepAsyncKernel<MINB, true, false>,
                 bulkStepAsyncKernel<MINB, false, true>, bulkStepAsyncKernel<MINB, true, true>})
    EMCG_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  return EMCG_OK;
}

// the warp-asynchronous kernel for a register cap; one: every ensemble of the
// batch has one valley, so the drift reads that valley's constants once;
// grain: some model of the batch has a grain mechanism
template <int MINB> static auto asyncKernel(bool one, bool grain) {
  if (grain)
    return one ? bulkStepAsyncKernel<MINB, true, true> : bulkStepAsyncKernel<MINB, false, true>;
  return one ? bulkStepAsyncKernel<MINB, true, false> : bulkStepAsyncKernel<MINB, false, false>;
}

// drift() known-answer kernel: independent particles, per-particle force/dt
template <class T>
__global__ void driftKatKernel(const ModelK<T> *__restrict__ models, int valley, int64_t n,
                               const int32_t *__restrict__ sub, const double *__restrict__ dt,
                               const double *__restrict__ force, double *__restrict__ k,
                               double *__restrict__ pos, double *__restrict__ energy) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  const ValleyK<T> &V = models[0].v[valley];
  int s = sub[i];
  T F[3] = {(T)force[i], (T)force[n + i], (T)force[2 * n + i]};
  T fE[3];
  toEcs(V.rot[s], F[0], F[1], F[2], fE);
  T fv[3] = {fE[0] * V.cF[0], fE[1] * V.cF[1], fE[2] * V.cF[2]};
  T kk[3] = {(T)k[i], (T)k[n + i], (T)k[2 * n + i]};
  T p[3] = {(T)pos[i], (T)pos[n + i], (T)pos[2 * n + i]};
  T E = (T)energy[i], kN[3];
  drift<T, 3>(V, s, fv, (T)dt[i], kk, E, p, kN);
  for (int d = 0; d < 3; d++) {
    k[d * n + i] = (double)kk[d];
    pos[d * n + i] = (double)p[d];
  }
  energy[i] = (double)E;
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct BulkImpl {
  int precision = EMCG_FP64;
  size_t tsz = 8;
  int nModels = 0, nEns = 0, nVmax = 1;
  bool anyGrain = false; // some model has a grain mechanism
  std::vector<emcg_ensemble_desc> ens;
  std::vector<emcg_model_desc> modelDescs;       // shallow copies (valleys)
  std::vector<std::vector<emcg_valley_desc>> valleyCopies;
  std::vector<int> ensNV;
  std::vector<int64_t> begin, count, cap;
  int64_t totalCap = 0;
  void *dModels = nullptr;
  std::vector<void *> dTables;
  std::vector<RateLayout> rates; // table layout per model (rate-table rebuild)
  RateScratch rateScratch;        // device scratch of rebuilds
  void *dEns = nullptr;
  Tile *dTiles = nullptr;
  int nTiles = 0, tilesCap = 0;
  bool tilesDirty = true;
  void *dState[9] = {};
  uint32_t *dMeta = nullptr;
  double *dObs = nullptr;
  size_t obsCap = 0;
  double *hObs = nullptr; // page-locked copy of dObs (asynchronous readback)
  int *hErr = nullptr;    // page-locked copy of dErr
  int *dErr = nullptr;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  int blockThreads = 256;
  bool autoBlock = true; // block size chosen per launch (emcg_set_launch, -1)
  int minBlocks = 1; // register cap variant of the step kernel (1, 3 or 4)
  int queued = 0; // step kernel: 0 lockstep, 1 block-queued, 2 warp-asynchronous (float)
  int passActions = kPassActions; // warp-asynchronous kernel: free flights per drift pass
  bool passAuto = true;           // not set by the caller or the autotuner: by launch length
  int stepsPerLaunch = 0;
  int chunk = 16;
  uint64_t *dWords = nullptr;
  int64_t wordsCap = 0;
  int64_t *dOff = nullptr;
  int64_t offCap = 0;
  bool replay = false;
  double lastMs = 0;
  // device staging of state uploads, the caller's arrays as they are (grown
  // on demand), and the first bad particle index the conversion found
  void *dStage = nullptr;
  size_t stageBytes = 0;
  unsigned long long *dBad = nullptr;
  // particle-particle Coulomb steps (FMMBulkParticleHandler)
  bool coulomb = false;
  double coulEpsR = 1., coulInvCut = 1e9;
  int coulImages = 0, sms = 0;
  std::vector<int64_t> nFixed;       // fixed charges per ensemble
  std::vector<double *> dFixed;      // their x, y, z, q planes
  double *dSrc = nullptr, *dPart = nullptr, *dCoulF = nullptr;
  int64_t srcCap = 0, partCap = 0;
  // graph replay of one launch of steps: [observable reset] -> [step kernel],
  // instantiated per launch shape, the step offset updated before each replay
  bool useGraph = false;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  cudaGraphNode_t gKernel = nullptr;
  cudaKernelNodeParams gKp = {};
  int gNs = -1, gBlock = 0, gMinb = 0, gQueued = -1, gTiles = -1, gPass = -1;
  alignas(16) unsigned char gArgs[256] = {};
  void *gParams[14] = {};
};

// arguments of the step kernels, in parameter order
template <class T> struct StepArgs {
  StateK<T> st;
  StateK<T> src; // the warp-asynchronous kernel's start state (st: the device's)
  int srcEns;
  const ModelK<T> *mp;
  const EnsK<T> *ep;
  const Tile *tiles;
  int ns;
  uint32_t step0;
  int chunk;
  int nVmax;
  int pass;
  double *obs;
  const uint64_t *words;
  const int64_t *off;
  int *err;
};

template <class T> static StateK<T> stateOf(BulkImpl *b) {
  StateK<T> s;
  T **f[9] = {&s.kx, &s.ky, &s.kz, &s.px, &s.py, &s.pz, &s.E, &s.tau, &s.gtau};
  for (int i = 0; i < 9; i++)
    *f[i] = (T *)b->dState[i];
  s.meta = b->dMeta;
  return s;
}

template <class T>
static void buildEnsK(const emcg_ensemble_desc &d, const ModelK<T> &M,
                      const emcg_model_desc &md, int64_t begin, int64_t n, EnsK<T> &E) {
  std::memset(&E, 0, sizeof(E));
  E.model = d.model;
  E.nV = md.n_valleys;
  E.begin = begin;
  E.n = n;
  double F[3], dir[3];
  for (int i = 0; i < 3; i++)
    F[i] = d.field[i] * d.charge; // scale(appliedField, charge) (:186)
  double nrm = std::sqrt(d.field_dir[0] * d.field_dir[0] + d.field_dir[1] * d.field_dir[1] +
                         d.field_dir[2] * d.field_dir[2]);
  for (int i = 0; i < 3; i++)
    dir[i] = nrm > 0 ? d.field_dir[i] / nrm : 0.;
  for (int v = 0; v < md.n_valleys; v++) {
    const emcg_valley_desc &V = md.valleys[v];
    ValleyDerived dv = deriveValley(V);
    for (int s = 0; s < V.deg; s++) {
      const double *R = V.rot[s];
      for (int i = 0; i < 3; i++) {
        double fe = F[0] * R[3 * i] + F[1] * R[3 * i + 1] + F[2] * R[3 * i + 2];
        double de = dir[0] * R[3 * i] + dir[1] * R[3 * i + 1] + dir[2] * R[3 * i + 2];
        E.fv[v][s][i] = (T)(fe * dv.vogt[i] / kHBAR);
        E.g[v][s][i] = (T)(dv.vogt[i] * de);
      }
    }
  }
  for (int i = 0; i < 3; i++) {
    E.box[i] = (T)d.box[i];
    E.F[i] = (T)F[i];
  }
  E.charge = (T)d.charge;
  E.dt = (T)d.dt;
  E.key0 = (uint32_t)d.seed;
  E.key1 = (uint32_t)(d.seed >> 32);
  E.stream = d.stream;
  E.floatDraws = (d.flags & EMCG_ENS_FLOAT_DRAWS) ? 1u : 0u;
  (void)M;
}

template <class T>
static int32_t createTyped(BulkImpl *b, const emcg_model_desc *models, int nModels,
                           const emcg_ensemble_desc *ens, int nEns) {
  std::vector<ModelK<T>> mk(nModels);
  b->dTables.assign(nModels, nullptr);
  b->rates.resize(nModels);
  for (int i = 0; i < nModels; i++) {
    std::vector<T> tab;
    EMCG_TRY(buildModelK<T>(models[i], mk[i], tab));
    b->rates[i] = rateLayoutOf(models[i]);
    EMCG_CUDA(cudaMalloc(&b->dTables[i], tab.size() * sizeof(T)));
    EMCG_CUDA(cudaMemcpy(b->dTables[i], tab.data(), tab.size() * sizeof(T),
                         cudaMemcpyHostToDevice));
    mk[i].tables = (const T *)b->dTables[i];
  }
  EMCG_CUDA(cudaMalloc(&b->dModels, sizeof(ModelK<T>) * nModels));
  EMCG_CUDA(cudaMemcpy(b->dModels, mk.data(), sizeof(ModelK<T>) * nModels,
                       cudaMemcpyHostToDevice));
  std::vector<EnsK<T>> ek(nEns);
  for (int e = 0; e < nEns; e++)
    buildEnsK<T>(ens[e], mk[ens[e].model], models[ens[e].model], b->begin[e], 0, ek[e]);
  EMCG_CUDA(cudaMalloc(&b->dEns, sizeof(EnsK<T>) * nEns));
  EMCG_CUDA(cudaMemcpy(b->dEns, ek.data(), sizeof(EnsK<T>) * nEns, cudaMemcpyHostToDevice));
  return EMCG_OK;
}

static int32_t ensureTiles(BulkImpl *b) {
  if (!b->tilesDirty)
    return EMCG_OK;
  std::vector<Tile> t;
  for (int e = 0; e < b->nEns; e++) {
    for (int64_t o = 0; o < b->count[e]; o += b->blockThreads) {
      Tile x;
      x.ens = e;
      x.pad_ = 0;
      x.begin = b->begin[e] + o;
      x.end = b->begin[e] + std::min<int64_t>(o + b->blockThreads, b->count[e]);
      t.push_back(x);
    }
  }
  if ((int)t.size() > b->tilesCap) {
    cudaFree(b->dTiles);
    b->dTiles = nullptr;
    b->tilesCap = std::max<int>((int)t.size(), 1);
    EMCG_CUDA(cudaMalloc(&b->dTiles, sizeof(Tile) * b->tilesCap));
  }
  if (!t.empty())
    EMCG_CUDA(cudaMemcpyAsync(b->dTiles, t.data(), sizeof(Tile) * t.size(),
                              cudaMemcpyHostToDevice, b->stream));
  EMCG_CUDA(cudaStreamSynchronize(b->stream));
  b->nTiles = (int)t.size();
  b->tilesDirty = false;
  return EMCG_OK;
}

// The error word already copied to hErr (the stream synchronised since).
static int32_t takeError(BulkImpl *b) {
  const int e = *b->hErr;
  if (e) {
    *b->hErr = 0;
    EMCG_CUDA(cudaMemsetAsync(b->dErr, 0, sizeof(int), b->stream));
    setError("bulk kernel reported: %s", statusName(e));
    return e;
  }
  return EMCG_OK;
}

static int32_t readError(BulkImpl *b) {
  EMCG_CUDA(cudaMemcpyAsync(b->hErr, b->dErr, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
  EMCG_CUDA(cudaStreamSynchronize(b->stream));
  return takeError(b);
}

static void dropGraph(BulkImpl *b) {
  if (b->gexec)
    cudaGraphExecDestroy(b->gexec);
  if (b->graph)
    cudaGraphDestroy(b->graph);
  b->gexec = nullptr;
  b->graph = nullptr;
  b->gKernel = nullptr;
  b->gNs = -1;
}

// The observable buffers (device sums and their page-locked readback) for at
// least need doubles.
static int32_t growObs(BulkImpl *b, size_t need) {
  if (need <= b->obsCap)
    return EMCG_OK;
  EMCG_CUDA(cudaStreamSynchronize(b->stream));
  dropGraph(b); // it holds the old buffer
  cudaFree(b->dObs);
  cudaFreeHost(b->hObs);
  b->dObs = nullptr;
  b->hObs = nullptr;
  b->obsCap = 0;
  EMCG_CUDA(cudaMalloc(&b->dObs, need * sizeof(double)));
  EMCG_CUDA(cudaHostAlloc(&b->hObs, need * sizeof(double), cudaHostAllocDefault));
  b->obsCap = need;
  return EMCG_OK;
}

// the step kernel of the current launch configuration (Philox streams)
template <class T> static void *stepKernelFn(const BulkImpl *b, bool *queued) {
  *queued = b->queued != 0;
  if constexpr (sizeof(T) == 4) {
    if (b->queued == 2) {
      const bool one = b->nVmax == 1;
      if (b->minBlocks >= 4 && b->blockThreads <= 256)
        return (void *)asyncKernel<4>(one, b->anyGrain);
      if (b->minBlocks == 3 && b->blockThreads <= 256)
        return (void *)asyncKernel<3>(one, b->anyGrain);
      return (void *)asyncKernel<1>(one, b->anyGrain);
    }
  }
  if (b->queued) {
    if (b->minBlocks >= 4 && b->blockThreads <= 256)
      return (void *)bulkStepQueuedKernel<T, 4>;
    if (b->minBlocks == 3 && b->blockThreads <= 256)
      return (void *)bulkStepQueuedKernel<T, 3>;
    return (void *)bulkStepQueuedKernel<T, 1>;
  }
  if (b->minBlocks >= 4 && b->blockThreads <= 256)
    return (void *)bulkStepKernel<T, false, 4>;
  if (b->minBlocks == 3 && b->blockThreads <= 256)
    return (void *)bulkStepKernel<T, false, 3>;
  return (void *)bulkStepKernel<T, false, 1>;
}

// (Re)build the graph of one launch of ns steps for the current configuration.
template <class T> static int32_t graphFor(BulkImpl *b, int ns, size_t smem, size_t qsmem) {
  if (b->gexec && b->gNs == ns && b->gBlock == b->blockThreads && b->gMinb == b->minBlocks &&
      b->gQueued == b->queued && b->gTiles == b->nTiles && b->gPass == b->passActions)
    return EMCG_OK;
  dropGraph(b);
  static_assert(sizeof(StepArgs<T>) <= sizeof(b->gArgs), "step arguments exceed the buffer");
  StepArgs<T> &a = *reinterpret_cast<StepArgs<T> *>(b->gArgs);
  a.st = stateOf<T>(b);
  a.src = a.st;
  a.srcEns = -1;
  a.mp = (const ModelK<T> *)b->dModels;
  a.ep = (const EnsK<T> *)b->dEns;
  a.tiles = b->dTiles;
  a.ns = ns;
  a.step0 = 0;
  a.chunk = b->chunk;
  a.nVmax = b->nVmax;
  a.pass = b->passActions;
  a.obs = b->dObs;
  a.words = nullptr;
  a.off = nullptr;
  a.err = b->dErr;
  bool queued = false;
  void *fn = stepKernelFn<T>(b, &queued);
  void *lock[12] = {&a.st,    &a.mp,   &a.ep,  &a.tiles, &a.ns,    &a.step0,
                    &a.chunk, &a.nVmax, &a.obs, &a.words, &a.off, &a.err};
  void *que[10] = {&a.st, &a.mp, &a.ep, &a.tiles, &a.ns, &a.step0, &a.chunk, &a.nVmax, &a.obs,
                   &a.err};
  void *asy[13] = {&a.st,   &a.src,   &a.srcEns, &a.mp,   &a.ep,  &a.tiles, &a.ns,
                   &a.step0, &a.chunk, &a.nVmax,  &a.pass, &a.obs, &a.err};
  static_assert(sizeof(asy) <= sizeof(b->gParams), "kernel parameters exceed the buffer");
  if (b->queued == 2 && sizeof(T) == 4)
    std::memcpy(b->gParams, asy, sizeof(asy));
  else if (queued)
    std::memcpy(b->gParams, que, sizeof(que));
  else
    std::memcpy(b->gParams, lock, sizeof(lock));
  const int Q = b->nVmax * 3;
  const size_t obsBytes = (size_t)b->nEns * ns * Q * sizeof(double);
  EMCG_CUDA(cudaGraphCreate(&b->graph, 0));
  cudaMemsetParams mp = {};
  mp.dst = b->dObs;
  mp.value = 0;
  mp.elementSize = 4;
  mp.width = obsBytes / 4;
  mp.height = 1;
  mp.pitch = 0;
  cudaGraphNode_t mn;
  EMCG_CUDA(cudaGraphAddMemsetNode(&mn, b->graph, nullptr, 0, &mp));
  cudaKernelNodeParams &kp = b->gKp;
  kp = {};
  kp.func = fn;
  kp.gridDim = dim3(b->nTiles, 1, 1);
  kp.blockDim = dim3(b->blockThreads, 1, 1);
  kp.sharedMemBytes = (unsigned)(b->queued == 2 && sizeof(T) == 4
                                      ? asyncSmemBytes(b->blockThreads / 32, ns, b->nVmax * 3)
                                      : (queued ? qsmem : smem));
  kp.kernelParams = b->gParams;
  if (kp.sharedMemBytes > 48 * 1024) // above the default needs the kernel's opt-in
    EMCG_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)kp.sharedMemBytes));
  EMCG_CUDA(cudaGraphAddKernelNode(&b->gKernel, b->graph, &mn, 1, &kp));
  EMCG_CUDA(cudaGraphInstantiate(&b->gexec, b->graph, 0));
  b->gNs = ns;
  b->gBlock = b->blockThreads;
  b->gMinb = b->minBlocks;
  b->gQueued = b->queued;
  b->gPass = b->passActions;
  b->gTiles = b->nTiles;
  return EMCG_OK;
}

// Grow a device buffer of doubles to n (after draining the stream).
static int32_t growDoubles(BulkImpl *b, double **p, int64_t *cap, int64_t n) {
  if (*cap >= n)
    return EMCG_OK;
  EMCG_CUDA(cudaStreamSynchronize(b->stream));
  cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  EMCG_CUDA(cudaMalloc(p, (size_t)std::max<int64_t>(n, 1) * sizeof(double)));
  *cap = n;
  return EMCG_OK;
}

// reference constants (include/emcConstants.hpp:9, 21, 27)
constexpr double kCoulombKe = 1. / (4 * 3.14159265358979323846 * 8.85419e-12);

// Steps with particle-particle Coulomb forces, one per launch.
template <class T>
static int32_t coulombStepTyped(BulkImpl *b, int nSteps, uint32_t step0, double *obsHost) {
  EMCG_TRY(ensureTiles(b));
  const int Q = b->nVmax * 3;
  if (!b->sms) {
    int dev = 0;
    EMCG_CUDA(cudaGetDevice(&dev));
    EMCG_CUDA(cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev));
  }
  int64_t srcNeed = 1, partNeed = 1;
  for (int e = 0; e < b->nEns; e++) {
    const int64_t n = b->count[e], m = n + b->nFixed[e];
    srcNeed = std::max(srcNeed, 4 * m);
    partNeed = std::max(partNeed, 4 * n * (int64_t)p2pChunks(std::max<int64_t>(n, 1), b->sms));
  }
  EMCG_TRY(growDoubles(b, &b->dSrc, &b->srcCap, srcNeed));
  EMCG_TRY(growDoubles(b, &b->dPart, &b->partCap, partNeed));
  if (!b->dCoulF) {
    EMCG_CUDA(cudaMalloc(&b->dCoulF, (size_t)std::max<int64_t>(b->totalCap, 1) * 4 *
                                         sizeof(double)));
    EMCG_CUDA(cudaMemsetAsync(b->dCoulF, 0, (size_t)std::max<int64_t>(b->totalCap, 1) * 4 *
                                                 sizeof(double), b->stream));
  }
  EMCG_TRY(growObs(b, (size_t)b->nEns * Q));
  StateK<T> st = stateOf<T>(b);
  const T coulFactor = (T)(-kCoulombKe / b->coulEpsR);
  EMCG_CUDA(cudaEventRecord(b->ev0, b->stream));
  for (int s = 0; s < nSteps; s++) {
    EMCG_CUDA(cudaMemsetAsync(b->dObs, 0, (size_t)b->nEns * Q * sizeof(double), b->stream));
    for (int e = 0; e < b->nEns; e++) {
      const int64_t n = b->count[e], nf = b->nFixed[e], m = n + nf;
      if (n == 0)
        continue;
      coulombGatherKernel<T><<<(unsigned)((m + 255) / 256), 256, 0, b->stream>>>(
          st, b->begin[e], n, b->ens[e].charge, b->dFixed[e], nf, b->dSrc);
      EMCG_CUDA(cudaGetLastError());
      EMCG_CUDA(p2pLaunch<T>(b->dSrc, b->dSrc + m, b->dSrc + 2 * m, b->dSrc + 3 * m, m, n,
                             b->coulInvCut, b->ens[e].box[0], b->coulImages,
                             p2pChunks(n, b->sms), b->dPart, b->dCoulF + b->begin[e],
                             b->totalCap, b->stream));
    }
    if (b->nTiles > 0) {
      bulkForceStepKernel<T><<<b->nTiles, b->blockThreads, 0, b->stream>>>(
          st, (const ModelK<T> *)b->dModels, (const EnsK<T> *)b->dEns, b->dTiles,
          step0 + (uint32_t)s, b->nVmax, b->dCoulF, b->totalCap, coulFactor, b->dObs, b->dErr);
      EMCG_CUDA(cudaGetLastError());
    }
    if (obsHost)
      for (int e = 0; e < b->nEns; e++)
        EMCG_CUDA(cudaMemcpyAsync(obsHost + ((size_t)e * nSteps + s) * Q, b->dObs + (size_t)e * Q,
                                  (size_t)Q * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  }
  EMCG_CUDA(cudaEventRecord(b->ev1, b->stream));
  EMCG_CUDA(cudaEventSynchronize(b->ev1));
  float ms = 0;
  EMCG_CUDA(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
  b->lastMs = ms;
  return readError(b);
}

// Launches of the warp-asynchronous kernel shorter than this run in 128-thread
// blocks when the block size is automatic.  A block keeps its SM resources
// until its slowest warp ends, and over few steps the warps of a block end far
// apart: measured on 2^20 electrons, 20-step launches took 0.312 ms in blocks
// of 128 threads (0.311 in 64) against 0.334 ms in 256; 100-step launches were
// even; 500-step launches took 5.81 ms in 128 against 5.64 ms in 256.
constexpr int kShortLaunchSteps = 100;

// One launch of ns steps over the tiles [tiles, tiles + nT) (the direct form;
// graph replay builds its own node).
template <class T>
static int32_t launchStepTiles(BulkImpl *b, const StateK<T> &st, int ns, uint32_t s0,
                               const Tile *tiles, int nT, size_t smem, bool async,
                               const StateK<T> &src, int srcEns) {
  const int Q = b->nVmax * 3;
  const ModelK<T> *mp = (const ModelK<T> *)b->dModels;
  const EnsK<T> *ep = (const EnsK<T> *)b->dEns;
  if (b->replay) {
    if constexpr (sizeof(T) == 8)
      bulkStepKernel<T, true, 1><<<nT, b->blockThreads, smem, b->stream>>>(
          st, mp, ep, tiles, ns, s0, b->chunk, b->nVmax, b->dObs, b->dWords,
          b->dOff, b->dErr);
  } else if (async) {
    if constexpr (sizeof(T) == 4) {
      const size_t asmem = asyncSmemBytes(b->blockThreads / 32, ns, Q);
      if (b->minBlocks >= 4 && b->blockThreads <= 256) {
        EMCG_TRY(asyncSmemOptIn<4>(asmem));
        asyncKernel<4>(b->nVmax == 1, b->anyGrain)<<<nT, b->blockThreads, asmem, b->stream>>>(
            st, src, srcEns, mp, ep, tiles, ns, s0, b->chunk, b->nVmax, b->passActions,
            b->dObs, b->dErr);
      } else if (b->minBlocks == 3 && b->blockThreads <= 256) {
        EMCG_TRY(asyncSmemOptIn<3>(asmem));
        asyncKernel<3>(b->nVmax == 1, b->anyGrain)<<<nT, b->blockThreads, asmem, b->stream>>>(
            st, src, srcEns, mp, ep, tiles, ns, s0, b->chunk, b->nVmax, b->passActions,
            b->dObs, b->dErr);
      } else {
        EMCG_TRY(asyncSmemOptIn<1>(asmem));
        asyncKernel<1>(b->nVmax == 1, b->anyGrain)<<<nT, b->blockThreads, asmem, b->stream>>>(
            st, src, srcEns, mp, ep, tiles, ns, s0, b->chunk, b->nVmax, b->passActions,
            b->dObs, b->dErr);
      }
    }
  } else if (b->queued) {
    const size_t qsmem = ((smem + 15) & ~size_t(15)) + blockStateBytes<T>(b->blockThreads);
    if (b->minBlocks >= 4 && b->blockThreads <= 256)
      bulkStepQueuedKernel<T, 4><<<nT, b->blockThreads, qsmem, b->stream>>>(
          st, mp, ep, tiles, ns, s0, b->chunk, b->nVmax, b->dObs, b->dErr);
    else if (b->minBlocks == 3 && b->blockThreads <= 256)
      bulkStepQueuedKernel<T, 3><<<nT, b->blockThreads, qsmem, b->stream>>>(
          st, mp, ep, tiles, ns, s0, b->chunk, b->nVmax, b->dObs, b->dErr);
    else
      bulkStepQueuedKernel<T, 1><<<nT, b->blockThreads, qsmem, b->stream>>>(
          st, mp, ep, tiles, ns, s0, b->chunk, b->nVmax, b->dObs, b->dErr);
  } else if (b->minBlocks >= 4 && b->blockThreads <= 256) {
    bulkStepKernel<T, false, 4><<<nT, b->blockThreads, smem, b->stream>>>(
        st, mp, ep, tiles, ns, s0, b->chunk, b->nVmax, b->dObs, nullptr,
        nullptr, b->dErr);
  } else if (b->minBlocks == 3 && b->blockThreads <= 256) {
    bulkStepKernel<T, false, 3><<<nT, b->blockThreads, smem, b->stream>>>(
        st, mp, ep, tiles, ns, s0, b->chunk, b->nVmax, b->dObs, nullptr,
        nullptr, b->dErr);
  } else {
    bulkStepKernel<T, false, 1><<<nT, b->blockThreads, smem, b->stream>>>(
        st, mp, ep, tiles, ns, s0, b->chunk, b->nVmax, b->dObs, nullptr,
        nullptr, b->dErr);
  }
  EMCG_CUDA(cudaGetLastError());
  return EMCG_OK;
}

// src/srcEns: the first launch reads ensemble srcEns's start state from src
// (the warp-asynchronous kernel only; nullptr: the device state)
template <class T>
static int32_t stepTyped(BulkImpl *b, int nSteps, uint32_t step0, double *obsHost,
                         const StateK<T> *src = nullptr, int srcEns = -1) {
  if (b->coulomb) // set_coulomb and set_replay exclude each other
    return coulombStepTyped<T>(b, nSteps, step0, obsHost);
  if (b->autoBlock) {
    const bool asyncK = b->queued == 2 && sizeof(T) == 4 && !b->replay;
    const int first = std::min(b->stepsPerLaunch > 0 ? b->stepsPerLaunch : nSteps, nSteps);
    const int want = asyncK && first < kShortLaunchSteps ? 128 : 256;
    if (want != b->blockThreads) {
      b->blockThreads = want;
      b->tilesDirty = true;
    }
  }
  if (b->passAuto) {
    const int first = std::min(b->stepsPerLaunch > 0 ? b->stepsPerLaunch : nSteps, nSteps);
    b->passActions = first < kShortLaunchSteps ? kPassActionsShort : kPassActions;
  }
  EMCG_TRY(ensureTiles(b));
  const int Q = b->nVmax * 3;
  int per = b->stepsPerLaunch > 0 ? b->stepsPerLaunch : nSteps;
  if (b->replay)
    per = 1;
  const bool async = b->queued == 2 && sizeof(T) == 4 && !b->replay;
  if (async) // the block's step sums live in shared memory
    per = std::min(per, asyncMaxSteps(b->blockThreads / 32, Q));
  EMCG_TRY(growObs(b, (size_t)b->nEns * per * Q));
  const int nWarps = b->blockThreads / 32;
  const size_t smem = (size_t)b->chunk * nWarps * Q * sizeof(T);
  StateK<T> st = stateOf<T>(b);
  double totalMs = 0;
  const bool graph = b->useGraph && !b->replay && b->nTiles > 0;
  for (int done = 0; done < nSteps; done += per) {
    int ns = std::min(per, nSteps - done);
    const bool fromSrc = done == 0 && src != nullptr;
    if (graph && !fromSrc) {
      const size_t qsmem = ((smem + 15) & ~size_t(15)) + blockStateBytes<T>(b->blockThreads);
      EMCG_TRY(graphFor<T>(b, ns, smem, qsmem));
      reinterpret_cast<StepArgs<T> *>(b->gArgs)->step0 = step0 + done;
      EMCG_CUDA(cudaGraphExecKernelNodeSetParams(b->gexec, b->gKernel, &b->gKp));
      EMCG_CUDA(cudaEventRecord(b->ev0, b->stream));
      EMCG_CUDA(cudaGraphLaunch(b->gexec, b->stream));
    } else {
      EMCG_CUDA(cudaMemsetAsync(b->dObs, 0, (size_t)b->nEns * ns * Q * sizeof(double), b->stream));
      EMCG_CUDA(cudaEventRecord(b->ev0, b->stream));
      if (b->nTiles > 0)
        EMCG_TRY(launchStepTiles<T>(b, st, ns, step0 + done, b->dTiles, b->nTiles, smem, async,
                                    fromSrc ? *src : st, fromSrc ? srcEns : -1));
    }
    EMCG_CUDA(cudaEventRecord(b->ev1, b->stream));
    // the launch's sums and, after the last, the error word: one page-locked
    // readback and one synchronisation per launch
    const size_t nObs = (size_t)b->nEns * ns * Q;
    if (obsHost)
      EMCG_CUDA(cudaMemcpyAsync(b->hObs, b->dObs, nObs * sizeof(double), cudaMemcpyDeviceToHost,
                                b->stream));
    if (done + ns >= nSteps)
      EMCG_CUDA(cudaMemcpyAsync(b->hErr, b->dErr, sizeof(int), cudaMemcpyDeviceToHost,
                                b->stream));
    EMCG_CUDA(cudaStreamSynchronize(b->stream));
    float ms = 0;
    EMCG_CUDA(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
    totalMs += ms;
    if (obsHost) // gather [ens][ns][Q] of this launch into [ens][nSteps][Q]
      for (int e = 0; e < b->nEns; e++)
        std::memcpy(obsHost + ((size_t)e * nSteps + done) * Q, b->hObs + (size_t)e * ns * Q,
                    (size_t)ns * Q * sizeof(double));
  }
  b->lastMs = totalMs;
  if (b->replay)
    b->replay = false;
  return takeError(b);
}

static void freeBulk(BulkImpl *b) {
  if (!b)
    return;
  if (b->stream)
    cudaStreamSynchronize(b->stream);
  for (void *p : b->dTables)
    cudaFree(p);
  cudaFree(b->dModels);
  cudaFree(b->dEns);
  cudaFree(b->dTiles);
  for (void *p : b->dState)
    cudaFree(p);
  cudaFree(b->dMeta);
  cudaFree(b->dObs);
  cudaFreeHost(b->hObs);
  cudaFree(b->dErr);
  cudaFreeHost(b->hErr);
  cudaFree(b->dWords);
  cudaFree(b->dOff);
  freeRateScratch(b->rateScratch);
  cudaFree(b->dStage);
  cudaFree(b->dBad);
  for (double *p : b->dFixed)
    cudaFree(p);
  cudaFree(b->dSrc);
  cudaFree(b->dPart);
  cudaFree(b->dCoulF);
  dropGraph(b);
  if (b->ev0)
    cudaEventDestroy(b->ev0);
  if (b->ev1)
    cudaEventDestroy(b->ev1);
  if (b->stream)
    cudaStreamDestroy(b->stream);
  delete b;
}

static int32_t bulkOf(emcg_handle *h, BulkImpl **out) {
  EMCG_CHECK_ARG(h && h->kind == 1 && h->bulk, "handle is not a bulk engine");
  *out = h->bulk;
  return EMCG_OK;
}

int32_t bulkUpdateRates(emcg_handle *h, int model, const double *raw, bool onDevice) {
  BulkImpl *b;
  EMCG_TRY(bulkOf(h, &b));
  EMCG_CHECK_ARG(model >= 0 && model < b->nModels, "model %d out of range", model);
  const size_t mb = b->precision == EMCG_FP64 ? sizeof(ModelK<double>) : sizeof(ModelK<float>);
  void *dm = (char *)b->dModels + (size_t)model * mb;
  if (b->precision == EMCG_FP64)
    return launchRateUpdate<double>(dm, b->dTables[model], b->rates[model], raw, onDevice,
                                    b->rateScratch, b->dErr, b->stream);
  return launchRateUpdate<float>(dm, b->dTables[model], b->rates[model], raw, onDevice,
                                 b->rateScratch, b->dErr, b->stream);
}

int32_t bulkGetRates(emcg_handle *h, int model, double *tables, double *tau) {
  BulkImpl *b;
  EMCG_TRY(bulkOf(h, &b));
  EMCG_CHECK_ARG(model >= 0 && model < b->nModels, "model %d out of range", model);
  const size_t mb = b->precision == EMCG_FP64 ? sizeof(ModelK<double>) : sizeof(ModelK<float>);
  const void *dm = (const char *)b->dModels + (size_t)model * mb;
  EMCG_TRY(b->precision == EMCG_FP64
               ? readRateTables<double>(dm, b->dTables[model], b->rates[model], tables, tau,
                                        b->stream)
               : readRateTables<float>(dm, b->dTables[model], b->rates[model], tables, tau,
                                       b->stream));
  return readError(b);
}

} // namespace emcg

using namespace emcg;

extern "C" int32_t emcg_bulk_create(const emcg_model_desc *models, int32_t n_models,
                                    const emcg_ensemble_desc *ens, int32_t n_ens,
                                    int32_t precision, emcg_handle **out) {
  EMCG_CHECK_ARG(out, "out is NULL");
  *out = nullptr;
  EMCG_CHECK_ARG(models && n_models >= 1, "need at least one model");
  EMCG_CHECK_ARG(ens && n_ens >= 1, "need at least one ensemble");
  EMCG_CHECK_ARG(precision == EMCG_FP64 || precision == EMCG_FP32, "bad precision %d",
                 precision);
  for (int e = 0; e < n_ens; e++) {
    const emcg_ensemble_desc &d = ens[e];
    EMCG_CHECK_ARG(d.model >= 0 && d.model < n_models, "ensemble %d: bad model index", e);
    EMCG_CHECK_ARG(d.capacity >= 0 && d.capacity < (int64_t(1) << 32),
                   "ensemble %d: capacity out of range", e);
    EMCG_CHECK_ARG(d.dt > 0 && std::isfinite(d.dt), "ensemble %d: dt must be positive", e);
    for (int i = 0; i < 3; i++)
      EMCG_CHECK_ARG(d.box[i] > 0 && std::isfinite(d.field[i]), "ensemble %d: bad box/field", e);
  }
  BulkImpl *b = new BulkImpl();
  b->precision = precision;
  // defaults measured on GB300: the float engine runs the warp-asynchronous
  // kernel with a 4-blocks-per-SM register cap, the double engine the
  // lockstep kernel without a cap
  b->queued = precision == EMCG_FP32 ? 2 : 0;
  b->minBlocks = precision == EMCG_FP32 ? 4 : 1;
  b->tsz = precision == EMCG_FP64 ? 8 : 4;
  b->nModels = n_models;
  b->nEns = n_ens;
  b->ens.assign(ens, ens + n_ens);
  b->valleyCopies.resize(n_models);
  for (int i = 0; i < n_models; i++) {
    b->valleyCopies[i].assign(models[i].valleys, models[i].valleys + models[i].n_valleys);
    emcg_model_desc md = models[i];
    md.valleys = b->valleyCopies[i].data();
    md.mechs = nullptr;
    md.tablesets = nullptr;
    md.tables = nullptr;
    b->modelDescs.push_back(md);
    b->anyGrain = b->anyGrain || md.grain != 0;
  }
  b->begin.resize(n_ens);
  b->count.assign(n_ens, 0);
  b->cap.resize(n_ens);
  b->ensNV.resize(n_ens);
  b->nFixed.assign(n_ens, 0);
  b->dFixed.assign(n_ens, nullptr);
  int64_t off = 0;
  for (int e = 0; e < n_ens; e++) {
    b->begin[e] = off;
    b->cap[e] = ens[e].capacity;
    off += ens[e].capacity;
    b->ensNV[e] = models[ens[e].model].n_valleys;
    b->nVmax = std::max(b->nVmax, models[ens[e].model].n_valleys);
  }
  b->totalCap = off;
  auto fail = [&](int32_t s) {
    freeBulk(b);
    return s;
  };
  int32_t s = precision == EMCG_FP64
                  ? createTyped<double>(b, models, n_models, ens, n_ens)
                  : createTyped<float>(b, models, n_models, ens, n_ens);
  if (s)
    return fail(s);
  size_t n = (size_t)std::max<int64_t>(off, 1);
  for (int i = 0; i < 9; i++)
    if (cudaMalloc(&b->dState[i], n * b->tsz) != cudaSuccess) {
      setError("cudaMalloc of particle state (%zu slots) failed", n);
      return fail(EMCG_ERR_CUDA);
    }
  if (cudaMalloc(&b->dMeta, n * sizeof(uint32_t)) != cudaSuccess ||
      cudaMalloc(&b->dErr, sizeof(int)) != cudaSuccess ||
      cudaMemset(b->dErr, 0, sizeof(int)) != cudaSuccess ||
      cudaHostAlloc(&b->hErr, sizeof(int), cudaHostAllocDefault) != cudaSuccess ||
      cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&b->ev0) != cudaSuccess || cudaEventCreate(&b->ev1) != cudaSuccess) {
    setError("CUDA allocation failed: %s", cudaGetErrorString(cudaGetLastError()));
    return fail(EMCG_ERR_CUDA);
  }
  *b->hErr = 0;
  emcg_handle *h = new emcg_handle();
  h->kind = 1;
  h->bulk = b;
  *out = h;
  return EMCG_OK;
}

extern "C" int32_t emcg_destroy(emcg_handle *h) {
  if (!h)
    return EMCG_OK;
  if (h->kind == 1)
    freeBulk(h->bulk);
  if (h->kind == 2)
    emcg::destroyDevice(h);
  delete h;
  return EMCG_OK;
}

extern "C" int64_t emcg_num_particles(emcg_handle *h, int32_t e) {
  if (h && h->kind == 2)
    return e == 0 ? emcg::deviceNumParticles(h) : -1;
  BulkImpl *b = nullptr;
  if (bulkOf(h, &b) || e < 0 || e >= b->nEns)
    return -1;
  return b->count[e];
}

// Upload check: the first particle whose valley, subvalley or region is out
// of range (the caller's int32 indices, copied to the device as they are).
__global__ void stateCheckKernel(int64_t n, const int32_t *__restrict__ idx, int nValleys,
                                 unsigned long long *__restrict__ bad) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  const int32_t v = idx[i], sb = idx[n + i], r = idx[2 * n + i];
  if (v < 0 || v >= nValleys || sb < 0 || sb >= EMCG_MAX_DEG || r < 0 || r >= EMCG_MAX_REGIONS)
    atomicMin(bad, (unsigned long long)i);
}

// Upload conversion into the engine's precision and packed meta; nothing is
// written if the check found a bad particle, so the old state stays.
template <class T>
__global__ void stateConvertKernel(StateK<T> st, int64_t base, int64_t n,
                                   const double *__restrict__ src,
                                   const int32_t *__restrict__ idx,
                                   const unsigned long long *__restrict__ bad) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || *bad != ~0ull)
    return;
  T *dst[9] = {st.kx, st.ky, st.kz, st.px, st.py, st.pz, st.E, st.tau, st.gtau};
#pragma unroll
  for (int f = 0; f < 9; f++)
    dst[f][base + i] = (T)src[(size_t)f * n + i];
  st.meta[base + i] = packMeta(idx[i], idx[n + i], idx[2 * n + i]);
}

// Upload a host state: one asynchronous copy per field of the caller's arrays
// into device staging (at the full host link rate when the caller's memory is
// pinned), then one conversion kernel.
template <class T>
static int32_t setStateTyped(BulkImpl *b, int e, const emcg_state *s) {
  const int64_t n = s->n, base = b->begin[e];
  const double *src[9] = {s->kx, s->ky, s->kz, s->px, s->py, s->pz, s->energy, s->tau,
                          s->grain_tau};
  for (int f = 0; f < 9; f++)
    EMCG_CHECK_ARG(src[f] != nullptr, "state field %d is NULL", f);
  EMCG_CHECK_ARG(s->valley && s->sub && s->region, "state index arrays are NULL");
  if (n == 0)
    return EMCG_OK;
  const size_t need = (size_t)n * (9 * sizeof(double) + 3 * sizeof(int32_t));
  if (b->stageBytes < need) {
    EMCG_CUDA(cudaStreamSynchronize(b->stream)); // an earlier upload may still read it
    cudaFree(b->dStage);
    b->dStage = nullptr;
    b->stageBytes = 0;
    EMCG_CUDA(cudaMalloc(&b->dStage, need));
    b->stageBytes = need;
  }
  if (!b->dBad)
    EMCG_CUDA(cudaMalloc(&b->dBad, sizeof(unsigned long long)));
  double *dsrc = static_cast<double *>(b->dStage);
  int32_t *didx = reinterpret_cast<int32_t *>(dsrc + (size_t)9 * n);
  for (int f = 0; f < 9; f++)
    EMCG_CUDA(cudaMemcpyAsync(dsrc + (size_t)f * n, src[f], n * sizeof(double),
                              cudaMemcpyHostToDevice, b->stream));
  const int32_t *isrc[3] = {s->valley, s->sub, s->region};
  for (int f = 0; f < 3; f++)
    EMCG_CUDA(cudaMemcpyAsync(didx + (size_t)f * n, isrc[f], n * sizeof(int32_t),
                              cudaMemcpyHostToDevice, b->stream));
  EMCG_CUDA(cudaMemsetAsync(b->dBad, 0xff, sizeof(unsigned long long), b->stream));
  const unsigned grid = (unsigned)((n + 255) / 256);
  stateCheckKernel<<<grid, 256, 0, b->stream>>>(n, didx, b->ensNV[e], b->dBad);
  stateConvertKernel<T><<<grid, 256, 0, b->stream>>>(stateOf<T>(b), base, n, dsrc, didx, b->dBad);
  EMCG_CUDA(cudaGetLastError());
  unsigned long long bad = 0;
  EMCG_CUDA(cudaMemcpyAsync(&bad, b->dBad, sizeof(bad), cudaMemcpyDeviceToHost, b->stream));
  EMCG_CUDA(cudaStreamSynchronize(b->stream));
  EMCG_CHECK_ARG(bad == ~0ull, "particle %llu: valley/sub/region out of range", bad);
  return EMCG_OK;
}

// The float layout: staged as it is, meta checked on the device, the fields
// and meta written (a double engine widens them) only if every particle is in
// range.
__global__ void metaCheckKernel(int64_t n, const uint32_t *__restrict__ meta, int nValleys,
                                unsigned long long *__restrict__ bad) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  const uint32_t m = meta[i];
  if ((int)(m & 0xff) >= nValleys || ((m >> 8) & 0xff) >= EMCG_MAX_DEG ||
      (m >> 16) >= EMCG_MAX_REGIONS)
    atomicMin(bad, (unsigned long long)i);
}

template <class T>
__global__ void stateConvertF32Kernel(StateK<T> st, int64_t base, int64_t n,
                                      const float *__restrict__ src,
                                      const uint32_t *__restrict__ meta,
                                      const unsigned long long *__restrict__ bad) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || *bad != ~0ull)
    return;
  T *dst[9] = {st.kx, st.ky, st.kz, st.px, st.py, st.pz, st.E, st.tau, st.gtau};
#pragma unroll
  for (int f = 0; f < 9; f++)
    dst[f][base + i] = (T)src[(size_t)f * n + i];
  st.meta[base + i] = meta[i];
}

template <class T>
static int32_t setStateF32Typed(BulkImpl *b, int e, const emcg_state_f32 *s) {
  const int64_t n = s->n, base = b->begin[e];
  const float *src[9] = {s->kx, s->ky, s->kz, s->px, s->py, s->pz, s->energy, s->tau,
                         s->grain_tau};
  for (int f = 0; f < 9; f++)
    EMCG_CHECK_ARG(src[f] != nullptr, "state field %d is NULL", f);
  EMCG_CHECK_ARG(s->meta, "state meta array is NULL");
  if (n == 0)
    return EMCG_OK;
  const size_t need = (size_t)n * (9 * sizeof(float) + sizeof(uint32_t));
  if (b->stageBytes < need) {
    EMCG_CUDA(cudaStreamSynchronize(b->stream));
    cudaFree(b->dStage);
    b->dStage = nullptr;
    b->stageBytes = 0;
    EMCG_CUDA(cudaMalloc(&b->dStage, need));
    b->stageBytes = need;
  }
  if (!b->dBad)
    EMCG_CUDA(cudaMalloc(&b->dBad, sizeof(unsigned long long)));
  float *dsrc = static_cast<float *>(b->dStage);
  uint32_t *dmeta = reinterpret_cast<uint32_t *>(dsrc + (size_t)9 * n);
  for (int f = 0; f < 9; f++)
    EMCG_CUDA(cudaMemcpyAsync(dsrc + (size_t)f * n, src[f], n * sizeof(float),
                              cudaMemcpyHostToDevice, b->stream));
  EMCG_CUDA(cudaMemcpyAsync(dmeta, s->meta, n * sizeof(uint32_t), cudaMemcpyHostToDevice,
                            b->stream));
  EMCG_CUDA(cudaMemsetAsync(b->dBad, 0xff, sizeof(unsigned long long), b->stream));
  const unsigned grid = (unsigned)((n + 255) / 256);
  metaCheckKernel<<<grid, 256, 0, b->stream>>>(n, dmeta, b->ensNV[e], b->dBad);
  stateConvertF32Kernel<T><<<grid, 256, 0, b->stream>>>(stateOf<T>(b), base, n, dsrc, dmeta,
                                                        b->dBad);
  EMCG_CUDA(cudaGetLastError());
  unsigned long long bad = 0;
  EMCG_CUDA(cudaMemcpyAsync(&bad, b->dBad, sizeof(bad), cudaMemcpyDeviceToHost, b->stream));
  EMCG_CUDA(cudaStreamSynchronize(b->stream));
  EMCG_CHECK_ARG(bad == ~0ull, "particle %llu: valley/sub/region out of range", bad);
  return EMCG_OK;
}

extern "C" int32_t emcg_set_state_f32(emcg_handle *h, int32_t e, const emcg_state_f32 *s) {
  BulkImpl *b;
  EMCG_TRY(bulkOf(h, &b));
  EMCG_CHECK_ARG(s && e >= 0 && e < b->nEns, "bad ensemble or state");
  EMCG_CHECK_ARG(s->n >= 0 && s->n <= b->cap[e], "ensemble %d: %lld particles exceed capacity %lld",
                 e, (long long)s->n, (long long)b->cap[e]);
  int32_t r = b->precision == EMCG_FP64 ? setStateF32Typed<double>(b, e, s)
                                        : setStateF32Typed<float>(b, e, s);
  if (r)
    return r;
  b->count[e] = s->n;
  b->tilesDirty = true;
  return EMCG_OK;
}

extern "C" int32_t emcg_bulk_step_from_host(emcg_handle *h, int32_t e, const emcg_state_f32 *s,
                                            int32_t n_steps, uint32_t step0, double *obs) {
  BulkImpl *b;
  EMCG_TRY(bulkOf(h, &b));
  EMCG_CHECK_ARG(s && e >= 0 && e < b->nEns, "bad ensemble or state");
  EMCG_CHECK_ARG(n_steps >= 0, "n_steps must be >= 0");
  EMCG_CHECK_ARG(s->n >= 0 && s->n <= b->cap[e], "ensemble %d: %lld particles exceed capacity %lld",
                 e, (long long)s->n, (long long)b->cap[e]);
  const float *f[9] = {s->kx, s->ky, s->kz, s->px, s->py, s->pz, s->energy, s->tau, s->grain_tau};
  for (int i = 0; i < 9; i++)
    EMCG_CHECK_ARG(f[i] != nullptr, "state field %d is NULL", i);
  EMCG_CHECK_ARG(s->meta, "state meta array is NULL");
  // The fused form: a float engine stepping with the warp-asynchronous kernel
  // reads the start state straight from emcg_host_alloc blocks.
  StateK<float> src{};
  bool fused = b->precision == EMCG_FP32 && b->queued == 2 && !b->replay && !b->coulomb &&
               n_steps > 0 && s->n > 0;
  const int64_t n = s->n, base = b->begin[e];
  if (fused) {
    float **d[9] = {&src.kx, &src.ky, &src.kz, &src.px, &src.py, &src.pz, &src.E, &src.tau,
                    &src.gtau};
    for (int i = 0; i < 9 && fused; i++) {
      const void *p = reinterpret_cast<uintptr_t>(f[i]) % alignof(float) == 0
                          ? mappedHostRange(f[i], (size_t)n * sizeof(float))
                          : nullptr;
      fused = p != nullptr;
      // indexed by the particle's place in the handle's arrays (base + i)
      *d[i] = const_cast<float *>(static_cast<const float *>(p)) - base;
    }
    const void *m = reinterpret_cast<uintptr_t>(s->meta) % alignof(uint32_t) == 0
                        ? mappedHostRange(s->meta, (size_t)n * sizeof(uint32_t))
                        : nullptr;
    fused = fused && m != nullptr;
    src.meta = const_cast<uint32_t *>(static_cast<const uint32_t *>(m)) - base;
  }
  if (!fused) {
    EMCG_TRY(emcg_set_state_f32(h, e, s));
    return emcg_bulk_step(h, n_steps, step0, obs);
  }
  if (b->count[e] != n) {
    b->count[e] = n;
    b->tilesDirty = true;
  }
  const int32_t r = stepTyped<float>(b, n_steps, step0, obs, &src, e);
  if (r == EMCG_ERR_ARG)
    setError("ensemble %d: a particle's valley, subvalley or region is out of range; "
             "its state is unspecified until set again", e);
  return r;
}

extern "C" int32_t emcg_get_state_f32(emcg_handle *h, int32_t e, emcg_state_f32 *s) {
  BulkImpl *b;
  EMCG_TRY(bulkOf(h, &b));
  EMCG_CHECK_ARG(s && e >= 0 && e < b->nEns, "bad ensemble or state");
  EMCG_CHECK_ARG(b->precision == EMCG_FP32, "a double engine's state is read with emcg_get_state");
  const int64_t n = b->count[e], base = b->begin[e];
  EMCG_CUDA(cudaStreamSynchronize(b->stream));
  float *dst[9] = {s->kx, s->ky, s->kz, s->px, s->py, s->pz, s->energy, s->tau, s->grain_tau};
  for (int f = 0; f < 9; f++)
    if (dst[f] && n)
      EMCG_CUDA(cudaMemcpyAsync(dst[f], static_cast<float *>(b->dState[f]) + base,
                                n * sizeof(float), cudaMemcpyDeviceToHost, b->stream));
  if (s->meta && n)
    EMCG_CUDA(cudaMemcpyAsync(s->meta, b->dMeta + base, n * sizeof(uint32_t),
                              cudaMemcpyDeviceToHost, b->stream));
  EMCG_CUDA(cudaStreamSynchronize(b->stream));
  s->n = n;
  return EMCG_OK;
}

extern "C" int32_t emcg_set_state(emcg_handle *h, int32_t e, const emcg_state *s) {
  if (h && h->kind == 2) {
    EMCG_CHECK_ARG(e == 0, "a device engine has one ensemble");
    return emcg::deviceSetState(h, s);
  }
  BulkImpl *b;
  EMCG_TRY(bulkOf(h, &b));
  EMCG_CHECK_ARG(s && e >= 0 && e < b->nEns, "bad ensemble or state");
  EMCG_CHECK_ARG(s->n >= 0 && s->n <= b->cap[e], "ensemble %d: %lld particles exceed capacity %lld",
                 e, (long long)s->n, (long long)b->cap[e]);
  int32_t r = b->precision == EMCG_FP64 ? setStateTyped<double>(b, e, s)
                                        : setStateTyped<float>(b, e, s);
  if (r)
    return r;
  b->count[e] = s->n;
  b->tilesDirty = true;
  return EMCG_OK;
}

template <class T> static int32_t getStateTyped(BulkImpl *b, int e, emcg_state *s) {
  const int64_t n = b->count[e], base = b->begin[e];
  double *dst[9] = {s->kx, s->ky, s->kz, s->px, s->py, s->pz, s->energy, s->tau, s->grain_tau};
  std::vector<T> tmp((size_t)std::max<int64_t>(n, 1));
  for (int f = 0; f < 9; f++) {
    if (!dst[f])
      continue;
    if (n)
      EMCG_CUDA(cudaMemcpy(tmp.data(), (T *)b->dState[f] + base, n * sizeof(T),
                           cudaMemcpyDeviceToHost));
    for (int64_t i = 0; i < n; i++)
      dst[f][i] = (double)tmp[i];
  }
  std::vector<uint32_t> meta((size_t)std::max<int64_t>(n, 1));
  if (n)
    EMCG_CUDA(cudaMemcpy(meta.data(), b->dMeta + base, n * sizeof(uint32_t),
                         cudaMemcpyDeviceToHost));
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

extern "C" int32_t emcg_get_state(emcg_handle *h, int32_t e, emcg_state *s) {
  if (h && h->kind == 2) {
    EMCG_CHECK_ARG(e == 0, "a device engine has one ensemble");
    return emcg::deviceGetState(h, s);
  }
  BulkImpl *b;
  EMCG_TRY(bulkOf(h, &b));
  EMCG_CHECK_ARG(s && e >= 0 && e < b->nEns, "bad ensemble or state");
  return b->precision == EMCG_FP64 ? getStateTyped<double>(b, e, s)
                                   : getStateTyped<float>(b, e, s);
}

extern "C" int32_t emcg_bulk_init(emcg_handle *h, int32_t e, int64_t n, const int64_t *coords,
                                  const int64_t extent[3], const double spacing[3],
                                  double thermal_voltage) {
  BulkImpl *b;
  EMCG_TRY(bulkOf(h, &b));
  EMCG_CHECK_ARG(e >= 0 && e < b->nEns, "bad ensemble %d", e);
  EMCG_CHECK_ARG(n >= 0 && n <= b->cap[e], "ensemble %d: %lld particles exceed capacity", e,
                 (long long)n);
  EMCG_CHECK_ARG(thermal_voltage > 0, "thermal voltage must be positive");
  int64_t ext[3] = {1, 1, 1};
  double hsp[3] = {1, 1, 1};
  int64_t *dC = nullptr;
  if (coords) {
    EMCG_CHECK_ARG(extent && spacing, "coords need extent and spacing");
    for (int d = 0; d < 3; d++) {
      ext[d] = extent[d];
      hsp[d] = spacing[d];
      EMCG_CHECK_ARG(ext[d] >= 1 && hsp[d] > 0, "bad extent/spacing");
    }
    for (int64_t i = 0; i < 3 * n; i++)
      EMCG_CHECK_ARG(coords[i] >= 0 && coords[i] < ext[i % 3], "coordinate out of the grid");
    if (n) {
      EMCG_CUDA(cudaMalloc(&dC, sizeof(int64_t) * 3 * n));
      EMCG_CUDA(cudaMemcpy(dC, coords, sizeof(int64_t) * 3 * n, cudaMemcpyHostToDevice));
    }
  }
  const emcg_ensemble_desc &d = b->ens[e];
  uint32_t k0 = (uint32_t)d.seed, k1 = (uint32_t)(d.seed >> 32);
  int blocks = (int)((n + 255) / 256);
  if (n) {
    if (b->precision == EMCG_FP64)
      bulkInitKernel<double><<<blocks, 256, 0, b->stream>>>(
          stateOf<double>(b), (const ModelK<double> *)b->dModels, d.model, b->begin[e], n, dC,
          ext[0], ext[1], ext[2], hsp[0], hsp[1], hsp[2], thermal_voltage, d.box[0], d.box[1],
          d.box[2], k0, k1, d.stream);
    else
      bulkInitKernel<float><<<blocks, 256, 0, b->stream>>>(
          stateOf<float>(b), (const ModelK<float> *)b->dModels, d.model, b->begin[e], n, dC,
          ext[0], ext[1], ext[2], hsp[0], hsp[1], hsp[2], thermal_voltage, d.box[0], d.box[1],
          d.box[2], k0, k1, d.stream);
    EMCG_CUDA(cudaGetLastError());
  }
  EMCG_CUDA(cudaStreamSynchronize(b->stream));
  cudaFree(dC);
  b->count[e] = n;
  b->tilesDirty = true;
  return EMCG_OK;
}

extern "C" int32_t emcg_bulk_step(emcg_handle *h, int32_t n_steps, uint32_t step0, double *obs) {
  BulkImpl *b;
  EMCG_TRY(bulkOf(h, &b));
  EMCG_CHECK_ARG(n_steps >= 0, "n_steps must be >= 0");
  if (n_steps == 0)
    return EMCG_OK;
  if (b->replay) {
    EMCG_CHECK_ARG(n_steps == 1, "replay mode advances one step per call");
    EMCG_CHECK_ARG(b->nEns == 1, "replay mode needs exactly one ensemble");
  }
  return b->precision == EMCG_FP64 ? stepTyped<double>(b, n_steps, step0, obs)
                                   : stepTyped<float>(b, n_steps, step0, obs);
}

extern "C" int32_t emcg_set_replay(emcg_handle *h, const uint64_t *words, int64_t nwords,
                                   const int64_t *offsets, int64_t n_offsets) {
  BulkImpl *b;
  EMCG_TRY(bulkOf(h, &b));
  if (!words) {
    b->replay = false;
    return EMCG_OK;
  }
  EMCG_CHECK_ARG(b->precision == EMCG_FP64, "replay needs the FP64 engine");
  EMCG_CHECK_ARG(b->nEns == 1, "replay needs exactly one ensemble");
  EMCG_CHECK_ARG(!b->coulomb, "replay does not run Coulomb steps; switch them off first");
  EMCG_CHECK_ARG(offsets && n_offsets == b->count[0] + 1,
                 "replay: need n+1 = %lld offsets, got %lld", (long long)(b->count[0] + 1),
                 (long long)n_offsets);
  EMCG_CHECK_ARG(nwords >= 0, "replay: negative word count");
  for (int64_t i = 0; i + 1 < n_offsets; i++)
    EMCG_CHECK_ARG(offsets[i] >= 0 && offsets[i] <= offsets[i + 1] && offsets[i + 1] <= nwords,
                   "replay: offsets not monotone within [0, nwords]");
  if (nwords > b->wordsCap) {
    cudaFree(b->dWords);
    b->dWords = nullptr;
    EMCG_CUDA(cudaMalloc(&b->dWords, sizeof(uint64_t) * std::max<int64_t>(nwords, 1)));
    b->wordsCap = nwords;
  }
  if (n_offsets > b->offCap) {
    cudaFree(b->dOff);
    b->dOff = nullptr;
    EMCG_CUDA(cudaMalloc(&b->dOff, sizeof(int64_t) * n_offsets));
    b->offCap = n_offsets;
  }
  if (nwords)
    EMCG_CUDA(cudaMemcpy(b->dWords, words, sizeof(uint64_t) * nwords, cudaMemcpyHostToDevice));
  EMCG_CUDA(cudaMemcpy(b->dOff, offsets, sizeof(int64_t) * n_offsets, cudaMemcpyHostToDevice));
  b->replay = true;
  return EMCG_OK;
}

extern "C" int32_t emcg_last_kernel_ms(emcg_handle *h, double *ms) {
  BulkImpl *b;
  EMCG_TRY(bulkOf(h, &b));
  EMCG_CHECK_ARG(ms, "ms is NULL");
  *ms = b->lastMs;
  return EMCG_OK;
}

extern "C" int32_t emcg_set_scatter_mode(emcg_handle *h, int32_t queued) {
  BulkImpl *b;
  EMCG_TRY(bulkOf(h, &b));
  EMCG_CHECK_ARG(queued >= 0 && queued <= 2, "scatter mode must be 0, 1 or 2");
  EMCG_CHECK_ARG(queued != 2 || b->precision == EMCG_FP32,
                 "the warp-asynchronous kernel (mode 2) is float only");
  b->queued = queued;
  return EMCG_OK;
}

extern "C" int32_t emcg_set_pass_actions(emcg_handle *h, int32_t n) {
  BulkImpl *b;
  EMCG_TRY(bulkOf(h, &b));
  EMCG_CHECK_ARG(n >= 0 && n <= kAsyncWindow, "pass actions must be in [0, %d]", kAsyncWindow);
  b->passAuto = n == 0;
  if (n > 0)
    b->passActions = n;
  return EMCG_OK;
}

extern "C" int32_t emcg_get_pass_actions(emcg_handle *h, int32_t *n) {
  BulkImpl *b;
  EMCG_TRY(bulkOf(h, &b));
  EMCG_CHECK_ARG(n, "NULL output");
  *n = b->passActions;
  return EMCG_OK;
}

extern "C" int32_t emcg_set_occupancy(emcg_handle *h, int32_t min_blocks_per_sm) {
  BulkImpl *b;
  EMCG_TRY(bulkOf(h, &b));
  EMCG_CHECK_ARG(min_blocks_per_sm == 1 || min_blocks_per_sm == 3 || min_blocks_per_sm == 4,
                 "min_blocks_per_sm must be 1, 3 or 4");
  b->minBlocks = min_blocks_per_sm;
  return EMCG_OK;
}

extern "C" int32_t emcg_set_launch(emcg_handle *h, int32_t block_threads,
                                   int32_t steps_per_launch) {
  BulkImpl *b;
  EMCG_TRY(bulkOf(h, &b));
  if (block_threads == -1) {
    b->autoBlock = true;
  } else if (block_threads) {
    EMCG_CHECK_ARG(block_threads % 32 == 0 && block_threads >= 32 && block_threads <= 1024,
                   "block_threads must be -1 or a multiple of 32 in [32, 1024]");
    if (block_threads != b->blockThreads)
      b->tilesDirty = true;
    b->blockThreads = block_threads;
    b->autoBlock = false;
  }
  if (steps_per_launch) {
    EMCG_CHECK_ARG(steps_per_launch > 0, "steps_per_launch must be positive");
    b->stepsPerLaunch = steps_per_launch;
  }
  return EMCG_OK;
}

extern "C" int32_t emcg_get_launch(emcg_handle *h, int32_t *block_threads,
                                   int32_t *steps_per_launch) {
  BulkImpl *b;
  EMCG_TRY(bulkOf(h, &b));
  if (block_threads)
    *block_threads = b->blockThreads;
  if (steps_per_launch)
    *steps_per_launch = b->stepsPerLaunch;
  return EMCG_OK;
}

extern "C" int32_t emcg_bulk_set_graph(emcg_handle *h, int32_t enable) {
  BulkImpl *b;
  EMCG_TRY(bulkOf(h, &b));
  b->useGraph = enable != 0;
  if (!b->useGraph)
    dropGraph(b);
  return EMCG_OK;
}

extern "C" int32_t emcg_bulk_set_coulomb(emcg_handle *h, int32_t enable, double eps_r,
                                         double inv_cutoff, int32_t images) {
  BulkImpl *b;
  EMCG_TRY(bulkOf(h, &b));
  if (enable) {
    EMCG_CHECK_ARG(eps_r > 0 && std::isfinite(eps_r), "eps_r must be positive");
    EMCG_CHECK_ARG(inv_cutoff >= 0 && std::isfinite(inv_cutoff), "inv_cutoff must be >= 0");
    EMCG_CHECK_ARG(images >= 0 && images <= 8, "images must be in [0, 8]");
    if (images > 0)
      for (int e = 0; e < b->nEns; e++) {
        const double *bx = b->ens[e].box;
        EMCG_CHECK_ARG(bx[0] == bx[1] && bx[1] == bx[2],
                       "ensemble %d: periodic copies need a cubic box", e);
      }
    EMCG_CHECK_ARG(!b->replay, "Coulomb steps run on Philox streams; clear replay first");
  }
  b->coulomb = enable != 0;
  b->coulEpsR = eps_r;
  b->coulInvCut = inv_cutoff;
  b->coulImages = images;
  return EMCG_OK;
}

extern "C" int32_t emcg_bulk_set_fixed_charges(emcg_handle *h, int32_t e, const double *pos,
                                               const double *q, int64_t n) {
  BulkImpl *b;
  EMCG_TRY(bulkOf(h, &b));
  EMCG_CHECK_ARG(e >= 0 && e < b->nEns, "ensemble %d out of range", e);
  EMCG_CHECK_ARG(n >= 0 && (n == 0 || (pos && q)), "bad fixed charges");
  EMCG_CUDA(cudaStreamSynchronize(b->stream));
  cudaFree(b->dFixed[e]);
  b->dFixed[e] = nullptr;
  b->nFixed[e] = 0;
  if (n == 0)
    return EMCG_OK;
  std::vector<double> planes((size_t)4 * n);
  std::memcpy(planes.data(), pos, (size_t)3 * n * sizeof(double));
  std::memcpy(planes.data() + 3 * n, q, (size_t)n * sizeof(double));
  for (double v : planes)
    EMCG_CHECK_ARG(std::isfinite(v), "fixed charges: non-finite value");
  EMCG_CUDA(cudaMalloc(&b->dFixed[e], planes.size() * sizeof(double)));
  EMCG_CUDA(cudaMemcpy(b->dFixed[e], planes.data(), planes.size() * sizeof(double),
                       cudaMemcpyHostToDevice));
  b->nFixed[e] = n;
  return EMCG_OK;
}

extern "C" int32_t emcg_bulk_get_coulomb(emcg_handle *h, int32_t e, double *force,
                                         double *potential) {
  BulkImpl *b;
  EMCG_TRY(bulkOf(h, &b));
  EMCG_CHECK_ARG(e >= 0 && e < b->nEns, "ensemble %d out of range", e);
  EMCG_CHECK_ARG(b->dCoulF, "no Coulomb step has run");
  const int64_t n = b->count[e];
  EMCG_CUDA(cudaStreamSynchronize(b->stream));
  for (int v = 0; v < 4; v++) {
    double *dst = v < 3 ? (force ? force + (size_t)v * n : nullptr) : potential;
    if (dst && n)
      EMCG_CUDA(cudaMemcpy(dst, b->dCoulF + (size_t)v * b->totalCap + b->begin[e],
                           (size_t)n * sizeof(double), cudaMemcpyDeviceToHost));
  }
  return EMCG_OK;
}

extern "C" int32_t emcg_bulk_autotune(emcg_handle *h, int32_t trial_steps, uint32_t step0,
                                      int32_t *steps_used, int32_t *block_threads,
                                      int32_t *min_blocks, int32_t *queued) {
  BulkImpl *b;
  EMCG_TRY(bulkOf(h, &b));
  EMCG_CHECK_ARG(trial_steps > 0, "trial_steps must be positive");
  EMCG_CHECK_ARG(!b->replay, "autotuning runs Philox steps; clear replay first");
  // launch shapes: block threads x register cap (resident blocks per SM) x
  // scatter scheme.  Each runs trial_steps steps (advancing the ensembles)
  // twice, once in a forward and once in a backward pass over the shapes, so
  // that the ensembles' warming up from the initial distribution (events get
  // more frequent) weighs on every shape alike; the least total device time
  // wins
  // (the warp-asynchronous kernel with 3 and with 6 free flights per pass)
  struct Cand {
    int block, minb, queued, pass;
  };
  const Cand cands[] = {{256, 4, 0, 0}, {256, 3, 0, 0}, {256, 1, 0, 0}, {128, 4, 0, 0},
                        {128, 1, 0, 0}, {256, 4, 1, 0}, {256, 3, 1, 0}, {128, 4, 1, 0},
                        {256, 4, 2, 3}, {256, 3, 2, 3}, {128, 4, 2, 3}, {256, 4, 2, 6},
                        {128, 4, 2, 6}};
  constexpr int kCands = sizeof(cands) / sizeof(cands[0]);
  const int nCands = b->precision == EMCG_FP32 ? kCands : 8; // mode 2 is float only
  const int keepPer = b->stepsPerLaunch, keepPass = b->passActions;
  const bool keepPassAuto = b->passAuto;
  b->autoBlock = false; // the tuner sets the block size
  b->passAuto = false;  // and the free flights per pass of each shape
  b->stepsPerLaunch = trial_steps;
  double ms[kCands] = {};
  uint32_t s = step0;
  for (int pass = 0; pass < 2 * nCands; pass++) {
    const int ci = pass < nCands ? pass : 2 * nCands - 1 - pass;
    const Cand &c = cands[ci];
    if (c.block != b->blockThreads)
      b->tilesDirty = true;
    b->blockThreads = c.block;
    b->minBlocks = c.minb;
    b->queued = c.queued;
    b->passActions = c.pass ? c.pass : keepPass;
    int32_t st = b->precision == EMCG_FP64 ? stepTyped<double>(b, trial_steps, s, nullptr)
                                           : stepTyped<float>(b, trial_steps, s, nullptr);
    s += trial_steps;
    if (st != EMCG_OK) {
      b->stepsPerLaunch = keepPer;
      b->passActions = keepPass;
      b->passAuto = keepPassAuto;
      return st;
    }
    ms[ci] += b->lastMs;
  }
  int bi = 0;
  for (int ci = 1; ci < nCands; ci++)
    if (ms[ci] < ms[bi])
      bi = ci;
  const Cand bestC = cands[bi];
  if (bestC.block != b->blockThreads)
    b->tilesDirty = true;
  b->blockThreads = bestC.block;
  b->minBlocks = bestC.minb;
  b->queued = bestC.queued;
  b->passActions = bestC.pass ? bestC.pass : keepPass;
  b->passAuto = bestC.pass ? false : keepPassAuto;
  b->stepsPerLaunch = keepPer;
  if (steps_used)
    *steps_used = (int32_t)(s - step0);
  if (block_threads)
    *block_threads = bestC.block;
  if (min_blocks)
    *min_blocks = bestC.minb;
  if (queued)
    *queued = bestC.queued;
  return EMCG_OK;
}

// grainScatter (emcGrainScatterMechanism::scatterParticle) of model 0 for n
// independent wave vectors (known-answer tests of the reference)
template <class T>
__global__ void grainKatKernel(const ModelK<T> *__restrict__ models, int64_t n,
                               double *__restrict__ k, uint32_t step) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  PhiloxSrc<T> rng;
  rng.init((uint32_t)i, step, 0x47524149u, 0x5eedu, 0u);
  T kk[3] = {(T)k[i], (T)k[n + i], (T)k[2 * n + i]};
  grainScatter(models[0], kk, rng);
  for (int j = 0; j < 3; j++)
    k[j * n + i] = (double)kk[j];
}

extern "C" int32_t emcg_grain_kat(emcg_handle *h, int64_t n, double *k, uint32_t step) {
  BulkImpl *b;
  EMCG_TRY(bulkOf(h, &b));
  EMCG_CHECK_ARG(n >= 0 && k, "bad grain arguments");
  EMCG_CHECK_ARG(b->modelDescs[0].grain, "model 0 has no grain mechanism");
  if (n == 0)
    return EMCG_OK;
  double *dK = nullptr;
  EMCG_CUDA(cudaMalloc(&dK, 3 * n * sizeof(double)));
  int32_t st = EMCG_OK;
  if (cudaMemcpy(dK, k, 3 * n * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) {
    st = EMCG_ERR_CUDA;
  } else {
    const int blocks = (int)((n + 127) / 128);
    if (b->precision == EMCG_FP64)
      grainKatKernel<double><<<blocks, 128, 0, b->stream>>>((const ModelK<double> *)b->dModels, n,
                                                            dK, step);
    else
      grainKatKernel<float><<<blocks, 128, 0, b->stream>>>((const ModelK<float> *)b->dModels, n,
                                                           dK, step);
    if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(b->stream) != cudaSuccess ||
        cudaMemcpy(k, dK, 3 * n * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
      st = EMCG_ERR_CUDA;
  }
  if (st)
    setError("grain known-answer kernel failed");
  cudaFree(dK);
  return st;
}

extern "C" int32_t emcg_drift_kat(emcg_handle *h, int32_t valley, int64_t n, const int32_t *sub,
                                  const double *dt, const double *force, double *k, double *pos,
                                  double *energy) {
  BulkImpl *b;
  EMCG_TRY(bulkOf(h, &b));
  EMCG_CHECK_ARG(n >= 0 && sub && dt && force && k && pos && energy, "bad drift arguments");
  if (n == 0)
    return EMCG_OK;
  // one scratch block: dt | force | k | pos | E (doubles) | sub (int32)
  void *buf = nullptr;
  EMCG_CUDA(cudaMalloc(&buf, n * sizeof(double) * 11 + n * sizeof(int32_t)));
  double *base = (double *)buf;
  double *dDt = base, *dF = base + n, *dK = base + 4 * n, *dP = base + 7 * n,
         *dE = base + 10 * n;
  int32_t *dSub = (int32_t *)(base + 11 * n);
  EMCG_CUDA(cudaMemcpy(dSub, sub, n * sizeof(int32_t), cudaMemcpyHostToDevice));
  EMCG_CUDA(cudaMemcpy(dDt, dt, n * sizeof(double), cudaMemcpyHostToDevice));
  EMCG_CUDA(cudaMemcpy(dF, force, 3 * n * sizeof(double), cudaMemcpyHostToDevice));
  EMCG_CUDA(cudaMemcpy(dK, k, 3 * n * sizeof(double), cudaMemcpyHostToDevice));
  EMCG_CUDA(cudaMemcpy(dP, pos, 3 * n * sizeof(double), cudaMemcpyHostToDevice));
  EMCG_CUDA(cudaMemcpy(dE, energy, n * sizeof(double), cudaMemcpyHostToDevice));
  int blocks = (int)((n + 127) / 128);
  if (b->precision == EMCG_FP64)
    driftKatKernel<double><<<blocks, 128, 0, b->stream>>>((const ModelK<double> *)b->dModels,
                                                          valley, n, dSub, dDt, dF, dK, dP, dE);
  else
    driftKatKernel<float><<<blocks, 128, 0, b->stream>>>((const ModelK<float> *)b->dModels,
                                                         valley, n, dSub, dDt, dF, dK, dP, dE);
  EMCG_CUDA(cudaGetLastError());
  EMCG_CUDA(cudaStreamSynchronize(b->stream));
  EMCG_CUDA(cudaMemcpy(k, dK, 3 * n * sizeof(double), cudaMemcpyDeviceToHost));
  EMCG_CUDA(cudaMemcpy(pos, dP, 3 * n * sizeof(double), cudaMemcpyDeviceToHost));
  EMCG_CUDA(cudaMemcpy(energy, dE, n * sizeof(double), cudaMemcpyDeviceToHost));
  cudaFree(buf);
  return EMCG_OK;
}

template <class T>
static int32_t updateEnsTyped(BulkImpl *b, int e, const emcg_ensemble_desc &d) {
  EnsK<T> ek;
  ModelK<T> dummy;
  buildEnsK<T>(d, dummy, b->modelDescs[d.model], b->begin[e], 0, ek);
  EMCG_CUDA(cudaMemcpyAsync((EnsK<T> *)b->dEns + e, &ek, sizeof(EnsK<T>), cudaMemcpyHostToDevice,
                            b->stream));
  EMCG_CUDA(cudaStreamSynchronize(b->stream));
  return EMCG_OK;
}

extern "C" int32_t emcg_bulk_update_ensemble(emcg_handle *h, int32_t e,
                                             const emcg_ensemble_desc *d) {
  BulkImpl *b;
  EMCG_TRY(bulkOf(h, &b));
  EMCG_CHECK_ARG(d && e >= 0 && e < b->nEns, "bad ensemble or descriptor");
  EMCG_CHECK_ARG(d->model == b->ens[e].model && d->capacity == b->ens[e].capacity,
                 "ensemble %d: model and capacity cannot change", e);
  EMCG_CHECK_ARG(d->dt > 0 && std::isfinite(d->dt), "dt must be positive");
  for (int i = 0; i < 3; i++)
    EMCG_CHECK_ARG(d->box[i] > 0 && std::isfinite(d->field[i]), "bad box/field");
  int32_t r = b->precision == EMCG_FP64 ? updateEnsTyped<double>(b, e, *d)
                                        : updateEnsTyped<float>(b, e, *d);
  if (r == EMCG_OK)
    b->ens[e] = *d;
  return r;
}
