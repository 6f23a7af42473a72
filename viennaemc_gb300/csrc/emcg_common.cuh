// Device-side building blocks of the sm_103a EMC engine: kernel-side model
// structs, random-number sources, valley kinematics, free flight, scatter
// selection and final-state sampling.  Templated on the arithmetic type T
// (double: parity engine, float: throughput engine).
//
// Reference (ViennaEMC) functions restated here are cited file:line.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "emcgpu.h"

namespace emcg {

// include/emcConstants.hpp:12-24
constexpr double kQ = 1.60219e-19;
constexpr double kKB = 1.38066e-23;
constexpr double kHBAR = 1.05459e-34;
constexpr double kPI = 3.14159265358979323846;
constexpr double kEPS0 = 8.85419e-12;

// ---------------------------------------------------------------------------
// kernel-side model (built on the host from emcg_model_desc)
// ---------------------------------------------------------------------------
template <class T> struct ValleyK {
  T rot[EMCG_MAX_DEG][9]; // rows = ellipse axes of each subvalley
  T vogt[3];              // Herring-Vogt factors sqrt(mc / m_i)
  T cE;                   // hbar^2 / (mc q):  gamma' = cE |k|^2        [eV m^2]
  T alpha;                // non-parabolicity [1/eV]
  T cK;                   // sqrt(2 mc q) / hbar: |k|(E) = cK sqrt(gamma)
  T cX;                   // hbar / mc: velocity and displacement factor
  T cF[3];                // vogt_i / hbar: dk_ecs = F_ecs cF dt
  int32_t deg;
  int32_t pad_;
};

template <class T> struct MechK {
  int32_t kind, finalValley, nF, pad_;
  T shift;                    // intervalley energy change [eV]
  T debye[EMCG_MAX_REGIONS];  // Coulomb: |doping| / (sc2 mc)   [eV]
  uint8_t finalSub[EMCG_MAX_DEG][EMCG_MAX_NF];
};

template <class T> struct ModelK {
  ValleyK<T> v[EMCG_MAX_VALLEYS];
  MechK<T> m[EMCG_MAX_MECH];
  int32_t nV, nLevels, nTS, grain; // grain: a grain mechanism is set
  T dE, invdE, grainTau, grainProb; // grainProb: its transmission probability
  int8_t tsIndex[EMCG_MAX_VALLEYS][EMCG_MAX_REGIONS]; // -1: no table set
  int32_t tsN[EMCG_MAX_TABLESETS];
  int64_t tsOff[EMCG_MAX_TABLESETS];   // offset of the set in `tables`
  T tauMax[EMCG_MAX_TABLESETS];
  uint8_t tsMech[EMCG_MAX_TABLESETS][EMCG_MAX_MECH];
  const T *tables; // level-major per set: tables[tsOff + L * nT + t]
  int32_t surfKind[4]; // EMCG_SURFACE_* per device boundary (XMIN, XMAX, YMIN, YMAX)
  T surfParam[4];      // its specularity or roughness height [m]
};

// per-ensemble constants of a bulk launch
template <class T> struct EnsK {
  int32_t model, nV;
  int64_t begin, n;                       // global particle index range
  T fv[EMCG_MAX_VALLEYS][EMCG_MAX_DEG][3]; // R F vogt / hbar   [1/(m s)]
  T g[EMCG_MAX_VALLEYS][EMCG_MAX_DEG][3];  // vogt o (R dir): v.dir = cX g.k_ecs / npf
  T box[3];
  T dt;
  T F[3];   // applied force charge x field [N] (particle-particle Coulomb steps)
  T charge; // [C]
  uint32_t key0, key1, stream;
  uint32_t floatDraws; // EMCG_ENS_FLOAT_DRAWS: the double engine draws as the float one
};

struct Tile {
  int32_t ens, pad_;
  int64_t begin, end;
};

template <class T> struct StateK {
  T *kx, *ky, *kz, *px, *py, *pz, *E, *tau, *gtau;
  uint32_t *meta; // valley | sub << 8 | region << 16
};

__host__ __device__ inline uint32_t packMeta(int v, int s, int r) {
  return (uint32_t)v | ((uint32_t)s << 8) | ((uint32_t)r << 16);
}

// ---------------------------------------------------------------------------
// precision-dispatched math.  Float uses the SFU approximations: the float
// engine is a statistical engine checked against the double one.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double m_sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float m_sqrt(float x) {
  float r;
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ double m_div(double a, double b) { return a / b; }
__device__ __forceinline__ float m_div(float a, float b) { return __fdividef(a, b); }
__device__ __forceinline__ double m_log(double x) { return log(x); }
__device__ __forceinline__ float m_log(float x) { return __logf(x); }
__device__ __forceinline__ double m_floor(double x) { return floor(x); }
__device__ __forceinline__ float m_floor(float x) { return floorf(x); }
__device__ __forceinline__ double m_exp(double x) { return exp(x); }
__device__ __forceinline__ float m_exp(float x) { return expf(x); }
__device__ __forceinline__ void m_sincos(double x, double *s, double *c) { sincos(x, s, c); }
__device__ __forceinline__ void m_sincos(float x, float *s, float *c) { sincosf(x, s, c); }
__device__ __forceinline__ void m_sincos2pi(double u, double *s, double *c) {
  double phi = 2 * kPI * u; // 2 * emcPi<T>() * rand (include/emcUtil.hpp:132)
  *s = sin(phi);
  *c = cos(phi);
}
__device__ __forceinline__ void m_sincos2pi(float u, float *s, float *c) {
  // the angle 2 pi u - pi in [-pi, pi) keeps the SFU in its accurate range;
  // sin and cos of 2 pi u are their negatives, so a draw gives the same
  // direction as in the double engine (the float and double engines stay on
  // the same path when they consume the same numbers)
  float sm, cm;
  __sincosf(6.2831853f * (u - 0.5f), &sm, &cm);
  *s = -sm;
  *c = -cm;
}

template <class T> __device__ __forceinline__ T ldg(const T *p) { return __ldg(p); }

// ---------------------------------------------------------------------------
// random numbers
// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon et al., SC'11): 10 rounds with Weyl key schedule.
__device__ __forceinline__ void philox4x32_10(uint32_t c0, uint32_t c1,
                                              uint32_t c2, uint32_t c3,
                                              uint32_t k0, uint32_t k1,
                                              uint32_t o[4]) {
#pragma unroll
  for (int r = 0; r < 10; r++) {
    uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
    uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
    uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  o[0] = c0;
  o[1] = c1;
  o[2] = c2;
  o[3] = c3;
}

// libstdc++ generate_canonical<double,53>(mt19937_64): (double)w / 2^64,
// clamped below 1; then uniform_real_distribution: u * (b - a) + a.
__device__ __forceinline__ double canonical53(uint64_t w) {
  double r = __dmul_rn(__ull2double_rn(w), 0x1p-64);
  return r >= 1.0 ? 0x1.fffffffffffffp-1 : r;
}

// Counter-based source: counter = (particle, step, call, stream), key = seed.
// double: 64-bit words (two per call), same layout as the oracle.
// float:  32-bit words (four per call).
template <class T> struct PhiloxSrc;

// Double draws: one 64-bit word per draw.  With f32 set (EMCG_ENS_FLOAT_DRAWS)
// one 32-bit word per draw and exactly the float source's values, widened.
template <> struct PhiloxSrc<double> {
  uint32_t c0, c1, c2, c3, k0, k1;
  uint64_t b0, b1;
  int nb;
  bool f32;
  __device__ __forceinline__ void init(uint32_t pid, uint32_t step,
                                       uint32_t stream, uint32_t key0,
                                       uint32_t key1, uint32_t floatDraws = 0) {
    c0 = pid;
    c1 = step;
    c2 = 0;
    c3 = stream;
    k0 = key0;
    k1 = key1;
    nb = 0;
    f32 = floatDraws != 0;
  }
  __device__ __forceinline__ void block() {
    uint32_t o[4];
    philox4x32_10(c0, c1, c2, c3, k0, k1, o);
    c2++;
    b0 = (uint64_t)o[0] | ((uint64_t)o[1] << 32);
    b1 = (uint64_t)o[2] | ((uint64_t)o[3] << 32);
  }
  __device__ __forceinline__ uint64_t word() {
    if (nb == 0) {
      block();
      nb = 2;
    }
    uint64_t w = (nb == 2) ? b0 : b1;
    nb--;
    return w;
  }
  // the float source's word sequence: o[0], o[1], o[2], o[3] of each block
  __device__ __forceinline__ uint32_t word32() {
    if (nb == 0) {
      block();
      nb = 4;
    }
    const uint32_t w = nb == 4 ? (uint32_t)b0 : nb == 3 ? (uint32_t)(b0 >> 32)
                     : nb == 2 ? (uint32_t)b1 : (uint32_t)(b1 >> 32);
    nb--;
    return w;
  }
  __device__ __forceinline__ uint32_t pick(uint32_t n) {
    return f32 ? __umulhi(word32(), n) : (uint32_t)(word() % (uint64_t)n);
  }
  __device__ __forceinline__ double u01() {
    return f32 ? (double)((float)(word32() >> 8) * 0x1p-24f) : canonical53(word());
  }
  __device__ __forceinline__ double ulog() {
    if (f32)
      return (double)fmaf((float)(word32() >> 8) * 0x1p-24f, 1.f - 1e-6f, 1e-6f);
    return __dadd_rn(__dmul_rn(canonical53(word()), 1. - 1e-6), 1e-6);
  }
  __device__ __forceinline__ bool failed() const { return false; }
};

template <> struct PhiloxSrc<float> {
  uint32_t c0, c1, c2, c3, k0, k1;
  uint32_t b0, b1, b2, b3; // scalars, not an array: a dynamically indexed
                           // array would live in local memory
  int nb;
  __device__ __forceinline__ void init(uint32_t pid, uint32_t step,
                                       uint32_t stream, uint32_t key0,
                                       uint32_t key1, uint32_t = 0) {
    c0 = pid;
    c1 = step;
    c2 = 0;
    c3 = stream;
    k0 = key0;
    k1 = key1;
    nb = 0;
  }
  // init() for another step of the same particle and stream
  __device__ __forceinline__ void restart(uint32_t step) {
    c1 = step;
    c2 = 0;
    nb = 0;
  }
  __device__ __forceinline__ uint32_t word() {
    if (nb == 0) {
      uint32_t o[4];
      philox4x32_10(c0, c1, c2, c3, k0, k1, o);
      b0 = o[0];
      b1 = o[1];
      b2 = o[2];
      b3 = o[3];
      c2++;
      nb = 4;
    }
    const uint32_t w = nb == 4 ? b0 : nb == 3 ? b1 : nb == 2 ? b2 : b3;
    nb--;
    return w;
  }
  __device__ __forceinline__ uint32_t pick(uint32_t n) {
    return __umulhi(word(), n);
  }
  __device__ __forceinline__ float u01() {
    return (float)(word() >> 8) * 0x1p-24f;
  }
  __device__ __forceinline__ float ulog() {
    return fmaf(u01(), 1.f - 1e-6f, 1e-6f);
  }
  __device__ __forceinline__ bool failed() const { return false; }
};

// Replay of a recorded std::mt19937_64 stream (double engine only).
struct ReplaySrc {
  const uint64_t *w;
  int64_t pos, end;
  int bad;
  __device__ __forceinline__ uint64_t word() {
    if (pos < end)
      return w[pos++];
    bad = 1;
    return 0;
  }
  __device__ __forceinline__ uint32_t pick(uint32_t n) {
    return (uint32_t)(word() % (uint64_t)n);
  }
  __device__ __forceinline__ double u01() { return canonical53(word()); }
  __device__ __forceinline__ double ulog() {
    return __dadd_rn(__dmul_rn(canonical53(word()), 1. - 1e-6), 1e-6);
  }
  __device__ __forceinline__ bool failed() const { return bad != 0; }
};

// ---------------------------------------------------------------------------
// valley kinematics (include/ValleyTypes/emcNonParabolicAnistropValley.hpp)
// ---------------------------------------------------------------------------
template <class T>
__device__ __forceinline__ void toEcs(const T *R, T a0, T a1, T a2, T o[3]) {
  o[0] = a0 * R[0] + a1 * R[1] + a2 * R[2]; // :140-153
  o[1] = a0 * R[3] + a1 * R[4] + a2 * R[5];
  o[2] = a0 * R[6] + a1 * R[7] + a2 * R[8];
}
template <class T>
__device__ __forceinline__ void toDev(const T *R, T a0, T a1, T a2, T o[3]) {
  o[0] = a0 * R[0] + a1 * R[3] + a2 * R[6]; // :157-170
  o[1] = a0 * R[1] + a1 * R[4] + a2 * R[7];
  o[2] = a0 * R[2] + a1 * R[5] + a2 * R[8];
}

// E(k) = gamma / (1 + sqrt(1 + 2 alpha gamma)), gamma = hbar^2 k^2/(mc q)  (:109-113)
template <class T>
__device__ __forceinline__ T energyOf(const ValleyK<T> &V, T sq) {
  T g = V.cE * sq;
  return m_div(g, T(1) + m_sqrt(T(1) + T(2) * V.alpha * g));
}
// gamma(E) = E (1 + alpha E)  (:122)
template <class T> __device__ __forceinline__ T gammaOf(const ValleyK<T> &V, T E) {
  return E * (T(1) + V.alpha * E);
}

// Free flight for time dt under the ellipse-frame force term fv = R F vogt/hbar
// (include/emcParticleDrift.hpp:11-36).  k, E and pos are updated in place;
// kN receives the new wave vector in the ellipse frame.
template <class T, int DIM>
__device__ __forceinline__ void drift(const ValleyK<T> &V, int sub,
                                      const T fv[3], T dt, T k[3], T &E,
                                      T *pos, T kN[3]) {
  const T *R = V.rot[sub];
  T kO[3];
  toEcs(R, k[0], k[1], k[2], kO);
#pragma unroll
  for (int i = 0; i < 3; i++)
    kN[i] = kO[i] + fv[i] * dt;
  toDev(R, kN[0], kN[1], kN[2], k);
  E = energyOf(V, k[0] * k[0] + k[1] * k[1] + k[2] * k[2]);
  // leapfrog displacement hbar vogt avgK dt / (mc (1 + 2 E alpha))
  T c = m_div(V.cX * dt, T(1) + T(2) * E * V.alpha) * T(0.5);
  T d[3], dd[3];
#pragma unroll
  for (int i = 0; i < 3; i++)
    d[i] = V.vogt[i] * (kN[i] + kO[i]) * c;
  toDev(R, d[0], d[1], d[2], dd);
#pragma unroll
  for (int i = 0; i < DIM; i++)
    pos[i] += dd[i];
}

// ---------------------------------------------------------------------------
// scattering (include/emcScatterHandler.hpp, include/ScatterMechanisms/)
// ---------------------------------------------------------------------------
// Energy level floor(E/dE) - 1 with the reference's size_t conversion:
// -1 -> 0, other negative values and NaN -> top level  (:237-244)
template <class T>
__device__ __forceinline__ int energyLevel(const ModelK<T> &M, T E);
template <>
__device__ __forceinline__ int energyLevel<double>(const ModelK<double> &M,
                                                   double E) {
  double f = floor(E / M.dE) - 1;
  if (!(f >= 0.))
    return (f == -1.) ? 0 : M.nLevels - 1;
  return f > (double)(M.nLevels - 1) ? M.nLevels - 1 : (int)f;
}
template <>
__device__ __forceinline__ int energyLevel<float>(const ModelK<float> &M,
                                                  float E) {
  float f = floorf(E * M.invdE) - 1.f;
  if (!(f >= 0.f))
    return (f == -1.f) ? 0 : M.nLevels - 1;
  return f > (float)(M.nLevels - 1) ? M.nLevels - 1 : (int)f;
}

// isotropic direction of norm n (include/emcUtil.hpp:131-139); the compiled
// reference evaluates initRandomDirection(n, dist(rng), dist(rng)) right to
// left, so cos(theta)'s number is drawn first.
template <class T, class R>
__device__ __forceinline__ void randomDirection(T n, R &rng, T k[3]) {
  T r2 = rng.u01();
  T r1 = rng.u01();
  T s, c;
  m_sincos2pi(r1, &s, &c);
  T ct = T(1) - T(2) * r2;
  T st = m_sqrt(T(1) - ct * ct);
  k[0] = n * st * c;
  k[1] = n * st * s;
  k[2] = n * ct;
}

// direction at polar angle acos(ct) about the current k
// (include/emcUtil.hpp:141-175)
template <class T>
__device__ __forceinline__ void directionAboutK(T k[3], T ct, T rnd) {
  T kxy = m_sqrt(k[0] * k[0] + k[1] * k[1]);
  T nK = m_sqrt(kxy * kxy + k[2] * k[2]);
  if (nK == T(0)) {
    k[0] = k[1] = k[2] = T(0);
    return;
  }
  T ct0 = m_div(k[2], nK), st0 = m_div(kxy, nK);
  T cfi0 = kxy > T(0) ? m_div(k[0], kxy) : T(1);
  T sfi0 = kxy > T(0) ? m_div(k[1], kxy) : T(0);
  T st = m_sqrt(T(1) - ct * ct);
  T s, c;
  m_sincos2pi(rnd, &s, &c);
  T kxp = nK * st * c, kyp = nK * st * s, kzp = nK * ct;
  k[0] = kxp * cfi0 * ct0 - kyp * sfi0 + kzp * cfi0 * st0;
  k[1] = kxp * sfi0 * ct0 + kyp * cfi0 + kzp * sfi0 * st0;
  k[2] = -kxp * st0 + kzp * ct0;
}

// emcGrainScatterMechanism::scatterParticle (include/emcGrainScatterMechanism.hpp:
// 41-80) with k in the device frame: reflected into the opposite hemisphere
// (cos(theta) <= 0 about k) when a draw exceeds the transmission probability,
// else transmitted into the same one; |k| is kept and the energy is not
// updated.  Only with a grain mechanism set (M.grain): without one the
// reference's scatterParticleAtGrain is a no-op (include/emcScatterHandler.hpp:
// 193-196).
template <class T, class R>
__device__ __forceinline__ void grainScatter(const ModelK<T> &M, T k[3], R &rng) {
  const bool reflect = rng.u01() > M.grainProb;
  T rnd = rng.u01();
  if (reflect) {
    if (rnd < T(0.5))
      rnd += T(0.5);
  } else if (rnd > T(0.5)) {
    rnd -= T(0.5);
  }
  directionAboutK(k, T(1) - T(2) * rnd, rng.u01());
}

// Selected mechanism's final state.
template <class T, class R>
__device__ __forceinline__ void applyMechanism(const ModelK<T> &M,
                                               const MechK<T> &me, T k[3],
                                               T &E, int &valley, int &sub,
                                               int region, R &rng) {
  switch (me.kind) {
  case EMCG_MECH_ACOUSTIC: { // elastic, isotropic (emcAcousticScatterMechanism.hpp:124-126)
    T n = m_sqrt(k[0] * k[0] + k[1] * k[1] + k[2] * k[2]);
    randomDirection(n, rng, k);
    break;
  }
  case EMCG_MECH_COULOMB: { // Brooks-Herring (emcCoulombScatterMechanism.hpp:48-59)
    const ValleyK<T> &V = M.v[valley];
    T g = gammaOf(V, E);
    T rnd = rng.u01();
    T ct = T(1) - m_div(rnd * T(2), m_div((T(1) - rnd) * g, me.debye[region]) + T(1));
    directionAboutK(k, ct, rng.u01());
    break;
  }
  default: { // intervalley absorption / emission, zero or first order
    valley = me.finalValley;
    sub = me.finalSub[sub][rng.pick((uint32_t)me.nF)];
    E += me.shift;
    const ValleyK<T> &V = M.v[valley];
    randomDirection(V.cK * m_sqrt(gammaOf(V, E)), rng, k);
    break;
  }
  }
}

// emcScatterHandler::scatterParticle (include/emcScatterHandler.hpp:148-170).
// Returns EMCG_ERR_OUT_OF_TABLE if the (valley, region) pair has no tables.
template <class T, class R>
__device__ __forceinline__ int scatterParticle(const ModelK<T> &M, T k[3],
                                               T &E, int &valley, int &sub,
                                               int region, R &rng) {
  int ts = M.tsIndex[valley][region];
  if (ts < 0)
    return EMCG_ERR_OUT_OF_TABLE;
  int nT = M.tsN[ts];
  if (nT == 0)
    return 0;
  int L = energyLevel(M, E);
  T rnd = rng.u01();
  const T *row = M.tables + M.tsOff[ts] + (int64_t)L * nT;
  if (rnd > ldg(row + nT - 1))
    return 0; // self-scattering
  // the first t with row[t-1] <= rnd < row[t] (row[-1] = 0): the row is
  // cumulative, so nondecreasing, and t is the number of entries <= rnd.  The
  // loads are independent, so the search costs one load latency, not nT.
  int t = 0;
#pragma unroll 4
  for (int q = 0; q < nT; q++)
    t += ldg(row + q) <= rnd ? 1 : 0;
  if (t < nT) // t = nT: rnd equals the last entry, no mechanism (as the loop above)
    applyMechanism(M, M.m[M.tsMech[ts][t]], k, E, valley, sub, region, rng);
  return 0;
}

// free-flight constant of (valley, region); 2e-15 s without tables
// (include/emcScatterHandler.hpp:79-84)
template <class T>
__device__ __forceinline__ T tauOf(const ModelK<T> &M, int valley, int region) {
  int ts = M.tsIndex[valley][region];
  return ts >= 0 ? M.tauMax[ts] : T(2e-15);
}

} // namespace emcg
