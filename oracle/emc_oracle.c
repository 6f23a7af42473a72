/*
 * CPU oracle for the ViennaEMC bulk hot path -- TEST INFRASTRUCTURE ONLY.
 * See emc_oracle.h.  Every function cites the reference file:line it
 * restates; paths are relative to the ViennaEMC project root.
 *
 * Build with -ffp-contract=off: the reference is compiled without FMA and the
 * oracle must reproduce its doubles exactly.
 */
#include "emc_oracle.h"
#include "emc_oracle_internal.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* include/emcConstants.hpp:12-24 */
#define C_PI 3.14159265358979323846
#define C_Q 1.60219e-19
#define C_KB 1.38066e-23
#define C_HBAR 1.05459e-34
#define C_EPS0 8.85419e-12

/* GCC on x86-64 evaluates the two dist(rng) arguments of
   initRandomDirection(norm, dist(rng), dist(rng)) right to left: the second
   argument (cos theta) is drawn first.  Pinned against the compiled reference
   by tests/test_oracle_golden.py. */
#define OC_ARGS_RIGHT_TO_LEFT 1

typedef struct {
  double relMass[3], pmass, alpha, bottom;
  int32_t deg;
  double rot[OC_MAX_DEG][9];
  double mc, mdos, vogt[3];
} oc_valley;

typedef struct {
  int32_t kind, valley, finalValley, nF;
  double p0, p1;
  int32_t finalSub[OC_MAX_DEG][OC_MAX_NF];
  double sc, sc1, sc2;
  double deltaValley;
} oc_mech;

struct oc_model {
  double T, rho, vs, epsR, Ni, maxE, dE, Vt;
  int32_t nLevels;
  int32_t nV, nM;
  oc_valley v[OC_MAX_VALLEYS];
  oc_mech mech[OC_MAX_MECH];
  double regionDoping[OC_MAX_REGIONS];
  int32_t tsUsed[OC_MAX_VALLEYS][OC_MAX_REGIONS];
  int32_t tsN[OC_MAX_VALLEYS][OC_MAX_REGIONS];
  int32_t tsMech[OC_MAX_VALLEYS][OC_MAX_REGIONS][OC_MAX_MECH];
  double *raw[OC_MAX_VALLEYS][OC_MAX_REGIONS];
  double *norm[OC_MAX_VALLEYS][OC_MAX_REGIONS];
  double tau[OC_MAX_VALLEYS][OC_MAX_REGIONS];
  /* grain mechanism (include/emcScatterHandler.hpp:61-62, 233-234):
     grainTau = 1 / rate with one set, 1 without */
  int32_t grain;
  double grainProb, grainTau;
  /* surface mechanism per boundary (XMIN, XMAX, YMIN, YMAX):
     include/emcScatterHandler.hpp:63-65, 114-124; OC_SURFACE_* */
  int32_t surfKind[4];
  double surfParam[4];
  int32_t built;
};

/* ======================================================================== */
/* random numbers                                                           */
/* ======================================================================== */

/* mt19937_64 (Matsumoto & Nishimura, 64-bit variant; the parameters are the
   ones fixed by the C++11 standard for std::mt19937_64, which the reference
   uses as emcRNG: include/emcUtil.hpp:15) */
#define MT_N 312
#define MT_M 156
void oc_mt_seed(oc_rng *r, uint64_t seed) {
  r->mt[0] = seed;
  for (int i = 1; i < MT_N; i++)
    r->mt[i] = 6364136223846793005ULL * (r->mt[i - 1] ^ (r->mt[i - 1] >> 62)) +
               (uint64_t)i;
  r->mt_idx = MT_N;
}

static void mt_twist(uint64_t *mt) {
  const uint64_t UM = 0xFFFFFFFF80000000ULL, LM = 0x7FFFFFFFULL;
  for (int i = 0; i < MT_N; i++) {
    uint64_t x = (mt[i] & UM) | (mt[(i + 1) % MT_N] & LM);
    uint64_t xa = x >> 1;
    if (x & 1ULL)
      xa ^= 0xB5026F5AA96619E9ULL;
    mt[i] = mt[(i + MT_M) % MT_N] ^ xa;
  }
}

uint64_t oc_mt_next(oc_rng *r) {
  if (r->mt_idx >= MT_N) {
    mt_twist(r->mt);
    r->mt_idx = 0;
  }
  uint64_t y = r->mt[r->mt_idx++];
  y ^= (y >> 29) & 0x5555555555555555ULL;
  y ^= (y << 17) & 0x71D67FFFEDA60000ULL;
  y ^= (y << 37) & 0xFFF7EEE000000000ULL;
  y ^= (y >> 43);
  return y;
}

/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11 "Parallel random numbers:
   as easy as 1, 2, 3"): 10 rounds, Weyl key schedule. */
void oc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2],
                      uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; r++) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
    uint32_t n1 = (uint32_t)p1;
    uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
    uint32_t n3 = (uint32_t)p0;
    c0 = n0;
    c1 = n1;
    c2 = n2;
    c3 = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0;
  out[1] = c1;
  out[2] = c2;
  out[3] = c3;
}

/* libstdc++ generate_canonical<double,53>(mt19937_64): one 64-bit word,
   (double)word / 2^64, clamped below 1 (bits/random.tcc generate_canonical) */
double oc_canonical(uint64_t w) {
  double s = (double)w;
  double ret = s / 18446744073709551616.0;
  if (ret >= 1.0)
    ret = nextafter(1.0, 0.0);
  return ret;
}

void oci_dctx_init(dctx *d, oc_rng *r, uint32_t pid, uint32_t step,
                      uint32_t streamWord) {
  d->r = r;
  d->mode = r->mode;
  d->ctr[0] = pid;
  d->ctr[1] = step;
  d->ctr[2] = 0;
  d->ctr[3] = streamWord;
  d->key[0] = (uint32_t)r->seed;
  d->key[1] = (uint32_t)(r->seed >> 32);
  d->nbuf = 0;
  d->fail = 0;
}

uint64_t oci_draw_u64(dctx *d) {
  uint64_t w;
  if (d->mode == OC_RNG_MT) {
    w = oc_mt_next(d->r);
  } else if (d->mode == OC_RNG_PHILOX) {
    if (d->nbuf == 0) {
      uint32_t o[4];
      oc_philox4x32_10(d->ctr, d->key, o);
      d->ctr[2]++;
      d->buf[0] = (uint64_t)o[0] | ((uint64_t)o[1] << 32);
      d->buf[1] = (uint64_t)o[2] | ((uint64_t)o[3] << 32);
      d->nbuf = 2;
    }
    w = d->buf[2 - d->nbuf];
    d->nbuf--;
  } else if (d->mode == OC_RNG_PHILOX32) {
    /* the engine's float source: o[0], o[1], o[2], o[3] of each block */
    if (d->nbuf == 0) {
      uint32_t o[4];
      oc_philox4x32_10(d->ctr, d->key, o);
      d->ctr[2]++;
      d->buf[0] = (uint64_t)o[0] | ((uint64_t)o[1] << 32);
      d->buf[1] = (uint64_t)o[2] | ((uint64_t)o[3] << 32);
      d->nbuf = 4;
    }
    const uint64_t b = d->buf[(4 - d->nbuf) >> 1];
    w = (d->nbuf & 1) ? (b >> 32) : (b & 0xFFFFFFFFu);
    d->nbuf--;
  } else {
    if (d->r->pos < d->r->nwords) {
      w = d->r->words[d->r->pos++];
    } else {
      d->fail = 1;
      w = 0;
    }
  }
  oc_rng *r = d->r;
  if (r->rec) {
    if (r->rec_n < r->rec_cap)
      r->rec[r->rec_n] = w;
    else
      r->rec_overflow = 1;
    r->rec_n++;
  }
  return w;
}

/* std::uniform_real_distribution<double>(a, b)(rng) = canonical*(b-a)+a
   (bits/random.h uniform_real_distribution::operator()).  OC_RNG_PHILOX32:
   the engine's float draws, a 24-bit uniform from the top of one 32-bit word
   and U[1e-6, 1) by one float fused multiply-add, widened to double. */
static float draw_f32(dctx *d) { return (float)(oci_draw_u64(d) >> 8) * 0x1p-24f; }
double oci_draw_u01(dctx *d) {
  if (d->mode == OC_RNG_PHILOX32)
    return (double)draw_f32(d);
  return oc_canonical(oci_draw_u64(d)) * (1.0 - 0.0) + 0.0;
}
double oci_draw_ulog(dctx *d) {
  if (d->mode == OC_RNG_PHILOX32)
    return (double)fmaf(draw_f32(d), 1.f - 1e-6f, 1e-6f);
  return oc_canonical(oci_draw_u64(d)) * (1. - 1e-6) + 1e-6;
}
/* rng() % n of the reference; OC_RNG_PHILOX32: the engine's float pick, the
   high word of the 32-bit draw times n */
uint32_t oci_draw_pick(dctx *d, uint32_t n) {
  const uint64_t w = oci_draw_u64(d);
  if (d->mode == OC_RNG_PHILOX32)
    return (uint32_t)((w * (uint64_t)n) >> 32);
  return (uint32_t)(w % (uint64_t)n);
}

/* ======================================================================== */
/* model                                                                    */
/* ======================================================================== */

oc_model *oc_model_new(double temperature, double rho, double vSound,
                       double epsR, double Ni, int32_t nLevels,
                       double maxEnergy) {
  oc_model *m = (oc_model *)calloc(1, sizeof(oc_model));
  m->T = temperature;
  m->rho = rho;
  m->vs = vSound;
  m->epsR = epsR;
  m->Ni = Ni;
  m->nLevels = nLevels;
  m->maxE = maxEnergy;
  /* include/emcScatterHandler.hpp:73-75: dE = maxEnergy / nrEnergyLevels */
  m->dE = maxEnergy / (double)nLevels;
  /* include/emcDevice.hpp:87: Vt = kB / q * T */
  m->Vt = C_KB / C_Q * temperature;
  for (int r = 0; r < OC_MAX_REGIONS; r++)
    m->regionDoping[r] = Ni;
  m->grainTau = 1.;
  return m;
}

void oc_model_free(oc_model *m) {
  if (!m)
    return;
  for (int v = 0; v < OC_MAX_VALLEYS; v++)
    for (int r = 0; r < OC_MAX_REGIONS; r++) {
      free(m->raw[v][r]);
      free(m->norm[v][r]);
    }
  free(m);
}

/* include/ValleyTypes/emcNonParabolicAnistropValley.hpp:48-56, 174-204 */
int32_t oc_add_valley(oc_model *m, const double relMass[3],
                      double particleMass, int32_t deg, double alpha,
                      double bottom) {
  if (m->nV >= OC_MAX_VALLEYS || deg < 1 || deg > OC_MAX_DEG)
    return -1;
  oc_valley *v = &m->v[m->nV];
  memcpy(v->relMass, relMass, sizeof(double) * 3);
  v->pmass = particleMass;
  v->deg = deg;
  v->alpha = alpha;
  v->bottom = bottom;
  for (int s = 0; s < deg; s++) {
    memset(v->rot[s], 0, sizeof(double) * 9);
    v->rot[s][0] = v->rot[s][4] = v->rot[s][8] = 1.0;
  }
  /* initEffMasses :185-194 */
  double dos = 1.;
  for (int i = 0; i < 3; i++)
    dos = dos * relMass[i];
  v->mdos = pow(dos, 1. / 3.) * particleMass;
  double acc = 0.;
  for (int i = 0; i < 3; i++)
    acc += 1. / relMass[i];
  v->mc = 3. * particleMass / acc;
  /* initVogtFactor :198-204 (getEffMassCond() at energy 0) */
  for (int i = 0; i < 3; i++)
    v->vogt[i] = sqrt(v->mc * (1 + 2 * 0. * alpha) / (relMass[i] * particleMass));
  return m->nV++;
}

/* include/emcUtil.hpp:40-49 (norm, normalize) */
static void oc_normalize(double d[3]) {
  double s = 0;
  for (int i = 0; i < 3; i++)
    s += d[i] * d[i];
  double n = sqrt(s);
  if (n == 0.)
    return;
  for (int i = 0; i < 3; i++)
    d[i] /= n;
}

/* emcNonParabolicAnistropValley.hpp:68-80 */
int32_t oc_set_frame(oc_model *m, int32_t valley, int32_t sub,
                     const double d1[3], const double d2[3],
                     const double d3[3]) {
  if (valley < 0 || valley >= m->nV || sub < 0 || sub >= m->v[valley].deg)
    return -1;
  double a[3], b[3], c[3];
  memcpy(a, d1, 24);
  memcpy(b, d2, 24);
  memcpy(c, d3, 24);
  oc_normalize(a);
  oc_normalize(b);
  oc_normalize(c);
  double *R = m->v[valley].rot[sub];
  memcpy(R, a, 24);
  memcpy(R + 3, b, 24);
  memcpy(R + 6, c, 24);
  return 0;
}

/* zero-order: emcZeroOrderInterValleyScatterMechanism.hpp:12-21;
   first-order: emcFirstOrderInterValleyScatterMechanism.hpp:11-20 */
static double zero_order_const(double D, double ph, double rho, double T,
                               int32_t nF, int abs) {
  double result = (double)nF * sqrt(C_Q) * pow(D / C_HBAR, 2.) * C_Q /
                  (C_PI * rho * ph * sqrt(2.));
  double nrPh = 1. / (exp(C_Q * ph / (C_KB * T)) - 1.);
  return abs ? result * nrPh : result * (nrPh + 1);
}
static double first_order_const(double D, double ph, double rho, double T,
                                int32_t nF, int abs) {
  double result = (double)nF * sqrt(2.) * pow(C_Q, 5. / 2.) * pow(D, 2.) /
                  (C_PI * rho * pow(C_HBAR, 4.) * ph);
  double nrPh = 1. / (exp(C_Q * ph / (C_KB * T)) - 1.);
  return abs ? result * nrPh : result * (nrPh + 1);
}

int32_t oc_add_mech(oc_model *m, int32_t kind, int32_t valley,
                    int32_t finalValley, double p0, double p1, int32_t nF,
                    const int32_t *finalSub, const int32_t *regions,
                    int32_t nRegions) {
  if (m->nM >= OC_MAX_MECH || valley < 0 || valley >= m->nV)
    return -1;
  int32_t idx = m->nM;
  oc_mech *me = &m->mech[idx];
  memset(me, 0, sizeof(*me));
  me->kind = kind;
  me->valley = valley;
  me->finalValley = (kind >= OC_ZERO_IV_ABS && kind <= OC_FIRST_IV_EMI)
                        ? finalValley
                        : valley;
  me->p0 = p0;
  me->p1 = p1;
  me->nF = nF;
  if (kind >= OC_ZERO_IV_ABS && kind <= OC_FIRST_IV_EMI) {
    if (nF < 1 || nF > OC_MAX_NF || finalValley < 0 || finalValley >= m->nV)
      return -1;
    for (int s = 0; s < m->v[valley].deg; s++)
      for (int f = 0; f < nF; f++)
        me->finalSub[s][f] = finalSub[s * nF + f];
    /* deltaValley = bottom(final) - bottom(initial), set by getScatterRate */
    me->deltaValley = m->v[me->finalValley].bottom - m->v[valley].bottom;
  }
  switch (kind) {
  case OC_ACOUSTIC: { /* emcAcousticScatterMechanism.hpp:100-110 */
    double cL = m->rho * pow(m->vs, 2.);
    me->sc = sqrt(2.0 * C_Q) * pow(p0 * C_Q, 2.) * C_KB * m->T /
             (C_PI * cL * pow(C_HBAR, 4.));
    break;
  }
  case OC_ZERO_IV_ABS:
  case OC_ZERO_IV_EMI:
    me->sc = zero_order_const(p0, p1, m->rho, m->T, nF, kind == OC_ZERO_IV_ABS);
    break;
  case OC_FIRST_IV_ABS:
  case OC_FIRST_IV_EMI:
    me->sc = first_order_const(p0, p1, m->rho, m->T, nF, kind == OC_FIRST_IV_ABS);
    break;
  case OC_COULOMB: { /* emcCoulombScatterMechanism.hpp:23-32 */
    double epsMat = C_EPS0 * p0;
    double Vt = C_KB / C_Q * m->T;
    me->sc1 = sqrt(2 * C_Q) * pow(C_KB * m->T, 2.) / (C_PI * pow(C_HBAR, 4.));
    me->sc2 = 8 * epsMat * Vt / (C_HBAR * C_HBAR);
    break;
  }
  default:
    return -1;
  }
  /* include/emcScatterHandler.hpp:127-145 */
  for (int i = 0; i < nRegions; i++) {
    int r = regions[i];
    if (r < 0 || r >= OC_MAX_REGIONS)
      return -1;
    m->tsUsed[valley][r] = 1;
    m->tsMech[valley][r][m->tsN[valley][r]++] = idx;
  }
  m->nM++;
  return idx;
}

/* emcScatterHandler::setGrainScatterMechanism with an
   emcGrainScatterMechanism(transmissionProb, scatterRate)
   (include/emcGrainScatterMechanism.hpp:27-29); the grain free-flight
   constant becomes 1 / scatterRate (include/emcScatterHandler.hpp:233-234) */
int32_t oc_set_grain(oc_model *m, double transmissionProb, double scatterRate) {
  if (!(scatterRate > 0))
    return -1;
  m->grain = 1;
  m->grainProb = transmissionProb;
  m->grainTau = 1. / scatterRate;
  return 0;
}

double oci_grain_tau(const oc_model *m) { return m->grainTau; }

/* emcScatterHandler::setSurfaceScatterMechanism (include/emcScatterHandler.hpp:
   114-124) for one boundary: OC_SURFACE_CONSTANT with the specularity
   parameter (emcConstantSurfaceScatterMechanism), OC_SURFACE_ROUGHNESS with
   the roughness height [m] (emcMomentumDependentSurfaceScatterMechanism),
   OC_SURFACE_SPECULAR for none */
int32_t oc_set_surface(oc_model *m, int32_t boundary, int32_t kind, double param) {
  if (boundary < 0 || boundary > 3 || kind < OC_SURFACE_SPECULAR || kind > OC_SURFACE_ROUGHNESS)
    return -1;
  m->surfKind[boundary] = kind;
  m->surfParam[boundary] = param;
  return 0;
}

int32_t oci_surface(const oc_model *m, int32_t boundary, double *param) {
  *param = m->surfParam[boundary];
  return m->surfKind[boundary];
}

int32_t oc_set_region_doping(oc_model *m, int32_t region, double doping) {
  if (region < 0 || region >= OC_MAX_REGIONS)
    return -1;
  m->regionDoping[region] = doping;
  return 0;
}

/* emcNonParabolicAnistropValley.hpp:122 */
static double gamma_of(const oc_valley *v, double E) {
  return E * (1 + v->alpha * E);
}
/* emcNonParabolicAnistropValley.hpp:84-92 at energy 0 */
static double mdos0(const oc_valley *v) { return v->mdos * pow(1 + 2 * v->alpha * 0., 3.); }

/* per-mechanism getScatterRate */
static double scatter_rate(const oc_model *m, const oc_mech *me, double E,
                           int32_t region) {
  const oc_valley *vi = &m->v[me->valley];
  const oc_valley *vf = &m->v[me->finalValley];
  switch (me->kind) {
  case OC_ACOUSTIC: { /* emcAcousticScatterMechanism.hpp:114-121 */
    double md = mdos0(vi);
    double alpha = vi->alpha;
    double g = gamma_of(vi, E);
    return me->sc * pow(md, 3. / 2.) * sqrt(g) * (2 * alpha * E + 1.0);
  }
  case OC_ZERO_IV_ABS:
  case OC_ZERO_IV_EMI: { /* ...ZeroOrder...hpp:231-245, 374-388 */
    double Ef = me->kind == OC_ZERO_IV_ABS ? E + me->p1 - me->deltaValley
                                           : E - me->p1 - me->deltaValley;
    if (Ef > 0) {
      double md = mdos0(vf);
      double alpha = vf->alpha;
      double g = gamma_of(vf, Ef);
      return me->sc * pow(md, 3. / 2.) * sqrt(g) * (2 * alpha * Ef + 1.0);
    }
    return 0;
  }
  case OC_FIRST_IV_ABS:
  case OC_FIRST_IV_EMI: { /* ...FirstOrder...hpp:102-119, 252-269 */
    double Ef = me->kind == OC_FIRST_IV_ABS ? E + me->p1 - me->deltaValley
                                            : E - me->p1 - me->deltaValley;
    if (Ef > 0) {
      double md = mdos0(vf);
      double alpha = vf->alpha;
      double g = gamma_of(vi, E);
      double gF = gamma_of(vf, Ef);
      return me->sc * pow(md, 5. / 2.) * sqrt(gF) * (2 * alpha * Ef + 1.0) *
             (g + gF);
    }
    return 0;
  }
  case OC_COULOMB: { /* emcCoulombScatterMechanism.hpp:36-46 */
    double doping = fabs(m->regionDoping[region]);
    double md = mdos0(vi);
    double mc = vi->mc * (1 + 2 * 0. * vi->alpha);
    double alpha = vi->alpha;
    double g = gamma_of(vi, E);
    return me->sc1 * pow(md, 3. / 2.) / doping * sqrt(g) * (2 * alpha * E + 1.0) /
           (1 + (me->sc2 * mc * g / doping));
  }
  }
  return 0;
}

/* include/emcScatterHandler.hpp:248-273: cumulative sums in table order
   (std::transform with std::plus, :256-261), the maximum of the last row
   (:264-265), every table divided by it (:267-270), tau = 1 / maximum (:271). */
static void renormalize_set(oc_model *m, int v, int r) {
  int L = m->nLevels, nT = m->tsN[v][r];
  if (nT == 0) {
    m->tau[v][r] = 2e-15;
    return;
  }
  double *nt = m->norm[v][r];
  memcpy(nt, m->raw[v][r], sizeof(double) * (size_t)nT * L);
  for (int t = 1; t < nT; t++)
    for (int l = 0; l < L; l++)
      nt[t * L + l] = nt[t * L + l] + nt[(t - 1) * L + l];
  double mx = nt[(nT - 1) * L];
  for (int l = 1; l < L; l++)
    if (mx < nt[(nT - 1) * L + l])
      mx = nt[(nT - 1) * L + l];
  for (int i = 0; i < nT * L; i++)
    nt[i] /= mx;
  m->tau[v][r] = 1. / mx;
}

/* include/emcScatterHandler.hpp:100-108 (reinitScatterTables) with the
   refilled rates supplied by the caller: nT x nLevels doubles, table-major. */
int32_t oc_set_raw_tables(oc_model *m, int32_t v, int32_t r, const double *raw) {
  if (oc_n_tables(m, v, r) < 0 || !m->built)
    return -1;
  memcpy(m->raw[v][r], raw, sizeof(double) * (size_t)m->tsN[v][r] * m->nLevels);
  renormalize_set(m, v, r);
  return 0;
}

/* include/emcScatterHandler.hpp:220-235 (fill) and :248-273 (renormalize) */
int32_t oc_build_tables(oc_model *m) {
  int L = m->nLevels;
  for (int v = 0; v < OC_MAX_VALLEYS; v++)
    for (int r = 0; r < OC_MAX_REGIONS; r++) {
      if (!m->tsUsed[v][r])
        continue;
      int nT = m->tsN[v][r];
      free(m->raw[v][r]);
      free(m->norm[v][r]);
      m->raw[v][r] = (double *)malloc(sizeof(double) * (size_t)(nT > 0 ? nT : 1) * L);
      m->norm[v][r] = (double *)malloc(sizeof(double) * (size_t)(nT > 0 ? nT : 1) * L);
      for (int t = 0; t < nT; t++) {
        const oc_mech *me = &m->mech[m->tsMech[v][r][t]];
        for (int l = 0; l < L; l++)
          m->raw[v][r][t * L + l] = scatter_rate(m, me, (l + 1) * m->dE, r);
      }
      renormalize_set(m, v, r);
    }
  m->built = 1;
  return 0;
}

int32_t oc_n_tables(const oc_model *m, int32_t v, int32_t r) {
  if (v < 0 || v >= OC_MAX_VALLEYS || r < 0 || r >= OC_MAX_REGIONS || !m->tsUsed[v][r])
    return -1;
  return m->tsN[v][r];
}
int32_t oc_table_mech(const oc_model *m, int32_t v, int32_t r, int32_t t) {
  if (oc_n_tables(m, v, r) <= t)
    return -1;
  return m->tsMech[v][r][t];
}
int32_t oc_get_raw_table(const oc_model *m, int32_t v, int32_t r, int32_t t,
                         double *out) {
  if (oc_n_tables(m, v, r) <= t || !m->built)
    return -1;
  memcpy(out, m->raw[v][r] + (size_t)t * m->nLevels, sizeof(double) * m->nLevels);
  return 0;
}
int32_t oc_get_norm_table(const oc_model *m, int32_t v, int32_t r, int32_t t,
                          double *out) {
  if (oc_n_tables(m, v, r) <= t || !m->built)
    return -1;
  memcpy(out, m->norm[v][r] + (size_t)t * m->nLevels, sizeof(double) * m->nLevels);
  return 0;
}

/* include/emcScatterHandler.hpp:79-84 */
double oc_get_tau(const oc_model *m, int32_t v, int32_t r) {
  if (v >= 0 && v < OC_MAX_VALLEYS && r >= 0 && r < OC_MAX_REGIONS && m->tsUsed[v][r])
    return m->tau[v][r];
  return 2e-15;
}

void oc_valley_consts(const oc_model *m, int32_t valley, double out[8]) {
  const oc_valley *v = &m->v[valley];
  out[0] = v->mc;
  out[1] = v->mdos;
  out[2] = v->alpha;
  out[3] = v->vogt[0];
  out[4] = v->vogt[1];
  out[5] = v->vogt[2];
  out[6] = v->bottom;
  out[7] = v->deg;
}
void oc_valley_rot(const oc_model *m, int32_t valley, double *out) {
  memcpy(out, m->v[valley].rot, sizeof(double) * 9 * m->v[valley].deg);
}

/* ======================================================================== */
/* valley kinematics (emcNonParabolicAnistropValley.hpp)                    */
/* ======================================================================== */

/* :140-153 */
static void to_ecs(const double *R, const double *a, double *o) {
  o[0] = a[0] * R[0] + a[1] * R[1] + a[2] * R[2];
  o[1] = a[0] * R[3] + a[1] * R[4] + a[2] * R[5];
  o[2] = a[0] * R[6] + a[1] * R[7] + a[2] * R[8];
}
/* :157-170 */
static void to_dev(const double *R, const double *a, double *o) {
  o[0] = a[0] * R[0] + a[1] * R[3] + a[2] * R[6];
  o[1] = a[0] * R[1] + a[1] * R[4] + a[2] * R[7];
  o[2] = a[0] * R[2] + a[1] * R[5] + a[2] * R[8];
}

/* :109-113 */
double oc_energy(const oc_model *m, int32_t valley, const double k[3]) {
  const oc_valley *v = &m->v[valley];
  double sq = 0;
  for (int i = 0; i < 3; i++)
    sq += k[i] * k[i];
  double g = C_HBAR * C_HBAR * sq / (v->mc * C_Q);
  return g / (1 + sqrt(1 + 2 * v->alpha * g));
}

/* :103-106 */
double oc_norm_wave_vec(const oc_model *m, int32_t valley, double E) {
  const oc_valley *v = &m->v[valley];
  return sqrt(2 * v->mc * gamma_of(v, E) * C_Q) / C_HBAR;
}

/* :126-136 */
void oc_velocity(const oc_model *m, int32_t valley, int32_t sub,
                 const double k[3], double E, double out[3]) {
  const oc_valley *v = &m->v[valley];
  double ve[3], w[3];
  to_ecs(v->rot[sub], k, ve);
  double npf = sqrt(1 + 4 * v->alpha * gamma_of(v, E));
  for (int i = 0; i < 3; i++)
    w[i] = C_HBAR * v->vogt[i] * ve[i] / (v->mc * npf);
  to_dev(v->rot[sub], w, out);
}

/* include/emcParticleDrift.hpp:11-36 */
void oc_drift(const oc_model *m, double dt, double k[3], double *E,
              int32_t valley, int32_t sub, double *pos, int32_t dim,
              const double force[3]) {
  const oc_valley *v = &m->v[valley];
  const double *R = v->rot[sub];
  double kOld[3], kNew[3], fE[3], dPos[3], dd[3];
  to_ecs(R, k, kOld);
  memcpy(kNew, kOld, 24);
  to_ecs(R, force, fE);
  for (int i = 0; i < 3; i++)
    kNew[i] += fE[i] * dt * v->vogt[i] / C_HBAR;
  to_dev(R, kNew, k);
  *E = oc_energy(m, valley, k);
  double mcE = v->mc * (1 + 2 * *E * v->alpha);
  for (int i = 0; i < 3; i++) {
    double avgK = (kNew[i] + kOld[i]) / 2;
    dPos[i] = C_HBAR * v->vogt[i] * avgK * dt / mcE;
  }
  to_dev(R, dPos, dd);
  for (int i = 0; i < dim; i++)
    pos[i] = pos[i] + dd[i];
}

/* include/emcUtil.hpp:131-139 */
static void random_direction(double nrm, double r1, double r2, double *o) {
  double phi = 2 * C_PI * r1;
  double ct = 1 - 2 * r2;
  o[0] = nrm * sqrt(1 - ct * ct) * cos(phi);
  o[1] = nrm * sqrt(1 - ct * ct) * sin(phi);
  o[2] = nrm * ct;
}

/* two draws in the compiled reference's argument order */
static void random_direction_draw(double nrm, dctx *d, double *o) {
#if OC_ARGS_RIGHT_TO_LEFT
  double r2 = oci_draw_u01(d);
  double r1 = oci_draw_u01(d);
#else
  double r1 = oci_draw_u01(d);
  double r2 = oci_draw_u01(d);
#endif
  random_direction(nrm, r1, r2, o);
}

/* include/emcUtil.hpp:141-175 */
static void random_direction_wrt_k(const double *k, double ct, double rnd,
                                   double *o) {
  double kxy = sqrt(k[0] * k[0] + k[1] * k[1]);
  double nK = sqrt(kxy * kxy + k[2] * k[2]);
  if (nK == 0.) {
    o[0] = o[1] = o[2] = 0.;
    return;
  }
  double ct0 = k[2] / nK;
  double st0 = kxy / nK;
  double cfi0 = (kxy > 0.) ? k[0] / kxy : 1.;
  double sfi0 = (kxy > 0.) ? k[1] / kxy : 0.;
  double st = sqrt(1.0 - ct * ct);
  double phi = 2.0 * C_PI * rnd;
  double kxp = nK * st * cos(phi);
  double kyp = nK * st * sin(phi);
  double kzp = nK * ct;
  o[0] = kxp * cfi0 * ct0 - kyp * sfi0 + kzp * cfi0 * st0;
  o[1] = kxp * sfi0 * ct0 + kyp * cfi0 + kzp * sfi0 * st0;
  o[2] = -kxp * st0 + kzp * ct0;
}

/* emcGrainScatterMechanism::scatterParticle
   (include/emcGrainScatterMechanism.hpp:41-80): reflected (into the opposite
   hemisphere, cos(theta) <= 0) when a draw exceeds the transmission
   probability, else transmitted (same hemisphere); |k| is kept and the
   energy is not updated.  No mechanism: a no-op
   (include/emcScatterHandler.hpp:193-196). */
void oci_grain_scatter(const oc_model *m, double *k, dctx *d) {
  if (!m->grain)
    return;
  const int reflect = oci_draw_u01(d) > m->grainProb;
  double rnd = oci_draw_u01(d);
  if (reflect) {
    if (rnd < 0.5)
      rnd += 0.5;
  } else if (rnd > 0.5) {
    rnd -= 0.5;
  }
  const double kin[3] = {k[0], k[1], k[2]};
  random_direction_wrt_k(kin, 1 - 2 * rnd, oci_draw_u01(d), k);
}

/* include/emcScatterHandler.hpp:237-244 with the x86-64 size_t conversion of
   floor(E/dE) - 1 (-1 -> 0; other negatives and NaN wrap to the top level) */
static int32_t energy_level(const oc_model *m, double E) {
  double f = floor(E / m->dE) - 1;
  if (!(f >= 0.))
    return (f == -1.) ? 0 : m->nLevels - 1;
  if (f > (double)(m->nLevels - 1))
    return m->nLevels - 1;
  return (int32_t)f;
}

/* per-mechanism scatterParticle */
static void mech_scatter(const oc_model *m, const oc_mech *me, double *k,
                         double *E, int32_t *valley, int32_t *sub,
                         int32_t region, dctx *d) {
  switch (me->kind) {
  case OC_ACOUSTIC: { /* emcAcousticScatterMechanism.hpp:124-126 */
    double s = 0;
    for (int i = 0; i < 3; i++)
      s += k[i] * k[i];
    random_direction_draw(sqrt(s), d, k);
    break;
  }
  case OC_ZERO_IV_ABS:
  case OC_FIRST_IV_ABS:
  case OC_ZERO_IV_EMI:
  case OC_FIRST_IV_EMI: { /* ...ZeroOrder...hpp:247-257, 390-400 etc. */
    *valley = me->finalValley;
    *sub = me->finalSub[*sub][oci_draw_pick(d, (uint32_t)me->nF)];
    if (me->kind == OC_ZERO_IV_ABS || me->kind == OC_FIRST_IV_ABS)
      *E += (me->p1 - me->deltaValley);
    else
      *E -= (me->p1 + me->deltaValley);
    double knew = oc_norm_wave_vec(m, me->finalValley, *E);
    random_direction_draw(knew, d, k);
    break;
  }
  case OC_COULOMB: { /* emcCoulombScatterMechanism.hpp:48-59 */
    const oc_valley *v = &m->v[me->valley];
    double g = gamma_of(v, *E);
    double doping = fabs(m->regionDoping[region]);
    double mc = v->mc * (1 + 2 * 0. * v->alpha);
    double rnd = oci_draw_u01(d);
    double debye = doping / (me->sc2 * mc);
    double ct = 1.0 - rnd * 2.0 / ((1 - rnd) * g / debye + 1.0);
    double kin[3] = {k[0], k[1], k[2]};
    random_direction_wrt_k(kin, ct, oci_draw_u01(d), k);
    break;
  }
  }
}

/* include/emcScatterHandler.hpp:148-170; returns -1 if the (valley, region)
   pair has no table set (the reference's std::map::at throws there) */
int32_t oci_handler_scatter(const oc_model *m, double *k, double *E,
                               int32_t *valley, int32_t *sub, int32_t region,
                               dctx *d) {
  int v = *valley;
  if (v < 0 || v >= OC_MAX_VALLEYS || region < 0 || region >= OC_MAX_REGIONS ||
      !m->tsUsed[v][region])
    return -1;
  int nT = m->tsN[v][region];
  if (nT == 0)
    return 0;
  const double *nt = m->norm[v][region];
  int L = m->nLevels;
  int32_t lvl = energy_level(m, *E);
  double rnd = oci_draw_u01(d);
  if (rnd > nt[(nT - 1) * L + lvl])
    return 0;
  double lo = 0, hi;
  for (int t = 0; t < nT; t++) {
    hi = nt[t * L + lvl];
    if (rnd >= lo && rnd < hi) {
      mech_scatter(m, &m->mech[m->tsMech[v][region][t]], k, E, valley, sub,
                   region, d);
      break;
    }
    lo = hi;
  }
  return 0;
}

/* include/ParticleType/emcParticleType.hpp:187-189 */
double oci_new_tau(const oc_model *m, int32_t valley, int32_t region,
                      dctx *d) {
  return -log(oci_draw_ulog(d)) * oc_get_tau(m, valley, region);
}

/* ======================================================================== */
/* bulk path                                                                */
/* ======================================================================== */

/* examples/bulkSimulation/basicBulkParticleHandler.hpp:600-613 */
static void bulk_drift(const oc_model *m, double dt, double *k, double *E,
                       int32_t valley, int32_t sub, double *pos,
                       const double force[3], const double box[3]) {
  oc_drift(m, dt, k, E, valley, sub, pos, 3, force);
  for (int i = 0; i < 3; i++) {
    double c = pos[i];
    if (c < 0)
      pos[i] = c + box[i];
    else if (c > box[i])
      pos[i] = c - box[i];
  }
}

/* basicBulkParticleHandler.hpp:195-220 for one particle */
static int32_t bulk_particle_step(const oc_model *m, oc_particles *p, int64_t i,
                                  double dt, const double force[3],
                                  const double box[3], dctx *d) {
  double k[3] = {p->kx[i], p->ky[i], p->kz[i]};
  double pos[3] = {p->px[i], p->py[i], p->pz[i]};
  double E = p->E[i], tau = p->tau[i], gtau = p->gtau[i];
  int32_t valley = p->valley[i], sub = p->sub[i], region = p->region[i];
  int32_t st = 0;
  bulk_drift(m, (dt < tau) ? dt : tau, k, &E, valley, sub, pos, force, box);
  double tRem = dt - tau;
  while (tRem > 0) {
    if (oci_handler_scatter(m, k, &E, &valley, &sub, region, d) < 0) {
      st = -1;
      break;
    }
    double nt = oci_new_tau(m, valley, region, d);
    tau += nt;
    bulk_drift(m, (nt < tRem) ? nt : tRem, k, &E, valley, sub, pos, force, box);
    tRem -= nt;
  }
  tau -= dt;
  gtau -= dt;
  if (gtau <= 0) { /* basicBulkParticleHandler.hpp:215-219 */
    oci_grain_scatter(m, k, d);
    gtau = -log(oci_draw_ulog(d)) * m->grainTau;
  }
  p->kx[i] = k[0];
  p->ky[i] = k[1];
  p->kz[i] = k[2];
  p->px[i] = pos[0];
  p->py[i] = pos[1];
  p->pz[i] = pos[2];
  p->E[i] = E;
  p->tau[i] = tau;
  p->gtau[i] = gtau;
  p->valley[i] = valley;
  p->sub[i] = sub;
  return d->fail ? -2 : st;
}

int32_t oc_bulk_step(const oc_model *m, oc_particles *p, double dt,
                     const double force[3], const double box[3], oc_rng *r,
                     uint32_t step, int64_t *offsets) {
  int32_t st = 0;
  for (int64_t i = 0; i < p->n; i++) {
    dctx d;
    oci_dctx_init(&d, r, (uint32_t)i, step, r->stream);
    if (offsets)
      offsets[i] = r->rec_n;
    int32_t s = bulk_particle_step(m, p, i, dt, force, box, &d);
    if (s && !st)
      st = s;
  }
  if (offsets)
    offsets[p->n] = r->rec_n;
  return st;
}

static void accum_obs(const oc_model *m, const oc_particles *p, int64_t i,
                      const double dir[3], double *acc /* nV*3 */) {
  int32_t v = p->valley[i];
  double k[3] = {p->kx[i], p->ky[i], p->kz[i]}, vel[3];
  oc_velocity(m, v, p->sub[i], k, p->E[i], vel);
  acc[v * 3 + 0] += p->E[i];
  acc[v * 3 + 1] += vel[0] * dir[0] + vel[1] * dir[1] + vel[2] * dir[2];
  acc[v * 3 + 2] += 1.;
}

int32_t oc_bulk_run_philox(const oc_model *m, oc_particles *p, double dt,
                           const double force[3], const double box[3],
                           const double fieldDir[3], uint64_t seed,
                           uint32_t stream, uint32_t step0, int32_t nSteps,
                           int32_t nThreads, double *obs, int32_t words32) {
  int nV = m->nV;
  int32_t status = 0;
#ifdef _OPENMP
  if (nThreads > 0)
    omp_set_num_threads(nThreads);
#endif
  for (int s = 0; s < nSteps; s++) {
    double tot[OC_MAX_VALLEYS * 3];
    memset(tot, 0, sizeof(tot));
#ifdef _OPENMP
#pragma omp parallel
#endif
    {
      double acc[OC_MAX_VALLEYS * 3];
      memset(acc, 0, sizeof(acc));
      oc_rng r;
      memset(&r, 0, sizeof(r));
      r.mode = words32 ? OC_RNG_PHILOX32 : OC_RNG_PHILOX;
      r.seed = seed;
      r.stream = stream;
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
      for (int64_t i = 0; i < p->n; i++) {
        dctx d;
        oci_dctx_init(&d, &r, (uint32_t)i, step0 + (uint32_t)s, stream);
        if (bulk_particle_step(m, p, i, dt, force, box, &d))
          status = -1;
        if (obs)
          accum_obs(m, p, i, fieldDir, acc);
      }
#ifdef _OPENMP
#pragma omp critical
#endif
      for (int j = 0; j < nV * 3; j++)
        tot[j] += acc[j];
    }
    if (obs)
      for (int j = 0; j < nV * 3; j++)
        obs[(size_t)s * nV * 3 + j] = tot[j];
  }
  return status;
}

int32_t oc_model_n_valleys(const oc_model *m) { return m->nV; }

/* One Philox step of every particle with its own force (3 x n planes):
   FMMBulkParticleHandler::moveParticles
   (examples/bulkSimulationFMM/FMMBulkParticleHandler.hpp:233-277), whose
   per-particle step is the bulk handler's with that force. */
int32_t oc_bulk_step_forces(const oc_model *m, oc_particles *p, double dt,
                            const double *forces, const double box[3],
                            const double fieldDir[3], uint64_t seed, uint32_t stream,
                            uint32_t step, int32_t nThreads, double *obs) {
  int nV = m->nV;
  int32_t status = 0;
  const int64_t n = p->n;
  double tot[OC_MAX_VALLEYS * 3];
  memset(tot, 0, sizeof(tot));
#ifdef _OPENMP
  if (nThreads > 0)
    omp_set_num_threads(nThreads);
#pragma omp parallel
#endif
  {
    double acc[OC_MAX_VALLEYS * 3];
    memset(acc, 0, sizeof(acc));
    oc_rng r;
    memset(&r, 0, sizeof(r));
    r.mode = OC_RNG_PHILOX;
    r.seed = seed;
    r.stream = stream;
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
    for (int64_t i = 0; i < n; i++) {
      dctx d;
      oci_dctx_init(&d, &r, (uint32_t)i, step, stream);
      const double f[3] = {forces[i], forces[n + i], forces[2 * n + i]};
      if (bulk_particle_step(m, p, i, dt, f, box, &d))
        status = -1;
      if (obs)
        accum_obs(m, p, i, fieldDir, acc);
    }
#ifdef _OPENMP
#pragma omp critical
#endif
    for (int j = 0; j < nV * 3; j++)
      tot[j] += acc[j];
  }
  if (obs)
    for (int j = 0; j < nV * 3; j++)
      obs[j] = tot[j];
  return status;
}

/* examples/bulkSimulation/basicBulkParticleHandler.hpp:289-347 */
void oc_observables(const oc_model *m, const oc_particles *p,
                    const double dir[3], double *out) {
  int nV = m->nV;
  double sE[OC_MAX_VALLEYS] = {0}, sV[OC_MAX_VALLEYS] = {0};
  double cnt[OC_MAX_VALLEYS] = {0};
  int64_t ci[OC_MAX_VALLEYS] = {0};
  for (int64_t i = 0; i < p->n; i++) {
    int32_t v = p->valley[i];
    double k[3] = {p->kx[i], p->ky[i], p->kz[i]}, vel[3];
    oc_velocity(m, v, p->sub[i], k, p->E[i], vel);
    sE[v] += p->E[i];
    sV[v] += vel[0] * dir[0] + vel[1] * dir[1] + vel[2] * dir[2];
    cnt[v]++;
    ci[v]++;
  }
  for (int v = 0; v < nV; v++) {
    out[v * 3 + 0] = ci[v] ? sE[v] / (double)ci[v] : 0.;
    out[v * 3 + 1] = ci[v] ? sV[v] / (double)ci[v] : 0.;
    out[v * 3 + 2] = p->n ? cnt[v] / (double)p->n : 0.;
  }
}

/* include/emcParticleInitialization.hpp:14-29 */
void oci_init_pos(const int64_t *coord, const int64_t *ext,
                     const double *h, int32_t dim, dctx *d, double *pos) {
  for (int i = 0; i < dim; i++) {
    if (coord[i] == ext[i] - 1)
      pos[i] = ((double)coord[i] - oci_draw_u01(d) * 0.5) * h[i];
    else if (coord[i] == 0)
      pos[i] = oci_draw_u01(d) * 0.5 * h[i];
    else
      pos[i] = ((double)coord[i] + oci_draw_u01(d) - 0.5) * h[i];
  }
}

/* include/ParticleType/emcElectron.hpp:75-90 (+ initParticleKSpaceMaxwellian,
   include/emcParticleInitialization.hpp:36-51).  tauRegionIsValley mirrors
   examples/mosfet2D/electronVWD.hpp:73 (getNewTau(valley, valley)). */
void oci_init_particle(const oc_model *m, const int64_t *coord,
                            const int64_t *ext, const double *h, int32_t dim,
                            int32_t region, double Vt, dctx *d,
                            oc_particles *p, int64_t idx,
                            int32_t tauRegionIsValley) {
  double pos[3] = {0, 0, 0};
  oci_init_pos(coord, ext, h, dim, d, pos);
  int32_t valley = (int32_t)floor((double)m->nV * oci_draw_ulog(d));
  int32_t sub = (int32_t)floor((double)m->v[valley].deg * oci_draw_ulog(d));
  double E = -1.5 * Vt * log(oci_draw_ulog(d));
  double k[3];
  random_direction_draw(oc_norm_wave_vec(m, valley, E), d, k);
  for (int i = 0; i < dim; i++)
    if ((coord[i] == 0 && k[i] < 0) || (coord[i] == ext[i] - 1 && k[i] > 0))
      k[i] *= -1;
  double tau = -log(oci_draw_ulog(d)) *
               oc_get_tau(m, valley, tauRegionIsValley ? valley : region);
  double gtau = -log(oci_draw_ulog(d)) * m->grainTau;
  p->kx[idx] = k[0];
  p->ky[idx] = k[1];
  p->kz[idx] = k[2];
  p->px[idx] = pos[0];
  p->py[idx] = pos[1];
  if (p->pz)
    p->pz[idx] = pos[2];
  p->E[idx] = E;
  p->tau[idx] = tau;
  p->gtau[idx] = gtau;
  p->valley[idx] = valley;
  p->sub[idx] = sub;
  p->region[idx] = region;
}

void oc_init_particle(const oc_model *m, const int64_t coord[3],
                      const int64_t extent[3], const double spacing[3],
                      int32_t dim, int32_t region, double thermalVoltage,
                      oc_rng *r, oc_particles *p, int64_t idx,
                      int32_t tauRegionIsValley) {
  dctx d;
  oci_dctx_init(&d, r, (uint32_t)idx, 0xFFFFFFFFu, r->stream);
  oci_init_particle(m, coord, extent, spacing, dim, region, thermalVoltage, &d, p,
                  idx, tauRegionIsValley);
}

/* examples/bulkSimulation/basicBulkParticleHandler.hpp:143-159 with
   emcElectron::getInitialNrParticles (usePotentialForInit = false),
   include/ParticleType/emcElectron.hpp:48-61 */
int64_t oc_bulk_init(const oc_model *m, const double maxPos[3],
                     const double spacing[3], double doping, oc_rng *r,
                     oc_particles *p, int64_t cap) {
  int64_t ext[3];
  for (int i = 0; i < 3; i++)
    ext[i] = (int64_t)round(maxPos[i] / spacing[i]) + 1;
  double cellVol = 1.;
  for (int i = 0; i < 3; i++)
    cellVol = cellVol * spacing[i];
  double Vt = C_KB / C_Q * m->T;
  int64_t n = 0;
  int64_t c[3];
  for (c[2] = 0; c[2] < ext[2]; c[2]++)
    for (c[1] = 0; c[1] < ext[1]; c[1]++)
      for (c[0] = 0; c[0] < ext[0]; c[0]++) {
        double nr = doping;
        for (int i = 0; i < 3; i++)
          if (c[i] == 0 || c[i] == ext[i] - 1)
            nr *= 0.5;
        nr = nr * cellVol;
        while (nr >= 1) {
          if (n >= cap)
            return -1;
          dctx d;
          oci_dctx_init(&d, r, (uint32_t)n, 0xFFFFFFFFu, r->stream);
          oci_init_particle(m, c, ext, spacing, 3, 0, Vt, &d, p, n, 0);
          n++;
          nr--;
        }
        dctx d;
        oci_dctx_init(&d, r, (uint32_t)n, 0xFFFFFFFEu, r->stream);
        if (oci_draw_u01(&d) < nr) {
          if (n >= cap)
            return -1;
          oci_dctx_init(&d, r, (uint32_t)n, 0xFFFFFFFFu, r->stream);
          oci_init_particle(m, c, ext, spacing, 3, 0, Vt, &d, p, n, 0);
          n++;
        }
      }
  p->n = n;
  return n;
}
int32_t oci_nvalleys(const oc_model *m) { return m->nV; }
