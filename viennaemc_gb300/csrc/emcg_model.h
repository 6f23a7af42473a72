// Host-side conversion and validation of emcg_model_desc into the kernel
// structs of emcg_common.cuh.  Shared by the bulk and device engines.
#pragma once

#include <cmath>
#include <cstring>
#include <vector>

#include "emcg_common.cuh"
#include "emcg_host.h"

namespace emcg {

struct ValleyDerived {
  double mc;      // conduction mass [kg]
  double vogt[3]; // Herring-Vogt factors
};

// include/ValleyTypes/emcNonParabolicAnistropValley.hpp:185-204
inline ValleyDerived deriveValley(const emcg_valley_desc &v) {
  ValleyDerived d;
  double acc = 0.;
  for (int i = 0; i < 3; i++)
    acc += 1. / v.rel_mass[i];
  d.mc = 3. * v.particle_mass / acc;
  for (int i = 0; i < 3; i++)
    d.vogt[i] = std::sqrt(d.mc / (v.rel_mass[i] * v.particle_mass));
  return d;
}

inline int32_t validateModel(const emcg_model_desc &m) {
  EMCG_CHECK_ARG(m.n_valleys >= 1 && m.n_valleys <= EMCG_MAX_VALLEYS,
                 "model: n_valleys=%d out of [1,%d]", m.n_valleys, EMCG_MAX_VALLEYS);
  EMCG_CHECK_ARG(m.valleys != nullptr, "model: valleys is NULL");
  EMCG_CHECK_ARG(m.n_mechs >= 0 && m.n_mechs <= EMCG_MAX_MECH,
                 "model: n_mechs=%d out of [0,%d]", m.n_mechs, EMCG_MAX_MECH);
  EMCG_CHECK_ARG(m.n_mechs == 0 || m.mechs != nullptr, "model: mechs is NULL");
  EMCG_CHECK_ARG(m.n_tablesets >= 0 && m.n_tablesets <= EMCG_MAX_TABLESETS,
                 "model: n_tablesets=%d out of range", m.n_tablesets);
  EMCG_CHECK_ARG(m.n_tablesets == 0 || m.tablesets != nullptr, "model: tablesets is NULL");
  EMCG_CHECK_ARG(m.n_levels >= 1 && m.n_levels <= (1 << 24), "model: n_levels=%d invalid",
                 m.n_levels);
  EMCG_CHECK_ARG(m.max_energy > 0 && std::isfinite(m.max_energy),
                 "model: max_energy must be positive");
  EMCG_CHECK_ARG(m.grain_tau > 0 && std::isfinite(m.grain_tau),
                 "model: grain_tau must be positive");
  EMCG_CHECK_ARG(m.grain == 0 || m.grain == 1, "model: grain must be 0 or 1");
  EMCG_CHECK_ARG(m.grain == 0 || std::isfinite(m.grain_transmission),
                 "model: grain_transmission must be finite");
  for (int b = 0; b < 4; b++) {
    EMCG_CHECK_ARG(m.surface_kind[b] >= EMCG_SURFACE_SPECULAR &&
                       m.surface_kind[b] <= EMCG_SURFACE_ROUGHNESS,
                   "model: surface_kind[%d]=%d unknown", b, m.surface_kind[b]);
    EMCG_CHECK_ARG(m.surface_kind[b] != EMCG_SURFACE_ROUGHNESS ||
                       (m.surface_param[b] > 0 && std::isfinite(m.surface_param[b])),
                   "model: surface_param[%d] (roughness height) must be positive", b);
    EMCG_CHECK_ARG(m.surface_kind[b] != EMCG_SURFACE_CONSTANT ||
                       std::isfinite(m.surface_param[b]),
                   "model: surface_param[%d] (specularity) must be finite", b);
  }
  for (int v = 0; v < m.n_valleys; v++) {
    const emcg_valley_desc &V = m.valleys[v];
    EMCG_CHECK_ARG(V.deg >= 1 && V.deg <= EMCG_MAX_DEG, "valley %d: deg=%d out of [1,%d]", v,
                   V.deg, EMCG_MAX_DEG);
    EMCG_CHECK_ARG(V.particle_mass > 0 && V.alpha >= 0, "valley %d: bad mass or alpha", v);
    for (int i = 0; i < 3; i++)
      EMCG_CHECK_ARG(V.rel_mass[i] > 0, "valley %d: relative mass must be positive", v);
  }
  for (int i = 0; i < m.n_mechs; i++) {
    const emcg_mech_desc &M = m.mechs[i];
    EMCG_CHECK_ARG(M.kind >= EMCG_MECH_ACOUSTIC && M.kind <= EMCG_MECH_COULOMB,
                   "mechanism %d: unknown kind %d", i, M.kind);
    EMCG_CHECK_ARG(M.valley >= 0 && M.valley < m.n_valleys, "mechanism %d: bad valley", i);
    if (M.kind >= EMCG_MECH_ZERO_IV_ABS && M.kind <= EMCG_MECH_FIRST_IV_EMI) {
      EMCG_CHECK_ARG(M.final_valley >= 0 && M.final_valley < m.n_valleys,
                     "mechanism %d: bad final valley", i);
      EMCG_CHECK_ARG(M.n_final >= 1 && M.n_final <= EMCG_MAX_NF,
                     "mechanism %d: n_final=%d out of [1,%d]", i, M.n_final, EMCG_MAX_NF);
      int degI = m.valleys[M.valley].deg, degF = m.valleys[M.final_valley].deg;
      for (int s = 0; s < degI; s++)
        for (int f = 0; f < M.n_final; f++)
          EMCG_CHECK_ARG(M.final_sub[s][f] >= 0 && M.final_sub[s][f] < degF,
                         "mechanism %d: final subvalley %d invalid", i, M.final_sub[s][f]);
    }
    if (M.kind == EMCG_MECH_COULOMB)
      EMCG_CHECK_ARG(M.coulomb_sc2 > 0, "mechanism %d: coulomb_sc2 must be positive", i);
  }
  bool seen[EMCG_MAX_VALLEYS][EMCG_MAX_REGIONS] = {};
  bool anyTables = false;
  for (int t = 0; t < m.n_tablesets; t++) {
    const emcg_tableset_desc &S = m.tablesets[t];
    EMCG_CHECK_ARG(S.valley >= 0 && S.valley < m.n_valleys && S.region >= 0 &&
                       S.region < EMCG_MAX_REGIONS,
                   "tableset %d: bad (valley, region)", t);
    EMCG_CHECK_ARG(!seen[S.valley][S.region], "tableset %d: duplicate (valley, region)", t);
    seen[S.valley][S.region] = true;
    EMCG_CHECK_ARG(S.n_tables >= 0 && S.n_tables <= EMCG_MAX_MECH, "tableset %d: bad n_tables",
                   t);
    for (int j = 0; j < S.n_tables; j++) {
      EMCG_CHECK_ARG(S.mech[j] >= 0 && S.mech[j] < m.n_mechs,
                     "tableset %d: mechanism index %d invalid", t, S.mech[j]);
      EMCG_CHECK_ARG(m.mechs[S.mech[j]].valley == S.valley,
                     "tableset %d: mechanism %d belongs to another valley", t, S.mech[j]);
    }
    if (S.n_tables > 0) {
      anyTables = true;
      EMCG_CHECK_ARG(S.tau_max > 0 && std::isfinite(S.tau_max), "tableset %d: bad tau_max", t);
    }
  }
  EMCG_CHECK_ARG(!anyTables || m.tables != nullptr, "model: tables is NULL");
  return EMCG_OK;
}

// Fill the kernel model (without the tables pointer) and the level-major
// table array of one model.
template <class T>
int32_t buildModelK(const emcg_model_desc &m, ModelK<T> &K, std::vector<T> &tables) {
  EMCG_TRY(validateModel(m));
  std::memset(&K, 0, sizeof(K));
  K.nV = m.n_valleys;
  K.nLevels = m.n_levels;
  K.nTS = m.n_tablesets;
  double dE = m.max_energy / (double)m.n_levels;
  K.dE = (T)dE;
  K.invdE = (T)(1.0 / dE);
  K.grainTau = (T)m.grain_tau;
  K.grain = m.grain;
  K.grainProb = m.grain ? (T)m.grain_transmission : T(0);
  for (int b = 0; b < 4; b++) {
    K.surfKind[b] = m.surface_kind[b];
    K.surfParam[b] = (T)m.surface_param[b];
  }
  std::vector<double> mcOf(m.n_valleys);
  for (int v = 0; v < m.n_valleys; v++) {
    const emcg_valley_desc &V = m.valleys[v];
    ValleyDerived d = deriveValley(V);
    mcOf[v] = d.mc;
    ValleyK<T> &O = K.v[v];
    for (int s = 0; s < V.deg; s++)
      for (int i = 0; i < 9; i++)
        O.rot[s][i] = (T)V.rot[s][i];
    for (int i = 0; i < 3; i++) {
      O.vogt[i] = (T)d.vogt[i];
      O.cF[i] = (T)(d.vogt[i] / kHBAR);
    }
    O.cE = (T)(kHBAR * kHBAR / (d.mc * kQ));
    O.alpha = (T)V.alpha;
    O.cK = (T)(std::sqrt(2 * d.mc * kQ) / kHBAR);
    O.cX = (T)(kHBAR / d.mc);
    O.deg = V.deg;
  }
  for (int i = 0; i < m.n_mechs; i++) {
    const emcg_mech_desc &M = m.mechs[i];
    MechK<T> &O = K.m[i];
    O.kind = M.kind;
    O.finalValley = (M.kind >= EMCG_MECH_ZERO_IV_ABS && M.kind <= EMCG_MECH_FIRST_IV_EMI)
                        ? M.final_valley
                        : M.valley;
    O.nF = M.n_final;
    O.shift = (T)M.shift;
    for (int s = 0; s < EMCG_MAX_DEG; s++)
      for (int f = 0; f < EMCG_MAX_NF; f++)
        O.finalSub[s][f] = (uint8_t)M.final_sub[s][f];
    if (M.kind == EMCG_MECH_COULOMB)
      for (int r = 0; r < EMCG_MAX_REGIONS; r++) // debyeEnergy (:55)
        O.debye[r] = (T)(std::fabs(m.region_doping[r]) / (M.coulomb_sc2 * mcOf[M.valley]));
  }
  for (int v = 0; v < EMCG_MAX_VALLEYS; v++)
    for (int r = 0; r < EMCG_MAX_REGIONS; r++)
      K.tsIndex[v][r] = -1;
  int64_t off = 0;
  tables.clear();
  const int L = m.n_levels;
  int64_t srcOff = 0;
  for (int t = 0; t < m.n_tablesets; t++) {
    const emcg_tableset_desc &S = m.tablesets[t];
    K.tsIndex[S.valley][S.region] = (int8_t)t;
    K.tsN[t] = S.n_tables;
    K.tsOff[t] = off;
    K.tauMax[t] = (T)(S.n_tables > 0 ? S.tau_max : 2e-15);
    for (int j = 0; j < S.n_tables; j++)
      K.tsMech[t][j] = (uint8_t)S.mech[j];
    const int nT = S.n_tables;
    tables.resize((size_t)(off + (int64_t)nT * L));
    for (int j = 0; j < nT; j++)
      for (int l = 0; l < L; l++)
        tables[(size_t)(off + (int64_t)l * nT + j)] = (T)m.tables[srcOff + (int64_t)j * L + l];
    off += (int64_t)nT * L;
    srcOff += (int64_t)nT * L;
  }
  if (tables.empty())
    tables.push_back(T(0));
  return EMCG_OK;
}

} // namespace emcg
