// A recording stand-in of libemcgpu's device entry points, for running the
// C++ plugins under the reference's emcSimulation on a machine without a GPU
// (tests/test_adapter.py).  It does no physics: each call is written to the
// log named by EMCG_STUB_LOG, and returns values the test can predict:
//   Poisson:   phi <- phi / 2 + 1 (equilibrium) or phi / 2 + 0.1
//   field:     Ex = 1000 phi, Ey = -1000 phi
//   move:      3 - c particles removed at contact c
//   contacts:  c + 1 injected minus deleted at contact c
//   assign:    2 particles at every node
// Particle states are kept as uploaded.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <vector>

#include "emcgpu.h"

struct emcg_handle {
  int nx = 0, ny = 0, nc = 0;
  std::map<int, std::vector<double>> grid;
  std::vector<double> f[9];
  std::vector<int32_t> idx[3];
  int64_t n = 0;
};

static FILE *logf() {
  static FILE *f = std::fopen(std::getenv("EMCG_STUB_LOG") ? std::getenv("EMCG_STUB_LOG")
                                                           : "/dev/null",
                              "w");
  return f;
}

extern "C" {
const char *emcg_last_error(void) { return "stub"; }

int32_t emcg_device_create(const emcg_model_desc *m, const emcg_device_desc *d,
                           const emcg_device_config *c, int32_t precision, emcg_handle **out) {
  auto *h = new emcg_handle;
  h->nx = d->nx;
  h->ny = d->ny;
  h->nc = d->n_contacts;
  for (int w = 0; w < 5; w++)
    h->grid[w].assign((size_t)h->nx * h->ny, 0.);
  std::fprintf(logf(), "create %d %d %d pm=%d dt=%a seed=%llu carriers=%a charge=%a cap=%lld "
                       "prec=%d mechs=%d levels=%d\n",
               h->nx, h->ny, h->nc, c->pm_scheme, c->dt, (unsigned long long)c->seed,
               c->carriers_per_particle, c->charge, (long long)c->capacity, precision,
               m->n_mechs, m->n_levels);
  *out = h;
  return EMCG_OK;
}
int32_t emcg_destroy(emcg_handle *h) {
  std::fprintf(logf(), "destroy\n");
  std::fflush(logf());
  delete h;
  return EMCG_OK;
}
int32_t emcg_device_set_grid(emcg_handle *h, int32_t which, const double *v) {
  auto &g = h->grid[which];
  double sum = 0;
  for (size_t i = 0; i < g.size(); i++)
    sum += (g[i] = v[i]);
  std::fprintf(logf(), "set %d %a %a\n", which, sum, g[g.size() / 2 + 3]);
  return EMCG_OK;
}
int32_t emcg_device_get_grid(emcg_handle *h, int32_t which, double *v) {
  const auto &g = h->grid[which];
  for (size_t i = 0; i < g.size(); i++)
    v[i] = g[i];
  std::fprintf(logf(), "get %d\n", which);
  return EMCG_OK;
}
int32_t emcg_device_poisson(emcg_handle *h, int32_t equilibrium, int32_t reset_bc,
                            double *rel, int32_t *cycles) {
  for (double &p : h->grid[EMCG_GRID_POTENTIAL])
    p = p / 2 + (equilibrium ? 1. : 0.1);
  *rel = 0;
  *cycles = 1;
  std::fprintf(logf(), "poisson %d %d\n", equilibrium, reset_bc);
  return EMCG_OK;
}
int32_t emcg_device_efield(emcg_handle *h) {
  const auto &p = h->grid[EMCG_GRID_POTENTIAL];
  for (size_t i = 0; i < p.size(); i++) {
    h->grid[EMCG_GRID_EX][i] = 1000 * p[i];
    h->grid[EMCG_GRID_EY][i] = -1000 * p[i];
  }
  std::fprintf(logf(), "efield\n");
  return EMCG_OK;
}
int32_t emcg_device_move(emcg_handle *h, uint32_t step, int32_t *netto) {
  for (int c = 0; c < h->nc; c++)
    netto[c] = 3 - c;
  std::fprintf(logf(), "move %u\n", step);
  return EMCG_OK;
}
int32_t emcg_device_contacts(emcg_handle *h, uint32_t step, int32_t *rem_inj) {
  for (int c = 0; c < h->nc; c++)
    rem_inj[c] = c + 1;
  std::fprintf(logf(), "contacts %u\n", step);
  return EMCG_OK;
}
int32_t emcg_device_assign(emcg_handle *h) {
  for (double &x : h->grid[EMCG_GRID_NRPART])
    x = 2.;
  std::fprintf(logf(), "assign\n");
  return EMCG_OK;
}
int32_t emcg_set_state(emcg_handle *h, int32_t ens, const emcg_state *s) {
  const double *src[9] = {s->kx, s->ky, s->kz, s->px, s->py, s->pz, s->energy, s->tau,
                          s->grain_tau};
  const int32_t *isrc[3] = {s->valley, s->sub, s->region};
  double esum = 0;
  for (int k = 0; k < 9; k++)
    h->f[k].assign(src[k], src[k] + s->n);
  for (int k = 0; k < 3; k++)
    h->idx[k].assign(isrc[k], isrc[k] + s->n);
  for (int64_t i = 0; i < s->n; i++)
    esum += s->energy[i];
  h->n = s->n;
  std::fprintf(logf(), "state %d %lld %a\n", ens, (long long)s->n, esum);
  return EMCG_OK;
}
int32_t emcg_get_state(emcg_handle *h, int32_t ens, emcg_state *s) {
  double *dst[9] = {s->kx, s->ky, s->kz, s->px, s->py, s->pz, s->energy, s->tau, s->grain_tau};
  int32_t *idst[3] = {s->valley, s->sub, s->region};
  for (int k = 0; k < 9; k++)
    for (int64_t i = 0; i < h->n; i++)
      dst[k][i] = h->f[k][i];
  for (int k = 0; k < 3; k++)
    for (int64_t i = 0; i < h->n; i++)
      idst[k][i] = h->idx[k][i];
  s->n = h->n;
  std::fprintf(logf(), "getstate %d\n", ens);
  return EMCG_OK;
}
int64_t emcg_num_particles(emcg_handle *h, int32_t) { return h->n; }
}
