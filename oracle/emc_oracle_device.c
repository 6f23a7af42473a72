/*
 * CPU oracle for the ViennaEMC device (2-D) path -- TEST INFRASTRUCTURE ONLY.
 * Restates, operation by operation, the reference's particle-mesh schemes,
 * boundary handling, device drift/scatter loop, ohmic contacts, carrier
 * concentration and SOR Poisson solver (paths relative to the reference
 * project root).  Build with -ffp-contract=off.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "emc_oracle.h"
#include "emc_oracle_internal.h"

#define C_Q 1.60219e-19
#define C_KB 1.38066e-23
#define C_EPS0 8.85419e-12

static double vt_of(const oc_dev *d) { return C_KB / C_Q * d->T; }

/* include/emcDevice.hpp:88-90 */
double oc_dev_debye(const oc_dev *d) {
  return sqrt(C_EPS0 * d->epsR * vt_of(d) / C_Q / d->Ni);
}

/* include/emcDevice.hpp:333-343 (2-D: times the device width) */
double oc_dev_cell_volume(const oc_dev *d) {
  double v = 1.;
  v = v * d->hx;
  v = v * d->hy;
  return v * d->width;
}

/* ---- surface (include/emcSurface.hpp) ---------------------------------- */
static int on_boundary(const oc_dev *d, int x, int y, int b) {
  switch (b) {
  case OC_XMIN: return x == 0;
  case OC_XMAX: return x == d->nx - 1;
  case OC_YMIN: return y == 0;
  default: return y == d->ny - 1;
  }
}
/* getBoundaryPos: the first boundary (XMIN, XMAX, YMIN, YMAX) holding the
   node (:340-349) */
static int boundary_pos(const oc_dev *d, int x, int y) {
  for (int b = 0; b < 4; b++)
    if (on_boundary(d, x, y, b))
      return b;
  return -1;
}
static int coord_on(int x, int y, int b) { return b < 2 ? y : x; } /* :303-315 */
static int idx_at(const oc_dev *d, int b, int c) { return d->bnd[b][c]; }

/* :87-94 */
int32_t oc_dev_contact_idx(const oc_dev *d, int32_t x, int32_t y) {
  int b = boundary_pos(d, x, y);
  return b < 0 ? -1 : idx_at(d, b, coord_on(x, y, b));
}
static int is_type_at(const oc_dev *d, int b, int c, int type) { /* :233-237 */
  int i = idx_at(d, b, c);
  return i != -1 && d->ctype[i] == type;
}
static int is_ohmic(const oc_dev *d, int x, int y) { /* :240-246 */
  int b = boundary_pos(d, x, y);
  return b >= 0 && is_type_at(d, b, coord_on(x, y, b), OC_OHMIC);
}
int32_t oc_dev_is_reservoir(const oc_dev *d, int32_t x, int32_t y) { /* :260-262 */
  int b = boundary_pos(d, x, y);
  if (b < 0)
    return 0;
  int c = coord_on(x, y, b);
  return is_type_at(d, b, c, OC_OHMIC) || is_type_at(d, b, c, OC_SCHOTTKY);
}

/* include/emcDevice.hpp:290-297 */
static void pos_to_coord(const oc_dev *d, const double *pos, int64_t *c) {
  c[0] = (int64_t)round(pos[0] / d->hx);
  c[1] = (int64_t)round(pos[1] / d->hy);
}

/* ---- E field (include/PMSchemes/emcEFieldCalculation.hpp:13-30, 58-81) --- */
static void efield_boundary(const oc_dev *d, double *Ex, double *Ey);

void oc_dev_efield(const oc_dev *d, const double *pot, double *Ex, double *Ey) {
  const int nx = d->nx, ny = d->ny;
  const double Vt = vt_of(d);
  for (int y = 0; y < ny; y++)
    for (int x = 0; x < nx; x++) {
      int i = y * nx + x;
      if (x != 0 && x != nx - 1)
        Ex[i] = (pot[i - 1] - pot[i + 1]) * Vt / (2 * d->hx);
      if (y != 0 && y != ny - 1)
        Ey[i] = (pot[i - nx] - pot[i + nx]) * Vt / (2 * d->hy);
    }
  efield_boundary(d, Ex, Ey);
}

/* The field of a PM scheme.  NGP, CIC: at the grid points (above).  NEC
   (include/PMSchemes/emcNECScheme.hpp:115-119 with calcEFieldAtEdgeMidPts,
   emcEFieldCalculation.hpp:35-52): forward differences on the edges, the
   boundary values as for the grid-point field.  NEC-VWD
   (examples/mosfet2D/NECSchemeVWD.hpp, calcEField): forward differences, 0 on
   the last edge of each direction, no boundary pass. */
void oc_dev_efield_pm(const oc_dev *d, int32_t scheme, const double *pot, double *Ex,
                      double *Ey) {
  const int nx = d->nx, ny = d->ny;
  const double Vt = vt_of(d);
  if (scheme == OC_NGP || scheme == OC_CIC) {
    oc_dev_efield(d, pot, Ex, Ey);
    return;
  }
  for (int y = 0; y < ny; y++)
    for (int x = 0; x < nx; x++) {
      int i = y * nx + x;
      if (scheme == OC_NEC) {
        if (x != 0 && x != nx - 1)
          Ex[i] = (pot[i] - pot[i + 1]) * Vt / d->hx;
        if (y != 0 && y != ny - 1)
          Ey[i] = (pot[i] - pot[i + nx]) * Vt / d->hy;
      } else {
        Ex[i] = x != nx - 1 ? (pot[i] - pot[i + 1]) * Vt / d->hx : 0.;
        Ey[i] = y != ny - 1 ? (pot[i] - pot[i + nx]) * Vt / d->hy : 0.;
      }
    }
  if (scheme == OC_NEC)
    efield_boundary(d, Ex, Ey);
}

/* boundary values: 0 normal to an artificial boundary, else the neighbour */
static void efield_boundary(const oc_dev *d, double *Ex, double *Ey) {
  const int nx = d->nx, ny = d->ny;
  for (int b = 0; b < 4; b++) {
    int n = b < 2 ? ny : nx;
    for (int c = 0; c < n; c++) {
      int x = b < 2 ? (b == OC_XMIN ? 0 : nx - 1) : c;
      int y = b < 2 ? c : (b == OC_YMIN ? 0 : ny - 1);
      int i = y * nx + x;
      double *E = b < 2 ? Ex : Ey;
      int stride = b < 2 ? 1 : nx;
      if (idx_at(d, b, c) == -1)
        E[i] = 0;
      else if (b % 2 == 0)
        E[i] = E[i + stride];
      else
        E[i] = E[i - stride];
    }
  }
}

/* ---- particle -> mesh (NGP: emcNGPScheme.hpp:21-44; CIC: emcCICScheme.hpp:
   30-42 with the reference's weight wX on the lower node) -------------- */
static void grid_add(const oc_dev *d, double *g, int64_t x, int64_t y, double v) {
  /* out-of-grid corners (a particle exactly on the far boundary) are
     dropped; the reference aborts there */
  if (x < 0 || y < 0 || x >= d->nx || y >= d->ny)
    return;
  g[y * d->nx + x] += v;
}

void oc_dev_assign(const oc_dev *d, int32_t scheme, const double *px,
                   const double *py, int64_t n, double nrC, double *grid) {
  for (int64_t i = 0; i < n; i++) {
    if (scheme == OC_NEC || scheme == OC_NEC_VWD) {
      /* a quarter to each corner of the element (emcNECScheme.hpp:24-33,
         NECSchemeVWD.hpp assignToMesh) */
      int64_t mx = (int64_t)floor(px[i] / d->hx), my = (int64_t)floor(py[i] / d->hy);
      double w = 0.25 * nrC;
      grid_add(d, grid, mx, my, w);
      grid_add(d, grid, mx + 1, my, w);
      grid_add(d, grid, mx, my + 1, w);
      grid_add(d, grid, mx + 1, my + 1, w);
    } else if (scheme == OC_NGP) {
      int64_t x = (int64_t)round(px[i] / d->hx), y = (int64_t)round(py[i] / d->hy);
      grid_add(d, grid, x, y, nrC);
    } else {
      int64_t mx = (int64_t)floor(px[i] / d->hx), my = (int64_t)floor(py[i] / d->hy);
      double wX = px[i] / d->hx - (double)mx;
      double wY = py[i] / d->hy - (double)my;
      grid_add(d, grid, mx, my, wX * wY * nrC);
      grid_add(d, grid, mx + 1, my, (1 - wX) * wY * nrC);
      grid_add(d, grid, mx, my + 1, wX * (1 - wY) * nrC);
      grid_add(d, grid, mx + 1, my + 1, (1 - wX) * (1 - wY) * nrC);
    }
  }
}

static double grid_get(const oc_dev *d, const double *g, int64_t x, int64_t y) {
  if (x < 0 || y < 0 || x >= d->nx || y >= d->ny)
    return 0;
  return g[y * d->nx + x];
}

/* NGP: emcNGPScheme.hpp:46-57; CIC: emcCICScheme.hpp:126-143, including its
   (1 - wY)(1 - wY) weight on the upper-right node */
void oc_dev_force(const oc_dev *d, int32_t scheme, const double *Ex,
                  const double *Ey, double x, double y, double charge,
                  double F[3]) {
  const double *E[2] = {Ex, Ey};
  if (scheme == OC_NEC || scheme == OC_NEC_VWD) {
    /* NEC (emcNECScheme.hpp:102-113): the two edges of the element along each
       direction; NEC-VWD (NECSchemeVWD.hpp interpolateForce) takes the nearest
       column and only the edge below on the last one */
    int64_t mx = scheme == OC_NEC ? (int64_t)floor(x / d->hx) : (int64_t)round(x / d->hx);
    int64_t my = (int64_t)floor(y / d->hy);
    F[0] = charge * (grid_get(d, Ex, mx, my) + grid_get(d, Ex, mx, my + 1)) / 2;
    if (scheme == OC_NEC_VWD && mx == d->nx - 1)
      F[1] = charge * grid_get(d, Ey, mx, my);
    else
      F[1] = charge * (grid_get(d, Ey, mx, my) + grid_get(d, Ey, mx + 1, my)) / 2;
  } else if (scheme == OC_NGP) {
    int64_t cx = (int64_t)round(x / d->hx), cy = (int64_t)round(y / d->hy);
    for (int k = 0; k < 2; k++)
      F[k] = charge * grid_get(d, E[k], cx, cy);
  } else {
    int64_t mx = (int64_t)floor(x / d->hx), my = (int64_t)floor(y / d->hy);
    double wX = x / d->hx - (double)mx;
    double wY = y / d->hy - (double)my;
    for (int k = 0; k < 2; k++)
      F[k] = charge * (grid_get(d, E[k], mx, my) * wX * wY +
                       grid_get(d, E[k], mx + 1, my) * (1 - wX) * wY +
                       grid_get(d, E[k], mx, my + 1) * wX * (1 - wY) +
                       grid_get(d, E[k], mx + 1, my + 1) * (1 - wY) * (1 - wY));
  }
  F[2] = 0;
}

/* ---- boundary (include/emcParticleDrift.hpp:41-66 with the default specular
   reflection of include/emcScatterHandler.hpp:172-191) ------------------ */
/* emcSurfaceScatterMechanism::scatterParticleSpecularly
   (include/SurfaceScatterMechanisms/emcSurfaceScatterMechanism.hpp:75-86):
   back into the device, k turned inwards only where it points out */
static void surface_specular(const oc_dev *d, double *pos, double *k) {
  const double mx[2] = {d->maxX, d->maxY};
  for (int i = 0; i < 2; i++)
    if (pos[i] < 0) {
      pos[i] *= -1;
      if (k[i] < 0)
        k[i] *= -1;
    } else if (pos[i] > mx[i]) {
      pos[i] = 2 * mx[i] - pos[i];
      if (k[i] > 0)
        k[i] *= -1;
    }
}

/* emcMomentumDependentSurfaceScatterMechanism::solveForTheta
   (include/SurfaceScatterMechanisms/emcMomentumDependentSurfaceScatterMechanism.hpp:
   38-66), the reference's fixed-point iteration as it stands (at most 10000
   steps, stopping below 1e-10) */
static double solve_for_theta(double r, double height, double speed) {
  const double c = pow(2 * height * speed, 2);
  const double e = exp(-c);
  const double start = sqrt(r * (1 / (1 - e) - 1 / c));
  double error = 1, x = start, x1;
  const double tol = 1e-10;
  int it = 0;
  const int maxIt = 10000;
  while (error > tol && it < maxIt) {
    const double co = cos(x), si = sin(x);
    const double ecos = exp(-c * pow(co, 2));
    const double esin = exp(-c * pow(si, 2));
    x1 = x - (((e - ecos) / c + pow(si, 2) - r * (1 - (1 - e) / c)) *
              (2 * esin * c * si * co * (ecos - 1)) / (e * (c - 1) - 1));
    error = fabs(x1 - x);
    x = x1;
    it++;
  }
  return x;
}

/* emcScatterHandler::scatterParticleAtBoundary (include/emcScatterHandler.hpp:
   172-191) with a surface mechanism at boundary b
   (emcSurfaceScatterMechanism::scatterParticle, :38-44, and
   calculateAndAssignKAndPos, :128-148): diffuse with the mechanism's
   probability (new direction into the device at polar angle theta from the
   normal), else specular */
static void surface_scatter(const oc_model *m, const oc_dev *d, int b, double *pos, double *k,
                            dctx *dc) {
  double param;
  const int kind = oci_surface(m, b, &param);
  const int perp = b / 2;
  double pDiff;
  if (kind == OC_SURFACE_CONSTANT) /* emcConstantSurfaceScatterMechanism.hpp:33 */
    pDiff = 1 - param;
  else /* emcMomentumDependentSurfaceScatterMechanism.hpp:23-27 */
    pDiff = 1 - (exp(-pow(2 * param * k[perp], 2)));
  if (oci_draw_u01(dc) < pDiff) {
    double theta;
    if (kind == OC_SURFACE_CONSTANT)
      theta = asin(sqrt(oci_draw_u01(dc)));
    else {
      const double sp = sqrt(k[0] * k[0] + k[1] * k[1] + k[2] * k[2]);
      theta = solve_for_theta(oci_draw_u01(dc), param, sp);
    }
    const double phi = 2 * 3.14159265358979323846 * oci_draw_u01(dc); /* constants::pi */
    const double speed = sqrt(k[0] * k[0] + k[1] * k[1] + k[2] * k[2]);
    const double sign = (b % 2 == 1) ? -1. : 1.;
    k[perp] = speed * cos(theta) * sign;
    k[(perp + 1) % 3] = speed * sin(theta) * cos(phi);
    k[(perp + 2) % 3] = speed * sin(theta) * sin(phi);
  }
  surface_specular(d, pos, k);
}

static int at_boundary(const oc_model *m, const oc_dev *d, double *pos, double *k, dctx *dc) {
  const double mx[2] = {d->maxX, d->maxY};
  int out = 0;
  for (int i = 0; i < 2; i++)
    if (pos[i] < 0 || pos[i] > mx[i])
      out = 1;
  if (!out)
    return 0;
  double pb[2];
  for (int i = 0; i < 2; i++) {
    double a = (mx[i] < pos[i]) ? mx[i] : pos[i]; /* std::min(pos, max) */
    pb[i] = (0. < a) ? a : 0.;                    /* std::max(0., .) */
  }
  int64_t c[2];
  pos_to_coord(d, pb, c);
  if (is_ohmic(d, (int)c[0], (int)c[1])) {
    pos[0] = pb[0];
    pos[1] = pb[1];
    return 1;
  }
  double sp;
  const int b = boundary_pos(d, (int)c[0], (int)c[1]);
  if (b >= 0 && oci_surface(m, b, &sp) != OC_SURFACE_SPECULAR) {
    surface_scatter(m, d, b, pos, k, dc);
    return 0;
  }
  for (int i = 0; i < 2; i++) {
    if (pos[i] < 0) {
      pos[i] = -pos[i];
      k[i] = -k[i];
    } else if (pos[i] > mx[i]) {
      pos[i] = 2 * mx[i] - pos[i];
      k[i] = -k[i];
    }
  }
  return 0;
}

/* emcAbstractParticleHandler::driftParticle (:238-249) */
static int dev_drift(const oc_model *m, const oc_dev *d, double dt, double *k,
                     double *E, int32_t valley, int32_t sub, int32_t *region,
                     double *pos, const double *F, dctx *dc) {
  oc_drift(m, dt, k, E, valley, sub, pos, 2, F);
  int removed = at_boundary(m, d, pos, k, dc);
  if (!removed) {
    int64_t c[2];
    pos_to_coord(d, pos, c);
    *region = d->region[c[1] * d->nx + c[0]];
  }
  return removed;
}

static void copy_particle(oc_particles *p, int64_t dst, int64_t src) {
  p->kx[dst] = p->kx[src];
  p->ky[dst] = p->ky[src];
  p->kz[dst] = p->kz[src];
  p->px[dst] = p->px[src];
  p->py[dst] = p->py[src];
  if (p->pz)
    p->pz[dst] = p->pz[src];
  p->E[dst] = p->E[src];
  p->tau[dst] = p->tau[src];
  p->gtau[dst] = p->gtau[src];
  p->valley[dst] = p->valley[src];
  p->sub[dst] = p->sub[src];
  p->region[dst] = p->region[src];
}

int32_t oc_dev_move(const oc_model *m, const oc_dev *d, int32_t scheme,
                    oc_particles *p, const double *Ex, const double *Ey,
                    double dt, double charge, oc_rng *r, uint32_t step,
                    int32_t *netto, int64_t *offsets) {
  int32_t status = 0;
  unsigned char *rem = (unsigned char *)calloc((size_t)(p->n > 0 ? p->n : 1), 1);
  for (int64_t i = 0; i < p->n; i++) {
    dctx dc;
    oci_dctx_init(&dc, r, (uint32_t)i, step, r->stream);
    if (offsets)
      offsets[i] = r->rec_n;
    double k[3] = {p->kx[i], p->ky[i], p->kz[i]};
    double pos[3] = {p->px[i], p->py[i], 0.};
    double E = p->E[i], tau = p->tau[i], gtau = p->gtau[i];
    int32_t valley = p->valley[i], sub = p->sub[i], region = p->region[i];
    double F[3];
    oc_dev_force(d, scheme, Ex, Ey, pos[0], pos[1], charge, F);
    int removed = 0;
    if (tau >= dt) {
      removed = dev_drift(m, d, dt, k, &E, valley, sub, &region, pos, F, &dc);
    } else {
      removed = dev_drift(m, d, tau, k, &E, valley, sub, &region, pos, F, &dc);
      double tRem = dt - tau;
      while (tRem > 0 && !removed) {
        if (oci_handler_scatter(m, k, &E, &valley, &sub, region, &dc) < 0) {
          status = -5;
          break;
        }
        double nt = oci_new_tau(m, valley, region, &dc);
        tau += nt;
        oc_dev_force(d, scheme, Ex, Ey, pos[0], pos[1], charge, F);
        removed = dev_drift(m, d, (nt < tRem) ? nt : tRem, k, &E, valley, sub, &region, pos, F,
                            &dc);
        tRem -= nt;
      }
    }
    tau -= dt;
    if (removed) {
      int64_t c[2];
      pos_to_coord(d, pos, c);
      int ci = oc_dev_contact_idx(d, (int)c[0], (int)c[1]);
      if (ci >= 0)
        netto[ci]++;
      rem[i] = 1;
    }
    gtau -= dt;
    if (gtau <= 0 && !removed) { /* emcBasicParticleHandler.hpp:131-138 */
      oci_grain_scatter(m, k, &dc);
      gtau = -log(oci_draw_ulog(&dc)) * oci_grain_tau(m);
    }
    p->kx[i] = k[0];
    p->ky[i] = k[1];
    p->kz[i] = k[2];
    p->px[i] = pos[0];
    p->py[i] = pos[1];
    p->E[i] = E;
    p->tau[i] = tau;
    p->gtau[i] = gtau;
    p->valley[i] = valley;
    p->sub[i] = sub;
    p->region[i] = region;
    if (dc.fail)
      status = -6;
  }
  if (offsets)
    offsets[p->n] = r->rec_n;
  /* removeParticles (:267-277): stable erase */
  int64_t w = 0;
  for (int64_t i = 0; i < p->n; i++)
    if (!rem[i]) {
      if (w != i)
        copy_particle(p, w, i);
      w++;
    }
  p->n = w;
  free(rem);
  return status;
}

/* include/ParticleType/emcElectron.hpp:63-73 (examples/mosfet2D/
   electronVWD.hpp:52-62 rounds the count) */
void oc_dev_exp_nr(const oc_dev *d, double *expNr, int32_t roundCounts) {
  double cv = oc_dev_cell_volume(d);
  for (int y = 0; y < d->ny; y++)
    for (int x = 0; x < d->nx; x++) {
      int i = y * d->nx + x;
      expNr[i] = 0;
      if (!oc_dev_is_reservoir(d, x, y))
        continue;
      double e = cv * d->doping[i];
      if (x == 0 || x == d->nx - 1)
        e *= 0.5;
      if (y == 0 || y == d->ny - 1)
        e *= 0.5;
      expNr[i] = roundCounts ? round(e) : e;
    }
}

int64_t oc_dev_contacts(const oc_model *m, const oc_dev *d, oc_particles *p,
                        int64_t cap, const double *expNr, double nrC,
                        oc_rng *r, uint32_t step, int32_t *remInj,
                        int32_t tauRegionIsValley) {
  const int nx = d->nx, ny = d->ny;
  double *nrPart = (double *)calloc((size_t)nx * ny, sizeof(double));
  /* count in index order, remove the excess (stable) */
  int64_t w = 0;
  for (int64_t i = 0; i < p->n; i++) {
    double pos[2] = {p->px[i], p->py[i]};
    int64_t c[2];
    pos_to_coord(d, pos, c);
    int keep = 1;
    if (oc_dev_is_reservoir(d, (int)c[0], (int)c[1])) {
      int64_t g = c[1] * nx + c[0];
      if (nrPart[g] < expNr[g])
        nrPart[g] += nrC;
      else {
        keep = 0;
        remInj[oc_dev_contact_idx(d, (int)c[0], (int)c[1])]--;
      }
    }
    if (keep) {
      if (w != i)
        copy_particle(p, w, i);
      w++;
    }
  }
  p->n = w;
  /* inject missing particles in grid order */
  const int64_t ext[3] = {nx, ny, 1};
  const double h[3] = {d->hx, d->hy, 0};
  const double Vt = vt_of(d);
  uint32_t serial = 0;
  for (int y = 0; y < ny; y++)
    for (int x = 0; x < nx; x++) {
      if (!oc_dev_is_reservoir(d, x, y))
        continue;
      int64_t g = (int64_t)y * nx + x;
      double diff = expNr[g] - nrPart[g];
      while (diff > 0) {
        if (p->n >= cap) {
          free(nrPart);
          return -7;
        }
        dctx dc;
        oci_dctx_init(&dc, r, serial++, step, r->stream | 0x80000000u);
        const int64_t c[3] = {x, y, 0};
        oci_init_particle(m, c, ext, h, 2, d->region[g], Vt, &dc, p, p->n,
                          tauRegionIsValley);
        p->n++;
        remInj[oc_dev_contact_idx(d, x, y)]++;
        diff -= nrC;
      }
    }
  free(nrPart);
  return p->n;
}

/* include/emcSimulationResults.hpp:98-116 */
void oc_dev_concentration(const oc_dev *d, const double *nrPart, double *conc) {
  double factor = 1. / oc_dev_cell_volume(d);
  for (int y = 0; y < d->ny; y++)
    for (int x = 0; x < d->nx; x++) {
      int i = y * d->nx + x;
      double c = nrPart[i] / d->Ni * factor;
      if (x == 0 || x == d->nx - 1)
        c *= 2;
      if (y == 0 || y == d->ny - 1)
        c *= 2;
      conc[i] = c;
    }
}

/* include/emcSimulationResults.hpp:208-213 */
void oc_dev_init_potential(const oc_dev *d, double *pot) {
  for (int i = 0; i < d->nx * d->ny; i++)
    pot[i] = asinh(0.5 * (d->doping[i] / d->Ni));
}

/* ---- SOR Poisson (include/PoissonSolver/emcSORSolver.hpp) --------------- */
int64_t oc_dev_sor(const oc_dev *d, double *pot, const double *eConc,
                   double omega, double accuracyVolt, int32_t resetBC,
                   int64_t maxSweeps) {
  const int nx = d->nx, ny = d->ny;
  const double Vt = vt_of(d), L = oc_dev_debye(d);
  const double h[2] = {d->hx / L, d->hy / L};                /* :31, normalised */
  const double hF[2] = {h[1] / h[0], h[0] / h[1]};           /* :332-334 */
  double hFsum = 0.;
  hFsum += hF[0];
  hFsum += hF[1];
  double hP = 1.;
  hP = hP * h[0];
  hP = hP * h[1];
  const double acc = accuracyVolt / Vt;
  const int maxC[2] = {nx - 1, ny - 1};
  double gF[64], gV[64], gB[64];
  for (int c = 0; c < d->nContacts && c < 64; c++) { /* :356-367 */
    gV[c] = d->cvolt[c] / Vt;
    gF[c] = gB[c] = 0;
    if (d->ctype[c] == OC_GATE) {
      double gamma = d->cpar[3 * c + 0] / d->epsR;
      double tox = d->cpar[3 * c + 1] / L;
      gF[c] = 2 * gamma / tox;
      gB[c] = d->cpar[3 * c + 2] / Vt;
    }
  }
  if (resetBC) { /* :137-153 (:55-69 without applied voltage) */
    for (int b = 0; b < 4; b++) {
      int n = b < 2 ? ny : nx;
      for (int c = 0; c < n; c++) {
        int ci = idx_at(d, b, c);
        if (ci < 0 || d->ctype[ci] != OC_OHMIC)
          continue;
        int x = b < 2 ? (b == OC_XMIN ? 0 : nx - 1) : c;
        int y = b < 2 ? c : (b == OC_YMIN ? 0 : ny - 1);
        int i = y * nx + x;
        double bi = asinh(0.5 * (d->doping[i] / d->Ni));
        pot[i] = eConc ? gV[ci] + bi : bi;
      }
    }
  }
  int64_t sweeps = 0;
  double error;
  do {
    error = 0;
    for (int y = 0; y < ny; y++)
      for (int x = 0; x < nx; x++) {
        if (oc_dev_is_reservoir(d, x, y))
          continue;
        int i = y * nx + x;
        double cur = pot[i], n, p, nom, den;
        double C = d->doping[i] / d->Ni;
        if (eConc) {
          p = exp(-cur);
          n = eConc[i];
        } else {
          n = exp(cur);
          p = 1. / n;
        }
        nom = hP * (p - n + C + cur * (p + n));
        den = 2 * hFsum + hP * (n + p);
        const int co[2] = {x, y};
        const int st[2] = {1, nx};
        for (int k = 0; k < 2; k++) {
          if (co[k] != 0)
            nom += pot[i - st[k]] * hF[k];
          else {
            nom += pot[i + st[k]] * hF[k];
            int b = 2 * k, cb = k == 0 ? y : x;
            if (is_type_at(d, b, cb, OC_GATE)) { /* :399-412 */
              int ci = idx_at(d, b, cb);
              double Vg = gB[ci];
              if (eConc)
                Vg += gV[ci];
              nom += gF[ci] * Vg * hF[k] * h[k];
              den += gF[ci] * hF[k] * h[k];
            }
          }
          if (co[k] != maxC[k])
            nom += pot[i + st[k]] * hF[k];
          else {
            nom += pot[i - st[k]] * hF[k];
            int b = 2 * k + 1, cb = k == 0 ? y : x;
            if (is_type_at(d, b, cb, OC_GATE)) {
              int ci = idx_at(d, b, cb);
              double Vg = gB[ci];
              if (eConc)
                Vg += gV[ci];
              nom += gF[ci] * Vg * hF[k] * h[k];
              den += gF[ci] * hF[k] * h[k];
            }
          }
        }
        double delta = omega * (nom / den - cur);
        pot[i] = cur + delta;
        if (fabs(delta) > error)
          error = fabs(delta);
      }
    sweeps++;
    if (sweeps >= maxSweeps)
      return error > acc ? -sweeps : sweeps;
  } while (error > acc);
  return sweeps;
}

int64_t oc_dev_init(const oc_model *m, const oc_dev *d, const double *pot,
                    int32_t roundCounts, double nrC, oc_rng *r, oc_particles *p,
                    int64_t cap, int32_t tauRegionIsValley) {
  const int nx = d->nx, ny = d->ny;
  const int64_t ext[3] = {nx, ny, 1};
  const double h[3] = {d->hx, d->hy, 0};
  const double Vt = vt_of(d), cv = oc_dev_cell_volume(d);
  int64_t n = 0;
  for (int y = 0; y < ny; y++)
    for (int x = 0; x < nx; x++) {
      int64_t g = (int64_t)y * nx + x;
      double e = pot ? exp(pot[g]) * d->Ni : d->doping[g];
      if (x == 0 || x == nx - 1)
        e *= 0.5;
      if (y == 0 || y == ny - 1)
        e *= 0.5;
      double nr = roundCounts ? round(e * cv) : e * cv;
      const int64_t c[3] = {x, y, 0};
      while (nr >= 1) {
        if (n >= cap)
          return -7;
        dctx dc;
        oci_dctx_init(&dc, r, (uint32_t)n, 0xFFFFFFFFu, r->stream);
        oci_init_particle(m, c, ext, h, 2, d->region[g], Vt, &dc, p, n, tauRegionIsValley);
        n++;
        nr -= nrC;
      }
      dctx dc;
      oci_dctx_init(&dc, r, (uint32_t)n, 0xFFFFFFFEu, r->stream);
      if (oci_draw_u01(&dc) < nr) {
        if (n >= cap)
          return -7;
        oci_dctx_init(&dc, r, (uint32_t)n, 0xFFFFFFFFu, r->stream);
        oci_init_particle(m, c, ext, h, 2, d->region[g], Vt, &dc, p, n, tauRegionIsValley);
        n++;
      }
    }
  p->n = n;
  return n;
}
