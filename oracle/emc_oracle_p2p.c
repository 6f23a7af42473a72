/* Oracle (test infrastructure only): the particle-particle Coulomb sums of
 * the reference's FMM handlers, evaluated directly.
 *
 * The pair kernel restates FP2PRCutoff::NonMutualParticles
 * (include/ParticleHandler/FMM/FP2PRCutoff.hpp:64-100): for target t and
 * source s, d = x_t - x_s, 1/r^2, 1/r; closer than the cutoff radius the
 * separation is rescaled to the cutoff (:76-86); then
 *   force_t += -q_t q_s d / r^3,   potential_t += q_s / r.
 * The FMM (scalFMM, absent here) evaluates the same sum with multipole
 * expansions for far pairs; the direct sum is its exact value.  Periodic
 * images: the box is repeated `images` times on each side in x, y and z, and
 * every target sums over all copies (its own copies included, itself in the
 * central box excluded).  The reference's own pair kernel, compiled by the
 * harness, pins this restatement bit for bit. */
#include <math.h>
#include <stdint.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include <stdlib.h>
#include <string.h>

#include "emc_oracle.h"

void oc_p2p_pair(double xt, double yt, double zt, double qt, double xs, double ys, double zs,
                 double qs, double invCut, double out[4]) {
  double dx = xt - xs, dy = yt - ys, dz = zt - zs;
  double inv2 = 1.0 / (dx * dx + dy * dy + dz * dz);
  double inv = sqrt(inv2);
  if (invCut > 0 && inv > invCut) { /* :76-86 */
    double f = inv * (1.0 / invCut);
    dx *= f;
    dy *= f;
    dz *= f;
    inv = invCut;
    inv2 = invCut * invCut;
  }
  inv2 *= inv;
  inv2 *= qt * qs;
  out[0] = dx * -inv2;
  out[1] = dy * -inv2;
  out[2] = dz * -inv2;
  out[3] = inv * qs;
}

int32_t oc_p2p_coulomb(const double *pos, const double *q, int64_t n, double invCut,
                       double box, int32_t images, double *force, double *pot,
                       int32_t threads) {
  if (n < 0 || images < 0 || (images > 0 && !(box > 0)))
    return -1;
  const double *x = pos, *y = pos + n, *z = pos + 2 * n;
#ifdef _OPENMP
  if (threads > 0)
    omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 64)
#endif
  for (int64_t i = 0; i < n; i++) {
    double fx = 0, fy = 0, fz = 0, p = 0, o[4];
    for (int a = -images; a <= images; a++)
      for (int b = -images; b <= images; b++)
        for (int c = -images; c <= images; c++) {
          const double ox = a * box, oy = b * box, oz = c * box;
          const int central = a == 0 && b == 0 && c == 0;
          for (int64_t j = 0; j < n; j++) {
            if (central && j == i)
              continue;
            oc_p2p_pair(x[i], y[i], z[i], q[i], x[j] + ox, y[j] + oy, z[j] + oz, q[j], invCut,
                        o);
            fx += o[0];
            fy += o[1];
            fz += o[2];
            p += o[3];
          }
        }
    force[i] = fx;
    force[n + i] = fy;
    force[2 * n + i] = fz;
    pot[i] = p;
  }
  return 0;
}

/* FMMBulkParticleHandler's step loop (examples/bulkSimulationFMM/
   bulkSimulationFMM.cpp:150-168): executeFMM (the Coulomb sums over the moving
   particles, charge q, and the fixed charges) then moveParticles with
   force = q field - (ke / epsR) x sum (getForceAtParticle,
   FMMBulkParticleHandler.hpp:433-440), ke from the reference's constants
   (include/emcConstants.hpp:9, 21, 27). */
int32_t oc_bulk_run_coulomb(const oc_model *m, oc_particles *p, double dt, double q,
                            const double field[3], const double box[3],
                            const double fieldDir[3], const double *fixedPos,
                            const double *fixedQ, int64_t nFixed, double epsR, double invCut,
                            int32_t images, uint64_t seed, uint32_t stream, uint32_t step0,
                            int32_t nSteps, int32_t threads, double *obs) {
  const double ke = 1. / (4 * 3.14159265358979323846 * 8.85419e-12);
  const int64_t n = p->n, mm = n + nFixed;
  double *src = (double *)malloc(sizeof(double) * (size_t)(4 * mm + 1));
  double *fc = (double *)malloc(sizeof(double) * (size_t)(3 * mm + 1));
  double *pot = (double *)malloc(sizeof(double) * (size_t)(mm + 1));
  double *force = (double *)malloc(sizeof(double) * (size_t)(3 * n + 1));
  int32_t st = 0;
  for (int s = 0; s < nSteps && !st; s++) {
    for (int64_t i = 0; i < n; i++) {
      src[i] = p->px[i];
      src[mm + i] = p->py[i];
      src[2 * mm + i] = p->pz[i];
      src[3 * mm + i] = q;
    }
    for (int64_t j = 0; j < nFixed; j++) {
      src[n + j] = fixedPos[j];
      src[mm + n + j] = fixedPos[nFixed + j];
      src[2 * mm + n + j] = fixedPos[2 * nFixed + j];
      src[3 * mm + n + j] = fixedQ[j];
    }
    if (oc_p2p_coulomb(src, src + 3 * mm, mm, invCut, box[0], images, fc, pot, threads)) {
      st = -1;
      break;
    }
    for (int64_t i = 0; i < n; i++)
      for (int v = 0; v < 3; v++)
        force[v * n + i] = q * field[v] + -(ke / epsR) * fc[v * mm + i];
    st = oc_bulk_step_forces(m, p, dt, force, box, fieldDir, seed, stream, step0 + (uint32_t)s,
                             threads, obs ? obs + (size_t)s * oc_model_n_valleys(m) * 3 : NULL);
  }
  free(src);
  free(fc);
  free(pot);
  free(force);
  return st;
}
