// Grid Poisson solver of the device engine.
//
// Discrete equation (include/PoissonSolver/emcSORSolver.hpp:131-197,
// 330-412), Debye-normalised, at every node that is not a reservoir contact:
//   F_i(phi) = sum_d hF_d (phi_{i-d} + phi_{i+d} - 2 phi_i)      (mirror at
//              artificial boundaries)
//            + hP (p_i - n_i + C_i) + G_i (Vg_i - phi_i) = 0
// with p = exp(-phi), n = the carrier concentration (non-equilibrium) or
// exp(phi) (equilibrium), G the gate Robin coefficient.  The reference's
// lexicographic SOR reaches the fixed point of this equation; here it is
// solved by Newton / defect correction in double precision whose correction
// equation J d = -F is solved approximately by a few multigrid V-cycles
// per iteration (red-black Gauss-Seidel, bilinear transfer, finite-volume
// coarse operators), in float or double.  The solve stops when
// max|F| <= rtol * max(hP (|C| + n + p)), the scale taken at the first
// iteration.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

namespace emcg {

// static per-node data of the fine grid (host arrays)
struct PoissonSetup {
  int nx = 0, ny = 0;
  double h[2] = {0, 0};       // normalised spacing
  std::vector<uint8_t> fixed; // Dirichlet (reservoir) nodes
  std::vector<double> C;      // normalised doping
  std::vector<double> gSum;   // sum of gate coefficients G at the node
  std::vector<double> gVeq;   // sum of G * barrier
  std::vector<double> gVne;   // sum of G * (barrier + applied)
  std::vector<double> gDensX; // FV Robin density of an x-side gate (gF / 2)
  std::vector<double> gDensY; // FV Robin density of a y-side gate
  std::vector<uint8_t> resetMask; // nodes whose value resetBC sets
  std::vector<double> resetEq, resetNe; // and the values it sets
};

struct MGLevel {
  int nx, ny;
  // FV coefficients (w, e, s, n), area and static diagonal (couplings + Robin)
  float *cw, *ce, *cs, *cn, *area, *diag0;
  double *dcw, *dce, *dcs, *dcn, *darea, *ddiag0;
  uint8_t *fixed;
  float *d, *r, *rho;    // correction, right-hand side, reaction density (float MG)
  double *dd, *dr, *drho; // the same in double (double MG)
  // transfer to the next coarser level
  int *rxIdx, *ryIdx;      // restriction: 3 fine indices per coarse index
  float *rxW, *ryW;
  int *pxIdx, *pyIdx;      // prolongation: lower coarse index per fine index
  float *pxW, *pyW;        // weight of the lower coarse node
  int *mapX, *mapY;        // coarse index -> fine index (injection)
  // coefficient classes of the cluster solve: per node an index into a table
  // of the distinct (cw, ce, cs, cn, area, diag0, fixed) tuples of the level,
  // 8 entries of the multigrid type per class; nCls = 0: more than 255 classes
  uint8_t *cls;
  void *clsTab;
  int nCls;
};

struct PoissonMG {
  PoissonSetup S;
  std::vector<MGLevel> L;
  // fine-grid device data (double)
  double *C = nullptr, *gSum = nullptr, *gVeq = nullptr, *gVne = nullptr;
  uint8_t *resetMask = nullptr;
  double *resetEq = nullptr, *resetNe = nullptr;
  double *stats = nullptr; // [max|F|, scale, max|d|] as ordered bits
  double *expTab = nullptr; // 2^(j/256), j < 256, for the residual's exp
  // red-black sweeps before and after the coarse correction, and sweeps on
  // the coarsest level
  int pre = 3, post = 3, coarseSweeps = 16;
  // V-cycles on the correction equation per Newton step once the relative
  // residual is below twoCycleRel, one above it (and one under the update-size
  // rule below, which needs only a rough correction).  Measured on the 201 x 101
  // resistor (device steps of 5e5 electrons): three V-cycles of three sweeps
  // from the first Newton step take 2 Newton steps per solve and the least
  // time; two V-cycles of two sweeps from 1e-2 took 4.8 and 14 % longer.
  int vcyclesPerNewton = 3;
  double twoCycleRel = 1e30;
  // the reference's SOR stopping rule as an alternative: stop once a Newton
  // update changes no potential by more than updTol (thermal voltages; 0 = off)
  double updTol = 0.;
  bool fp32 = true;
  double hF[2], hP;
  // single-launch cluster solve: CTAs per cluster (0 = not available for this
  // grid) and its dynamic shared memory; useCluster = 0 forces the
  // multi-launch path
  int clusterSize = 0;
  size_t clusterSmem = 0;
  bool clusterEven = true; // the layout's bands have even rows (see clusterDesc)
  bool useCluster = true;
  // upper bound on clusterSize set by the caller (0: none)
  int clusterCap = 0;
  // the plan for batchFor solves side by side (emcg_device_step_many) under
  // the bound batchCap; batchFor = 0: none yet
  int batchFor = 0, batchCap = 0, batchSize = 0;
  size_t batchSmem = 0;
  bool batchEven = true;
  // page-locked block, mapped into the device's address space, into which an
  // enqueued cluster solve (poissonEnqueue) writes its [relative residual,
  // Newton steps, stopped by the update rule]
  double *hStats = nullptr, *hStatsDev = nullptr; // host and device addresses
};

int32_t poissonCreate(PoissonMG &P, const PoissonSetup &S, bool fp32, int smooth,
                      cudaStream_t st);
void poissonFree(PoissonMG &P);
// Solve for pot (device, normalised).  conc == nullptr: equilibrium.
// Returns EMCG_OK / EMCG_ERR_NONCONVERGED / EMCG_ERR_CUDA; outputs the final
// relative residual and the number of Newton steps.
int32_t poissonSolve(PoissonMG &P, double *pot, const double *conc, bool resetBC,
                     double rtol, int maxCycles, cudaStream_t st, double *relRes,
                     int *cycles);
// The cluster solve without waiting for it: enqueues the solve and the copy
// of its statistics on st and returns *queued = true; poissonFinish, once st
// has passed that copy, gives what poissonSolve returns.  Where the grid has
// no cluster solve it runs poissonSolve and returns *queued = false.
int32_t poissonEnqueue(PoissonMG &P, double *pot, const double *conc, bool resetBC, double rtol,
                       int maxCycles, cudaStream_t st, bool *queued, double *relRes,
                       int *cycles);
int32_t poissonFinish(PoissonMG &P, double rtol, double *relRes, int *cycles);
// Re-plan the cluster solve (clusterSize, clusterSmem) under P.clusterCap so
// that `concurrent` solves of this size fit on the device at once (engines
// stepped side by side); falls back to the plan for one solve at a time.
int32_t poissonPlanCluster(PoissonMG &P, int concurrent);

} // namespace emcg
