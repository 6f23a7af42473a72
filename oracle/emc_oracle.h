/*
 * CPU oracle for the ViennaEMC per-particle hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithm (ViennaTools/ViennaEMC, header-only C++17) used as the checker for
 * the sm_103a engine in viennaemc_gb300/.  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg may load it; the engine never calls it.
 *
 * Parity is pinned: oracle/ref_driver.cpp runs the reference's own classes
 * (compiled from its headers by oracle/Makefile) and tests/golden/ holds the
 * vectors it produced; tests/test_oracle_golden.py checks this restatement
 * against them bit for bit.
 *
 * Arithmetic follows the reference operation by operation (same association
 * order, no FMA contraction: build with -ffp-contract=off) so that with the
 * same mt19937_64 stream the oracle reproduces the reference's doubles exactly.
 */
#ifndef EMC_ORACLE_H
#define EMC_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OC_MAX_VALLEYS 4
#define OC_MAX_DEG 8
#define OC_MAX_MECH 32
#define OC_MAX_NF 8
#define OC_MAX_REGIONS 16
#define OC_MAX_TABLESETS (OC_MAX_VALLEYS * OC_MAX_REGIONS)

/* mechanism kinds (reference include/ScatterMechanisms/) */
enum {
  OC_ACOUSTIC = 0,     /* emcAcousticScatterMechanism.hpp:68-127 */
  OC_ZERO_IV_ABS = 1,  /* emcZeroOrderInterValleyScatterMechanism.hpp:165-257 */
  OC_ZERO_IV_EMI = 2,  /* emcZeroOrderInterValleyScatterMechanism.hpp:310-400 */
  OC_FIRST_IV_ABS = 3, /* emcFirstOrderInterValleyScatterMechanism.hpp:36-131 */
  OC_FIRST_IV_EMI = 4, /* emcFirstOrderInterValleyScatterMechanism.hpp:185-280 */
  OC_COULOMB = 5       /* emcCoulombScatterMechanism.hpp:11-60 */
};

/* random-number source modes */
enum {
  OC_RNG_MT = 0,     /* one sequential std::mt19937_64 (reference, no OpenMP) */
  OC_RNG_PHILOX = 1, /* Philox4x32-10, counter (particle, step, call, stream) */
  OC_RNG_REPLAY = 2, /* consume a recorded flat word log sequentially */
  OC_RNG_PHILOX32 = 3 /* Philox4x32-10 as the engine's float draws: one 32-bit
                         word per draw, 24-bit uniforms, multiply-high picks */
};

typedef struct oc_model oc_model;

typedef struct {
  double *kx, *ky, *kz; /* wave vector [1/m] */
  double *px, *py, *pz; /* position [m] (pz unused in 2-D) */
  double *E;            /* energy [eV] */
  double *tau;          /* remaining free-flight time [s] */
  double *gtau;         /* remaining grain free-flight time [s] */
  int32_t *valley, *sub, *region;
  int64_t n;
} oc_particles;

typedef struct {
  int32_t mode;
  uint32_t stream;
  uint64_t seed;
  /* mt19937_64 state (mode OC_RNG_MT), in/out */
  uint64_t mt[312];
  int32_t mt_idx;
  int32_t pad_;
  /* replay (mode OC_RNG_REPLAY): flat word log, consumed from pos */
  const uint64_t *words;
  int64_t nwords;
  int64_t pos;
  /* optional recording of every consumed word (any mode) */
  uint64_t *rec;
  int64_t rec_cap;
  int64_t rec_n;
  int32_t rec_overflow;
  int32_t pad2_;
} oc_rng;

/* ---- random numbers ---------------------------------------------------- */
void oc_mt_seed(oc_rng *r, uint64_t seed);
uint64_t oc_mt_next(oc_rng *r);
void oc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2],
                      uint32_t out[4]);
double oc_canonical(uint64_t word); /* libstdc++ generate_canonical<double,53> */

/* ---- model construction ------------------------------------------------ */
oc_model *oc_model_new(double temperature, double rho, double vSound,
                       double epsR, double Ni, int32_t nLevels,
                       double maxEnergy);
void oc_model_free(oc_model *m);
int32_t oc_add_valley(oc_model *m, const double relMass[3],
                      double particleMass, int32_t deg, double alpha,
                      double bottom);
int32_t oc_set_frame(oc_model *m, int32_t valley, int32_t sub,
                     const double d1[3], const double d2[3],
                     const double d3[3]);
/* p0: sigma [eV] (acoustic) | defPot [eV/m] (IV) | epsR (Coulomb)
   p1: phonon energy [eV] (IV)
   finalSub: deg(valley) x nF table of final subvalleys (IV) */
int32_t oc_add_mech(oc_model *m, int32_t kind, int32_t valley,
                    int32_t finalValley, double p0, double p1, int32_t nF,
                    const int32_t *finalSub, const int32_t *regions,
                    int32_t nRegions);
int32_t oc_set_region_doping(oc_model *m, int32_t region, double doping);
/* emcParticleType::setGrainScatterMechanism(emcGrainScatterMechanism(
   transmissionProb, scatterRate)), include/emcGrainScatterMechanism.hpp */
int32_t oc_set_grain(oc_model *m, double transmissionProb, double scatterRate);
/* surface scattering at a device boundary (XMIN 0, XMAX 1, YMIN 2, YMAX 3):
   emcParticleType::setSurfaceScatterMechanism with
   emcConstantSurfaceScatterMechanism(specularity) or
   emcMomentumDependentSurfaceScatterMechanism(roughness height)
   (include/SurfaceScatterMechanisms/) */
#define OC_SURFACE_SPECULAR 0
#define OC_SURFACE_CONSTANT 1
#define OC_SURFACE_ROUGHNESS 2
int32_t oc_set_surface(oc_model *m, int32_t boundary, int32_t kind, double param);
int32_t oc_build_tables(oc_model *m);
/* replace the rates of one built (valley, region) table set and
   renormalise it (reinitScatterTables with caller-filled rates) */
int32_t oc_set_raw_tables(oc_model *m, int32_t valley, int32_t region, const double *raw);

int32_t oc_model_n_valleys(const oc_model *m);
/* one Philox step of every particle with its own force (3 x n planes) */
int32_t oc_bulk_step_forces(const oc_model *m, oc_particles *p, double dt,
                            const double *forces, const double box[3],
                            const double fieldDir[3], uint64_t seed, uint32_t stream,
                            uint32_t step, int32_t nThreads, double *obs);
/* FMMBulkParticleHandler's step loop: Coulomb sums over the particles (charge q)
   and the fixed charges, then one step with charge x field - ke / epsR x sum;
   obs: nSteps x nV x 3 (may be NULL) */
int32_t oc_bulk_run_coulomb(const oc_model *m, oc_particles *p, double dt, double q,
                            const double field[3], const double box[3],
                            const double fieldDir[3], const double *fixedPos,
                            const double *fixedQ, int64_t nFixed, double epsR, double invCut,
                            int32_t images, uint64_t seed, uint32_t stream, uint32_t step0,
                            int32_t nSteps, int32_t threads, double *obs);

/* particle-particle Coulomb sums of the FMM handlers, direct (emc_oracle_p2p.c):
   pos 3 x n planes, q n; invCut = 1 / cutoff radius (0: no cutoff); box and
   images: periodic copies per side; force 3 x n, pot n */
void oc_p2p_pair(double xt, double yt, double zt, double qt, double xs, double ys, double zs,
                 double qs, double invCut, double out[4]);
int32_t oc_p2p_coulomb(const double *pos, const double *q, int64_t n, double invCut,
                       double box, int32_t images, double *force, double *pot,
                       int32_t threads);
int32_t oc_get_raw_table(const oc_model *m, int32_t valley, int32_t region,
                         int32_t idxTable, double *out);
int32_t oc_get_norm_table(const oc_model *m, int32_t valley, int32_t region,
                          int32_t idxTable, double *out);
int32_t oc_n_tables(const oc_model *m, int32_t valley, int32_t region);
int32_t oc_table_mech(const oc_model *m, int32_t valley, int32_t region,
                      int32_t idxTable);
double oc_get_tau(const oc_model *m, int32_t valley, int32_t region);
void oc_valley_consts(const oc_model *m, int32_t valley, double out[8]);
void oc_valley_rot(const oc_model *m, int32_t valley, double *out /*deg*9*/);

/* ---- valley kinematics ------------------------------------------------- */
double oc_energy(const oc_model *m, int32_t valley, const double k[3]);
double oc_norm_wave_vec(const oc_model *m, int32_t valley, double E);
void oc_velocity(const oc_model *m, int32_t valley, int32_t sub,
                 const double k[3], double E, double v[3]);
void oc_drift(const oc_model *m, double dt, double k[3], double *E,
              int32_t valley, int32_t sub, double *pos, int32_t dim,
              const double force[3]);

/* ---- bulk path --------------------------------------------------------- */
/* one reference time step for every particle (basicBulkParticleHandler::
   moveParticles); step is the global step index (Philox counter).  When
   offsets != NULL it receives n+1 word offsets into r->rec for this step. */
int32_t oc_bulk_step(const oc_model *m, oc_particles *p, double dt,
                     const double force[3], const double box[3], oc_rng *r,
                     uint32_t step, int64_t *offsets);
/* nSteps Philox steps with OpenMP over particles (CPU baseline); per-step
   per-valley observables written to obs[(s*nV + v)*3 + {E, vd, count}] */
int32_t oc_bulk_run_philox(const oc_model *m, oc_particles *p, double dt,
                           const double force[3], const double box[3],
                           const double fieldDir[3], uint64_t seed,
                           uint32_t stream, uint32_t step0, int32_t nSteps,
                           int32_t nThreads, double *obs, int32_t words32);
/* reference per-valley observables: out[v*3 + 0] = avg E, 1 = avg v.dir,
   2 = occupation probability */
void oc_observables(const oc_model *m, const oc_particles *p,
                    const double fieldDir[3], double *out);
/* bulk initial particles, reference generateInitialParticles order; returns
   particle count (<= cap), positions/k/E/tau/gtau/valley/sub/region filled */
int64_t oc_bulk_init(const oc_model *m, const double maxPos[3],
                     const double spacing[3], double doping, oc_rng *r,
                     oc_particles *p, int64_t cap);
/* one particle's initial state at grid node coord (emcElectron::
   generateInitialParticle + initParticlePos); used for replay of init */
void oc_init_particle(const oc_model *m, const int64_t coord[3],
                      const int64_t extent[3], const double spacing[3],
                      int32_t dim, int32_t region, double thermalVoltage,
                      oc_rng *r, oc_particles *p, int64_t idx,
                      int32_t tauRegionIsValley);

/* ---- device (2-D) path ------------------------------------------------- */
enum { OC_NGP = 0, OC_CIC = 1, OC_NEC = 2, OC_NEC_VWD = 3 };
enum { OC_OHMIC = 0, OC_SCHOTTKY = 1, OC_GATE = 2 };
enum { OC_XMIN = 0, OC_XMAX = 1, OC_YMIN = 2, OC_YMAX = 3 };

/* A 2-D emcDevice flattened: grids are x fastest (include/emcGrid.hpp:242-254);
   bnd[b] holds the contact index of each coordinate of boundary b (-1: none),
   XMIN/XMAX indexed by y, YMIN/YMAX by x (include/emcSurface.hpp:37-64). */
typedef struct {
  int32_t nx, ny;
  double hx, hy;
  double maxX, maxY;
  double width;
  double T, Ni, epsR;
  const double *doping;
  const int32_t *region;
  const int32_t *bnd[4];
  int32_t nContacts;
  int32_t pad_;
  const int32_t *ctype;
  const double *cvolt;
  const double *cpar; /* nContacts x 3: epsR oxide, thickness [m], barrier [V] */
} oc_dev;

double oc_dev_debye(const oc_dev *d);
double oc_dev_cell_volume(const oc_dev *d);
int32_t oc_dev_contact_idx(const oc_dev *d, int32_t x, int32_t y);
int32_t oc_dev_is_reservoir(const oc_dev *d, int32_t x, int32_t y);
void oc_dev_efield(const oc_dev *d, const double *pot, double *Ex, double *Ey);
/* the E field of PM scheme `scheme` (NGP and CIC: oc_dev_efield) */
void oc_dev_efield_pm(const oc_dev *d, int32_t scheme, const double *pot, double *Ex,
                      double *Ey);
void oc_dev_assign(const oc_dev *d, int32_t scheme, const double *px,
                   const double *py, int64_t n, double nrCarriers,
                   double *grid);
void oc_dev_force(const oc_dev *d, int32_t scheme, const double *Ex,
                  const double *Ey, double x, double y, double charge,
                  double F[3]);
/* driftScatterParticles (include/ParticleHandler/emcBasicParticleHandler.hpp:
   76-145): moves every particle, removes those that left through an ohmic
   contact (stable), netto[c] counts them per contact.  offsets (n+1, may be
   NULL) receive each particle's word offsets into r->rec. */
int32_t oc_dev_move(const oc_model *m, const oc_dev *d, int32_t scheme,
                    oc_particles *p, const double *Ex, const double *Ey,
                    double dt, double charge, oc_rng *r, uint32_t step,
                    int32_t *netto, int64_t *offsets);
/* expected particles at reservoir nodes (emcElectron.hpp:63-73) */
void oc_dev_exp_nr(const oc_dev *d, double *expNr, int32_t roundCounts);
/* handleOhmicContacts (emcBasicParticleHandler.hpp:158-192 with
   emcAbstractParticleHandler.hpp:200-216): removes excess particles at
   reservoir nodes, injects missing ones (appended, grid order).  remInj[c]
   gets -removed + injected per contact.  Returns the new particle count or a
   negative status. */
int64_t oc_dev_contacts(const oc_model *m, const oc_dev *d, oc_particles *p,
                        int64_t cap, const double *expNr, double nrCarriers,
                        oc_rng *r, uint32_t step, int32_t *remInj,
                        int32_t tauRegionIsValley);
/* generateInitialParticles (emcAbstractParticleHandler.hpp:133-148) with
   emcElectron::getInitialNrParticles (emcElectron.hpp:48-61): pot != NULL ->
   exp(pot) Ni, else the doping; roundCounts mirrors electronVWD. */
int64_t oc_dev_init(const oc_model *m, const oc_dev *d, const double *pot,
                    int32_t roundCounts, double nrCarriers, oc_rng *r,
                    oc_particles *p, int64_t cap, int32_t tauRegionIsValley);
void oc_dev_concentration(const oc_dev *d, const double *nrPart, double *conc);
void oc_dev_init_potential(const oc_dev *d, double *pot);
/* emcSORSolver (include/PoissonSolver/emcSORSolver.hpp:49-197): eConc NULL ->
   equilibrium, else non-equilibrium with the given normalised electron
   concentration.  Returns sweeps used (<= maxSweeps), negative on error. */
int64_t oc_dev_sor(const oc_dev *d, double *pot, const double *eConc,
                   double omega, double accuracyVolt, int32_t resetBC,
                   int64_t maxSweeps);

#ifdef __cplusplus
}
#endif
#endif
