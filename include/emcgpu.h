/*
 * emcgpu.h -- C ABI of libemcgpu, the sm_103a engine for the ViennaEMC
 * per-particle hot path (free flight, scatter selection and final states,
 * particle-mesh assignment / force interpolation, grid Poisson solve).
 *
 * Plain C: POD descriptors, plain pointers and sizes, no C++ or torch types.
 * Every entry point returns an int status (EMCG_OK == 0); emcg_last_error()
 * gives the message of the most recent failure on the calling thread.
 *
 * The reference interface each entry point replaces is cited beside it
 * (paths relative to the ViennaEMC project root).  A maintainer binds this
 * header from the reference's C++ through the adapter classes of
 * include/emcgpu_reference.hpp; the Python package viennaemc_gb300 binds it
 * with ctypes.
 *
 * Units are SI throughout (m, s, J, kg, V/m) except energies in eV, exactly
 * as in the reference.  Particle state crosses the boundary as
 * structure-of-arrays doubles/int32, whatever precision the engine computes in.
 */
#ifndef EMCGPU_H
#define EMCGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- limits ------------------------------------------------------------ */
#define EMCG_MAX_VALLEYS 4
#define EMCG_MAX_DEG 8       /* subvalleys per valley */
#define EMCG_MAX_MECH 32     /* mechanisms per model */
#define EMCG_MAX_NF 8        /* final subvalleys per initial subvalley */
#define EMCG_MAX_REGIONS 16  /* doping regions */
#define EMCG_MAX_TABLESETS (EMCG_MAX_VALLEYS * EMCG_MAX_REGIONS)

/* ---- status codes ------------------------------------------------------ */
#define EMCG_OK 0
#define EMCG_ERR_ARG (-1)          /* invalid argument (host-side check)   */
#define EMCG_ERR_CUDA (-2)         /* CUDA runtime failure                 */
#define EMCG_ERR_TIMEOUT (-3)      /* a bounded device wait gave up        */
#define EMCG_ERR_NONCONVERGED (-4) /* Poisson solve did not converge       */
#define EMCG_ERR_OUT_OF_TABLE (-5) /* particle in a (valley, region) pair
                                      without a rate-table set (the
                                      reference's std::map::at throws)    */
#define EMCG_ERR_REPLAY (-6)       /* replay word stream exhausted         */
#define EMCG_ERR_CAPACITY (-7)     /* particle capacity exceeded           */

/* ---- precision --------------------------------------------------------- */
#define EMCG_FP64 0 /* double state and arithmetic (parity engine)         */
#define EMCG_FP32 1 /* float state and arithmetic, double observable sums  */

/* ---- mechanism kinds (include/ScatterMechanisms/) ---------------------- */
#define EMCG_MECH_ACOUSTIC 0     /* emcAcousticScatterMechanism.hpp:124-126 */
#define EMCG_MECH_ZERO_IV_ABS 1  /* emcZeroOrderInterValleyScatterMechanism.hpp:247-257 */
#define EMCG_MECH_ZERO_IV_EMI 2  /* emcZeroOrderInterValleyScatterMechanism.hpp:390-400 */
#define EMCG_MECH_FIRST_IV_ABS 3 /* emcFirstOrderInterValleyScatterMechanism.hpp:121-131 */
#define EMCG_MECH_FIRST_IV_EMI 4 /* emcFirstOrderInterValleyScatterMechanism.hpp:269-279 */
#define EMCG_MECH_COULOMB 5      /* emcCoulombScatterMechanism.hpp:48-59 */
/* surface mechanisms at device boundaries (emcg_model_desc.surface_kind) */
#define EMCG_SURFACE_SPECULAR 0
#define EMCG_SURFACE_CONSTANT 1
#define EMCG_SURFACE_ROUGHNESS 2

/* ---- random-number modes ----------------------------------------------- */
#define EMCG_RNG_PHILOX 0 /* counter-based Philox4x32-10                   */
#define EMCG_RNG_REPLAY 1 /* consume a recorded std::mt19937_64 word stream */

/* One valley: emcNonParabolicAnisotropValley
   (include/ValleyTypes/emcNonParabolicAnistropValley.hpp:22-204).
   rot[s] holds the normalised ellipse-frame axes of subvalley s as rows
   (setSubValleyEllipseCoordSystem, :68-80). */
typedef struct {
  int32_t deg;
  int32_t pad_;
  double rel_mass[3];
  double particle_mass; /* kg */
  double alpha;         /* non-parabolicity [1/eV] */
  double bottom;        /* valley bottom energy [eV] */
  double rot[EMCG_MAX_DEG][9];
} emcg_valley_desc;

/* One scatter mechanism's final-state sampler.  The rates stay on the host
   (getScatterRate of the reference classes) and arrive as tables.
   shift:  energy change of an intervalley event [eV]
           (absorption: +(phononEnergy - deltaValley),
            emission:   -(phononEnergy + deltaValley));
   coulomb_sc2: 8 eps0 epsR Vt / hbar^2 (emcCoulombScatterMechanism.hpp:31). */
typedef struct {
  int32_t kind;
  int32_t valley;
  int32_t final_valley;
  int32_t n_final;
  double shift;
  double coulomb_sc2;
  int32_t final_sub[EMCG_MAX_DEG][EMCG_MAX_NF];
} emcg_mech_desc;

/* One (valley, region) table set (emcScatterHandler::scatterTables entry,
   include/emcScatterHandler.hpp:58-59).  mech[t] is the model mechanism index
   of table t in registration order; tau_max = 1 / Gamma_max (:271). */
typedef struct {
  int32_t valley;
  int32_t region;
  int32_t n_tables;
  int32_t pad_;
  int32_t mech[EMCG_MAX_MECH];
  double tau_max;
} emcg_tableset_desc;

/* A particle type's band + scattering model (emcParticleType +
   emcScatterHandler, include/ParticleType/emcParticleType.hpp:25-189).
   tables: for each table set in order, n_tables x n_levels doubles of the
   cumulative, Gamma_max-normalised rates (renormalizeTables, :248-273),
   table-major: tables[ts_offset + t * n_levels + level].
   region_doping: net doping per region [1/m^3] (Coulomb final state). */
typedef struct {
  int32_t n_valleys;
  int32_t n_mechs;
  int32_t n_tablesets;
  int32_t n_levels;
  double max_energy; /* eV; dE = max_energy / n_levels */
  double grain_tau;  /* grain free-flight constant (1.0 without a grain
                        mechanism, include/emcScatterHandler.hpp:62) */
  const emcg_valley_desc *valleys;
  const emcg_mech_desc *mechs;
  const emcg_tableset_desc *tablesets;
  const double *tables;
  double region_doping[EMCG_MAX_REGIONS];
  /* A grain mechanism (emcParticleType::setGrainScatterMechanism with an
     emcGrainScatterMechanism(transmissionProb, scatterRate),
     include/emcGrainScatterMechanism.hpp:27-80): grain = 1 scatters the
     particle at every grain event (basicBulkParticleHandler.hpp:215-219,
     emcBasicParticleHandler.hpp:131-138), reflected when a uniform draw
     exceeds grain_transmission, else transmitted, with |k| and the energy
     kept; grain_tau is then 1 / scatterRate.  grain = 0 (a zeroed
     descriptor): no mechanism, grain events only redraw the timer. */
  int32_t grain;
  int32_t grain_pad_;
  double grain_transmission;
  /* Surface mechanism per boundary of a device (XMIN, XMAX, YMIN, YMAX;
     emcParticleType::setSurfaceScatterMechanism, include/emcScatterHandler.hpp:
     114-124, 172-191): EMCG_SURFACE_SPECULAR (0, a zeroed descriptor) reflects
     specularly, the reference's default; EMCG_SURFACE_CONSTANT scatters
     diffusely with probability 1 - surface_param (the specularity,
     emcConstantSurfaceScatterMechanism); EMCG_SURFACE_ROUGHNESS with
     probability 1 - exp(-(2 surface_param k_perp)^2) (surface_param: the
     roughness height [m], emcMomentumDependentSurfaceScatterMechanism, its
     polar angle from the reference's fixed-point iteration of at most 10000
     steps).  Bulk engines ignore them. */
  int32_t surface_kind[4];
  double surface_param[4];
} emcg_model_desc;

/* One bulk ensemble (basicBulkParticleHandler,
   examples/bulkSimulation/basicBulkParticleHandler.hpp:93-120):
   force = charge * field (:186), periodic box [0, box] (:600-613),
   field_dir = normalised field direction for the drift velocity (:326-347).
   flags: EMCG_ENS_FLOAT_DRAWS or 0 (see below). */
typedef struct {
  int32_t model;      /* index into the handle's models */
  int32_t pad_;
  int64_t capacity;   /* particle slots reserved for this ensemble */
  double field[3];    /* V/m */
  double charge;      /* C (-q for electrons) */
  double field_dir[3];
  double box[3];      /* m */
  double dt;          /* s */
  uint64_t seed;
  uint32_t stream;
  uint32_t flags;
} emcg_ensemble_desc;

/* Ensemble flag, no reference counterpart: the double engine draws its random
   numbers as the float engine does -- one 32-bit Philox word per draw, the
   float engine's uniform (24 bits) or pick, widened to double -- in place of
   one 64-bit word per draw.  With the same seed, stream and initial state the
   two engines then consume the same numbers, and their results differ by the
   arithmetic alone: the double run is the float run's precision oracle.  The
   float engine ignores the flag. */
#define EMCG_ENS_FLOAT_DRAWS 1u

/* Host-side structure-of-arrays particle state (emcParticle +
   positionsParticles, include/emcParticle.hpp:10-18). */
typedef struct {
  double *kx, *ky, *kz;
  double *px, *py, *pz;
  double *energy;
  double *tau;
  double *grain_tau;
  int32_t *valley, *sub, *region;
  int64_t n;
} emcg_state;

typedef struct emcg_handle emcg_handle;

/* ---- errors ------------------------------------------------------------ */
/* Text of the last failure on this thread (replaces emcMessage::addError,
   include/emcMessage.hpp:43-66, which aborts). */
const char *emcg_last_error(void);
int32_t emcg_version(void);

/* Page-locked host memory for particle states (no reference counterpart):
   state uploads (emcg_set_state) and downloads from such memory run at the
   full host-link rate; from ordinary memory CUDA stages them.  The block is
   mapped into the device's address space, so emcg_bulk_step_from_host reads
   it from inside the step kernel.  bytes = 0 gives NULL. */
int32_t emcg_host_alloc(int64_t bytes, void **ptr);
int32_t emcg_host_free(void *ptr);

/* ---- bulk engine (examples/bulkSimulation/basicBulkParticleHandler.hpp) -- */

/* Create a bulk engine holding n_models particle-type models and n_ens
   ensembles (one ensemble = one basicBulkParticleHandler; several ensembles
   advance together in one launch).  precision: EMCG_FP64 | EMCG_FP32.
   Replaces the basicBulkParticleHandler constructor (:93-120) once the
   particle type's initScatterTables has run. */
int32_t emcg_bulk_create(const emcg_model_desc *models, int32_t n_models,
                         const emcg_ensemble_desc *ens, int32_t n_ens,
                         int32_t precision, emcg_handle **out);
int32_t emcg_destroy(emcg_handle *h);

/* Replace ensemble e's field, charge, direction, box, dt and Philox stream
   (resetAppliedFieldStrength, :135-137); model and capacity must not change. */
int32_t emcg_bulk_update_ensemble(emcg_handle *h, int32_t ens,
                                  const emcg_ensemble_desc *desc);

/* Upload / download ensemble e's particles (replaces direct access to the
   handler's particles / positionsParticles vectors, :58-59).  For a device
   engine (emcg_device_create) e must be 0 and pz is ignored. */
int32_t emcg_set_state(emcg_handle *h, int32_t ens, const emcg_state *s);
int32_t emcg_get_state(emcg_handle *h, int32_t ens, emcg_state *s);
int64_t emcg_num_particles(emcg_handle *h, int32_t ens);

/* The same for a bulk engine in the float engine's own layout (no reference
   counterpart): float fields and one packed word per particle,
   meta = valley | subvalley << 8 | region << 16.  40 bytes per particle cross
   the host link instead of 84, a host that keeps its ensembles in floats
   uploads them at half the cost (a double engine widens them).  The check of
   emcg_set_state applies: a field out of range is refused with the first bad
   particle's index and nothing is written. */
typedef struct {
  float *kx, *ky, *kz;
  float *px, *py, *pz;
  float *energy;
  float *tau;
  float *grain_tau;
  uint32_t *meta;
  int64_t n;
} emcg_state_f32;
int32_t emcg_set_state_f32(emcg_handle *h, int32_t ens, const emcg_state_f32 *s);
int32_t emcg_get_state_f32(emcg_handle *h, int32_t ens, emcg_state_f32 *s);

/* Generate n initial particles of ensemble e on the GPU (Philox stream
   (seed, stream), counter = (particle, 0xFFFFFFFF, call, stream)):
   emcElectron::generateInitialParticle + initParticlePos
   (include/ParticleType/emcElectron.hpp:75-90,
    include/emcParticleInitialization.hpp:14-51) at grid nodes coord[i]
   (3 x int64 per particle) of a grid with the given extent and spacing.
   coords == NULL places particles at nodes drawn uniformly. */
int32_t emcg_bulk_init(emcg_handle *h, int32_t ens, int64_t n,
                       const int64_t *coords, const int64_t extent[3],
                       const double spacing[3], double thermal_voltage);

/* Advance every ensemble by n_steps time steps (moveParticles(dt), :181-225)
   starting at global step index step0 (Philox counter).  obs (optional,
   host) receives, per ensemble, step and valley, the sums
   {sum E, sum v.field_dir, count}:
   obs[((e * n_steps + s) * n_valleys_max + v) * 3 + q]
   with n_valleys_max the largest n_valleys over the models.  Averages and
   occupations as returned by getAvgEnergy / getAvgDriftVelocity /
   getValleyOccupationProbability (:289-347) are sum/count and count/N. */
int32_t emcg_bulk_step(emcg_handle *h, int32_t n_steps, uint32_t step0,
                       double *obs);

/* emcg_set_state_f32(h, ens, s) followed by emcg_bulk_step(h, n_steps,
   step0, obs), with the upload fused into the first launch: when the engine
   is a float one stepping with the warp-asynchronous kernel and every array
   of s lies inside an emcg_host_alloc block, each thread of that launch reads
   its particle's start state from host memory over the host link, so the
   transfer overlaps the steps instead of preceding them (the reference's
   setParticles + moveParticles pair, :58-59 and :181-225).  Other engines and
   other host memory take the two calls.  In the fused form a particle whose
   valley, subvalley or region is out of range is neither stepped nor stored:
   the call returns EMCG_ERR_ARG and the ensemble's state is unspecified until
   it is set again. */
int32_t emcg_bulk_step_from_host(emcg_handle *h, int32_t ens,
                                 const emcg_state_f32 *s, int32_t n_steps,
                                 uint32_t step0, double *obs);

/* Replay mode: the next emcg_bulk_step (n_steps must be 1) of ensemble 0
   consumes words[offsets[i] .. offsets[i+1]) for particle i instead of
   Philox (the sequential std::mt19937_64 stream of the reference built
   without OpenMP, attributed to particles).  words/offsets are host
   arrays of nwords / n+1 entries; NULL words switches replay off. */
int32_t emcg_set_replay(emcg_handle *h, const uint64_t *words, int64_t nwords,
                        const int64_t *offsets, int64_t n_offsets);

/* Per-launch timing of the last emcg_bulk_step (device milliseconds). */
int32_t emcg_last_kernel_ms(emcg_handle *h, double *ms);

/* Tuning: threads per block (multiple of 32, <= 1024; -1 = automatic, the
   default: 256, or 128 for launches of the warp-asynchronous kernel shorter
   than 100 steps, whose blocks' warps end far apart) and steps fused per
   kernel launch (observables flushed every chunk). 0 keeps the current. */
int32_t emcg_set_launch(emcg_handle *h, int32_t block_threads,
                        int32_t steps_per_launch);
/* The block size of the last launch (or the set one) and the steps per
   launch setting (0: all steps of a call in one launch). */
int32_t emcg_get_launch(emcg_handle *h, int32_t *block_threads, int32_t *steps_per_launch);

/* Tuning, the step kernel: 0 lockstep (each warp advances its particles
   step by step and handles their events; the default of the double engine);
   1 block-queued (the events of a thread block are processed together by its
   first warps); 2 warp-asynchronous, float only and the float engine's
   default (each lane runs its particle from event to event across step
   boundaries, so a warp's lanes process their events together; per-step
   observables go through a per-warp window).  All follow the same
   per-particle algorithm; replay always uses the lockstep kernel.  In the
   queued kernel a grain event (the grain mechanism's draws and the timer
   redraw) takes its own Philox calls, so its stream differs from the
   lockstep kernel and the oracle in grain events only (without a grain
   mechanism they are rare timer redraws).  The warp-asynchronous kernel adds its
   per-step sums in float in an order that varies from run to run: particle
   states are reproducible bit for bit, observables to float rounding. */
int32_t emcg_set_scatter_mode(emcg_handle *h, int32_t queued);
/* Tuning of the warp-asynchronous kernel: free flights a lane may take in one
   drift pass before the warp checks its waiting lanes again, in [1, 20]; 0
   (the default) chooses by launch length: 5 below 100 steps per launch, 6
   from there.  emcg_get_pass_actions gives the value of the last launch (or
   the setting).  Only the schedule changes: particle states are the same bit
   for bit.  No reference counterpart. */
int32_t emcg_set_pass_actions(emcg_handle *h, int32_t n);
int32_t emcg_get_pass_actions(emcg_handle *h, int32_t *n);

/* Tuning: register cap of the step kernel, as the minimum number of resident
   256-thread blocks per SM (1 = uncapped, 3 or 4); capped variants apply to
   blocks of at most 256 threads. */
int32_t emcg_set_occupancy(emcg_handle *h, int32_t min_blocks_per_sm);
/* Graph replay (enable != 0): each launch of steps is an instantiated CUDA
   graph (observable reset -> step kernel) replayed with its step offset
   updated; results equal the direct launches.  No reference counterpart. */
int32_t emcg_bulk_set_graph(emcg_handle *h, int32_t enable);
/* Autotuner: runs trial_steps steps (from step0, advancing the ensembles --
   use it as warm-up) with each candidate launch shape (block threads 128 /
   256, register cap 1 / 3 / 4 resident blocks per SM, lockstep,
   block-queued or, for float, warp-asynchronous scatter with 3 or 6 free
   flights per pass), twice: in a forward and then a backward pass over the
   shapes.  It keeps the shape of least total device time (its pass actions:
   emcg_get_pass_actions).  *steps_used = steps run (2 x shapes x
   trial_steps: 13 float shapes, 8 double); outputs may be NULL.  No
   reference counterpart. */
int32_t emcg_bulk_autotune(emcg_handle *h, int32_t trial_steps, uint32_t step0,
                           int32_t *steps_used, int32_t *block_threads, int32_t *min_blocks,
                           int32_t *queued);

/* ---- rate-table rebuild (include/emcScatterHandler.hpp:100-108) -------- */
/* emcScatterHandler::reinitScatterTables for model `model` of a bulk
   handle, or of a device handle (model 0): the caller refills the rates --
   getScatterRate at (level + 1) dE of every table (fillScatterTables,
   :220-235), for instance after a phonon bath changed them -- and the GPU
   renormalises them (renormalizeTables, :248-273): cumulative sums in table
   order, their maximum Gmax over levels, tables / Gmax and tau = 1 / Gmax,
   in double, stored in the handle's precision in place of the old tables.
   raw: per table set in the model's order, n_tables x n_levels doubles,
   table-major (the layout of emcg_model_desc.tables before
   normalisation); the table sets, their mechanisms and the level grid stay
   those of the model.  raw_on_device == 0: host memory, checked (finite
   rates, positive Gmax) before anything is launched.  raw_on_device != 0:
   device memory of the handle's device, complete when the call is made and
   unchanged until the next step call returns; a set with a non-finite rate
   or Gmax <= 0 is left as it was and the next step call returns
   EMCG_ERR_ARG.  The rebuild is ordered on the handle's stream before the
   next step (graph replay included); the call does not wait for it. */
int32_t emcg_update_rates(emcg_handle *h, int32_t model, const double *raw,
                          int32_t raw_on_device);
/* The handle's current tables of model `model`, converted to double, in the
   layout of emcg_update_rates' raw (NULL to skip), and tau_max per table set
   (n_tablesets doubles, NULL to skip).  Waits for the handle's stream. */
int32_t emcg_get_rates(emcg_handle *h, int32_t model, double *tables, double *tau);

/* ---- particle-particle Coulomb (FMM handlers) ------------------------- */
/* The particle-particle sums that scalFMM computes for
   emcFMMParticleHandler (include/ParticleHandler/emcFMMParticleHandler.hpp:
   160-167, 381-393) and FMMBulkParticleHandler
   (examples/bulkSimulationFMM/FMMBulkParticleHandler.hpp:203-205, 433-440),
   evaluated directly on the GPU.  For every particle i, over every other
   particle j and every periodic copy of the box, the pair term of
   FP2PRCutoff::NonMutualParticles (include/ParticleHandler/FMM/
   FP2PRCutoff.hpp:64-100): force_i += -q_i q_j d / r^3, potential_i +=
   q_j / r, with d = x_i - x_j rescaled to the cutoff radius when the pair is
   closer.  These are the container values before the handlers' Coulomb factor.
   pos: 3 x n doubles (x plane, y plane, z plane) [m]; charge: n [C];
   inv_cutoff: 1 / cutoff radius [1/m] (1e9: the reference's 1 nm; 0: none);
   images: copies of the cubic box of width box on each side in x, y and z
   (0: the box alone; a particle sees its own copies, not itself);
   precision: EMCG_FP64 (the reference's arithmetic order) or EMCG_FP32
   (float pair terms, double sums per tile).  force: 3 x n, potential: n;
   *kernel_ms (may be NULL): device time of the sums. */
int32_t emcg_p2p_coulomb(const double *pos, const double *charge, int64_t n,
                         double inv_cutoff, double box, int32_t images,
                         int32_t precision, double *force, double *potential,
                         double *kernel_ms);

/* Particle-particle Coulomb steps in the bulk engine: FMMBulkParticleHandler
   (examples/bulkSimulationFMM/FMMBulkParticleHandler.hpp) on the GPU.
   enable != 0: every step first forms, for each ensemble, the sums of
   emcg_p2p_coulomb over its particles (charge of the ensemble) and its fixed
   charges, for each of its particles (executeFMM, :203-205), and then moves
   every particle one step with force = charge x field - (ke / eps_r) x force
   sum (getForceAtParticle, :433-440; ke = 1 / (4 pi eps0) with the
   reference's constants), the force rotated into each free flight's
   subvalley frame (moveParticles, :233-277).  inv_cutoff and images as
   emcg_p2p_coulomb, images over each ensemble's (cubic) box.  Steps then run
   one launch each; replay is not available.  enable == 0: back to the
   applied field alone. */
int32_t emcg_bulk_set_coulomb(emcg_handle *h, int32_t enable, double eps_r,
                              double inv_cutoff, int32_t images);
/* Fixed charges of ensemble e (the handler's particle types that do not
   move, e.g. donors): pos 3 x n planes [m], q n [C]; n = 0 removes them. */
int32_t emcg_bulk_set_fixed_charges(emcg_handle *h, int32_t e, const double *pos,
                                    const double *q, int64_t n);
/* The force sums (3 x n planes, may be NULL) and potential sums (n, may be
   NULL) of ensemble e's particles from the last Coulomb step (the container
   values, before the Coulomb factor). */
int32_t emcg_bulk_get_coulomb(emcg_handle *h, int32_t e, double *force, double *potential);

/* ---- single-particle kernels (known-answer tests of the reference) ----- */
/* emcGrainScatterMechanism::scatterParticle (include/emcGrainScatterMechanism.hpp:
   41-80) of model 0's grain mechanism for n independent wave vectors: k
   (3 x n, SoA) in/out, Philox draws of a fixed key at `step`.  Runs in the
   handle's precision; model 0 must have a grain mechanism. */
int32_t emcg_grain_kat(emcg_handle *h, int64_t n, double *k, uint32_t step);
/* drift() of include/emcParticleDrift.hpp:11-36 for n independent
   particles of valley v of model 0: k, pos (3 x n, SoA) and energy in/out,
   force 3 x n, dt per particle.  Runs in the handle's precision. */
int32_t emcg_drift_kat(emcg_handle *h, int32_t valley, int64_t n,
                       const int32_t *sub, const double *dt,
                       const double *force, double *k, double *pos,
                       double *energy);

/* ---- device engine (include/emcSimulation.hpp:164-193) ------------------ */
#define EMCG_PM_NGP 0     /* include/PMSchemes/emcNGPScheme.hpp */
#define EMCG_PM_CIC 1     /* include/PMSchemes/emcCICScheme.hpp */
#define EMCG_PM_NEC 2     /* include/PMSchemes/emcNECScheme.hpp */
#define EMCG_PM_NEC_VWD 3 /* examples/mosfet2D/NECSchemeVWD.hpp */
#define EMCG_CONTACT_OHMIC 0
#define EMCG_CONTACT_SCHOTTKY 1
#define EMCG_CONTACT_GATE 2
#define EMCG_GRID_POTENTIAL 0 /* phi / Vt (Debye-normalised)           */
#define EMCG_GRID_EX 1        /* V/m                                   */
#define EMCG_GRID_EY 2
#define EMCG_GRID_NRPART 3    /* particles assigned to each node       */
#define EMCG_GRID_CONC 4      /* electron concentration / Ni           */

/* A 2-D emcDevice (include/emcDevice.hpp:38-344) flattened; grids are x
   fastest (include/emcGrid.hpp:242-254).  boundary_contact[b] lists the
   contact index of every coordinate of boundary b (XMIN, XMAX: ny entries;
   YMIN, YMAX: nx entries; -1 = artificial boundary), as emcSurface's
   idxContactGrid (include/emcSurface.hpp:37-64, 199-222). */
typedef struct {
  int32_t nx, ny;
  double hx, hy;       /* m */
  double max_x, max_y; /* device extent maxPos [m]; 0: (n - 1) h */
  double width;        /* extent in the third dimension [m] */
  double temperature;  /* K */
  double ni;           /* intrinsic density [1/m^3] */
  double eps_r;
  const double *doping;  /* net doping [1/m^3] */
  const int32_t *region; /* doping-region index */
  const int32_t *boundary_contact[4];
  int32_t n_contacts;
  int32_t pad_;
  const int32_t *contact_type;
  const double *contact_voltage; /* V */
  const double *contact_param;   /* 3 per contact: oxide eps_r, oxide
                                    thickness [m], barrier height [V] */
} emcg_device_desc;

/* emcSimulationParameter + particle handler + solver settings. */
typedef struct {
  int32_t pm_scheme;            /* EMCG_PM_NGP | _CIC | _NEC | _NEC_VWD */
  int32_t tau_region_is_valley; /* injection draws tau with the valley as the
                                   region (examples/mosfet2D/electronVWD.hpp:87) */
  int64_t capacity;             /* particle slots */
  double dt;                    /* s */
  double charge;                /* C */
  double carriers_per_particle;
  uint64_t seed;
  uint32_t stream;
  int32_t poisson_max_cycles;   /* Newton / defect-correction iterations */
  double poisson_rtol;          /* relative residual target */
  int32_t poisson_smooth;       /* red-black sweeps before and after (0: 3) */
  int32_t poisson_fp32;         /* 1: float V-cycles in double refinement */
  int32_t round_expected;       /* 1: expected particles at the contacts rounded to
                                   whole particles, as electronVWD
                                   (examples/mosfet2D/electronVWD.hpp:46-56) */
  int32_t pad_;
  double poisson_update_tol;    /* V; > 0: also stop once a Newton update changes
                                   no node's potential by more than this, the
                                   reference SOR's rule (emcSORSolver.hpp:25-27,
                                   190-196); 0: the residual rule only */
} emcg_device_config;

/* Create a device engine (emcSimulation constructor: particle handler with
   expected contact counts, solver, PM scheme). */
int32_t emcg_device_create(const emcg_model_desc *model, const emcg_device_desc *dev,
                           const emcg_device_config *cfg, int32_t precision,
                           emcg_handle **out);
int32_t emcg_device_set_grid(emcg_handle *h, int32_t which, const double *v);
int32_t emcg_device_get_grid(emcg_handle *h, int32_t which, double *v);
/* emcAbstractSolver::calcEquilibriumPotential / calcNonEquilibriumPotential
   (include/PoissonSolver/emcAbstractSolver.hpp:9-58) on the potential grid,
   the latter with the current concentration grid. */
int32_t emcg_device_poisson(emcg_handle *h, int32_t equilibrium, int32_t reset_bc,
                            double *rel_residual, int32_t *cycles);
/* emcAbstractPMScheme::calcEField (include/PMSchemes/emcEFieldCalculation.hpp:13-81) */
int32_t emcg_device_efield(emcg_handle *h);
/* emcScatterHandler::scatterParticleAtBoundary (include/emcScatterHandler.hpp:
   172-191) at boundary b (0 XMIN, 1 XMAX, 2 YMIN, 3 YMAX) for n independent
   particles outside the device: the model's surface mechanism there, else
   the plain reflection.  k (3 x n) and pos (2 x n) SoA, in/out; Philox draws
   of the engine's seed and stream at `step`.  For known-answer tests of the
   reference (tests/testSurfaceScatterMechanisms). */
int32_t emcg_device_surface_kat(emcg_handle *h, int32_t boundary, int64_t n, double *k,
                                double *pos, uint32_t step);
/* driftScatterParticles (include/ParticleHandler/emcBasicParticleHandler.hpp:76-145):
   netto[c] += particles that left through contact c. */
int32_t emcg_device_move(emcg_handle *h, uint32_t step, int32_t *netto);
/* handleOhmicContacts (:158-192): rem_inj[c] = injected - removed at c. */
int32_t emcg_device_contacts(emcg_handle *h, uint32_t step, int32_t *rem_inj);
/* assignParticlesToMesh + updateCurrentParticleConcentrations
   (include/emcSimulation.hpp:207-213, include/emcSimulationResults.hpp:98-116) */
int32_t emcg_device_assign(emcg_handle *h);
/* performEMCStep (include/emcSimulation.hpp:164-193) n_steps times; netto
   (n_steps x n_contacts, may be NULL) receives removed - (injected - deleted)
   per step and contact, as emcSimulationResults::updateCurrent consumes.
   The single-launch Poisson solve of a step is checked at the end of that
   step: EMCG_ERR_NONCONVERGED returns after the step whose solve missed its
   target, its particle phase done on the potential the solve reached. */
int32_t emcg_device_step(emcg_handle *h, int32_t n_steps, uint32_t step0, int32_t *netto);
/* generateInitialParticles (include/ParticleHandler/emcAbstractParticleHandler.hpp:
   133-148): counts from exp(potential) Ni (potential_based) or the doping. */
int32_t emcg_device_init(emcg_handle *h, int32_t potential_based, int32_t round_counts);
/* Replay words for the next move (phase 0, offsets per particle) or
   contact injection (phase 1, offsets per injected particle). */
int32_t emcg_device_set_replay(emcg_handle *h, int32_t phase, const uint64_t *words,
                               int64_t nwords, const int64_t *offsets, int64_t n_offsets);
/* Device-side time of the last emcg_device_step / poisson call (ms). */
int32_t emcg_device_timing(emcg_handle *h, double *step_ms, double *poisson_ms);
/* emcg_device_step on n engines at once (a bias sweep, several devices): one
   host thread per engine, each on its engine's stream, so their kernels run
   concurrently.  netto (may be NULL) holds one n_steps x n_contacts array per
   engine.  Returns the first failing engine's status.  No reference
   counterpart (the reference runs one emcSimulation per process). */
int32_t emcg_device_step_many(emcg_handle **h, int32_t n, int32_t n_steps, uint32_t step0,
                              int32_t **netto);
/* Poisson execution: mode 1 = the whole solve in one launch of a thread-block
   cluster (default where the grid fits), 0 = one launch per multigrid phase,
   -1 = leave as is.  *cluster_size (may be NULL) receives the CTAs per
   cluster of the solve in use, 0 for the multi-launch path. */
int32_t emcg_device_poisson_mode(emcg_handle *h, int32_t mode, int32_t *cluster_size);
/* Upper bound on the CTAs of the single-launch Poisson cluster (0: none; the
   largest size whose layout fits is taken, 16, 14, 12, 10, 8, 4, 2 or 1).
   The result does not depend on the size.  *cluster_size (may be NULL)
   receives the size now in use (0 for the multi-launch path).
   emcg_device_step_many plans its engines' clusters for the batch by itself:
   sizes of which the device holds all n at once.  No reference counterpart. */
int32_t emcg_device_set_poisson_cluster(emcg_handle *h, int32_t max_ctas, int32_t *cluster_size);
/* Change the Poisson settings of a device engine (negative: keep):
   relative-residual target, Newton-step limit, update tolerance [V]. */
int32_t emcg_device_set_poisson(emcg_handle *h, double rtol, int32_t max_cycles,
                                double update_tol);
/* Newton steps (*cycles) and Poisson solves of the last emcg_device_step call. */
int32_t emcg_device_poisson_counts(emcg_handle *h, int64_t *cycles, int64_t *solves);

/* Poisson solve that allocates nothing.  No counterpart in the reference: it
   is the solve of emcg_device_poisson (float multigrid V-cycles inside double
   Newton / defect correction) for callers that must not allocate device
   memory when they solve -- a host whose memory pool owns the GPU, or an
   embedder that fixes its device footprint at start-up.
   Works on caller-owned device arrays of nx * ny doubles: d_pot (in/out) is
   the potential in thermal voltages and d_conc the electron concentration
   normalised to ni (the units of EMCG_GRID_POTENTIAL / EMCG_GRID_CONC), or
   NULL for the equilibrium equation.  reset_bc, the smoothing sweeps (0 = 3),
   rtol and max_cycles mean what they mean for emcg_device_create's
   configuration and emcg_device_poisson.  cuda_stream may be NULL (default
   stream); the call returns after the solve has finished on that stream.
   Working memory is one fixed device array of about 21 MB in this library:
   grids of up to 131072 nodes and 8192 nodes per dimension, at most 64
   contacts (ohmic or gate); larger inputs return EMCG_ERR_ARG and touch
   nothing.  Every call rebuilds the array's contents, including the
   statistics that must start at zero.
   The array belongs to this library's device code, which CUDA loads onto a
   device lazily by default: at the library's first kernel launch there or
   at the first call of this function, whichever comes first
   (CUDA_MODULE_LOADING=EAGER loads it when the context is created).  A
   caller whose memory pool will claim the rest of the GPU should therefore
   make one call at start-up, before the pool takes the device.
   The first call on each device also looks the array's address up
   (cudaGetSymbolAddress, with that device current) and keeps it for the
   life of the process; make it before any stream capture begins on that
   device.  The kept address is not valid after cudaDeviceReset on that
   device: do not call this function again after such a reset.
   All calls share the array: calls whose work can overlap on a device, from
   several host threads or on several streams, race and corrupt each other's
   results; serialise them.
   A potential, concentration or correction that is not finite (NaN or Inf)
   at some node ends the solve with EMCG_ERR_NONCONVERGED. */
int32_t emcg_poisson_solve_noalloc(const emcg_device_desc *dev, double *d_pot,
                                   const double *d_conc, int32_t reset_bc, int32_t smooth,
                                   double rtol, int32_t max_cycles, void *cuda_stream,
                                   double *rel_residual, int32_t *cycles);

#ifdef __cplusplus
}
#endif
#endif /* EMCGPU_H */
