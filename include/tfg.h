/*
 * tfg.h -- C ABI of the GB300 engine for Tissue Forge's per-step particle path.
 *
 * Every entry point is extern "C", takes plain pointers and sizes, and returns
 * an int status (TFG_OK == 0, negative TFG_E_* on failure).  The message of the
 * last failure on an engine is available from tfg_last_error().
 *
 * The data model mirrors the reference's mdcore engine:
 *   - an engine owns a periodic space split into cells (source/mdcore/include/tfSpace.h:127-243),
 *   - particles live in cells with cell-relative coordinates (tfParticle.h:101-287),
 *   - interactions come from tabulated Potential objects (tfPotential.h:213-253), DPD
 *     potentials (tfDPDPotential.h), Fluxes (tfFlux.h:53-62), Bonds (tfBond.h) and Angles
 *     (tfAngle.h),
 *   - one step runs force_prep -> force -> advance (tfEngine.cpp:1378-1557,
 *     tf_engine_advance.cpp:309-480).
 *
 * Threading: one host thread per engine handle; all device work of a handle is ordered
 * on that handle's CUDA stream (tfg_engine_set_stream may supply the caller's stream).
 */
#ifndef TFG_H
#define TFG_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define TFG_API __attribute__((visibility("default")))
#else
#define TFG_API
#endif

/* ---- status codes (the reference returns HRESULT S_OK / E_FAIL, include/tf_port.h:255-260) ---- */
#define TFG_OK            0
#define TFG_E_INVAL      -1   /* bad argument or unsupported configuration */
#define TFG_E_OOM        -2   /* device or host allocation failed / arena budget exceeded */
#define TFG_E_CUDA       -3   /* a CUDA runtime call failed */
#define TFG_E_TOOFAST    -4   /* a particle moved more than one cell in a step (tf_engine_advance.cpp:204-206) */
#define TFG_E_TIMEOUT    -5   /* a bounded device wait ran out */
#define TFG_E_OVERFLOW   -6   /* a per-cell or per-tile capacity was exceeded */
#define TFG_E_RANGE      -7   /* a particle lies outside the space (tfSpace.cpp:444-448) */
#define TFG_E_STATE      -8   /* call made in the wrong state (e.g. step before load) */
#define TFG_E_NAN        -9   /* a non-finite position or force was produced */
#define TFG_E_NODEVICE  -10   /* no CUDA device is available */

/* ---- potential kinds and flags: values of the reference enums (tfPotential.h:56-122) ---- */
#define TFG_POTENTIAL_KIND_POTENTIAL 0u   /* tabulated piecewise quintic */
#define TFG_POTENTIAL_KIND_DPD       1u   /* dissipative particle dynamics */

#define TFG_POTENTIAL_R2        (1u << 4)
#define TFG_POTENTIAL_ANGLE     (1u << 6)
#define TFG_POTENTIAL_HARMONIC  (1u << 7)
#define TFG_POTENTIAL_SCALED    (1u << 11)
#define TFG_POTENTIAL_SHIFTED   (1u << 12)
#define TFG_POTENTIAL_LJ126     (1u << 0)

/* Number of float coefficients per interval (potential_chunk, tfPotential.h:40). */
#define TFG_POTENTIAL_CHUNK 8
/* Largest interval count a table may have (potential_ivalsmax, tfPotential.h:45). */
#define TFG_POTENTIAL_IVALSMAX 3048

/*
 * A potential as the reference stores it (struct Potential, tfPotential.h:213-253):
 * table coefficients c[(n+1)*8] plus the index transform alpha[0..2].  For DPD the
 * table is empty (c == NULL) and dpd_alpha/gamma/sigma hold DPDPotential's fields
 * (tfDPDPotential.cpp:32-43); a = sqrt(FLT_EPSILON), b = cutoff.
 */
typedef struct tfg_potential {
    uint32_t kind;
    uint32_t flags;
    float alpha[4];
    float r0_plusone;
    float a, b;
    int32_t n;
    const float *c;          /* (n+1)*TFG_POTENTIAL_CHUNK floats; owned by the creator */
    float dpd_alpha, dpd_gamma, dpd_sigma;
} tfg_potential;

/* ---- table construction: the reference's Potential factories (tfPotential.cpp) ----
 * Each builds the table on the host exactly as potential_init() does
 * (tfPotential.cpp:1396-1634) and returns a library-owned object; free it with
 * tfg_potential_free().  Arguments and defaults follow the factories cited. */

/* Potential::morse (tfPotential.cpp:3068-3084 -> potential_create_morse :2249-2283) */
TFG_API int tfg_potential_morse(float d, float a, float r0, float min, float max, float tol,
                                int shifted, tfg_potential **out);
/* Potential::lennard_jones_12_6 (tfPotential.cpp:2741-2751 -> potential_create_LJ126 :1087-1109);
 * tol <= 0 selects the reference default 0.001*(max-min). */
TFG_API int tfg_potential_lennard_jones_12_6(float min, float max, float A, float B, float tol,
                                             tfg_potential **out);
/* Potential::harmonic (tfPotential.cpp:2961-2975 -> potential_create_harmonic :374-401);
 * min < 0 / max < 0 / tol <= 0 select the reference defaults r0-r0, r0+r0, 0.01*(max-min). */
TFG_API int tfg_potential_harmonic(float k, float r0, float min, float max, float tol,
                                   tfg_potential **out);
/* Potential::harmonic_angle (tfPotential.cpp:2991-3003 -> potential_create_harmonic_angle :594-626);
 * min < 0 / max < 0 / tol <= 0 select the defaults 0, pi, 0.005*(max-min). */
TFG_API int tfg_potential_harmonic_angle(float k, float theta0, float min, float max, float tol,
                                         tfg_potential **out);
/* Potential::dpd (tfPotential.cpp:3128-3142 -> DPDPotential ctor tfDPDPotential.cpp:32-43) */
TFG_API int tfg_potential_dpd(float alpha, float gamma, float sigma, float cutoff, int shifted,
                              tfg_potential **out);
TFG_API void tfg_potential_free(tfg_potential *p);
/* Evaluate a table the way potential_eval_ex does (tf_potential_eval.h:104-146), for
 * r2 = squared distance and radii ri, rj.  Returns 1 when in range, else 0. */
TFG_API int tfg_potential_eval(const tfg_potential *p, float ri, float rj, float r2,
                               float *e, float *f);

/* ---- fluxes (struct Flux, tfFlux.h:53-62; Fluxes::create tfFlux.cpp:56-112) ---- */
#define TFG_FLUX_FICK     0
#define TFG_FLUX_SECRETE  1
#define TFG_FLUX_UPTAKE   2
#define TFG_MAX_FLUX_PER_PAIR 8   /* TF_SIMD_SIZE (CMakeLists.txt:82) */

typedef struct tfg_flux {
    int32_t kind;          /* TFG_FLUX_* */
    int32_t type_a, type_b;  /* orientation (type_ids[i].a/.b) */
    int32_t index_a, index_b;/* species index in a's and b's state vector */
    float coef, decay, target, cutoff;  /* cutoff <= 0 -> engine cutoff (tfFlux.cpp:95-96) */
} tfg_flux;

/* ---- particle types (engine::types[], tfParticle.h ParticleType) ---- */
#define TFG_NEWTONIAN   0   /* PARTICLE_NEWTONIAN  (tfParticle.h:62-65) */
#define TFG_OVERDAMPED  1   /* PARTICLE_OVERDAMPED */

/* particle flags (ParticleFlags, tfParticle.h:68-78) */
#define TFG_PARTICLE_FROZEN_X (1u << 3)
#define TFG_PARTICLE_FROZEN_Y (1u << 4)
#define TFG_PARTICLE_FROZEN_Z (1u << 5)

/* ---- engine ---- */
typedef struct tfg_engine tfg_engine;

/* Engine description: UniverseConfig / engine_init arguments (tfUniverse.cpp:102-120,
 * tfEngine.cpp:1702-1874, tfSpace.cpp:715-770).  cells[k] is the cell count per axis
 * (space_init computes cdim = floor(dim/L)); every cell edge must be >= cutoff (a 27-cell
 * stencil, span 1) and every cells[k] >= 3. */
typedef struct tfg_engine_desc {
    float origin[3];
    float dim[3];
    int32_t cells[3];
    float cutoff;
    float dt;
    int32_t max_type;                 /* number of particle types */
    int32_t nr_species;               /* species per particle state vector (0 = none) */
    float particle_max_dist_fraction; /* reference default 0.05 (tfEngine.cpp:1865) */
    uint64_t seed;                    /* Philox key for the random terms */
    int32_t capacity;                 /* maximum particles (0 -> sized at first load) */
    int32_t max_bonds;                /* capacity for bonds (0 -> sized at load) */
    int32_t max_angles;               /* capacity for angles (0 -> sized at load) */
    int32_t device;                   /* CUDA device ordinal */
    uint32_t flags;                   /* TFG_ENGINE_* */
    int32_t nr_fluxsteps;             /* flux substeps per step, UniverseConfig::nr_fluxsteps
                                         (tfEngine.cpp:1742, tf_engine_advance.cpp:314-323); 0 -> 1 */
} tfg_engine_desc;

/* Engine flags.
 * TFG_ENGINE_DPD_REFERENCE_RANDOM: reproduce the reference's DPD "random" term, which
 *   is the constant sigma*omega/sqrt(dt) (tf_dpd_eval.h:64; the Gaussian argument is never
 *   used).  Without it the term is sigma*omega*xi/sqrt(dt) with xi ~ N(0,1) drawn from a
 *   Philox4x32-10 stream keyed on (seed, step, min id, max id).
 * TFG_ENGINE_NO_DENSITY: skip the number-density side output f[3]
 *   (tf_runner_dopair.cpp:175-177).
 * TFG_ENGINE_VERLET: the reference's engine_flag_verlet (tfEngine.h:74; engine_init
 *   tfEngine.cpp:1749-1752).  Particles stay in their cells between rebuilds: a step
 *   re-bins (space_shuffle_local) only when twice the largest displacement since the last
 *   rebuild exceeds the skin min(h) - cutoff (engine_verlet_update, tfEngine.cpp:214-354),
 *   and the integrator is the reference's Verlet branch (tf_engine_advance.cpp:367-427: no
 *   velocity clamp, frozen mask, wall reflection, migration or flux integration; computed
 *   volume 0).  The first step after a load, a boundary change or a change of a batch's
 *   membership rebuilds.  The displacement is measured as the
 *   reference's OpenMP branch measures it; its default branch discards it (the sum goes to
 *   a shadowing int), so the reference itself never rebuilds after the first step.  On the
 *   device, the rebuild step also records each home cell's interacting-pair candidates
 *   within the skin radius, and the other steps evaluate those lists instead of testing
 *   every candidate pair. */
#define TFG_ENGINE_DPD_REFERENCE_RANDOM (1u << 0)
#define TFG_ENGINE_NO_DENSITY           (1u << 1)
#define TFG_ENGINE_VERLET               (1u << 2)

/* ---- boundary conditions (BoundaryConditions, tfBoundaryConditions.h:39-261) ----
 * Walls: 0 left (x low), 1 right (x high), 2 front (y low), 3 back (y high), 4 bottom
 * (z low), 5 top (z high).  Every wall starts PERIODIC.  An axis is periodic when both its
 * walls are; a PERIODIC wall facing a non-periodic one makes both exactly PERIODIC
 * (check_periodicy, tfBoundaryConditions.cpp:192-216), while two PERIODIC walls keep their
 * other bits (RESETTING).  On a non-periodic axis no cell pair
 * crosses the box edge (space_init task list, tfSpace.cpp:905-1000).  Walls with FREESLIP or
 * VELOCITY reflect particles that cross them (apply_update_pos_vel,
 * tf_boundary_eval.h:46-134); NO_SLIP is VELOCITY with zero velocity
 * (BoundaryCondition::init, tfBoundaryConditions.cpp:151-158).  Potentials set on a wall act
 * on particles of their type within the potential's range when the wall is active
 * (FREESLIP, VELOCITY or POTENTIAL; boundary_eval, tf_boundary_eval.h:192-254). */
#define TFG_BOUNDARY_VELOCITY  (1u << 0)
#define TFG_BOUNDARY_PERIODIC  (1u << 1)
#define TFG_BOUNDARY_FREESLIP  (1u << 2)
#define TFG_BOUNDARY_POTENTIAL (1u << 3)
#define TFG_BOUNDARY_NO_SLIP   (1u << 4)
/* BOUNDARY_RESETTING (tfBoundaryConditions.h:44): with PERIODIC on both walls of an axis, a
 * particle that wraps around the box through this wall (moves into a cell on this wall from
 * the cell on the opposite wall) has its species values reset to the simulation's reset
 * values (StateVector::reset, state/tfStateVector.cpp:36-44: each species' initial
 * concentration, 0 when unset; tfg_set_species_reset); apply_boundary_particle_crossing,
 * tfBoundaryConditions.cpp:676-735, called at migration, tf_engine_advance.cpp:219. */
#define TFG_BOUNDARY_RESETTING (1u << 5)

typedef struct tfg_boundary {
    uint32_t kind;         /* TFG_BOUNDARY_* */
    float velocity[3];     /* wall velocity (VELOCITY) */
    float restore;         /* fraction of the velocity restored on reflection (default 1) */
    float radius;          /* wall radius for shifted/scaled wall potentials (default 0) */
} tfg_boundary;

/* FP64 per-step totals (the reference sums in FPTYPE: tf_engine_advance.cpp:459-470,
 * tfEngine.cpp:1893+). */
typedef struct tfg_reductions {
    double epot;             /* nonbond + bond + angle */
    double epot_nonbond;
    double epot_bond;
    double epot_angle;
    double kinetic;          /* 0.5 * m * |v|^2 summed, at force_prep (before the step) */
    double virial;           /* sum over pairs and bonds of f_ij . r_ij */
    double computed_volume;  /* sum of 1/number_density (tf_engine_advance.cpp:188,239) */
    double species_total[8]; /* per-species sum of state values after the step */
    int64_t steps;           /* engine time (number of steps taken) */
    int64_t migrations;      /* particles that changed cell in the last step */
} tfg_reductions;

TFG_API int tfg_engine_create(const tfg_engine_desc *desc, tfg_engine **out);
TFG_API int tfg_engine_destroy(tfg_engine *eng);
TFG_API const char *tfg_last_error(const tfg_engine *eng);
/* Use the caller's CUDA stream (a cudaStream_t passed as void*); NULL restores the engine's own. */
TFG_API int tfg_engine_set_stream(tfg_engine *eng, void *stream);

/* ParticleType dynamics and mass (mass only enters the kinetic energy, tfEngine.cpp:1912). */
TFG_API int tfg_set_type(tfg_engine *eng, int type, int dynamics, float mass);
/* engine_addpot (tfEngine.cpp:1054-1077): stores p for (ti,tj) and (tj,ti).  The table is copied. */
TFG_API int tfg_set_potential(tfg_engine *eng, int ti, int tj, const tfg_potential *p);
/* engine_addfluxes (tfEngine.cpp:1079-1099) + Fluxes::addFlux (tfFlux.cpp:204-246): appends one
 * flux to the (ti,tj) Fluxes (at most TFG_MAX_FLUX_PER_PAIR). */
TFG_API int tfg_add_flux(tfg_engine *eng, int ti, int tj, const tfg_flux *flux);
/* Species flags per species index: bit0 = SPECIES_KONSTANT (tfFlux.cpp:177-179). */
TFG_API int tfg_set_species_flags(tfg_engine *eng, int nr, const uint32_t *flags);
/* Species values a particle takes when it crosses a RESETTING boundary: nr values, one per
 * species index (default 0). */
TFG_API int tfg_set_species_reset(tfg_engine *eng, int nr, const float *values);
/* Stop the simulation when its clock (the step count, as tfg_get_reductions reports it)
 * reaches `step`; -1 (the default) runs on.  The step calls of a stopped simulation leave
 * it exactly as it is: positions, velocities, species, clock and the totals of its last
 * step.  Raising the stop later lets it continue as if it had not paused.  This lets a
 * batch step past the end of some of its members (tfg_batch_set_stop), which the serving
 * loop uses to run whole chunks.  The reference has no counterpart: Universe::step runs
 * one universe until its caller stops calling (tfUniverse.cpp). */
TFG_API int tfg_set_stop(tfg_engine *eng, int64_t step);
/* Gaussian single-body force per type (Force::random, tfForce.cpp:111-245): redraw
 * when (time + id) % duration_steps == 0; std <= 0 disables. */
TFG_API int tfg_set_random_force(tfg_engine *eng, int type, float mean, float std, int duration_steps);

/* Load n particles with GLOBAL positions (space_addpart -> space_setpartp,
 * tfSpace.cpp:432-475).  Particle i gets id i.  Any pointer except x may be NULL:
 * v -> 0, type -> 0, radius -> 1, imass -> 1, flags -> 0, species -> 0, force_i -> 0. */
TFG_API int tfg_load_particles(tfg_engine *eng, int n, const float *x, const float *v,
                               const int32_t *type, const float *radius, const float *imass,
                               const uint32_t *flags, const float *species, const float *force_i);
/* Load n particles already binned: cell index (space_cellid order, x-major) and
 * cell-relative position, as the reference stores them (tfSpace_cell.h:103-156).
 * Used for bit-exact state transfer from a reference engine. */
TFG_API int tfg_load_particles_binned(tfg_engine *eng, int n, const int32_t *cell, const float *xrel,
                                      const float *v, const int32_t *type, const float *radius,
                                      const float *imass, const uint32_t *flags,
                                      const float *species, const float *force_i);
/* Bond potentials live in numbered slots; bonds and angles name a slot. */
TFG_API int tfg_set_bonded_potential(tfg_engine *eng, int slot, const tfg_potential *p);
/* Bond::create (tfBond.cpp:638) for n bonds (i[k], j[k]) using potential slot[k] (NULL -> 0). */
TFG_API int tfg_load_bonds(tfg_engine *eng, int n, const int32_t *i, const int32_t *j, const int32_t *slot);
/* Angle::create for n angles (i,j,k) with j the vertex (tfAngle.cpp:90-382). */
TFG_API int tfg_load_angles(tfg_engine *eng, int n, const int32_t *i, const int32_t *j,
                            const int32_t *k, const int32_t *slot);

/* Run nsteps full engine steps on the device (engine_step, tfEngine.cpp:1378-1429):
 * re-bin -> nonbond pair pass -> bonds -> angles -> forward-Euler advance -> flux
 * integration -> FP64 reductions.  Asynchronous on the engine's stream unless an error
 * needs reporting; tfg_sync() waits and returns any device-side error. */
TFG_API int tfg_step(tfg_engine *eng, int nsteps);
/* Forces only: the reference's engine_nonbond_cuda (tfRunner_cuda.cu:2940-3354) + bonded
 * forces, without the advance.  Leaves f, number density and flux increments readable. */
TFG_API int tfg_force_only(tfg_engine *eng, int with_bonded);
TFG_API int tfg_sync(tfg_engine *eng);
/* *idle = 1 when the engine's stream has no unfinished work, else 0 (never blocks). */
TFG_API int tfg_query(tfg_engine *eng, int *idle);
/* Replay steps from CUDA graphs (default on): after any change of layout, tables, work
 * split or stream one step runs eagerly, and the following steps replay a captured
 * single-step graph (one per particle-buffer parity), phase events included. */
TFG_API int tfg_set_graphs(tfg_engine *eng, int enable);
/* Pair lists for simulations in Verlet mode (default on): the tiled pass records each home
 * cell's pairs within the list radius at a rebuild and evaluates those lists until the
 * next one; off, every step tests all candidate pairs of the cell stencil.  The pair set
 * is the same either way. */
TFG_API int tfg_set_pair_lists(tfg_engine *eng, int enable);
/* Autotune the nonbonded pass's form by timing each choice on the current state; the
 * state is left unchanged.  The choices are the tiled kernel's work split (warps per home
 * cell: 1, 2, 7 or 14) and, for engines whose potentials are all tabulated (no DPD, no
 * fluxes, no Verlet pair lists), TFG_PAIR_HOME_OUTER: the kernel that takes home particles
 * one at a time against targets held in registers.  tfg_step and tfg_force_only run it on
 * their first call, and time the work splits again whenever the particle count has grown
 * or shrunk more than 4x since (a batch that fills up or drains); tfg_set_split fixes the
 * choice instead (TFG_PAIR_HOME_OUTER falls back
 * to split 1 while the engine is not eligible).  The reference selects CUDA
 * blocks/threads by hand (cuda::EngineConfig::setBlocks / setThreads,
 * source/cuda/tfEngineConfig.cpp:98-124). */
#define TFG_PAIR_HOME_OUTER 32
TFG_API int tfg_autotune(tfg_engine *eng, int *split);
TFG_API int tfg_set_split(tfg_engine *eng, int split);
/* The whole tuple the autotuner picks: the split (as above), the warps per CTA of the tiled
 * kernel (8, or 4 for engines whose potentials are all tabulated: twice the CTAs per SM) and
 * the home cells a warp takes from the shared work counter at a time (1..8; it times 1, 2, 4).
 * The reference's counterparts are the hand-set blocks and threads of
 * cuda::EngineConfig::setBlocks / setThreads (source/cuda/tfEngineConfig.cpp:98-124). */
TFG_API int tfg_get_tuning(tfg_engine *eng, int *split, int *warps_per_cta, int *grab);
TFG_API int tfg_set_tuning(tfg_engine *eng, int split, int warps_per_cta, int grab);
/* Pair-set signature of the current binned state, per particle id: the number of
 * partners with r2 <= cutoff^2 and the wrap-around sum of a 32-bit mix of their ids.
 * It runs the pair pass's own stencil walk and pair decision (no forces).  Call it after
 * tfg_force_only to describe the pair set that pass used.  A simulation in Verlet mode
 * that did not rebuild at its last step is walked through its pair lists, as its next
 * force pass would be.  Verification hook; the reference has no counterpart. */
TFG_API int tfg_pair_signature(tfg_engine *eng, int32_t *count, uint32_t *hash);
/* The interacting pairs themselves, from the same kernels and pair decision as
 * tfg_pair_signature: up to cap pairs (lower id, higher id), 2*cap ints, in no particular
 * order; *count = all pairs found (cap 0: count only).  Ids are the arena's particle ids
 * (for a single simulation, its particle ids).  Verification hook; no reference counterpart
 * (the reference's pair set is the one its runner_dopair walk finds). */
TFG_API int tfg_pair_list(tfg_engine *eng, int64_t cap, int32_t *pairs, int64_t *count);

TFG_API int tfg_get_count(const tfg_engine *eng, int *n);
/* Download per-particle state in id order.  Any pointer may be NULL.
 *   x: global position (cell origin + relative), xrel: cell-relative, cell: cell index,
 *   f: force (f[0..2]), density: number density f[3], q: flux increments (n*nr_species),
 *   species: state values (n*nr_species). */
TFG_API int tfg_download(tfg_engine *eng, float *x, float *xrel, int32_t *cell, float *v, float *f,
                         float *density, float *species, float *q);
TFG_API int tfg_get_reductions(tfg_engine *eng, tfg_reductions *out);

/* Verlet state of simulation 0 (TFG_ENGINE_VERLET): rebuilds so far, including the first
 * step's, and the largest displacement since the last rebuild as of the last step
 * (space::maxdx, 0 on a rebuild step).  Either pointer may be NULL. */
TFG_API int tfg_get_verlet(tfg_engine *eng, int64_t *rebuilds, float *maxdx);

/* Per-step timing of the device phases of the last step, in milliseconds, from GPU
 * global-timer stamps written between the phases: [0] bin, [1] pair, [2] bonded,
 * [3] advance (-1 when no step has been timed). */
TFG_API int tfg_get_phase_ms(tfg_engine *eng, float ms[4]);
/* Phase stamps on (default) or off: five one-thread kernels per step; turn them off to time
 * whole steps without them. */
TFG_API int tfg_set_phase_timing(tfg_engine *eng, int enable);

/* Set one wall (0..5) of simulation 0; takes effect at the next step. */
TFG_API int tfg_set_boundary(tfg_engine *eng, int wall, const tfg_boundary *bc);
/* Wall potential for particles of `type` (BoundaryCondition::set_potential,
 * tfBoundaryConditions.cpp:504-513); wall -1 sets all six (BoundaryConditions::set_potential
 * :559-571); p NULL removes it.  Tables and DPD potentials are accepted. */
TFG_API int tfg_set_boundary_potential(tfg_engine *eng, int wall, int type, const tfg_potential *p);

/* ---- batches: many independent simulations in one device arena ----
 * The reference runs one engine per process (the global `_Engine`, tfEngine.cpp); it has no
 * counterpart to a batch.  An engine made by tfg_engine_create is a batch holding one
 * simulation, id 0, and the calls above act on it.  tfg_batch_create makes an empty batch;
 * every simulation added must share its max_type and nr_species, and each has its own space,
 * cutoff, dt, seed, flags, potentials, fluxes, types, particles, bonds and angles.  All
 * live simulations step together (tfg_step / tfg_batch_step), one launch per phase for the
 * whole arena; particle ids, random streams and results of a simulation do not depend on
 * what else is in the batch.  Additions, removals and loads take effect at the next step or
 * download, which re-lays the arena out.  Simulation ids are never reused. */
TFG_API int tfg_batch_create(int device, int max_type, int nr_species, tfg_engine **out);
TFG_API int tfg_batch_add_sim(tfg_engine *eng, const tfg_engine_desc *desc, int *sim);
TFG_API int tfg_batch_remove_sim(tfg_engine *eng, int sim);
TFG_API int tfg_batch_sim_count(const tfg_engine *eng, int *live);
TFG_API int tfg_batch_step(tfg_engine *eng, int nsteps);
TFG_API int tfg_batch_set_type(tfg_engine *eng, int sim, int type, int dynamics, float mass);
TFG_API int tfg_batch_set_potential(tfg_engine *eng, int sim, int ti, int tj, const tfg_potential *p);
TFG_API int tfg_batch_add_flux(tfg_engine *eng, int sim, int ti, int tj, const tfg_flux *flux);
TFG_API int tfg_batch_set_species_flags(tfg_engine *eng, int sim, int nr, const uint32_t *flags);
TFG_API int tfg_batch_set_species_reset(tfg_engine *eng, int sim, int nr, const float *values);
TFG_API int tfg_batch_set_stop(tfg_engine *eng, int sim, int64_t step);
TFG_API int tfg_batch_set_random_force(tfg_engine *eng, int sim, int type, float mean, float std,
                                       int duration_steps);
TFG_API int tfg_batch_load_particles(tfg_engine *eng, int sim, int n, const float *x, const float *v,
                                     const int32_t *type, const float *radius, const float *imass,
                                     const uint32_t *flags, const float *species, const float *force_i);
TFG_API int tfg_batch_load_particles_binned(tfg_engine *eng, int sim, int n, const int32_t *cell,
                                            const float *xrel, const float *v, const int32_t *type,
                                            const float *radius, const float *imass, const uint32_t *flags,
                                            const float *species, const float *force_i);
TFG_API int tfg_batch_load_bonds(tfg_engine *eng, int sim, int n, const int32_t *i, const int32_t *j,
                                 const int32_t *slot);
TFG_API int tfg_batch_load_angles(tfg_engine *eng, int sim, int n, const int32_t *i, const int32_t *j,
                                  const int32_t *k, const int32_t *slot);
TFG_API int tfg_batch_get_count(const tfg_engine *eng, int sim, int *n);
TFG_API int tfg_batch_download(tfg_engine *eng, int sim, float *x, float *xrel, int32_t *cell, float *v,
                               float *f, float *density, float *species, float *q);
TFG_API int tfg_batch_get_reductions(tfg_engine *eng, int sim, tfg_reductions *out);
TFG_API int tfg_batch_get_verlet(tfg_engine *eng, int sim, int64_t *rebuilds, float *maxdx);
/* Resume a simulation saved mid-run: after tfg_batch_load_particles_binned (cells and
 * cell-relative positions as tfg_download returns them), set its engine time (steps taken,
 * the counter every random stream is keyed on) and, when q is not NULL, the flux increments
 * its particles carry into the next step (n * nr_species in id order, tfg_download's q:
 * particles that changed cell integrate theirs a step late, tf_engine_advance.cpp:222-236).
 * The reference restores a saved Universe through FIO (tfSimulator.cpp:940-1020). */
TFG_API int tfg_batch_resume(tfg_engine *eng, int sim, int64_t steps, const float *q);
/* Deterministic pair pass (default off): the nonbonded forces are accumulated per particle
 * in a fixed order (the stencil kernel, no atomics), so a run gives the same bits every
 * time and a resumed run continues bit-identically.  Bonded forces still use atomics. */
TFG_API int tfg_set_deterministic(tfg_engine *eng, int enable);
/* Status of one simulation: TFG_OK, or the first error its particles raised (TFG_E_NAN,
 * TFG_E_TOOFAST, TFG_E_RANGE), kept until the simulation is removed.  The reference flags
 * the offending particle and fails the whole step (toofast_error,
 * tf_engine_advance.cpp:72-85, 204-206); in a batch each simulation fails alone: the step
 * call (or tfg_sync) that observes an error returns it, its message names the failed
 * simulations, and the others are unaffected and keep stepping once the failed ones are
 * removed (tfg_batch_remove_sim) or even while they stay.  Waits for the engine's stream. */
TFG_API int tfg_batch_sim_status(tfg_engine *eng, int sim, int *status);
TFG_API int tfg_batch_set_boundary(tfg_engine *eng, int sim, int wall, const tfg_boundary *bc);
TFG_API int tfg_batch_set_boundary_potential(tfg_engine *eng, int sim, int wall, int type, const tfg_potential *p);

/* ---- serving: continuous batching of simulation requests ----
 * The reference runs one simulation per process; there is no counterpart to a server.  Its
 * C entry style (handle + HRESULT-like status, wraps/C/tfC_cuda.h:117-125,
 * wraps/C/tfCUniverse.h:153) is kept.  A request is a whole simulation recorded host-side
 * (tfg_request_*: the same operations as a batch member) plus a step count.  The server keeps
 * one batch (tfg_batch_*) per model family (max_type, nr_species), each on its own CUDA
 * stream, admits arrived requests while they fit an HBM budget and a cap on particles in
 * flight (least work, particles x steps, first; or first come, first served), advances each
 * batch in chunks of at most `quantum` steps cut so that no simulation overshoots, and at
 * every chunk boundary retires the finished simulations (results downloaded to host memory)
 * and admits waiting requests: requests that arrive while others run join at the next chunk.
 * A simulation whose particles raise an error (TFG_E_NAN, TFG_E_TOOFAST, TFG_E_RANGE) is
 * retired as failed with that status; the rest of its batch continues.
 * Threading: one host thread per server handle; tfg_server_poll does all device work. */
typedef struct tfg_server tfg_server;
typedef struct tfg_request tfg_request;

#define TFG_SERVER_LEAST_WORK 0
#define TFG_SERVER_FIFO       1

#define TFG_REQ_QUEUED  0   /* submitted, waiting for admission */
#define TFG_REQ_RUNNING 1   /* in a batch on the device */
#define TFG_REQ_DONE    2   /* finished; its result is ready */
#define TFG_REQ_FAILED  3   /* retired with an error status */

typedef struct tfg_server_desc {
    int32_t device;
    int32_t quantum;          /* largest chunk of steps between admissions (0 -> 50) */
    int64_t budget_bytes;     /* HBM admission budget (0 -> 150 GiB) */
    int64_t max_particles;    /* particles in flight (0 -> no cap); a lone request is always admitted */
    int32_t policy;           /* TFG_SERVER_LEAST_WORK or TFG_SERVER_FIFO */
    int32_t discard_results;  /* 1: do not download finished simulations (throughput runs) */
} tfg_server_desc;

typedef struct tfg_server_stats {
    int64_t submitted, completed, failed;
    int64_t queued, running;          /* now */
    int64_t particles_in_flight, bytes_in_flight;
    int64_t max_concurrent;           /* largest number of simulations in flight so far */
    int64_t chunks;                   /* chunks launched over all batches */
    /* host time spent, in seconds: admitting (recording requests into batches), starting
     * chunks (tfg_batch_step: a re-layout of the arena after a membership change, then the
     * graph launches), retiring (syncs, downloads, removals) */
    double admit_s, launch_s, retire_s;
    /* summed over the batches: wall time from starting a chunk to seeing it complete
     * (busy_s), and from a chunk's completion to the start of the batch's next chunk while
     * the batch still held simulations (gap_s: the host turn between chunks) */
    double busy_s, gap_s;
} tfg_server_stats;

TFG_API int tfg_server_create(const tfg_server_desc *desc, tfg_server **out);
TFG_API int tfg_server_destroy(tfg_server *srv);
/* A request for one simulation of `nsteps` steps; the engine description is a batch
 * member's (tfg_batch_add_sim).  Calls on the request record the model host-side. */
TFG_API int tfg_request_create(const tfg_engine_desc *desc, int max_type, int nr_species, int nsteps,
                               tfg_request **out);
TFG_API int tfg_request_free(tfg_request *req);
TFG_API int tfg_request_set_type(tfg_request *req, int type, int dynamics, float mass);
TFG_API int tfg_request_set_potential(tfg_request *req, int ti, int tj, const tfg_potential *p);
TFG_API int tfg_request_add_flux(tfg_request *req, int ti, int tj, const tfg_flux *flux);
TFG_API int tfg_request_set_species_flags(tfg_request *req, int nr, const uint32_t *flags);
TFG_API int tfg_request_set_species_reset(tfg_request *req, int nr, const float *values);
TFG_API int tfg_request_set_random_force(tfg_request *req, int type, float mean, float std, int duration_steps);
TFG_API int tfg_request_set_boundary(tfg_request *req, int wall, const tfg_boundary *bc);
TFG_API int tfg_request_set_boundary_potential(tfg_request *req, int wall, int type, const tfg_potential *p);
TFG_API int tfg_request_set_bonded_potential(tfg_request *req, int slot, const tfg_potential *p);
TFG_API int tfg_request_load_particles(tfg_request *req, int n, const float *x, const float *v, const int32_t *type,
                                       const float *radius, const float *imass, const uint32_t *flags,
                                       const float *species, const float *force_i);
TFG_API int tfg_request_load_bonds(tfg_request *req, int n, const int32_t *i, const int32_t *j, const int32_t *slot);
TFG_API int tfg_request_load_angles(tfg_request *req, int n, const int32_t *i, const int32_t *j, const int32_t *k,
                                    const int32_t *slot);
/* Submit (arrival = now); the server takes the request over (do not free it).  *id names
 * the request from now on.  A request larger than the whole budget is refused. */
TFG_API int tfg_server_submit(tfg_server *srv, tfg_request *req, int64_t *id);
/* One turn of the serving loop: admit, launch chunks on idle batches, retire finished
 * chunks.  If nothing finished, waits up to wait_us microseconds for a chunk to finish.
 * *completed (may be NULL) = requests finished or failed during this call. */
TFG_API int tfg_server_poll(tfg_server *srv, int wait_us, int *completed);
/* Ids of the requests finished or failed since the last call, up to cap; *n = how many. */
TFG_API int tfg_server_take_finished(tfg_server *srv, int64_t *ids, int cap, int *n);
/* State (TFG_REQ_*) and status (TFG_OK or the failure) of a request; times in seconds on
 * the server's clock (steady clock since creation): submitted, admitted, finished (-1 if
 * not yet).  Any pointer may be NULL. */
TFG_API int tfg_server_request_info(tfg_server *srv, int64_t id, int *state, int *status, double times[3]);
/* Result of a finished request: particle count, then positions (n*3, global), velocities
 * (n*3), species (n*nr_species) in id order and the FP64 totals.  Pass NULL arrays to read
 * n first.  tfg_server_release forgets a finished request. */
TFG_API int tfg_server_result(tfg_server *srv, int64_t id, int *n, float *x, float *v, float *species,
                              tfg_reductions *red);
TFG_API int tfg_server_release(tfg_server *srv, int64_t id);
TFG_API int tfg_server_get_stats(tfg_server *srv, tfg_server_stats *out);
TFG_API const char *tfg_server_last_error(const tfg_server *srv);

/* Measured FP32 FMA throughput of `device` in TFLOP/s (2 flops per FMA), from a
 * register-only kernel with eight independent FMA chains per thread.  Measurement
 * helper for roofline reporting; the reference has no counterpart. */
TFG_API int tfg_probe_fp32_tflops(int device, double *tflops);

/* ---- binning without allocation ----
 * For callers that cannot allocate device memory (code running inside someone else's
 * stream capture, plugins confined to a host application's memory pool, real-time loops
 * where a cudaMalloc/cudaFree would stall the device).  Bins n particles given by GLOBAL
 * positions exactly as tfg_load_particles does (space_setpartp, tfSpace.cpp:432-475) and
 * returns, in caller-owned device buffers: the cell index and cell-relative position of
 * each particle, `order` (particle indices in cell order, by index inside a cell) and
 * `cell_start` (ncells+1 offsets into `order`).  It calls no cudaMalloc, cudaFree or
 * allocating library routine: its temporaries live in one file-scope device array of
 * TFG_NOALLOC_SCRATCH_BYTES that every GPU loading this library holds until exit.
 *   - Limits: n <= TFG_NOALLOC_MAX_PARTICLES, every cells[k] and the product
 *     cells[0]*cells[1]*cells[2] <= TFG_NOALLOC_MAX_CELLS; larger requests return
 *     TFG_E_OVERFLOW and do nothing.  Any cells[k] >= 1 is accepted.
 *   - Work is linear in n however the particles are spread (a stable radix sort on the
 *     cell index): all of them in one cell costs what a uniform spread costs.
 *   - The first call in a CUDA context looks up the array's device address
 *     (cudaGetSymbolAddress, with the device current) and keeps it for that context; make
 *     that first call before any stream capture.  A context created later (the host
 *     application's own, or the primary context after cudaDeviceReset) gets its own lookup.
 *   - All calls share the one array, and each call clears what must start at zero: calls
 *     whose work overlaps on the GPU (other streams, other host threads) race.  Serialise
 *     them, e.g. on one stream.
 *   - Work is queued on `stream` (a cudaStream_t; NULL = legacy default stream).
 *   - TFG_E_CUDA reports a failure of this call's own launches only: earlier errors on the
 *     calling thread are neither read nor cleared (no cudaGetLastError).
 * No counterpart in the reference (its binning always runs on the host). */
#define TFG_NOALLOC_MAX_PARTICLES 1048576
#define TFG_NOALLOC_MAX_CELLS     262144
#define TFG_NOALLOC_SCRATCH_BYTES \
    ((TFG_NOALLOC_MAX_CELLS + 2 * 256 * (TFG_NOALLOC_MAX_PARTICLES / 1024) + 1 + 2 * TFG_NOALLOC_MAX_PARTICLES + 256) * 4)
TFG_API int tfg_bin_noalloc(const tfg_engine_desc *desc, int n, const float *x_dev, int32_t *cell_dev,
                            float *xrel_dev, int32_t *order_dev, int32_t *cell_start_dev, void *stream);

/* Library build information: returns a static string. */
TFG_API const char *tfg_build_info(void);

#ifdef __cplusplus
}
#endif
#endif /* TFG_H */
