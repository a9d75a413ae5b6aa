/*
 * solveit_gpu.h -- C ABI of the GB300 force-evaluation engine for SOLVEiT.
 *
 * One context (sv_ctx) owns one plume's particle state in GPU memory, a CUDA
 * stream and all method workspaces.  Host buffers belong to the caller.
 * Every call returns an sv_status; on failure sv_last_error() describes it.
 * Calls on one context are issued from one host thread and are ordered on the
 * context's stream; only the download / readback calls block.
 *
 * Each entry point names the reference interface it stands in for (paths are
 * inside the SOLVEiT-Code project).  The reference's force methods are
 * ForceCalculationMethod subclasses (force_calculation_methods.h:28-87) that
 * ADD acceleration (m/s^2) into ChargedParticles::acceleration[i].xyz for
 * inbound targets (w == 1) from sources with w in {1, 2}; the integrator
 * zeroes inbound accelerations first (integration_schemes.cpp:344).
 */
#ifndef SOLVEIT_GPU_H
#define SOLVEIT_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SV_ABI_VERSION 1

#if defined(__GNUC__)
#define SV_API __attribute__((visibility("default")))
#else
#define SV_API
#endif

typedef struct sv_ctx sv_ctx;

typedef enum {
    SV_OK = 0,
    SV_ERR_INVALID = 1,     /* bad argument (null pointer, n < 0, bad enum) */
    SV_ERR_CUDA = 2,        /* a CUDA call failed; see sv_last_error */
    SV_ERR_ALLOC = 3,       /* device or pinned allocation failed */
    SV_ERR_STATE = 4,       /* call out of order (e.g. compute before upload) */
    SV_ERR_CAPACITY = 5,    /* a fixed-capacity structure overflowed */
    SV_ERR_TIMEOUT = 6,     /* a bounded device wait gave up */
    SV_ERR_UNSUPPORTED = 7  /* method/symmetry/precision combination not built */
} sv_status;

/* Force method (the ForceCalculationMethod subclass it replaces). */
typedef enum {
    SV_METHOD_DIRECT = 0,      /* DirectForceCalculation, direct_force_method.cpp:347 */
    SV_METHOD_BARNES_HUT = 1,  /* BarnesHutForceCalculation, barnes_hut_force_calculation.cpp:574 */
    SV_METHOD_FMM = 2          /* MultipoleMethodForceCalculation, multipole_method_force_calculation.cpp:148 */
} sv_method;

/* SimulationParameters::symType (simulation_parameters.h:139, structures.h:200-204). */
typedef enum {
    SV_SYM_NONE = 0,
    SV_SYM_ROTATIONAL = 1,     /* 4-fold images about z (direct_force_method_rotational.cpp:48-94) */
    SV_SYM_TRANSLATIONAL = 2   /* finite periodic image lattice (lattice_point.h:65-131) */
} sv_symmetry;

/* Arithmetic of the pair / expansion work.  MIXED: FP32 pair and expansion
 * arithmetic on coordinates taken relative to a nearby FP64 origin, FP64
 * accumulation across tiles; FP64: every operation in FP64. */
typedef enum {
    SV_PREC_MIXED = 0,
    SV_PREC_FP64 = 1
} sv_precision;

/* FMM variant (FmmType, structures.h:283-288).  The treecode evaluates the
 * far-field multipoles directly at the particles (M2P) instead of M2L/L2L/L2P;
 * the outlier variants take particles whose position deviates from the median
 * by 3 or more scaled median absolute deviations on any axis
 * (DomainBoundsFunction::isOutlier, domain_bounds_functions.cpp:16-99) out of
 * the tree and sum every interaction that involves one of them directly. */
typedef enum {
    SV_FMM_FMM = 0,               /* FmmType::fmm */
    SV_FMM_FMM_OUTLIERS = 1,      /* FmmType::fmmOutliers */
    SV_FMM_TREECODE = 2,          /* FmmType::treecode */
    SV_FMM_TREECODE_OUTLIERS = 3  /* FmmType::treecodeOutliers */
} sv_fmm_type;

typedef struct {
    double softening2;       /* eps^2 in m^2 (constants.h:31 SOFTENING) */
    double k_const;          /* e^2/(4 pi eps0 amu) (constants.h:46 K_CONST) */
    double e_over_amu;       /* ELEM_CHARGE/AMU (particles.cpp:500) */
    double efield[3];        /* uniform background field in V/m, added in the kick */
    int32_t method;          /* sv_method */
    int32_t precision;       /* sv_precision */
    int32_t symmetry;        /* sv_symmetry */
    float theta;             /* BH opening parameter (setTheta, barnes_hut_force_calculation.cpp:110) */
    int32_t leaf_size;       /* BH leaf bucket size (reference: 1 particle per leaf) */
    int32_t fmm_order;       /* expansion order p (setNumExpansions), 1..10 */
    int32_t fmm_ws;          /* FMM well-separation in boxes (reference: 1) */
    int32_t fmm_leaf_target; /* mean particles per occupied leaf box when choosing the depth */
    int32_t sym_axes[3];     /* periodic axes (SimulationParameters::symmetryAxes) */
    int32_t sym_levels;      /* numSymmetryLevels: 3^levels cells per periodic axis */
    double domain_size[3];   /* periodic cell size in m (SimulationParameters::domainSize) */
    int32_t device;          /* CUDA device ordinal */
    int32_t profile_phases;  /* 1: record device time of each phase into sv_stats.ms_phase */
    int32_t fmm_type;        /* sv_fmm_type */
    float fmm_root_scale;    /* FMM root cube side = this x the smallest power of two >= the
                                plume's extent, rounded down to a multiple of 1/8 in [1, 2)
                                (0: 1): leaf boxes between two octree levels' sizes, so the
                                box side can follow the plume (sv_fmm_tune picks it) */
    int32_t fmm_direct_pairs;  /* leaf-level interaction-list entries whose two boxes hold fewer
                                particles multiplied than this are summed as direct pairs in the
                                near field instead of an M2L translation (up to 128 per box; single
                                plumes and a batch's FMM forest): 0 = 1024, < 0 = every entry by M2L */
    int32_t fmm_m2l_tc;        /* M2L translations: 1 = on the tensor cores (offset classes as dense TF32x3
                                contractions, tcgen05), -1 = the FP32 rotation kernel, 0 = the default
                                (the tensor cores) */
    float fmm_tune_err;        /* sv_fmm_tune's force-error bound: > 0 makes it choose the expansion order
                                and separation as well (the fastest that meets the bound on sampled
                                targets); 0 = it tunes the root scale only */
    int32_t fmm_near;          /* FMM near field at fmm_ws = 2: 1 = the full cube of 5^3 boxes, 2 = trimmed
                                (the 32 boxes at (2,2,1)- and (2,2,2)-type offsets go to the M2L, whose
                                worst separation ratio they do not raise), 0 = the default (the full
                                cube); ignored at fmm_ws = 1 */
} sv_params;

/* Per-call statistics of the last force evaluation. */
typedef struct {
    double pair_interactions;     /* particle-particle pairs evaluated */
    double cell_interactions;     /* BH accepted cells / FMM M2L translations */
    double flops_algorithmic;     /* 20 flop/pair + expansion flops (method's count) */
    double ms_total;              /* device time of the whole evaluation */
    double ms_phase[8];           /* sort, tree, lists, upward (P2M+M2M), downward (M2L+L2L),
                                     L2P, near field (P2P / direct / BH walk), scatter; the FMM
                                     runs its near field on a second stream beside the upward
                                     and downward passes, so its entry is the P2P's own device
                                     time and overlaps them */
    int32_t levels;               /* FMM leaf level / BH max depth */
    int32_t boxes;                /* occupied leaf boxes / BH nodes */
    int32_t m2l_tc;               /* FMM: 1 when the last evaluation's M2L ran on the tensor cores, 0 when
                                     it ran on the FP32 rotation kernel */
    int32_t reserved[5];
} sv_stats;

/* Fill p with the defaults of the reference configuration: softening
 * 6.4e-19 m^2, K and e/amu as constants.h evaluates them, direct method,
 * mixed precision, no symmetry, theta 0.5, leaf 16, p 8, ws 1. */
SV_API sv_status sv_default_params(sv_params *p);

/* Stands in for constructing a ForceCalculationMethod on a ParticleSystem
 * (force_calculation_methods.h:33-35). */
SV_API sv_status sv_create(const sv_params *p, sv_ctx **out);
SV_API void sv_destroy(sv_ctx *ctx);
/* setTheta / setNumExpansions / symType etc. in one call. */
SV_API sv_status sv_set_params(sv_ctx *ctx, const sv_params *p);
SV_API sv_status sv_get_params(const sv_ctx *ctx, sv_params *p);

/* Load a plume.  x3, v3: 3n interleaved (m, m/s); q in e; m_amu in amu;
 * status as ParticleStatus (1 inbound, 2 source only, 0 / -1 ignored);
 * t_inj: injection time in s (timeInjected).  Null v3 / t_inj mean zero. */
SV_API sv_status sv_upload(sv_ctx *ctx, int64_t n, const double *x3, const double *v3,
                    const double *q, const double *m_amu, const int32_t *status,
                    const double *t_inj);
/* Same from the reference's own arrays (particles.h:99-105): position =
 * (x,y,z,q), velocity = (vx,vy,vz,species), acceleration.w = status;
 * masses come from the species code (particles.h:65-87). */
SV_API sv_status sv_upload_ref32(sv_ctx *ctx, int64_t n, const float *pos4,
                          const float *vel4, const float *acc4,
                          const float *t_inj);
SV_API sv_status sv_download(sv_ctx *ctx, double *x3, double *v3, int32_t *status);
/* Replace the uploaded plume's positions, velocities and statuses (the arrays
 * the reference's integrator advances, particles.h:99-105: position,
 * velocity, acceleration.w) and keep its charges, masses, injection times and
 * run state (events, energy records, snapshot fields, substep levels).  n must
 * be the uploaded count; v3 and status may be null to keep them.  The same
 * transfers as sv_upload: pinned, mapped arrays are read in place. */
SV_API sv_status sv_update_state(sv_ctx *ctx, int64_t n, const double *x3, const double *v3,
                                 const int32_t *status);
SV_API sv_status sv_download_ref32(sv_ctx *ctx, float *pos4, float *vel4);

/* One force evaluation with the context's method: the body of
 * updateAcceleration() (direct_force_method.cpp:347-428,
 * barnes_hut_force_calculation.cpp:574-715,
 * multipole_method_force_calculation.cpp:148-522).  As there, only particles
 * with index in [first, last) take part: targets are the inbound ones, sources
 * those with status 1 or 2 (direct_force_method.cpp:374-377).  The result
 * (m/s^2, FP64) stays on the device; a3_out, if not null, receives a copy (3n
 * interleaved, zero for non-targets). */
SV_API sv_status sv_compute_accel(sv_ctx *ctx, int64_t first, int64_t last, double *a3_out);
/* acceleration[i].xyz += a_i for inbound i, i.e. the += contract of
 * ForceCalculationMethod::updateAcceleration on the reference's vec4 array. */
SV_API sv_status sv_add_accel_ref32(sv_ctx *ctx, float *acc4);

/* nsteps of LeapfrogDKD (integration_schemes.cpp:856-891): drift dt/2,
 * kick dt (force + uniform field), drift dt/2, with the reference's
 * injection-time clamps (particles.cpp:693-786).  t0 is the time at the start
 * of the first step.  Injection window (LeapfrogDKD::driftNew,
 * integration_schemes.cpp:705-723, and ChargedParticles::findMostRecentInjected,
 * particles.cpp:1328-1366): a half-step drift over [t, t + dt/2] acts on the
 * particles with t_inj <= t + dt/2, and the force and kick of a step act on the
 * particles with t_inj <= its mid time, as sources and as targets; particles
 * injected later keep their state.  With t_inj ascending in index order (the
 * reference's precondition) this is the reference's [firstParticle,
 * lastParticle) window.  The boundary set by sv_set_boundary is applied after
 * every drift. */
SV_API sv_status sv_leapfrog(sv_ctx *ctx, int32_t nsteps, double dt, double t0);

/* Crash and boundary conditions of the drift, as ParticleSystem::
 * propagatePositionNew (particles.cpp:33-40) applies them for every particle
 * in the injection window:
 * 1. crash (CrashParameters::checkExtractorGridCrash, structures.h:467-517,
 *    called from ChargedParticles::propagatePositionNew, particles.cpp:
 *    693-739): the segment of a status 1 or 2 particle's drift, in the (r, z)
 *    plane, against the extractor grid (the ring r >= crash_r between z =
 *    crash_z and crash_z + crash_width): on a hit the status becomes -1
 *    (crashed), z the hit's z, and x, y follow the straight path to that z;
 * 2. folding when fold != 0 (enforceSymmetryConditions, particles.cpp:
 *    199-333), of every particle in the window whatever its status: with the
 *    rotational symmetry into the first quadrant (positions and velocities),
 *    with the translational one into [-L/2, L/2) on each periodic axis;
 * 3. boundary conditions (enforceBoundaryConditions, particles.cpp:73-177) on
 *    inbound particles: spatial, |x| > bc_space[0], |y| > bc_space[1],
 *    |z| > bc_space[2] or sqrt(x^2 + y^2) > bc_space[3] (a zero limit is off),
 *    then temporal, t - t_inj > bc_time; either sets the status to 0 (out of
 *    bounds).
 * Every crash and boundary hit records an sv_event. */
typedef enum {
    SV_CRASH_NONE = 0,            /* CrashConditionOptions::none */
    SV_CRASH_EXTRACTOR_GRID = 1   /* CrashConditionOptions::extractorGrid */
} sv_crash_kind;

typedef enum {
    SV_BC_NONE = 0,               /* BoundaryConditionOptions::none */
    SV_BC_SPACE = 1,              /* ::space */
    SV_BC_TIME = 2,               /* ::time */
    SV_BC_SPACE_AND_TIME = 3      /* ::space_and_time */
} sv_bc_kind;

typedef struct {
    int32_t crash;          /* sv_crash_kind */
    int32_t bc;             /* sv_bc_kind */
    double crash_z;         /* z_distance: bottom of the grid (m) */
    double crash_width;     /* z_width: thickness of the grid (m) */
    double crash_r;         /* r_distance: inner radius of the grid (m) */
    double bc_space[4];     /* spatialBoundaryConditions x, y, z, w (m; 0 = off) */
    double bc_time;         /* temporalBoundaryCondition (s) */
    int32_t fold;           /* 1: fold into the symmetry domain of the context's symmetry */
    int32_t reserved[7];
} sv_boundary;

/* Default: no crash, no boundary conditions, no folding. */
SV_API sv_status sv_set_boundary(sv_ctx *ctx, const sv_boundary *b);
SV_API sv_status sv_get_boundary(const sv_ctx *ctx, sv_boundary *b);

/* One crash or boundary event: the 40-byte record that
 * ChargedParticles::writeToEventsFile (particles.cpp:666-684) appends to the
 * events file, field for field (time of the event; position and velocity
 * after the event; particle index; species code; status after the event,
 * -1 crashed or 0 out of bounds, written as its 32-bit pattern). */
typedef struct {
    float time;
    float x, y, z;
    float vx, vy, vz;
    int32_t index;
    uint32_t species;       /* velocity.w of the reference (0xffffffff: mass not in the species table) */
    int32_t status;
} sv_event;

/* Events recorded since the last call, in the reference's file order (by
 * drift, then crashes before spatial before temporal hits, then particle
 * index).  out may be null to query the count; otherwise up to cap records are
 * copied and all recorded events are released.  A context keeps up to
 * max(65536, n) events between calls; events past that are dropped, and the
 * next call returns SV_ERR_CAPACITY with count = events recorded + dropped. */
SV_API sv_status sv_get_events(sv_ctx *ctx, sv_event *out, int64_t cap, int64_t *count);

/* Snapshot records (Integrator::saveData, integration_schemes.cpp:266-331,
 * SaveDataOptions, structures.h:244-247): one record per particle with status
 * 1 or 2 and index in [first, last), in index order; last < 0 means n.
 *   SV_SNAPSHOT_ORIGINAL: x, y, z, vx, vy, vz, E1[3], E2[3] (float32), species
 *     (uint32), index (int32), lastParticle (int32): 60 bytes per record;
 *   SV_SNAPSHOT_NEW_ORIGINAL: a 12-byte header (0xffffffff, lastParticle,
 *     currentTime as float32), then index (int32), species (uint32), x, y, z,
 *     vx, vy, vz, E1[3], E2[3] (float32): 56 bytes per record.
 * lastParticle is `last`, currentTime is current_time.  E1 and E2 are the
 * particle-particle field, (amu/e)(m/q) a (Integrator::updateAcceleration,
 * :336-367), and the background field (particles.cpp:512) at the particle's
 * last kick of sv_leapfrog as a target (zero before its first one), as the
 * reference's Efield1 / Efield2 arrays hold them.
 * With SV_SNAPSHOT_FULL or-ed into the format, the records are those of
 * Integrator::saveFullCurrentConditions (integration_schemes.cpp:197-258):
 * every particle of [0, n) whatever its status and injection time (first is
 * ignored; last is still written as lastParticle).
 * *bytes receives the size; out (cap_bytes) may be null to query it.  The
 * records go to the file as they are (fwrite). */
typedef enum {
    SV_SNAPSHOT_ORIGINAL = 0,     /* SaveDataOptions::original */
    SV_SNAPSHOT_NEW_ORIGINAL = 1, /* SaveDataOptions::newOriginal */
    SV_SNAPSHOT_FULL = 16         /* flag: saveFullCurrentConditions */
} sv_snapshot_format;

SV_API sv_status sv_snapshot(sv_ctx *ctx, int32_t format, int64_t first, int64_t last, float current_time,
                             void *out, int64_t cap_bytes, int64_t *bytes);

/* Energy bookkeeping of the reference's integrator (Integrator::toggleEnergy,
 * integration_schemes.cpp:85-97; initializeEnergyData :757-775;
 * updateEnergyInjectionData :783-793; updateEnergyIntervalData :799-835).
 * enable = 1 arms it; the next step of sv_leapfrog first takes, for every
 * particle, its kinetic energy and the work of the emitter field along z from
 * (0, 0, z_max r0) and then along (x, y) (init_steps samples per leg; zero
 * without an emitter field).  Before each drift, the particles injected since
 * the previous drift add their kinetic energy and field energy of the set-up
 * and their potential energy at that moment to KE_inj, FE_inj, PE_inj.  After
 * every `interval`-th step (counted as the reference does: the step that
 * starts at t is number round(t / dt) + 1), each particle of the window
 * updates its field energy along the path it moved since the previous update
 * (max(min(dt interval, t - t_inj) steps / dt, 2) samples per leg), and one
 * record is kept: KE_inj, PE_inj, FE_inj and the window's KE, PE (halved) and
 * FE.  The window is the reference's [firstParticle, lastParticle): the
 * injected particles from the first one with status 1 or 2 on, whatever their
 * status; potential energies are q_i q_j e^2 / (4 pi eps0 sqrt(r^2 + eps^2))
 * over it.  Sums are FP64 (the reference's are FP32), the potential's pairs
 * FP32 on FP32 hi + lo offsets.  The potential energy costs a direct sum over
 * the window per record (O(n^2)), as in the reference.  sv_upload re-arms the
 * set-up and clears the records; enable = 0 releases everything.  Single-rate
 * leapfrog of a single-plume context only (batch, substeps and the adjoint
 * return SV_ERR_UNSUPPORTED). */
typedef struct {
    float ke_inj, pe_inj, fe_inj, ke, pe, fe;  /* J: the energy file's 24-byte record */
} sv_energy_record;

SV_API sv_status sv_set_energy(sv_ctx *ctx, int32_t enable, int32_t init_steps, int32_t steps, int32_t interval);
/* Copies up to cap records (oldest first) to out and releases them; *count
 * receives how many were kept.  out may be null to query the count. */
SV_API sv_status sv_get_energy_records(sv_ctx *ctx, sv_energy_record *out, int64_t cap, int64_t *count);

/* Multi-rate leapfrog (LeapfrogDKDSubsteps, integration_schemes.cpp:899-1528).
 * Each entry asks for steps of at most dt inside a region: spatial limits
 * bc_space (|x|, |y|, |z|, r; 0 = unbounded) and/or a limit bc_time on the
 * time since injection, of kind bc (sv_bc_kind).  The entries are resolved
 * into levels l = 0 .. L with steps time_step / 3^l exactly as
 * setSubstepTimes (:1361-1427) resolves them.  sv_leapfrog then runs
 * LeapfrogDKDSubsteps::runSimulation's recursion (:1494-1526): a level's drift
 * half is drift, kick, drift of the next finer level; only the finest level
 * drifts (every particle) and kicks; a kick makes the particles at levels >=
 * its top level targets (status 1) and the coarser ones sources only (status
 * 2, setParticleStatus :1216-1236), evaluates the force with the context's
 * method plus the background field, and kicks each target by its own level's
 * step (variableTimestepKick :1241-1262); particles are moved between levels
 * after each coarser drift half (crossoverParticles / checkConditions
 * :932-1111).  Every particle starts at the finest level (set and upload).
 * sv_leapfrog must then be called with dt = time_step.  n = 0 returns to the
 * single-rate leapfrog.  Single-plume contexts only; at most 16 levels. */
typedef struct {
    double dt;              /* largest step inside the region (s) */
    int32_t bc;             /* sv_bc_kind of the region */
    double bc_space[4];     /* |x|, |y|, |z|, r limits (m); 0 = unbounded */
    double bc_time;         /* limit on the time since injection (s); 0 = unbounded */
} sv_substep;

SV_API sv_status sv_set_substeps(sv_ctx *ctx, double time_step, int32_t n, const sv_substep *substeps);
/* The substep level of every particle (n bytes). */
SV_API sv_status sv_get_substep_levels(sv_ctx *ctx, int8_t *levels);

/* Background field of a single emitter (BackgroundEfield::singleEmitter), as
 * InterpolationScheme::computeEfieldSingleEmitter (interpolation_scheme.cpp:
 * 206-262) evaluates it from the field map the reference reads from its
 * Fields and Triangles files (fillInterpolationScheme / fillTriangleScheme,
 * interpolation_scheme.cpp:66-150):
 *   node_rz    2 n_nodes: (r, z) of the nodes in units of r0
 *   e_r, e_z   n_nodes: the field's radial and axial components in units of e0
 *   triangles  3 n_triangles node indices
 *   neighbors  3 n_triangles: the triangle across the edge opposite each
 *              vertex, -1 on the hull
 * At a particle (x, y, z), (r, z) = (sqrt(x^2 + y^2), z) / r0; for z outside
 * [0, z_max] there is no field (the reference uses z_max = 140).  Otherwise the
 * triangle holding (r, z) is found by the walk of triangulation_search_delaunay
 * (pwl_interp_2d_scattered.c:1762-1992; outside the hull the field is
 * extrapolated from the triangle where the walk stops), E_r and E_z are
 * interpolated linearly in it (pwl_interp_2d_scattered_value, :887-957), and
 * E = e0 (E_r x/r, E_r y/r, E_z).  sv_leapfrog's kick adds (e/amu)(q/m) E for
 * inbound particles (computeBackgroundAcceleration, particles.cpp:496-520),
 * with sv_params.efield on top.  Each particle's walk starts from its triangle
 * of the previous kick.  n_nodes = 0 removes the map.  A walk that does not end
 * (a triangulation with a cycle) or a degenerate triangle makes sv_leapfrog
 * return SV_ERR_INVALID. */
SV_API sv_status sv_set_emitter_field(sv_ctx *ctx, int32_t n_nodes, const double *node_rz, const double *e_r,
                                      const double *e_z, int32_t n_triangles, const int32_t *triangles,
                                      const int32_t *neighbors, double r0, double e0, double z_max);
/* The emitter field in V/m at n points (x3, e3: 3n interleaved, host); each
 * walk starts from the middle triangle, (n_triangles + 1)/2 - 1, as the
 * reference's first search does. */
SV_API sv_status sv_emitter_field_at(sv_ctx *ctx, int64_t n, const double *x3, double *e3);

/* Adjoint of sv_leapfrog with the direct sum (no reference counterpart: the
 * reference integrates forward only).  sv_adjoint_forward runs nsteps like
 * sv_leapfrog and keeps the state every checkpoint_every steps;
 * sv_adjoint_backward takes dL/dx and dL/dv of the final state (host, 3n
 * interleaved) and returns dL/dx0, dL/dv0 (3n, nullable) and dL/dE (3,
 * nullable, per V/m of the uniform field), re-running each checkpointed segment
 * and applying the transposed Jacobian of the softened Coulomb sum.  The
 * context's state is the final state again on return. */
SV_API sv_status sv_adjoint_forward(sv_ctx *ctx, int32_t nsteps, double dt, double t0,
                                    int32_t checkpoint_every);
SV_API sv_status sv_adjoint_backward(sv_ctx *ctx, const double *dl_dx3, const double *dl_dv3,
                                     double *dl_dx0, double *dl_dv0, double *dl_defield);

/* Outlier flags of the last evaluation with an outlier variant of the FMM, in
 * the caller's order, as the reference's outlierCheck
 * (domain_bounds_functions.cpp:78-89): 1 outlier, 0 source within bounds,
 * -1 no source; count receives the number of outliers.  Either may be null. */
SV_API sv_status sv_get_outliers(sv_ctx *ctx, int32_t *flags, int64_t *count);

/* Kinetic and softened potential energy in J, FP64, over all particles
 * (particles.cpp:535-578 with the halving of integration_schemes.cpp:815). */
SV_API sv_status sv_energy(sv_ctx *ctx, double *ke, double *pe);

/* Per-particle relative-L2 accuracy metric of Integrator::compareAcceleration
 * (integration_schemes.cpp:411-461) of the last evaluation's acceleration
 * against a host reference ref3 (3n interleaved, m/s^2), computed on the
 * device in FP64 over that evaluation's window [first, last) (the whole plume
 * after sv_leapfrog or a batch): l2 = sqrt(mean over inbound k of
 * |a_k - ref_k|^2 / |ref_k|^2), maxl2 = the largest per-particle term's square
 * root, argmax = its index (the first of equal largest terms; 0 when none is
 * positive).  maxl2 and argmax may be null. */
SV_API sv_status sv_compare_accel(sv_ctx *ctx, const double *ref3, double *l2, double *maxl2,
                           int64_t *argmax);

SV_API sv_status sv_get_stats(const sv_ctx *ctx, sv_stats *out);
SV_API sv_status sv_sync(sv_ctx *ctx);
/* The context's cudaStream_t, for callers that time or order work on it. */
SV_API void *sv_stream(sv_ctx *ctx);
/* Kernels this context has launched since creation. */
SV_API uint64_t sv_launch_count(const sv_ctx *ctx);
SV_API const char *sv_last_error(const sv_ctx *ctx);
SV_API int32_t sv_abi_version(void);

/* Many independent plumes in one context.  The reference runs one
 * ForceCalculationMethod and one LeapfrogDKD loop per ParticleSystem
 * (force_calculation_methods.h:28-87, integration_schemes.cpp:856-891); a
 * batch runs every plume of a study at once.  Plume p owns the caller
 * particles [counts[0] + ... + counts[p-1], + counts[p]) of the arrays (laid
 * out as sv_upload's), uses method[p] (SV_METHOD_DIRECT or SV_METHOD_FMM, the
 * FMM at the context's fmm_order and fmm_ws) and symmetry[p] (SV_SYM_NONE or
 * SV_SYM_ROTATIONAL), and interacts with no other plume.  Afterwards
 * sv_compute_accel (whole batch; first/last are ignored), sv_leapfrog,
 * sv_download, sv_download_ref32 and sv_compare_accel act on all plumes;
 * sv_energy and the adjoint return SV_ERR_UNSUPPORTED.  Each force evaluation
 * and each leapfrog step is one CUDA-graph launch.  Uploading a batch of the
 * same shape (plume counts, methods, symmetries) again keeps the plan and the
 * graphs; a later sv_upload or sv_upload_ref32 leaves batch mode.  At most
 * 512 plumes. */
SV_API sv_status sv_upload_batch(sv_ctx *ctx, int32_t nplumes, const int64_t *counts, const int32_t *method,
                                 const int32_t *symmetry, const double *x3, const double *v3, const double *q,
                                 const double *m_amu, const int32_t *status, const double *t_inj);
/* Autotuner of a batch (no reference counterpart): times the weight of the
 * FMM plumes' depth model (the cost of one M2L translation in pair
 * interactions; each plume's depth is chosen on the device at every
 * evaluation to minimise P2P pairs + weight * M2L translations) and the direct
 * plumes' work-item size on the uploaded state and keeps the fastest; among
 * weights within 3 % of the fastest it keeps the largest (shallower trees, whose
 * M2L work grows less as the plumes expand).  With fmm_tune_err > 0 it also
 * chooses the forest's expansion order (4, 6, 8) and, at fmm_ws = 2 with
 * fmm_near = 0, the near-field shape: the fastest whose force error (the
 * largest over up to four FMM plumes without symmetry images, 64 sampled
 * targets each, against an FP64 direct sum) is at most fmm_tune_err, else the
 * most accurate; sv_get_params and sv_batch_get_info show the choice.  Results
 * are cached per batch shape (plume count, size buckets, methods, symmetries,
 * order, separation, near field, M2L path, error bound) in the process and,
 * when cache_path is not null, in that text file (read first, appended to).
 * best_ms (nullable) receives the tuned force-evaluation time. */
SV_API sv_status sv_batch_tune(sv_ctx *ctx, const char *cache_path, double *best_ms);
/* Autotuner of a single-plume FMM context, after the reference's timing-driven
 * choice of the FMM's level (MultipoleMethodForceCalculation::setOptimumLevel,
 * multipole_method_force_calculation.cpp:835-881; Integrator::compareAcceleration
 * raising maxLevel from measured times, integration_schemes.cpp:470-570): times
 * force evaluations of the uploaded state at fmm_root_scale = 1, 1.125, ...,
 * 1.875 and keeps the fastest in the context's parameters (sv_get_params
 * shows it).  The root scale sets the leaf box side between two octree
 * levels' sides, so it is also the leaf-size choice.  With fmm_tune_err > 0
 * it also chooses the expansion order, separation and near-field shape, as
 * the reference's test cases sweep the order (test_cases.cpp:217-295): for
 * each of (p, ws) = (6, 2), (8, 1), (8, 2), (10, 1), (10, 2), with both
 * fmm_near shapes at ws = 2 unless fmm_near is set, it tunes the root scale, measures
 * the per-particle relative-L2 force error on 256 evenly spaced targets
 * against an FP64 direct sum, and keeps the fastest candidate whose error is
 * at most fmm_tune_err (the most accurate one when none is).  best_ms
 * (nullable) receives the kept force-evaluation time. */
SV_API sv_status sv_fmm_tune(sv_ctx *ctx, double *best_ms);
/* Sets the two tuned quantities directly (M2L weight >= 1, direct sources
 * per work item >= 256) and re-plans the batch. */
SV_API sv_status sv_batch_set_tuning(sv_ctx *ctx, int32_t m2l_weight, int32_t direct_chunk);
typedef struct {
    int32_t nplumes, fmm_plumes;
    int64_t slots, fmm_slots;       /* particles plus FMM rotational image copies */
    int32_t leaf_level;             /* leaf level of the FMM forest */
    int32_t m2l_weight;             /* tuned M2L cost in pair units of the depth model */
    int32_t direct_chunk;           /* tuned sources per direct work item */
    int32_t direct_items;
    int32_t graph_kernels_step;     /* kernel nodes of one captured leapfrog step */
    int32_t graph_kernels_accel;    /* kernel nodes of one captured force evaluation */
    double tuned_ms;                /* force-evaluation time measured by sv_batch_tune */
    double direct_pairs;            /* pair interactions of the direct plumes per evaluation */
    double fmm_m2l;                 /* M2L translations of the last FMM forest evaluation */
    double fmm_pairs;               /* P2P pair interactions of the last FMM forest evaluation */
    int32_t regrows;                /* times a box capacity overflowed and the work was redone */
    int32_t overflow_mask;          /* bit l: forest level l overflowed at the last regrow */
    int32_t level_boxes[22];        /* forest boxes per level at the last evaluation */
    int32_t level_cap[22];          /* box capacity per level */
    int32_t level_max[22];          /* largest box count per level since the last plan */
    int32_t max_leaf;               /* most slots in one leaf box at the last evaluation */
    int32_t m2l_tc;                 /* 1: the last forest evaluation's M2L ran on the tensor cores, 0: on the
                                       FP32 rotation kernel (selected, or its room was outgrown) */
    int32_t fmm_order;              /* the forest's expansion order (sv_batch_tune may choose it) */
    int32_t fmm_near;               /* the forest's near field (sv_params.fmm_near) */
    int32_t reserved[2];
} sv_batch_info;
SV_API sv_status sv_batch_get_info(const sv_ctx *ctx, sv_batch_info *out);

/* Direct sum that allocates no memory.  No counterpart in the reference: it
 * is for callers that cannot allocate device memory (an allocator owned by a
 * host framework, real-time loops that forbid cudaMalloc / cudaFree and their
 * implicit synchronisation).  Computes the same acceleration as
 * sv_compute_accel with SV_METHOD_DIRECT, SV_PREC_MIXED, SV_SYM_NONE: a3
 * (3n interleaved, m/s^2) for every particle with status 1, 0 for the others,
 * sources with status 1 or 2.  All pointers are DEVICE pointers on the current
 * device; x3 is 3n interleaved (m), q in e, m_amu in amu; stream is a
 * cudaStream_t (NULL = legacy default stream).  Working storage is one static
 * device array of SV_NOALLOC_SCRATCH_BYTES that each GPU loading the library
 * holds until exit; n above SV_NOALLOC_MAX_N returns SV_ERR_CAPACITY.  The
 * first call on a device is its set-up call: it looks the array up
 * (cudaGetSymbolAddress) and, under lazy module loading (the CUDA default),
 * loads the library's device code on that device, which commits the array's
 * memory and can synchronise the device; make it during set-up, before any
 * stream capture.  The looked-up address is kept for the life of the process,
 * so after a cudaDeviceReset the entry point must not be called on that device
 * again.  A CUDA error already pending on the calling thread makes the call
 * return SV_ERR_CUDA without work and is left pending.  Calls whose work
 * overlaps on the GPU race on the shared array. */
#define SV_NOALLOC_MAX_N 262144
#define SV_NOALLOC_SCRATCH_BYTES (40u << 20)
SV_API sv_status sv_direct_accel_noalloc(int64_t n, const double *x3, const double *q, const double *m_amu,
                                         const int32_t *status, double softening2, double k_const,
                                         double *a3, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* SOLVEIT_GPU_H */
