/*
 * sv_oracle.h -- CPU restatement of the SOLVEiT force-evaluation hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: the parity tests,
 * the smoke check and the CPU-baseline leg of bench.py call it to produce the
 * numbers the CUDA path is compared against.  Nothing in the product path
 * (libsolveit_gpu.so, the host adapter) links or calls it.
 *
 * Two families of functions:
 *   *_ref32  restate the reference arithmetic on its own FP32 vec4 state
 *            (position = x,y,z,q; velocity = vx,vy,vz,species;
 *            acceleration = ax,ay,az,status), operation by operation, so that
 *            they reproduce the reference's outputs bit for bit on the same
 *            machine (pinned against fixtures generated by running the
 *            reference itself, see tests/golden/make_golden.py).
 *   *_f64    are the FP64 ground truth (FP64 positions, FP64 accumulation)
 *            that the GPU results are measured against.
 */
#ifndef SV_ORACLE_H
#define SV_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Physical constants exactly as the reference evaluates them
 * (constants.h:28-47): K = e^2 / (4 pi eps0 amu), e/amu, 1/(4 pi eps0). */
double orc_k_const(void);
double orc_e_over_amu(void);
double orc_coulomb_ke(void);
double orc_elem_charge(void);
double orc_amu(void);
/* Species code (velocity.w) -> mass in amu (particles.h:65-87). */
double orc_species_mass(int species);

/* Reference direct sum, no symmetry (direct_force_method.cpp:153-190).
 * Adds into acc4[i].xyz for i in [i0,i1) with acc4[i].w == 1, sources
 * j in [j0,j1) with w in {1,2}, j != i. eps = softening squared (m^2). */
void orc_direct_ref32(const float *pos4, const float *vel4, float *acc4,
                      int i0, int i1, int j0, int j1, double eps, int nthreads);

/* Reference 4-fold rotational direct sum
 * (direct_force_method_rotational.cpp:28-94): quadrant k = 0..3 added in turn. */
void orc_direct_rot4_ref32(const float *pos4, const float *vel4, float *acc4,
                           int i0, int i1, int j0, int j1, double eps,
                           int nthreads);

/* Reference translational image sum
 * (direct_force_method_translational.cpp:28-367): images[3*k..3*k+2] are the
 * integer lattice offsets in summation order; the target is shifted by
 * -image*domain_size (FP32) before the pair loop. */
void orc_direct_trans_ref32(const float *pos4, const float *vel4, float *acc4,
                            int i0, int i1, int j0, int j1, double eps,
                            int nimg, const int *images,
                            const float domain_size[3], int nthreads);

/* Image list of the reference's periodic Grid (lattice_point.h:65-131)
 * expanded by the sign/permutation loops of
 * direct_force_method_translational.cpp:35-306.  lattice (3*nlat ints) is the
 * Grid's canonical point list in its stored order; pass NULL to build it here
 * (points sorted by descending norm, ties kept in generation order).
 * Returns the number of images written to out (capacity max_out). */
int orc_trans_images(int box_length, const int axes[3], const int *lattice,
                     int nlat, int *out, int max_out);

/* FP64 ground truth.  x: 3n interleaved metres; q: charge in e; m: mass in
 * amu; status: 1 inbound, 2 source-only, 0/-1 ignored.  Computes a (m/s^2)
 * for the given targets (NULL = all n) into a_out[3*ntargets].
 * sym 0: none (j != i);  1: 4-fold rotation about z;  2: images
 * (img_off = 3*nimg metres, target shifted by -offset, no j != i test,
 * matching the reference). */
void orc_direct_f64(int64_t n, const double *x, const double *q,
                    const double *m, const int32_t *status,
                    const int64_t *targets, int64_t ntargets, double eps2,
                    double kconst, int sym, int nimg, const double *img_off,
                    double *a_out, int nthreads);

/* Same sum with the potential (sum q_j / sqrt(r^2+eps2)) per target, FP64. */
void orc_potential_f64(int64_t n, const double *x, const double *q,
                       const int32_t *status, const int64_t *targets,
                       int64_t ntargets, double eps2, double *phi_out,
                       int nthreads);

/* Reference leapfrog DKD with the direct force (integration_schemes.cpp:
 * 856-891, 705-751; particles.cpp:693-786) and a uniform background field
 * E (V/m) added as computeBackgroundAcceleration does (particles.cpp:496-520).
 * sym as in orc_direct_f64 (images/domain used for sym 2). */
void orc_leapfrog_ref32(int n, float *pos4, float *vel4, float *acc4,
                        const float *t_inj, int nsteps, float dt, double eps,
                        const float efield[3], int sym, int nimg,
                        const int *images, const float domain_size[3],
                        int nthreads);

/* FP64 leapfrog DKD: x, v (3n interleaved) updated in place; a_out (3n,
 * nullable) receives the last kick's acceleration (force + field). */
void orc_leapfrog_f64(int64_t n, double *x, double *v, const double *q,
                      const double *m, int32_t *status, const double *t_inj,
                      int nsteps, double dt, double t0, double eps2,
                      double kconst, const double efield[3], int sym, int nimg,
                      const double *img_off, double *a_out, int nthreads);

/* Crash test, symmetry folding and boundary conditions of the drift
 * (ParticleSystem::propagatePositionNew, particles.cpp:33-40). */
typedef struct {
    int crash;              /* 1: CrashConditionOptions::extractorGrid */
    int bc;                 /* BoundaryConditionOptions: 0 none, 1 space, 2 time, 3 both */
    int fold;               /* f64 only: 0 none, 1 rotational, 2 translational */
    int axes[3];            /* symmetryAxes (translational folding) */
    double crash_z, crash_width, crash_r;   /* z_distance, z_width, r_distance */
    double bc_space[4];     /* spatialBoundaryConditions x, y, z, w */
    double bc_time;         /* temporalBoundaryCondition */
    double domain[3];       /* domainSize (translational folding) */
} orc_boundary;

/* One record of the events file (ChargedParticles::writeToEventsFile,
 * particles.cpp:666-684), 40 bytes. */
typedef struct {
    float time, x, y, z, vx, vy, vz;
    int32_t index;
    uint32_t species;
    int32_t status;
} orc_event;

/* Field map of a single emitter (InterpolationScheme, interpolation_scheme.cpp:
 * 66-262): node (r, z) in units of r0, field components in units of e0, a
 * triangulation and its neighbour table (the triangle across the edge
 * opposite each vertex, -1 on the hull). */
typedef struct {
    int n_nodes, n_tri;
    const double *node_rz;   /* 2 n_nodes */
    const double *er, *ez;   /* n_nodes */
    const int *tri, *nbr;    /* 3 n_tri each */
    double r0, e0, zmax;     /* the reference: zmax = 140 */
} orc_field;

/* InterpolationScheme::Efield for a singleEmitter map at the FP32 positions of
 * pos4, in index order, FP32 out (3n), as the reference evaluates it:
 * triangulation_search_delaunay's walk starts where the previous search
 * ended (its static triangle_index_save; *save = -1 before the first call). */
void orc_emitter_field_ref32(const orc_field *f, int n, const float *pos4, float *e3, int *save);

/* The same field in FP64 at FP64 points (3n), each walk starting from the
 * middle triangle, E = e0 (E_r x/r, E_r y/r, E_z). */
void orc_emitter_field_f64(const orc_field *f, int64_t n, const double *x3, double *e3);

/* orc_leapfrog_ref32 with the crash test, folding and boundary conditions of
 * bd (nullable; the folding follows sym as the reference's does), on the
 * reference's [firstParticle, lastParticle) window (LeapfrogDKD::driftNew,
 * findMostRecentInjected, resetFirstChargedParticle).  Events go to ev (up to
 * ev_cap; *ev_count receives the total). */
void orc_leapfrog_ref32_bc(int n, float *pos4, float *vel4, float *acc4,
                           const float *t_inj, int nsteps, float dt, double eps,
                           const float efield[3], int sym, int nimg,
                           const int *images, const float domain_size[3],
                           const orc_boundary *bd, const orc_field *field,
                           orc_event *ev, int ev_cap, int *ev_count, int nthreads);

/* Energy bookkeeping of Integrator (toggleEnergy, integration_schemes.cpp:
 * 85-97; initializeEnergyData :757-775; updateEnergyInjectionData :783-793;
 * updateEnergyIntervalData :799-835): init_steps / steps are the numbers of
 * integration steps of the field energy at initialisation and per interval;
 * every `interval` steps a record of six floats (KE_inj, PE_inj, FE_inj, KE,
 * PE, FE in J, the energy file's layout) goes to rec (up to rec_cap records;
 * rec_count receives the total). */
typedef struct {
    int init_steps, steps, interval;
    float *rec;
    int rec_cap, rec_count;
} orc_energy;

/* orc_leapfrog_ref32_bc with the energy bookkeeping of en, FP32 as the
 * reference keeps it: the potential of a particle sums over the window
 * [firstParticle, lastParticle) whatever the status, the field energy
 * integrates the emitter's field (field; none: zero) along z, then r. */
void orc_leapfrog_ref32_energy(int n, float *pos4, float *vel4, float *acc4,
                               const float *t_inj, int nsteps, float dt, double eps,
                               const float efield[3], const orc_boundary *bd,
                               const orc_field *field, orc_energy *en, int nthreads);

/* One substep request of LeapfrogDKDSubsteps::setSubstepTimes: the largest
 * step dt inside a region (bc: BoundaryConditionOptions; spatial limits s =
 * |x|, |y|, |z|, r; t: time since injection; 0 = unbounded). */
typedef struct {
    float dt;
    int bc;
    float s[4];
    float t;
} orc_substep;

/* LeapfrogDKDSubsteps::runSimulation (integration_schemes.cpp:899-1528) with
 * setSubstepTimes(subs, nsub) and the direct force, FP32 as the reference;
 * bd: crash / boundary conditions of the drift (nullable; folding follows sym
 * as the reference's does); efield: uniform field in the kick (the
 * reference's runSimulation has none: pass zeros to compare with it).
 * levels_out (n, nullable): each particle's substep level at the end. */
void orc_leapfrog_substeps_ref32(int n, float *pos4, float *vel4, float *acc4,
                                 const float *t_inj, int nsteps, float dt, double eps,
                                 const float efield[3], int sym, int nsub,
                                 const orc_substep *subs, const orc_boundary *bd,
                                 int8_t *levels_out, int nthreads);

/* orc_leapfrog_f64 with bd (nullable; folding per bd->fold) and the
 * injection window as a per-particle test (t_inj <= end of the half step;
 * force and kick: t_inj <= mid step), with species codes for the events.
 * field (nullable): the emitter's field added to efield in the kick; with
 * field, the ref32 loop replaces the uniform field by it, as the reference's
 * computeBackgroundAcceleration does. */
void orc_leapfrog_f64_bc(int64_t n, double *x, double *v, const double *q,
                         const double *m, int32_t *status, const double *t_inj,
                         int nsteps, double dt, double t0, double eps2,
                         double kconst, const double efield[3], int sym, int nimg,
                         const double *img_off, const orc_boundary *bd,
                         const orc_field *field, orc_event *ev, int ev_cap,
                         int *ev_count, int nthreads);

/* Energy diagnostic in FP64 (particles.cpp:535-578): kinetic
 * 0.5*amu*m*|v|^2 and potential 0.5*sum_{i!=j} q_i q_j e^2 ke/sqrt(r^2+eps2),
 * over all particles in [0,n) as the reference does (no status test). */
void orc_energy_f64(int64_t n, const double *x, const double *v,
                    const double *q, const double *m, double eps2,
                    double *ke, double *pe, int nthreads);

/* Accuracy metric of compareAcceleration (integration_schemes.cpp:411-461):
 * l2 = sqrt(mean_i |a_i - r_i|^2 / |r_i|^2) over status==1 particles (NULL
 * status = all), max = sqrt(max ratio), argmax its index. Also returns the
 * global form sqrt(sum|a-r|^2 / sum|r|^2). FP64. */
void orc_rel_l2(int64_t n, const double *a, const double *r,
                const int32_t *status, double *l2, double *maxl2,
                int64_t *argmax, double *global_l2);

/* Outlier classification of DomainBoundsFunction::isOutlier
 * (domain_bounds_functions.cpp:16-99) on FP32 positions: per axis the true
 * median of the sources' positions (findTrueMedian, outlier_detection.h:117:
 * middle element, or the mean of the two middle ones), the median of the
 * absolute deviations times 1.482602218505602, and a source is an outlier
 * when any axis deviates by >= 3 of those.  x3: 3n FP64 positions (rounded
 * to FP32 as the reference's state is); flags[i] = 1 outlier, 0 inlier
 * source, -1 not a source (status not 1 or 2).  Returns the outlier count.
 * The deviations' median is taken over the sources (the reference takes it
 * over its whole particle range; the two agree when every particle is a
 * source). */
int64_t orc_outliers(int64_t n, const double *x3, const int32_t *status, int32_t *flags);

#ifdef __cplusplus
}
#endif
#endif
