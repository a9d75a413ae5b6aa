// sv_internal.cuh -- shared definitions of the GB300 engine (not part of the ABI).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstring>

#include "solveit_gpu.h"
#include "field.cuh"

namespace sv {

constexpr int kMortonBits = 21;       // bits per axis of the Morton key (63-bit keys)
constexpr uint64_t kInactiveKey = ~0ull;
// Floor of r^2 + eps^2 (m^2) in the FP32 pair kernels: 1e-24 keeps 1/r^3 below
// FP32 overflow, so a zero-distance pair (the self pair, or zero-charge tile
// padding) contributes 0 * finite = 0 even with eps = 0; it only alters pairs
// closer than 1 pm.
constexpr float kMinR2 = 1e-24f;

// Morton-sorted working copy of the plume, rebuilt at every force evaluation.
// Sorting makes every block of consecutive targets spatially compact, which is
// what lets the mixed-precision kernels take FP32 coordinates relative to an
// FP64 origin per block (or per box) without losing the close pairs.
struct Sorted {
    double *x = nullptr, *y = nullptr, *z = nullptr;  // FP64 positions, sorted
    float *q = nullptr;        // source charge (0 when the particle is no source)
    double *qm = nullptr;      // K q / m for targets (0 when not a target)
    uint32_t *idx = nullptr;   // sorted slot -> caller's particle index
    uint64_t *keys = nullptr, *keys_alt = nullptr;
    uint32_t *idx_alt = nullptr;
    double *ax = nullptr, *ay = nullptr, *az = nullptr;  // acceleration, sorted order
    // a second field to add in the scatter (the FMM's far field: x, y, z at
    // far, far + far_stride, far + 2 far_stride), or null; cleared by it
    const double *far = nullptr;
    int64_t far_stride = 0;
    void *cub_tmp = nullptr;
    size_t cub_bytes = 0;
    double *root = nullptr;    // device [16]: origin xyz, cube side S, bbox max xyz, empty flag, 2^21/S
    double *red = nullptr;     // device reduction scratch
    int red_blocks = 0;
    int64_t cap = 0;
    // Morton levels the next sort must order (a one-shot request, reset to all
    // of them by the sort) and the levels the last sort ordered: an FMM tree
    // needs its keys ordered down to its leaf level only
    int want_levels = kMortonBits, key_levels = kMortonBits;
    bool resort = false;  // the FMM found its leaf level below key_levels: sort again, fully
    int64_t n = 0;       // sorted entries (caller particles plus any image copies)
    int64_t n_orig = 0;  // caller particles; sorted idx >= n_orig are image copies
};

// particle arrays to sort: the caller's state, or the caller's particles
// followed by source-only image copies (indices >= n_orig)
struct ParticleView {
    const double *x, *y, *z, *q, *m;
    const int32_t *status;
    int64_t n, n_orig;
    const double *qom = nullptr;  // q/m per particle (0 for m <= 0), or null: divide on the fly
};

struct Fmm;   // fmm.cu
struct Tree;  // tree.cu
struct Bh;    // bh.cu
struct Adj;   // adjoint.cu
struct Batch; // batch.cu
struct Outliers; // outliers.cu

}  // namespace sv

namespace sv {
// substep levels of the multi-rate leapfrog (substeps.cu): level l has the
// step dt[l] and the region limits (bs: |x|, |y|, |z|, r; bt: time since
// injection; 0 = unbounded) of kind type[l] (sv_bc_kind)
constexpr int kMaxSubLevels = 16;
struct SubTable {
    int on = 0, L = 0;  // L: finest level
    double dt[kMaxSubLevels] = {};
    int type[kMaxSubLevels] = {};
    double bs[kMaxSubLevels][4] = {};
    double bt[kMaxSubLevels] = {};
};

// energy bookkeeping of the reference's integrator (sv_set_energy, energy.cu)
struct EnergyBook {
    int on = 0, init_steps = 0, steps = 0, interval = 1;
    bool need_init = true;        // initialise at the next leapfrog step
    bool have_prev = false;       // an injection pass has run (t_prev is set)
    double t_prev = 0.0;          // particles with t_inj <= t_prev are counted as injected
    int64_t cap = 0;
    double *fe = nullptr, *ke_inj = nullptr;     // per particle: field energy, kinetic energy at set-up (J)
    double *ix = nullptr, *iy = nullptr, *iz = nullptr;  // end of the last field-energy path
    float4 *ph = nullptr, *pl = nullptr;         // positions as FP32 hi + lo, charge / index
    int *list = nullptr;                         // compacted particles of one pass
    double *pot = nullptr;                       // their sum of q_j / r over the window
    int *walk = nullptr;                         // per particle: start triangle of the field walk
    void *scan_tmp = nullptr;
    size_t scan_bytes = 0;
    unsigned long long *d_first = nullptr;       // [0] the window's first particle, [1] candidate
    int *d_cnt = nullptr;                        // compacted count
    double *d_acc = nullptr;                     // KE_inj, PE_inj, FE_inj, KE, PE, FE (J)
    sv_energy_record *recs = nullptr;            // host records not yet drained
    int64_t nrec = 0, rec_cap = 0;
};
}  // namespace sv

struct sv_ctx {
    sv_params P{};
    int device = 0;
    cudaStream_t stream = nullptr;
    int64_t n = 0, cap = 0;
    // caller-order state, FP64 SoA
    double *x = nullptr, *y = nullptr, *z = nullptr;
    double *vx = nullptr, *vy = nullptr, *vz = nullptr;
    double *q = nullptr, *m = nullptr, *t_inj = nullptr;
    double *qom = nullptr;  // q/m (0 where m <= 0), set at upload: no FP64 division per step
    int32_t *status = nullptr;
    int32_t *species = nullptr;  // species code per particle (event records), 0xffffffff unknown
    float *e2 = nullptr;         // 3n: background field (V/m) at each inbound particle's last kick (Efield2)
    float *e1 = nullptr;         // 3n: force acceleration (m/s^2) of each inbound particle's last kick (Efield1 / ((e/amu) q/m))
    // status the force and the kick see: the injection-windowed copy during a
    // leapfrog step (written by the first drift), else null (use status)
    int32_t *wstatus = nullptr;
    const int32_t *fstatus = nullptr;
    int32_t *rstatus = nullptr;  // status of an evaluation over a partial [first, last) range
    // crash / boundary / folding applied after every drift, and the event log
    sv_boundary B{};
    sv_event *d_events = nullptr;
    unsigned long long *d_ev_key = nullptr;  // file-order sort key per recorded event
    unsigned long long *d_ev_count = nullptr;
    int64_t ev_cap = 0;
    long long ev_seq = 0;       // drifts issued so far (event order across calls)
    const int8_t *pfold = nullptr;  // batch: per-particle folding (1 rotational plume), else null
    // emitter field map (sv_set_emitter_field): device copies; field.cache has
    // one start triangle per particle (field_cap entries)
    sv::FieldMesh field{};
    int64_t field_cap = 0;
    // multi-rate leapfrog (sv_set_substeps): level table and per-particle level
    sv::SubTable sub{};
    int8_t *sub_level = nullptr;
    int64_t sub_cap = 0;
    // energy bookkeeping (sv_set_energy)
    sv::EnergyBook en{};
    // last acceleration (force only), caller order, FP64
    double *ax = nullptr, *ay = nullptr, *az = nullptr;
    bool have_state = false, have_accel = false;
    int64_t acc_first = 0, acc_last = 0;  // window [first, last) of the last evaluation
    sv::Sorted S;
    sv::Tree *tree = nullptr;
    sv::Fmm *fmm = nullptr;
    sv::Bh *bh = nullptr;
    sv::Adj *adj = nullptr;
    sv::Batch *batch = nullptr;   // set by sv_upload_batch
    sv::Outliers *outliers = nullptr;  // outlier variants of the FMM
    // device staging for interleaved <-> SoA transfers
    void *d_stage = nullptr;
    size_t d_stage_bytes = 0;
    // copy streams of the host <-> device transfers (upload, download) and
    // their join events, the last one the fork from the context's stream
    cudaStream_t cps[4] = {};
    cudaEvent_t cpe[5] = {};
    double *h_accel = nullptr;    // page-locked host copy of the acceleration (sv_add_accel_ref32)
    int64_t h_accel_cap = 0;      // doubles
    double *d_scalar = nullptr;   // device scratch for small reductions
    double *h_scalar = nullptr;   // pinned mirror
    cudaEvent_t ev_begin = nullptr, ev_end = nullptr;
    // per-phase timing (sv_params.profile_phases): events 0..8 bracket the
    // phases sort, tree, lists, upward, downward, L2P, near field, scatter
    cudaEvent_t ph_ev[9] = {};
    // the FMM's near field on its own stream: its start / end events (phase 6
    // of the statistics is then its own duration, overlapping phases 3-5)
    cudaEvent_t near_ev[2] = {};
    unsigned long long launches = 0;
    sv_stats stats{};
    char err[512] = {0};
};

namespace sv {

sv_status set_error(sv_ctx *c, sv_status s, const char *fmt, ...);
sv_status cuda_error(sv_ctx *c, cudaError_t e, const char *what, const char *file, int line);

#define SV_CK(ctx, call)                                                    \
    do {                                                                    \
        cudaError_t _e = (call);                                            \
        if (_e != cudaSuccess) return ::sv::cuda_error((ctx), _e, #call, __FILE__, __LINE__); \
    } while (0)

#define SV_LAUNCHED(ctx)                                                    \
    do {                                                                    \
        (ctx)->launches++;                                                  \
        cudaError_t _e = cudaGetLastError();                                \
        if (_e != cudaSuccess) return ::sv::cuda_error((ctx), _e, "kernel launch", __FILE__, __LINE__); \
    } while (0)

#define SV_TRY(expr)                                                        \
    do {                                                                    \
        sv_status _s = (expr);                                              \
        if (_s != SV_OK) return _s;                                         \
    } while (0)

// 1/sqrt(x) by the special-function unit's approximation with denormal
// inputs and results flushed to zero: one instruction, where rsqrtf (built
// without -ftz) adds a range test and rescaling for denormal inputs.  The
// pair kernels' r^2 + eps^2 is never below kMinR2 (a normal float).
__device__ __forceinline__ float rsqrt_ftz(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Two consecutive staged sources (negated coordinates X, Y, Z, charges Q)
// against one target (T*, both halves the same), packed FP32x2: d = t + (-s),
// r^-3 per half, partial sums of the even and odd sources in g*.
template <bool CLAMP, bool UQ>
__device__ __forceinline__ void pair2(float2 X, float2 Y, float2 Z, float2 Q, float2 TX, float2 TY, float2 TZ,
                                      float2 E2, float2 &gx, float2 &gy, float2 &gz) {
    const float2 dx = __fadd2_rn(TX, X), dy = __fadd2_rn(TY, Y), dz = __fadd2_rn(TZ, Z);
    float2 r2 = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __ffma2_rn(dz, dz, E2)));
    if (CLAMP) r2 = make_float2(fmaxf(r2.x, kMinR2), fmaxf(r2.y, kMinR2));
    const float2 inv = make_float2(rsqrt_ftz(r2.x), rsqrt_ftz(r2.y));
    float2 w = __fmul2_rn(__fmul2_rn(inv, inv), inv);
    if (!UQ) w = __fmul2_rn(Q, w);
    gx = __ffma2_rn(dx, w, gx);
    gy = __ffma2_rn(dy, w, gy);
    gz = __ffma2_rn(dz, w, gz);
}

// two consecutive floats of a staged row
__device__ __forceinline__ float2 ld2(const float *p, int k) { return *reinterpret_cast<const float2 *>(p + k); }

// the low 21 bits of v spread to every third bit (Morton interleave: x at
// bit 0, y at bit 1, z at bit 2 of each level's triple)
__host__ __device__ __forceinline__ uint64_t morton_spread3(uint32_t v) {
    uint64_t x = v & 0x1fffffull;
    x = (x | (x << 32)) & 0x1f00000000ffffull;
    x = (x | (x << 16)) & 0x1f0000ff0000ffull;
    x = (x | (x << 8)) & 0x100f00f00f00f00full;
    x = (x | (x << 4)) & 0x10c30c30c30c30c3ull;
    x = (x | (x << 2)) & 0x1249249249249249ull;
    return x;
}

// 32-byte aligned quadruple of doubles (one shared-memory source record)
struct alignas(32) dbl4_t {
    double x, y, z, w;
};
__host__ __device__ inline dbl4_t dbl4(double x, double y, double z, double w) { return dbl4_t{x, y, z, w}; }

// record the boundary event k of the per-phase timing when profiling is on
inline void phase_mark(sv_ctx *c, int k) {
    if (c->P.profile_phases && c->ph_ev[k]) cudaEventRecord(c->ph_ev[k], c->stream);
}

inline int div_up(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }

// SM count of the current device (cudaDevAttrMultiProcessorCount), cached per
// device: grid-stride and persistent launches are sized in multiples of it
int device_sms();

// sort.cu
sv_status ensure_sorted_capacity(sv_ctx *c, int64_t n);
// Morton-sort the live plume into c->S (targets: inbound with index in [first,last)).
sv_status sort_state(sv_ctx *c, int64_t first, int64_t last);
sv_status sort_view(sv_ctx *c, const ParticleView &v, int64_t first, int64_t last);
// Scatter c->S.a{x,y,z} (plus S.far when set) back to caller order into
// c->a{x,y,z}; particles that are no target of the evaluation (K q/m of their
// sorted slot = 0) get zero.
sv_status unsort_accel(sv_ctx *c);

// direct.cu
sv_status direct_accel(sv_ctx *c);  // sorted -> c->S.a*
// the mixed-precision all-pairs kernel on caller-provided sorted arrays
// (no symmetry images); launches only, allocates nothing
cudaError_t launch_direct_mixed_sorted(const double *xs, const double *ys, const double *zs, const float *qs,
                                       const double *qm, int n, float eps2, double *ax, double *ay, double *az,
                                       cudaStream_t stream);

// tree.cu / bh.cu / fmm.cu
sv_status bh_accel(sv_ctx *c);
// Relative-L2 error of the last acceleration on up to k_max evenly spaced
// targets of [first, first + count) against the FP64 direct sum over that range
sv_status sampled_error_range(sv_ctx *c, int64_t first, int64_t count, int k_max, double *err);
// Morton levels the Barnes-Hut's next sort needs (its last tree's depth + 2, or all)
int bh_sort_levels(const sv_ctx *c);
// the last Barnes-Hut evaluation's cell and pair interaction counts (waits for the stream)
sv_status bh_counts(sv_ctx *c, double *cells, double *pairs);
sv_status fmm_accel(sv_ctx *c);
// Morton levels the FMM's next sort needs (its last leaf level + 1, or all)
int fmm_sort_levels(const sv_ctx *c);
// FMM with symmetry images: sorts the caller's particles plus their images
sv_status fmm_sort_images(sv_ctx *c, int64_t first, int64_t last);
void tree_free(sv_ctx *c);
void fmm_free(sv_ctx *c);
void bh_free(sv_ctx *c);
// M2L translations and P2P pairs of the last FMM evaluation (synchronises)
sv_status fmm_counts(sv_ctx *c, double *m2l, double *pairs);

// api.cu: one force evaluation into c->a{x,y,z} (caller order)
sv_status compute_accel_device(sv_ctx *c, int64_t first, int64_t last);

// adjoint.cu
void adjoint_free(sv_ctx *c);

// outliers.cu: detection (status with outliers masked for the tree), the
// direct sums of every interaction with an outlier, the flags of the last run
sv_status outliers_detect(sv_ctx *c, const int32_t **status_for_tree);
sv_status outliers_add(sv_ctx *c, int64_t first, int64_t last);
sv_status outliers_get(sv_ctx *c, int32_t *flags, int64_t *count);
void outliers_free(sv_ctx *c);

// batch.cu: many plumes in one context (sv_upload_batch)
sv_status batch_plan(sv_ctx *c, int32_t np, const int64_t *counts, const int32_t *method, const int32_t *sym);
sv_status batch_accel(sv_ctx *c);
sv_status batch_leapfrog(sv_ctx *c, int32_t nsteps, double dt, double t0);
sv_status batch_tune(sv_ctx *c, const char *cache_path, double *best_ms);
sv_status batch_set_tuning(sv_ctx *c, int m2l_weight, int direct_chunk);
sv_status batch_info(const sv_ctx *c, sv_batch_info *out);
void batch_invalidate(sv_ctx *c);
bool batch_same_shape(const sv_ctx *c, int32_t np, const int64_t *counts, const int32_t *method,
                      const int32_t *sym);
void batch_free(sv_ctx *c);

// integrate.cu.  With tb (device {t0, dt, k}), the step's start time
// t0 + dt * k is added to t_start on the device (CUDA-graph replays).
// Half-step drift over [t_start, t_start + h] with the injection window, the
// crash test, folding and boundary conditions of c->B.  window != null
// receives the status the following force and kick see (0 outside the
// window).  With tb (device {t0, dt, k}) t_start is taken relative to
// tb[0] + tb[1] * tb[2] and the event order from seq_base + 2 * tb[2].
sv_status drift(sv_ctx *c, double t_start, double h, int32_t *window, const double *tb = nullptr,
                long long seq_base = 0);
// Kick over [t_start, t_start + dt] of the particles with st == 1 (st: the
// windowed status of the step).
sv_status kick(sv_ctx *c, double t_start, double dt, const int32_t *st, const double *tb = nullptr);
// One DKD step of sv_leapfrog on a single-plume context (save_xh: mid-step positions, 3n, or null).
sv_status leapfrog_step(sv_ctx *c, double ts, double dt, double *save_xh = nullptr);
// status as the force sees it (windowed during a leapfrog step)
inline const int32_t *force_status(const sv_ctx *c) { return c->fstatus ? c->fstatus : c->status; }
// wstatus[i] = status[i] if t_inj[i] <= t_window else 0 (adjoint re-runs)
sv_status window_status(sv_ctx *c, double t_window);
sv_status events_reserve(sv_ctx *c);
void events_free(sv_ctx *c);
// field.cu: the per-particle walk caches of the emitter field (grown to n, reset to -1)
sv_status field_prepare(sv_ctx *c);
sv_status field_reset(sv_ctx *c);
sv_status field_check(sv_ctx *c);
void field_free(sv_ctx *c);
// substeps.cu: the multi-rate leapfrog
sv_status substeps_run(sv_ctx *c, int32_t nsteps, double dt, double t0);
sv_status substeps_reset_levels(sv_ctx *c);
void substeps_free(sv_ctx *c);
sv_status energy(sv_ctx *c, double *ke, double *pe);
// energy.cu: the bookkeeping hooks of a leapfrog step (no-ops when off).
// Before a drift that ends at t_end: count the particles injected since the
// previous one; after it: move the window's first particle; after the step
// that starts at ts: the interval record.
sv_status energy_inject(sv_ctx *c, double t_end);
sv_status energy_first(sv_ctx *c, double t_end);
sv_status energy_interval(sv_ctx *c, double ts, double dt);
void energy_free(sv_ctx *c);
// a new state: set-up again at the next step, records cleared
void energy_rearm(sv_ctx *c);

// image offsets (metres) of the translational lattice, in summation order
int trans_images(const sv_params &P, double *out, int max_out);

// constant memory copies per context are not used: parameters travel as
// kernel arguments so that several contexts can share a device.

}  // namespace sv
