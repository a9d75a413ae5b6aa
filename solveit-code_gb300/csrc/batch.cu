// batch.cu -- many independent plumes in one context, stepped by CUDA graphs.
//
// The reference runs one ForceCalculationMethod per ParticleSystem
// (force_calculation_methods.h:28-87) and one LeapfrogDKD time loop per plume
// (integration_schemes.cpp:856-891).  A batch holds every plume of a study in
// one context and evaluates all of them at once:
//
//  * view: one slot per (particle, image).  FMM plumes come first (plume ids
//    0..nfp-1), each particle followed by its source-only rotated copies for
//    the 4-fold rotational variant; direct plumes follow (their images are
//    formed on the fly by the pair kernel, as in direct.cu).
//  * one radix sort of all slots by key = plume id << 54 | 18-bit-per-axis
//    Morton code relative to the plume's own root cube, so each plume's slots
//    stay contiguous and spatially ordered.
//  * FMM plumes: one forest of octrees (forest.cuh).  Each plume's cube is
//    enlarged by 2^delta so that a single leaf level L is, for every plume,
//    the level its cost model picks.  delta is chosen on the device at every
//    evaluation from the plume's split-level histogram (dense plumes expand
//    radially by tens of percent within a few steps, which changes the best
//    depth), and applied by shifting the plume's sorted Morton keys right by
//    3*delta, which keeps their order.
//  * direct plumes: a persistent kernel pulls work items (256 targets x a
//    source chunk x images) from an atomic queue, largest first, on a second
//    stream that runs beside the FMM.
//  * every step (drift, force, kick, drift) is captured once in a CUDA graph
//    and replayed; the step time lives on the device.  Box capacities are
//    fixed per graph; an overflow sets a device flag, and the host restores
//    the state saved before that step, doubles the capacities and runs the
//    step again.
#include <cub/device/device_radix_sort.cuh>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "forest.cuh"
#include "sv_internal.cuh"

namespace sv {

constexpr int kBatchBits = 18;       // Morton bits per axis below the plume id
constexpr int kPidShift = 3 * kBatchBits;
constexpr int kMaxPlumes = 512;      // plume ids use bits 54..62; bit 63 stays clear
constexpr int kChunk = 8192;         // view slots per bounding-box partial
constexpr int kBLevels = kMortonBits + 1;

struct DirectItem {
    int t0, t1, j0, j1, nimg, pad0, pad1, pad2;
};

struct Batch {
    int np = 0, nfp = 0;
    std::vector<int64_t> count, off;  // caller order: plume p owns [off[p], off[p] + count[p])
    std::vector<int> method, sym;     // per plume
    std::vector<int> pid_of;          // plume -> plume id (FMM plumes first)
    std::vector<int> plume_of;        // plume id -> plume
    std::vector<int64_t> vbeg;        // plume id -> first view slot; vbeg[np] = view size
    int64_t nv = 0, nf = 0;           // view slots; FMM slots (the first nf)
    uint32_t *vsrc = nullptr;         // view slot -> caller particle
    uint32_t *vtag = nullptr;         // view slot -> plume id * 4 + image
    double *roots = nullptr;          // [8 * np]
    int *delta = nullptr;             // [np] cube enlargement exponents of the last evaluation
    std::vector<int> h_delta;
    int *d_hist = nullptr;            // [nfp * kBLevels] split-level histogram per FMM plume
    int *d_vbeg = nullptr;            // [np + 1] first view slot per plume id
    int nchunks = 0;
    int *chunk_beg = nullptr;         // [nchunks + 1]
    int *pid_chunk = nullptr;         // [np + 1]
    double *chunk_red = nullptr;      // [6 * nchunks]
    DirectItem *items = nullptr;
    int nitems = 0;
    double direct_pairs = 0;          // pair interactions of the direct plumes per evaluation
    int *queue = nullptr;
    void *cub_tmp = nullptr;
    size_t cub_bytes = 0;
    // forest
    ForestArgs fa;
    bool planned = false;
    int *d_nbox = nullptr, *d_err = nullptr, *h_err = nullptr;
    int overflow_mask = 0;            // levels that overflowed at the last regrow
    // graphs
    double *d_time = nullptr;         // {t0, dt, k, first event sequence number}
    double *h_time = nullptr;         // pinned
    cudaGraphExec_t g_accel = nullptr, g_step = nullptr;
    unsigned long long accel_kernels = 0, step_kernels = 0;
    cudaStream_t side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    double *backup = nullptr;         // 6 n: state at the start of a leapfrog call
    int32_t *backup_st = nullptr;     // n: status at the start of a leapfrog call
    unsigned long long *ev_count0 = nullptr;  // event count at the start of a leapfrog call
    int8_t *pfold = nullptr;          // n: 1 for the particles of rotational plumes (folding)
    double step_dt = 0;               // dt baked into g_step
    // tuning
    int m2l_weight = 400, direct_chunk = 2048;  // tuned: M2L cost in pair units, direct work-item size
    double tuned_ms = 0;
    int regrows = 0;
};

namespace {

__device__ __forceinline__ bool is_src(int32_t w) { return w == 1 || w == 2; }

// image g of a position: rotated by g*pi/2 about z (quadrantRotationFunction,
// auxiliary_functions.h:55-57)
__device__ __forceinline__ void rot_image(int g, double &x, double &y) {
    const double x0 = x, y0 = y;
    if (g == 1) { x = -y0; y = x0; }
    else if (g == 2) { x = -x0; y = -y0; }
    else if (g == 3) { x = y0; y = -x0; }
}

// position of a view slot: the rotated source, or the plume origin for a slot
// that is no source (it then carries zero charge and is no target)
__device__ __forceinline__ void slot_pos(uint32_t i, uint32_t tag, const double *__restrict__ x,
                                         const double *__restrict__ y, const double *__restrict__ z,
                                         const int32_t *__restrict__ st, const double *__restrict__ roots,
                                         double &px, double &py, double &pz, bool &src) {
    src = is_src(st[i]);
    if (src) {
        px = x[i];
        py = y[i];
        pz = z[i];
        rot_image((int)(tag & 3u), px, py);
    } else {
        const double *r = roots + 8 * (tag >> 2);
        px = r[0];
        py = r[1];
        pz = r[2];
    }
}

__global__ void bbox_chunks_kernel(const int *__restrict__ chunk_beg, const uint32_t *__restrict__ vsrc,
                                   const uint32_t *__restrict__ vtag, const double *__restrict__ x,
                                   const double *__restrict__ y, const double *__restrict__ z,
                                   const int32_t *__restrict__ st, double *__restrict__ red) {
    const int b0 = chunk_beg[blockIdx.x], b1 = chunk_beg[blockIdx.x + 1];
    double mn[3] = {1e300, 1e300, 1e300}, mx[3] = {-1e300, -1e300, -1e300};
    for (int v = b0 + threadIdx.x; v < b1; v += blockDim.x) {
        const uint32_t i = vsrc[v];
        if (!is_src(st[i])) continue;
        double p[3] = {x[i], y[i], z[i]};
        rot_image((int)(vtag[v] & 3u), p[0], p[1]);
#pragma unroll
        for (int d = 0; d < 3; d++) {
            mn[d] = fmin(mn[d], p[d]);
            mx[d] = fmax(mx[d], p[d]);
        }
    }
    __shared__ double sh[6][8];
#pragma unroll
    for (int d = 0; d < 3; d++) {
        for (int o = 16; o > 0; o >>= 1) {
            mn[d] = fmin(mn[d], __shfl_xor_sync(0xffffffffu, mn[d], o));
            mx[d] = fmax(mx[d], __shfl_xor_sync(0xffffffffu, mx[d], o));
        }
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        for (int d = 0; d < 3; d++) {
            sh[d][w] = mn[d];
            sh[3 + d][w] = mx[d];
        }
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        const int d = threadIdx.x;
        double v = d < 3 ? 1e300 : -1e300;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) v = d < 3 ? fmin(v, sh[d][k]) : fmax(v, sh[d][k]);
        red[blockIdx.x * 6 + d] = v;
    }
}

// Root record per plume: origin = bbox min, side = smallest power of two
// above the largest extent, bbox max, empty flag.
__global__ void plume_roots_kernel(int np, const int *__restrict__ pid_chunk, const double *__restrict__ red,
                                   double *__restrict__ roots) {
    const int pid = blockIdx.x * blockDim.x + threadIdx.x;
    if (pid >= np) return;
    double mn[3] = {1e300, 1e300, 1e300}, mx[3] = {-1e300, -1e300, -1e300};
    for (int k = pid_chunk[pid]; k < pid_chunk[pid + 1]; k++)
        for (int d = 0; d < 3; d++) {
            mn[d] = fmin(mn[d], red[6 * k + d]);
            mx[d] = fmax(mx[d], red[6 * k + 3 + d]);
        }
    const bool empty = mn[0] > mx[0];
    double ext = 0.0;
    if (empty) {
        for (int d = 0; d < 3; d++) mn[d] = mx[d] = 0.0;
    } else {
        for (int d = 0; d < 3; d++) ext = fmax(ext, mx[d] - mn[d]);
    }
    double S = 1e-12;
    if (ext > 0.0) {
        int e;
        frexp(ext, &e);
        S = ldexp(1.0, e);
    }
    double *r = roots + 8 * pid;
    r[0] = mn[0];
    r[1] = mn[1];
    r[2] = mn[2];
    r[3] = S;
    r[4] = mx[0];
    r[5] = mx[1];
    r[6] = mx[2];
    r[7] = empty ? 1.0 : 0.0;
}

__device__ __forceinline__ uint64_t spread3_18(uint32_t v) {
    uint64_t x = v & 0x3ffffull;
    x = (x | (x << 32)) & 0x1f00000000ffffull;
    x = (x | (x << 16)) & 0x1f0000ff0000ffull;
    x = (x | (x << 8)) & 0x100f00f00f00f00full;
    x = (x | (x << 4)) & 0x10c30c30c30c30c3ull;
    x = (x | (x << 2)) & 0x1249249249249249ull;
    return x;
}

__global__ void batch_keys_kernel(int64_t nv, const uint32_t *__restrict__ vsrc, const uint32_t *__restrict__ vtag,
                                  const double *__restrict__ x, const double *__restrict__ y,
                                  const double *__restrict__ z, const int32_t *__restrict__ st,
                                  const double *__restrict__ roots, uint64_t *__restrict__ keys,
                                  uint32_t *__restrict__ vals) {
    const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (v >= nv) return;
    const uint32_t i = vsrc[v], tag = vtag[v];
    double p[3];
    bool src;
    slot_pos(i, tag, x, y, z, st, roots, p[0], p[1], p[2], src);
    const double *r = roots + 8 * (tag >> 2);
    const double inv = (double)(1u << kBatchBits) / r[3];
    uint32_t cc[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
        double f = floor((p[d] - r[d]) * inv);
        f = fmin(fmax(f, 0.0), (double)((1u << kBatchBits) - 1));
        cc[d] = (uint32_t)f;
    }
    keys[v] = ((uint64_t)(tag >> 2) << kPidShift) | spread3_18(cc[0]) | (spread3_18(cc[1]) << 1) |
              (spread3_18(cc[2]) << 2);
    vals[v] = (uint32_t)v;
}

__global__ void batch_gather_kernel(int64_t nv, const uint32_t *__restrict__ idx, const uint32_t *__restrict__ vsrc,
                                    const uint32_t *__restrict__ vtag, const double *__restrict__ x,
                                    const double *__restrict__ y, const double *__restrict__ z,
                                    const double *__restrict__ q, const double *__restrict__ m,
                                    const double *__restrict__ qom, const int32_t *__restrict__ st,
                                    const double *__restrict__ roots, double kconst,
                                    double *__restrict__ xs, double *__restrict__ ys, double *__restrict__ zs,
                                    float *__restrict__ qs, double *__restrict__ qm) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= nv) return;
    const uint32_t v = idx[s];
    const uint32_t i = vsrc[v], tag = vtag[v];
    double px, py, pz;
    bool src;
    slot_pos(i, tag, x, y, z, st, roots, px, py, pz, src);
    xs[s] = px;
    ys[s] = py;
    zs[s] = pz;
    qs[s] = src ? (float)q[i] : 0.0f;
    const bool tgt = (tag & 3u) == 0 && st[i] == 1 && m[i] > 0.0;
    qm[s] = tgt ? kconst * qom[i] : 0.0;
}

__global__ void batch_scatter_kernel(int64_t nv, const uint32_t *__restrict__ idx, const uint32_t *__restrict__ vsrc,
                                     const uint32_t *__restrict__ vtag, const double *__restrict__ axs,
                                     const double *__restrict__ ays, const double *__restrict__ azs,
                                     double *__restrict__ ax, double *__restrict__ ay, double *__restrict__ az) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= nv) return;
    const uint32_t v = idx[s];
    if (vtag[v] & 3u) return;  // image copy
    const uint32_t i = vsrc[v];
    ax[i] = axs[s];
    ay[i] = ays[s];
    az[i] = azs[s];
}

// Split-level histogram per plume on the sorted keys: hist[pid][l] counts the
// slots that open a new box at level l (and below) of their plume.  A block of
// consecutive keys spans few plumes: the first kHistPids of them use shared
// counters, any further one global atomics.
constexpr int kHistPids = 4;
__global__ void __launch_bounds__(256) plume_levels_kernel(const uint64_t *__restrict__ keys, int64_t n,
                                                           int *__restrict__ hist) {
    __shared__ int sh[kHistPids * kBLevels];
    for (int t = threadIdx.x; t < kHistPids * kBLevels; t += blockDim.x) sh[t] = 0;
    const int64_t b0 = blockIdx.x * (int64_t)blockDim.x;
    const int pid0 = b0 < n ? (int)(keys[b0] >> kPidShift) : 0;
    __syncthreads();
    const int64_t i = b0 + threadIdx.x;
    if (i > 0 && i < n) {
        const uint64_t k = keys[i], kp = keys[i - 1];
        const uint64_t xx = k ^ kp;
        if ((k >> kPidShift) == (kp >> kPidShift) && xx) {
            const int b = 63 - __clzll((long long)xx);
            const int l = kBatchBits - b / 3;
            const int pid = (int)(k >> kPidShift), r = pid - pid0;
            if (r < kHistPids) atomicAdd(&sh[r * kBLevels + l], 1);
            else atomicAdd(&hist[pid * kBLevels + l], 1);
        }
    }
    __syncthreads();
    for (int t = threadIdx.x; t < kHistPids * kBLevels; t += blockDim.x)
        if (sh[t]) atomicAdd(&hist[(pid0 + t / kBLevels) * kBLevels + t % kBLevels], sh[t]);
}

// The leaf level of one plume from a cost model on its box counts per level:
//   cost(l) = P2P pairs(l) + W * (M2L translations of levels 2..l)
// with the occupied boxes' growth ratio g_k = boxes(k) / boxes(k-1) giving the
// dimension d_k = log2(g_k) in which the plume is resolved at level k (1 for a
// thin filament, 3 for a bulk), near boxes (2ws+1)^d and M2L boxes
// (4ws+2)^d - (2ws+1)^d per box, pairs = n * occupancy * near.  W is the cost
// of one M2L in pair units (tuned).  Levels below an occupancy of 2 are not
// considered.
__host__ __device__ inline int pick_level(double np_slots, const long long *boxes, double w, int ws) {
    const double a = 2.0 * ws + 1.0, b = 4.0 * ws + 2.0;
    int best = 2;
    double bestc = 1e300, m2l = 0.0;
    for (int l = 2; l <= kBatchBits; l++) {
        const double nb = (double)boxes[l];
        double g = nb / (double)boxes[l - 1];
        g = g < 1.0 ? 1.0 : (g > 8.0 ? 8.0 : g);
        const double d = log2(g);
        const double near = pow(a, d), far = pow(b, d) - near;
        m2l += nb * far;
        const double occ = np_slots / nb;
        if (occ < 2.0 && l > 2) break;
        const double cost = np_slots * occ * near + w * m2l;
        if (cost < bestc) {
            bestc = cost;
            best = l;
        }
    }
    return best;
}

// Per FMM plume: its own leaf level Lp, delta = L - Lp, and the root side
// scaled by 2^delta.
__global__ void choose_delta_kernel(int nfp, const int *__restrict__ hist, const int *__restrict__ vbeg, int L,
                                    double w, int ws, int *__restrict__ delta, double *__restrict__ roots) {
    const int pid = blockIdx.x * blockDim.x + threadIdx.x;
    if (pid >= nfp) return;
    const double np_slots = (double)(vbeg[pid + 1] - vbeg[pid]);
    long long boxes[kBatchBits + 1];
    boxes[0] = 1;
    for (int l = 1; l <= kBatchBits; l++) boxes[l] = boxes[l - 1] + hist[pid * kBLevels + l];
    const int lp = pick_level(np_slots, boxes, w, ws);
    const int d = L > lp ? L - lp : 0;
    delta[pid] = d;
    roots[8 * pid + 3] = ldexp(roots[8 * pid + 3], d);
}

// Apply each plume's delta to its sorted keys: Morton >> 3*delta is the key in
// the cube enlarged by 2^delta (same origin), and keeps the sorted order.
__global__ void shift_keys_kernel(uint64_t *__restrict__ keys, int64_t n, const int *__restrict__ delta) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t k = keys[i];
    const int pid = (int)(k >> kPidShift);
    const int d = delta[pid];
    if (d) keys[i] = ((uint64_t)pid << kPidShift) | ((k & ((1ull << kPidShift) - 1ull)) >> (3 * d));
}

constexpr int kDTPB = 128;  // threads per CTA of the direct batch kernel
constexpr int kDTPT = 2;    // targets per thread
constexpr int kDTile = 256; // sources per shared-memory tile

// Persistent all-pairs kernel over the direct plumes' work items.  Same
// arithmetic as direct_mixed_kernel (direct.cu): FP32 pairs on offsets from the
// item's first target, FP64 accumulation across tiles, atomics into the
// sorted acceleration (zeroed beforehand).
__global__ void __launch_bounds__(kDTPB)
direct_batch_kernel(const DirectItem *__restrict__ items, int nitems, int *__restrict__ queue,
                    const double *__restrict__ xs, const double *__restrict__ ys, const double *__restrict__ zs,
                    const float *__restrict__ qs, const double *__restrict__ qm, float eps2,
                    double *__restrict__ ax, double *__restrict__ ay, double *__restrict__ az) {
    __shared__ __align__(16) float tile[4][kDTile];  // staged sources: -x, -y, -z, charge
    __shared__ int item_sh;
    const float2 E2 = make_float2(eps2, eps2);
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) item_sh = atomicAdd(queue, 1);
        __syncthreads();
        const int it = item_sh;
        if (it >= nitems) break;
        const DirectItem w = items[it];
        const double ox = xs[w.t0], oy = ys[w.t0], oz = zs[w.t0];
        float2 TX[kDTPT], TY[kDTPT], TZ[kDTPT];
        double sx[kDTPT], sy[kDTPT], sz[kDTPT];
#pragma unroll
        for (int k = 0; k < kDTPT; k++) {
            const int ii = min(w.t0 + (int)threadIdx.x + k * kDTPB, w.t1 - 1);
            const float tx = (float)(xs[ii] - ox), ty = (float)(ys[ii] - oy), tz = (float)(zs[ii] - oz);
            TX[k] = make_float2(tx, tx);
            TY[k] = make_float2(ty, ty);
            TZ[k] = make_float2(tz, tz);
            sx[k] = sy[k] = sz[k] = 0.0;
        }
        for (int g = 0; g < w.nimg; g++) {
            for (int jt = w.j0; jt < w.j1; jt += kDTile) {
                __syncthreads();
                for (int s = threadIdx.x; s < kDTile; s += kDTPB) {
                    const int j = jt + s;
                    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (j < w.j1) {
                        double px = xs[j], py = ys[j];
                        rot_image(g, px, py);
                        v = make_float4((float)(px - ox), (float)(py - oy), (float)(zs[j] - oz), qs[j]);
                    }
                    tile[0][s] = -v.x;
                    tile[1][s] = -v.y;
                    tile[2][s] = -v.z;
                    tile[3][s] = v.w;
                }
                __syncthreads();
                // two sources per packed FP32x2 operation, r^2 floored at kMinR2
                float2 gx[kDTPT], gy[kDTPT], gz[kDTPT];
#pragma unroll
                for (int k = 0; k < kDTPT; k++) gx[k] = gy[k] = gz[k] = make_float2(0.f, 0.f);
#pragma unroll 4
                for (int s = 0; s < kDTile; s += 2) {
                    const float2 X = ld2(tile[0], s), Y = ld2(tile[1], s), Z = ld2(tile[2], s),
                                 Q = ld2(tile[3], s);
#pragma unroll
                    for (int k = 0; k < kDTPT; k++)
                        pair2<true, false>(X, Y, Z, Q, TX[k], TY[k], TZ[k], E2, gx[k], gy[k], gz[k]);
                }
#pragma unroll
                for (int k = 0; k < kDTPT; k++) {
                    sx[k] += gx[k].x + gx[k].y;
                    sy[k] += gy[k].x + gy[k].y;
                    sz[k] += gz[k].x + gz[k].y;
                }
            }
        }
#pragma unroll
        for (int k = 0; k < kDTPT; k++) {
            const int i = w.t0 + threadIdx.x + k * kDTPB;
            if (i >= w.t1) continue;
            const double cq = qm[i];
            if (cq == 0.0) continue;
            atomicAdd(&ax[i], sx[k] * cq);
            atomicAdd(&ay[i], sy[k] * cq);
            atomicAdd(&az[i], sz[k] * cq);
        }
    }
}

__global__ void advance_step_kernel(double *tb) { tb[2] += 1.0; }

// ------------------------------------------------------------------ host --

sv_status check_cuda(sv_ctx *c, cudaError_t e, const char *what) {
    if (e != cudaSuccess) return cuda_error(c, e, what, __FILE__, __LINE__);
    return SV_OK;
}

void drop_graphs(Batch &B) {
    if (B.g_accel) cudaGraphExecDestroy(B.g_accel);
    if (B.g_step) cudaGraphExecDestroy(B.g_step);
    B.g_accel = B.g_step = nullptr;
}

// Work items of the direct plumes: 256 targets x direct_chunk sources x images,
// largest first (longest-processing-time order for the persistent queue).
sv_status build_items(sv_ctx *c, Batch &B) {
    std::vector<DirectItem> it;
    B.direct_pairs = 0;
    for (int pid = B.nfp; pid < B.np; pid++) {
        const int p = B.plume_of[pid];
        const int s0 = (int)B.vbeg[pid], s1 = (int)B.vbeg[pid + 1];
        const int nimg = B.sym[p] == SV_SYM_ROTATIONAL ? 4 : 1;
        B.direct_pairs += (double)(s1 - s0) * (double)(s1 - s0) * nimg;
        const int ch = std::max(kDTile, B.direct_chunk / nimg / kDTile * kDTile);
        for (int t = s0; t < s1; t += kDTPB * kDTPT)
            for (int j = s0; j < s1; j += ch)
                it.push_back(DirectItem{t, std::min(s1, t + kDTPB * kDTPT), j, std::min(s1, j + ch), nimg, 0, 0, 0});
    }
    std::stable_sort(it.begin(), it.end(), [](const DirectItem &a, const DirectItem &b) {
        return (int64_t)(a.j1 - a.j0) * a.nimg * (a.t1 - a.t0) > (int64_t)(b.j1 - b.j0) * b.nimg * (b.t1 - b.t0);
    });
    cudaFree(B.items);
    B.items = nullptr;
    B.nitems = (int)it.size();
    if (B.nitems) {
        SV_CK(c, cudaMalloc(&B.items, sizeof(DirectItem) * it.size()));
        SV_CK(c, cudaMemcpy(B.items, it.data(), sizeof(DirectItem) * it.size(), cudaMemcpyHostToDevice));
    }
    return SV_OK;
}

// bbox, roots, keys, sort, (adapt: per-plume depth), gather (launches only)
sv_status sort_batch(sv_ctx *c, Batch &B, bool adapt) {
    Sorted &S = c->S;
    const int64_t nv = B.nv;
    bbox_chunks_kernel<<<B.nchunks, 256, 0, c->stream>>>(B.chunk_beg, B.vsrc, B.vtag, c->x, c->y, c->z, force_status(c),
                                                         B.chunk_red);
    SV_LAUNCHED(c);
    plume_roots_kernel<<<div_up(B.np, 128), 128, 0, c->stream>>>(B.np, B.pid_chunk, B.chunk_red, B.roots);
    SV_LAUNCHED(c);
    batch_keys_kernel<<<div_up(nv, 256), 256, 0, c->stream>>>(nv, B.vsrc, B.vtag, c->x, c->y, c->z, force_status(c),
                                                              B.roots, S.keys_alt, S.idx_alt);
    SV_LAUNCHED(c);
    size_t bytes = B.cub_bytes;
    SV_CK(c, cub::DeviceRadixSort::SortPairs(B.cub_tmp, bytes, S.keys_alt, S.keys, S.idx_alt, S.idx, (int)nv, 0,
                                             kPidShift + 9, c->stream));
    c->launches += 2 * ((kPidShift + 9 + 7) / 8);
    if (adapt && B.nfp > 0 && B.nf > 0) {
        SV_CK(c, cudaMemsetAsync(B.d_hist, 0, sizeof(int) * kBLevels * B.nfp, c->stream));
        plume_levels_kernel<<<div_up(B.nf, 256), 256, 0, c->stream>>>(S.keys, B.nf, B.d_hist);
        SV_LAUNCHED(c);
        choose_delta_kernel<<<div_up(B.nfp, 128), 128, 0, c->stream>>>(B.nfp, B.d_hist, B.d_vbeg, B.fa.spec.L,
                                                                       (double)B.m2l_weight, c->P.fmm_ws, B.delta,
                                                                       B.roots);
        SV_LAUNCHED(c);
        shift_keys_kernel<<<div_up(B.nf, 256), 256, 0, c->stream>>>(S.keys, B.nf, B.delta);
        SV_LAUNCHED(c);
    }
    batch_gather_kernel<<<div_up(nv, 256), 256, 0, c->stream>>>(nv, S.idx, B.vsrc, B.vtag, c->x, c->y, c->z, c->q,
                                                                c->m, c->qom, force_status(c), B.roots, c->P.k_const,
                                                                S.x, S.y, S.z, S.q, S.qm);
    SV_LAUNCHED(c);
    return SV_OK;
}

// one force evaluation of every plume into c->a{x,y,z} (launches only)
sv_status batch_force(sv_ctx *c, Batch &B) {
    Sorted &S = c->S;
    SV_TRY(sort_batch(c, B, true));
    const int64_t nd = B.nv - B.nf;
    if (B.nitems > 0) {
        SV_CK(c, cudaMemsetAsync(S.ax + B.nf, 0, sizeof(double) * nd, c->stream));
        SV_CK(c, cudaMemsetAsync(S.ay + B.nf, 0, sizeof(double) * nd, c->stream));
        SV_CK(c, cudaMemsetAsync(S.az + B.nf, 0, sizeof(double) * nd, c->stream));
        SV_CK(c, cudaMemsetAsync(B.queue, 0, sizeof(int), c->stream));
        SV_CK(c, cudaEventRecord(B.fork, c->stream));
        SV_CK(c, cudaStreamWaitEvent(B.side, B.fork, 0));
        const int dev_sms = device_sms();
        direct_batch_kernel<<<std::min(B.nitems, 8 * dev_sms), kDTPB, 0, B.side>>>(
            B.items, B.nitems, B.queue, S.x, S.y, S.z, S.q, S.qm, (float)c->P.softening2, S.ax, S.ay, S.az);
        SV_LAUNCHED(c);
        SV_CK(c, cudaEventRecord(B.join, B.side));
    }
    if (B.nf > 0) SV_TRY(fmm_forest_run(c, B.fa));
    if (B.nitems > 0) SV_CK(c, cudaStreamWaitEvent(c->stream, B.join, 0));
    batch_scatter_kernel<<<div_up(B.nv, 256), 256, 0, c->stream>>>(B.nv, S.idx, B.vsrc, B.vtag, S.ax, S.ay, S.az,
                                                                   c->ax, c->ay, c->az);
    SV_LAUNCHED(c);
    return SV_OK;
}

// Chooses the per-plume cube enlargement (delta), the forest's leaf level and
// the box capacities from the current state (blocking; not captured).
sv_status plan_forest(sv_ctx *c, Batch &B, int cap_scale) {
    drop_graphs(B);
    SV_TRY(sort_batch(c, B, false));
    B.fa.spec.n = (int)B.nf;
    if (B.nfp == 0 || B.nf == 0) {
        SV_CK(c, cudaStreamSynchronize(c->stream));
        B.planned = true;
        return SV_OK;
    }
    SV_CK(c, cudaMemsetAsync(B.d_hist, 0, sizeof(int) * kBLevels * B.nfp, c->stream));
    plume_levels_kernel<<<div_up(B.nf, 256), 256, 0, c->stream>>>(c->S.keys, B.nf, B.d_hist);
    SV_LAUNCHED(c);
    std::vector<int> hist((size_t)kBLevels * B.nfp);
    SV_CK(c, cudaMemcpyAsync(hist.data(), B.d_hist, sizeof(int) * hist.size(), cudaMemcpyDeviceToHost, c->stream));
    SV_CK(c, cudaStreamSynchronize(c->stream));
    // boxes of plume pid at its own level l: 1 + splits at levels 1..l
    std::vector<std::vector<long long>> boxes(B.nfp, std::vector<long long>(kBatchBits + 1, 1));
    std::vector<int> Lp(B.nfp, 2);
    for (int pid = 0; pid < B.nfp; pid++) {
        long long acc = 1;
        for (int l = 0; l <= kBatchBits; l++) {
            if (l > 0) acc += hist[(size_t)pid * kBLevels + l];
            boxes[pid][l] = acc;
        }
        Lp[pid] = pick_level((double)(B.vbeg[pid + 1] - B.vbeg[pid]), boxes[pid].data(), (double)B.m2l_weight,
                             c->P.fmm_ws);
    }
    // one level of headroom: a plume that contracts can still deepen
    int L = 2;
    for (int pid = 0; pid < B.nfp; pid++) L = std::max(L, Lp[pid]);
    L = std::min(L + 1, kBatchBits);
    B.h_delta.assign(B.np, 0);
    for (int pid = 0; pid < B.nfp; pid++) B.h_delta[pid] = L - Lp[pid];
    ForestSpec &f = B.fa.spec;
    f.L = L;
    f.mbits = kBatchBits;
    std::vector<int> caps(3 * kBLevels, 0);
    for (int l = 0; l <= L; l++) {
        int64_t tot = 0;
        for (int pid = 0; pid < B.nfp; pid++) {
            const int lo = l - B.h_delta[pid];
            tot += lo < 0 ? 1 : boxes[pid][lo];
        }
        int64_t cap = (2 * tot + 4096) * cap_scale;
        cap = std::min<int64_t>(cap, B.nf + 1);
        f.cap[l] = (int)cap;
        caps[kBLevels + l] = (int)cap;
    }
    SV_CK(c, cudaMemcpy(B.d_nbox, caps.data(), sizeof(int) * caps.size(), cudaMemcpyHostToDevice));
    B.fa.p = c->P.fmm_order;
    B.fa.ws = c->P.fmm_ws;
    B.fa.nroots = B.nfp;
    B.fa.roots = B.roots;
    B.fa.d_nbox = B.d_nbox;
    B.fa.d_err = B.d_err;
    SV_TRY(fmm_forest_reserve(c, B.fa));
    B.planned = true;
    return SV_OK;
}

// Capture fn's launches on c->stream into an executable graph.
template <typename Fn>
sv_status capture(sv_ctx *c, cudaGraphExec_t *out, unsigned long long *kernels, Fn fn) {
    cudaGraph_t g = nullptr;
    const unsigned long long before = c->launches;
    SV_CK(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    const sv_status st = fn();
    const cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    if (st != SV_OK) {
        if (g) cudaGraphDestroy(g);
        return st;
    }
    SV_TRY(check_cuda(c, e, "cudaStreamEndCapture"));
    const cudaError_t ei = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    SV_TRY(check_cuda(c, ei, "cudaGraphInstantiate"));
    *kernels = c->launches - before;
    c->launches = before;
    return SV_OK;
}

sv_status ensure_accel_graph(sv_ctx *c, Batch &B) {
    if (B.g_accel) return SV_OK;
    return capture(c, &B.g_accel, &B.accel_kernels, [&]() { return batch_force(c, B); });
}

sv_status ensure_step_graph(sv_ctx *c, Batch &B) {
    if (B.g_step) return SV_OK;
    return capture(c, &B.g_step, &B.step_kernels, [&]() -> sv_status {
        const double dt = B.step_dt, h = 0.5 * dt;
        SV_TRY(drift(c, 0.0, h, c->wstatus, B.d_time, 0));
        c->fstatus = c->wstatus;
        const sv_status s = batch_force(c, B);
        c->fstatus = nullptr;
        SV_TRY(s);
        SV_TRY(kick(c, 0.0, dt, c->wstatus, B.d_time));
        SV_TRY(drift(c, h, h, nullptr, B.d_time, 1));
        advance_step_kernel<<<1, 1, 0, c->stream>>>(B.d_time);
        SV_LAUNCHED(c);
        return SV_OK;
    });
}

sv_status read_err(sv_ctx *c, Batch &B, int *err) {
    SV_CK(c, cudaMemcpyAsync(B.h_err, B.d_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    SV_CK(c, cudaStreamSynchronize(c->stream));
    *err = *B.h_err;
    if (*err) B.overflow_mask = *err;
    return SV_OK;
}

sv_status grow(sv_ctx *c, Batch &B, int scale) {
    B.regrows++;
    SV_CK(c, cudaMemsetAsync(B.d_err, 0, sizeof(int), c->stream));
    return plan_forest(c, B, scale);
}

}  // namespace

void batch_free(sv_ctx *c) {
    if (!c->batch) return;
    Batch &B = *c->batch;
    drop_graphs(B);
    cudaFree(B.vsrc); cudaFree(B.vtag); cudaFree(B.roots); cudaFree(B.delta); cudaFree(B.d_hist);
    cudaFree(B.d_vbeg);
    cudaFree(B.chunk_beg); cudaFree(B.pid_chunk); cudaFree(B.chunk_red); cudaFree(B.items);
    cudaFree(B.queue); cudaFree(B.cub_tmp); cudaFree(B.d_nbox); cudaFree(B.d_err); cudaFree(B.d_time);
    cudaFree(B.backup);
    cudaFree(B.backup_st);
    cudaFree(B.ev_count0);
    cudaFree(B.pfold);
    c->pfold = nullptr;
    cudaFreeHost(B.h_err);
    cudaFreeHost(B.h_time);
    if (B.side) cudaStreamDestroy(B.side);
    if (B.fork) cudaEventDestroy(B.fork);
    if (B.join) cudaEventDestroy(B.join);
    delete c->batch;
    c->batch = nullptr;
}

// Parameters travel into the graphs as kernel arguments: a change of them
// needs a new plan and new graphs.
void batch_invalidate(sv_ctx *c) {
    if (!c->batch) return;
    drop_graphs(*c->batch);
    c->batch->planned = false;
}

bool batch_same_shape(const sv_ctx *c, int32_t np, const int64_t *counts, const int32_t *method,
                      const int32_t *sym) {
    if (!c->batch || c->batch->np != np) return false;
    const Batch &B = *c->batch;
    for (int p = 0; p < np; p++)
        if (B.count[p] != counts[p] || B.method[p] != method[p] || B.sym[p] != sym[p]) return false;
    return true;
}

// Builds the view and the static tables of a batch whose state is uploaded.
sv_status batch_plan(sv_ctx *c, int32_t np, const int64_t *counts, const int32_t *method, const int32_t *sym) {
    batch_free(c);
    if (np < 1 || np > kMaxPlumes) return set_error(c, SV_ERR_INVALID, "1..%d plumes per batch", kMaxPlumes);
    if (c->sub.on) return set_error(c, SV_ERR_UNSUPPORTED, "substeps run on single-plume contexts");
    c->batch = new Batch();
    Batch &B = *c->batch;
    B.np = np;
    B.count.assign(counts, counts + np);
    B.method.assign(method, method + np);
    B.sym.assign(sym, sym + np);
    B.off.assign(np + 1, 0);
    for (int p = 0; p < np; p++) {
        if (counts[p] < 0) return set_error(c, SV_ERR_INVALID, "plume %d: negative count", p);
        if (method[p] != SV_METHOD_DIRECT && method[p] != SV_METHOD_FMM)
            return set_error(c, SV_ERR_UNSUPPORTED, "plume %d: batches run the direct sum or the FMM", p);
        if (sym[p] != SV_SYM_NONE && sym[p] != SV_SYM_ROTATIONAL)
            return set_error(c, SV_ERR_UNSUPPORTED, "plume %d: batches support no symmetry or the rotational one", p);
        B.off[p + 1] = B.off[p] + counts[p];
    }
    if (B.off[np] != c->n) return set_error(c, SV_ERR_INVALID, "plume counts sum to %lld, state has %lld",
                                            (long long)B.off[np], (long long)c->n);
    if (c->P.fmm_order != 4 && c->P.fmm_order != 6 && c->P.fmm_order != 8 && c->P.fmm_order != 10)
        return set_error(c, SV_ERR_UNSUPPORTED, "FMM order %d not instantiated (4, 6, 8, 10)", c->P.fmm_order);
    if (c->P.fmm_type != SV_FMM_FMM)
        return set_error(c, SV_ERR_UNSUPPORTED, "batches run the plain FMM (no treecode or outlier variant)");
    // plume ids: FMM plumes first, in plume order, then the direct plumes
    B.pid_of.assign(np, -1);
    for (int p = 0; p < np; p++)
        if (method[p] == SV_METHOD_FMM) {
            B.pid_of[p] = (int)B.plume_of.size();
            B.plume_of.push_back(p);
        }
    B.nfp = (int)B.plume_of.size();
    for (int p = 0; p < np; p++)
        if (method[p] != SV_METHOD_FMM) {
            B.pid_of[p] = (int)B.plume_of.size();
            B.plume_of.push_back(p);
        }
    B.vbeg.assign(np + 1, 0);
    for (int pid = 0; pid < np; pid++) {
        const int p = B.plume_of[pid];
        const int nimg = (method[p] == SV_METHOD_FMM && sym[p] == SV_SYM_ROTATIONAL) ? 4 : 1;
        B.vbeg[pid + 1] = B.vbeg[pid] + counts[p] * nimg;
    }
    B.nv = B.vbeg[np];
    B.nf = B.vbeg[B.nfp];
    if (B.nv > (int64_t)INT32_MAX / 2) return set_error(c, SV_ERR_CAPACITY, "%lld slots", (long long)B.nv);
    std::vector<uint32_t> vsrc(B.nv), vtag(B.nv);
    for (int pid = 0; pid < np; pid++) {
        const int p = B.plume_of[pid];
        const int64_t n = counts[p];
        const int nimg = (int)((B.vbeg[pid + 1] - B.vbeg[pid]) / std::max<int64_t>(n, 1));
        int64_t v = B.vbeg[pid];
        for (int64_t i = 0; i < n; i++)
            for (int g = 0; g < nimg; g++) {
                vsrc[v] = (uint32_t)(B.off[p] + i);
                vtag[v] = (uint32_t)pid * 4u + (uint32_t)g;
                v++;
            }
    }
    std::vector<int> cbeg, pchunk(np + 1, 0);
    for (int pid = 0; pid < np; pid++) {
        pchunk[pid] = (int)cbeg.size();
        for (int64_t v = B.vbeg[pid]; v < B.vbeg[pid + 1]; v += kChunk) cbeg.push_back((int)v);
    }
    pchunk[np] = (int)cbeg.size();
    B.nchunks = (int)cbeg.size();
    cbeg.push_back((int)B.nv);
    const size_t nvb = (size_t)std::max<int64_t>(B.nv, 1);
    SV_CK(c, cudaMalloc(&B.vsrc, sizeof(uint32_t) * nvb));
    SV_CK(c, cudaMalloc(&B.vtag, sizeof(uint32_t) * nvb));
    SV_CK(c, cudaMalloc(&B.roots, sizeof(double) * 8 * np));
    SV_CK(c, cudaMalloc(&B.delta, sizeof(int) * np));
    SV_CK(c, cudaMemset(B.delta, 0, sizeof(int) * np));
    SV_CK(c, cudaMalloc(&B.d_hist, sizeof(int) * kBLevels * std::max(B.nfp, 1)));
    SV_CK(c, cudaMalloc(&B.d_vbeg, sizeof(int) * (np + 1)));
    {
        std::vector<int> vb(B.vbeg.begin(), B.vbeg.end());
        SV_CK(c, cudaMemcpy(B.d_vbeg, vb.data(), sizeof(int) * (np + 1), cudaMemcpyHostToDevice));
    }
    SV_CK(c, cudaMalloc(&B.chunk_beg, sizeof(int) * cbeg.size()));
    SV_CK(c, cudaMalloc(&B.pid_chunk, sizeof(int) * (np + 1)));
    SV_CK(c, cudaMalloc(&B.chunk_red, sizeof(double) * 6 * std::max(B.nchunks, 1)));
    SV_CK(c, cudaMalloc(&B.queue, sizeof(int)));
    SV_CK(c, cudaMalloc(&B.d_nbox, sizeof(int) * 3 * kBLevels));
    SV_CK(c, cudaMalloc(&B.d_err, sizeof(int)));
    SV_CK(c, cudaMalloc(&B.d_time, sizeof(double) * 4));
    SV_CK(c, cudaMallocHost(&B.h_err, sizeof(int)));
    SV_CK(c, cudaMallocHost(&B.h_time, sizeof(double) * 4));
    {
        std::vector<int8_t> pf((size_t)std::max<int64_t>(c->n, 1), 0);
        for (int p = 0; p < np; p++)
            if (sym[p] == SV_SYM_ROTATIONAL)
                std::fill(pf.begin() + B.off[p], pf.begin() + B.off[p] + counts[p], (int8_t)1);
        SV_CK(c, cudaMalloc(&B.pfold, pf.size()));
        SV_CK(c, cudaMemcpy(B.pfold, pf.data(), pf.size(), cudaMemcpyHostToDevice));
        c->pfold = B.pfold;
    }
    SV_CK(c, cudaMemset(B.d_err, 0, sizeof(int)));
    SV_CK(c, cudaMemset(B.d_nbox, 0, sizeof(int) * 3 * kBLevels));
    if (B.nv > 0) {
        SV_CK(c, cudaMemcpy(B.vsrc, vsrc.data(), sizeof(uint32_t) * B.nv, cudaMemcpyHostToDevice));
        SV_CK(c, cudaMemcpy(B.vtag, vtag.data(), sizeof(uint32_t) * B.nv, cudaMemcpyHostToDevice));
    }
    SV_CK(c, cudaMemcpy(B.chunk_beg, cbeg.data(), sizeof(int) * cbeg.size(), cudaMemcpyHostToDevice));
    SV_CK(c, cudaMemcpy(B.pid_chunk, pchunk.data(), sizeof(int) * (np + 1), cudaMemcpyHostToDevice));
    SV_CK(c, cudaStreamCreateWithFlags(&B.side, cudaStreamNonBlocking));
    SV_CK(c, cudaEventCreateWithFlags(&B.fork, cudaEventDisableTiming));
    SV_CK(c, cudaEventCreateWithFlags(&B.join, cudaEventDisableTiming));
    SV_TRY(ensure_sorted_capacity(c, std::max<int64_t>(B.nv, 1)));
    size_t bytes = 0;
    SV_CK(c, cub::DeviceRadixSort::SortPairs(nullptr, bytes, c->S.keys_alt, c->S.keys, c->S.idx_alt, c->S.idx,
                                             (int)std::max<int64_t>(B.nv, 1), 0, kPidShift + 9, c->stream));
    SV_CK(c, cudaMalloc(&B.cub_tmp, bytes));
    B.cub_bytes = bytes;
    c->S.n = B.nv;
    c->S.n_orig = c->n;
    SV_TRY(build_items(c, B));
    return SV_OK;
}

sv_status batch_accel(sv_ctx *c) {
    Batch &B = *c->batch;
    if (B.nv == 0) return SV_OK;
    if (!B.planned) SV_TRY(plan_forest(c, B, 1));
    for (int attempt = 0; attempt < 4; attempt++) {
        SV_TRY(ensure_accel_graph(c, B));
        SV_CK(c, cudaGraphLaunch(B.g_accel, c->stream));
        c->launches += B.accel_kernels;
        int err = 0;
        SV_TRY(read_err(c, B, &err));
        if (!err) {
            c->stats.pair_interactions = B.direct_pairs;
            // the result stands (the rotation M2L ran); the next run gets more room
            if (fmm_forest_tc_overflowed(c)) {
                SV_TRY(fmm_forest_tc_grow(c));
                drop_graphs(B);
            }
            return SV_OK;
        }
        SV_TRY(grow(c, B, 2 << attempt));
    }
    return set_error(c, SV_ERR_CAPACITY, "forest box capacity still exceeded after growing it");
}

sv_status batch_leapfrog(sv_ctx *c, int32_t nsteps, double dt, double t0) {
    Batch &B = *c->batch;
    if (nsteps == 0 || B.nv == 0) return SV_OK;
    if (!B.planned) SV_TRY(plan_forest(c, B, 1));
    const int64_t n = c->n;
    if (!B.backup) SV_CK(c, cudaMalloc(&B.backup, sizeof(double) * 6 * std::max<int64_t>(n, 1)));
    if (!B.backup_st) SV_CK(c, cudaMalloc(&B.backup_st, sizeof(int32_t) * std::max<int64_t>(n, 1)));
    if (!B.ev_count0) SV_CK(c, cudaMalloc(&B.ev_count0, sizeof(unsigned long long)));
    // the drift may change status and record events: both are part of the state a retry restores
    if (c->B.crash != SV_CRASH_NONE || c->B.bc != SV_BC_NONE) SV_TRY(events_reserve(c));
    SV_TRY(field_prepare(c));  // before capture: the graph keeps the walk caches' address
    double *st[6] = {c->x, c->y, c->z, c->vx, c->vy, c->vz};
    const bool watch_tc = B.nf > 0 && B.nfp > 0 && c->P.fmm_m2l_tc >= 0;
    // Step by step: each step's state is saved first (a device copy, ~0.1 ms
    // for 8M ions), and the step's capacity flags are read after it (one
    // host wait, small beside a batch step's device time).  A step that
    // overflowed a forest level is undone and run again with larger
    // capacities; only that step is repeated.  A step whose M2L translations
    // outgrew the tensor-core room ran the rotation kernel (its result
    // stands), and the room grows before the next step, so a run of steps
    // whose plumes expand keeps the tensor cores.
    for (int s = 0; s < nsteps; s++) {
        for (int attempt = 0;; attempt++) {
            if (attempt == 4) return set_error(c, SV_ERR_CAPACITY, "forest box capacity still exceeded after growing it");
            for (int k = 0; k < 6; k++)
                SV_CK(c, cudaMemcpyAsync(B.backup + k * n, st[k], sizeof(double) * n, cudaMemcpyDeviceToDevice,
                                         c->stream));
            SV_CK(c, cudaMemcpyAsync(B.backup_st, c->status, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, c->stream));
            if (c->d_ev_count)
                SV_CK(c, cudaMemcpyAsync(B.ev_count0, c->d_ev_count, sizeof(unsigned long long),
                                         cudaMemcpyDeviceToDevice, c->stream));
            // dt is baked into the step graph
            if (B.g_step && B.step_dt != dt) {
                cudaGraphExecDestroy(B.g_step);
                B.g_step = nullptr;
            }
            B.step_dt = dt;
            SV_TRY(ensure_step_graph(c, B));
            B.h_time[0] = t0;
            B.h_time[1] = dt;
            B.h_time[2] = (double)s;
            B.h_time[3] = (double)c->ev_seq;
            SV_CK(c, cudaMemcpyAsync(B.d_time, B.h_time, sizeof(double) * 4, cudaMemcpyHostToDevice, c->stream));
            SV_CK(c, cudaGraphLaunch(B.g_step, c->stream));
            c->launches += B.step_kernels;
            int err = 0;
            SV_TRY(read_err(c, B, &err));
            if (!err) break;
            for (int k = 0; k < 6; k++)
                SV_CK(c, cudaMemcpyAsync(st[k], B.backup + k * n, sizeof(double) * n, cudaMemcpyDeviceToDevice,
                                         c->stream));
            SV_CK(c, cudaMemcpyAsync(c->status, B.backup_st, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice,
                                     c->stream));
            if (c->d_ev_count)
                SV_CK(c, cudaMemcpyAsync(c->d_ev_count, B.ev_count0, sizeof(unsigned long long),
                                         cudaMemcpyDeviceToDevice, c->stream));
            SV_TRY(grow(c, B, 2 << attempt));
        }
        if (watch_tc && fmm_forest_tc_overflowed(c)) {
            SV_TRY(fmm_forest_tc_grow(c));
            drop_graphs(B);
        }
    }
    c->ev_seq += 2LL * nsteps;
    return SV_OK;
}

// ------------------------------------------------------------- autotuner --
namespace {

std::mutex g_tune_mu;
// shape -> the tuned choice: leaf target (M2L weight), direct chunk, FMM order and near field
struct Tuned {
    int lt, dc, p, near;
};
std::map<std::string, Tuned> g_tune_cache;

// The batch's shape: plume count, per method / symmetry the plume count and
// the log2 buckets of plume sizes, FMM order and well-separation (and the
// error bound when the order is tuned too).
std::string shape_key(const sv_ctx *c, const Batch &B) {
    std::map<std::string, int> hist;
    for (int p = 0; p < B.np; p++) {
        int bucket = 0;
        while ((int64_t)1 << (bucket + 1) <= std::max<int64_t>(B.count[p], 1)) bucket++;
        hist["m" + std::to_string(B.method[p]) + "s" + std::to_string(B.sym[p]) + "b" + std::to_string(bucket)]++;
    }
    std::string k = "np" + std::to_string(B.np) + "_p" + std::to_string(c->P.fmm_order) + "_ws" +
                    std::to_string(c->P.fmm_ws) + "_n" + std::to_string(c->P.fmm_near) +
                    (c->P.fmm_m2l_tc >= 0 ? "_tc" : "_rot");
    if (c->P.fmm_tune_err > 0.0f) {
        char e[32];
        snprintf(e, sizeof(e), "_err%.3g", (double)c->P.fmm_tune_err);
        k += e;
    }
    for (auto &kv : hist) k += "_" + kv.first + "x" + std::to_string(kv.second);
    return k;
}

// Cache file lines: key, leaf target, direct chunk, ms, then (optional) FMM
// order and near field.
void load_cache(const char *path) {
    if (!path) return;
    FILE *f = fopen(path, "r");
    if (!f) return;
    char line[8192], key[4096];
    while (fgets(line, sizeof(line), f)) {
        int lt, dc, po = 0, nr = 0;
        double ms;
        const int got = sscanf(line, "%4095s %d %d %lf %d %d", key, &lt, &dc, &ms, &po, &nr);
        if (got == 4 || got == 6) g_tune_cache[key] = Tuned{lt, dc, got == 6 ? po : 0, got == 6 ? nr : 0};
    }
    fclose(f);
}

void append_cache(const char *path, const std::string &key, const Tuned &t, double ms) {
    if (!path) return;
    FILE *f = fopen(path, "a");
    if (!f) return;
    fprintf(f, "%s %d %d %.6f %d %d\n", key.c_str(), t.lt, t.dc, ms, t.p, t.near);
    fclose(f);
}

// median device time of `reps` replays of the force graph
sv_status time_accel(sv_ctx *c, Batch &B, int reps, double *ms) {
    SV_TRY(ensure_accel_graph(c, B));
    for (int w = 0; w < 2; w++) SV_CK(c, cudaGraphLaunch(B.g_accel, c->stream));
    std::vector<float> t;
    for (int r = 0; r < reps; r++) {
        SV_CK(c, cudaEventRecord(c->ev_begin, c->stream));
        SV_CK(c, cudaGraphLaunch(B.g_accel, c->stream));
        SV_CK(c, cudaEventRecord(c->ev_end, c->stream));
        SV_CK(c, cudaEventSynchronize(c->ev_end));
        float e = 0;
        SV_CK(c, cudaEventElapsedTime(&e, c->ev_begin, c->ev_end));
        t.push_back(e);
    }
    int err = 0;
    SV_TRY(read_err(c, B, &err));
    std::sort(t.begin(), t.end());
    *ms = err ? 1e30 : t[t.size() / 2];
    return SV_OK;
}

// Leaf occupancy of the FMM plumes: the M2L weight of the depth model.
// Among the weights within 3 % of the fastest, the largest is kept: it
// chooses shallower trees, and as the plumes expand their M2L translations
// grow faster than their pairs (batch256 over 10 steps from a tie at the
// start: weight 400 95 ms per step, weight 200 107 ms).
sv_status sweep_weights(sv_ctx *c, Batch &B, int *best_lt, double *best_ms) {
    const int weights[6] = {100, 200, 400, 800, 1600, 3200};
    double t[6], best = 1e30;
    for (int k = 0; k < 6; k++) {
        B.m2l_weight = weights[k];
        SV_TRY(plan_forest(c, B, 1));
        SV_TRY(time_accel(c, B, 5, &t[k]));
        best = std::min(best, t[k]);
    }
    for (int k = 0; k < 6; k++)
        if (t[k] <= 1.03 * best) *best_lt = weights[k];
    *best_ms = best;
    return SV_OK;
}

// The force error of the current plan: the largest over up to four FMM
// plumes without symmetry images (the biggest), 64 sampled targets each,
// against the FP64 direct sum of the plume.
sv_status batch_sampled_error(sv_ctx *c, Batch &B, double *err) {
    std::vector<int> cand;
    for (int p = 0; p < B.np; p++)
        if (B.method[p] == SV_METHOD_FMM && B.sym[p] == SV_SYM_NONE) cand.push_back(p);
    std::sort(cand.begin(), cand.end(), [&](int a, int b) { return B.count[a] > B.count[b]; });
    if (cand.size() > 4) cand.resize(4);
    *err = 0.0;
    for (int p : cand) {
        double e = 0.0;
        SV_TRY(sampled_error_range(c, B.off[p], B.count[p], 64, &e));
        *err = std::max(*err, e);
    }
    return SV_OK;
}

}  // namespace

sv_status batch_tune(sv_ctx *c, const char *cache_path, double *best_ms) {
    Batch &B = *c->batch;
    if (B.nv == 0) {
        if (best_ms) *best_ms = 0.0;
        return SV_OK;
    }
    std::lock_guard<std::mutex> lk(g_tune_mu);
    load_cache(cache_path);
    const std::string key = shape_key(c, B);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) {
        const Tuned &t = it->second;
        if (t.p > 0 && (t.p != c->P.fmm_order || t.near != c->P.fmm_near)) {
            c->P.fmm_order = t.p;
            c->P.fmm_near = t.near;
            batch_invalidate(c);
        }
        B.m2l_weight = t.lt;
        B.direct_chunk = t.dc;
        SV_TRY(build_items(c, B));
        drop_graphs(B);
        SV_TRY(plan_forest(c, B, 1));
        double ms = 0;
        SV_TRY(time_accel(c, B, 3, &ms));
        B.tuned_ms = ms;
        if (best_ms) *best_ms = ms;
        return SV_OK;
    }
    int best_lt = B.m2l_weight, best_dc = B.direct_chunk;
    double best = 1e30;
    if (B.nfp > 0 && c->P.fmm_tune_err > 0.0f) {
        // the expansion order and near field too: the fastest (order, shape)
        // whose sampled force error meets fmm_tune_err (else the most accurate)
        struct Cand {
            int p, near;
        };
        std::vector<Cand> cands;
        const int fixed_near = c->P.fmm_near;
        for (const int p : {4, 6, 8}) {
            if (c->P.fmm_ws == 2 && fixed_near == 0) {
                cands.push_back({p, 2});
                cands.push_back({p, 1});
            } else {
                cands.push_back({p, fixed_near});
            }
        }
        int kept = -1, most_acc = 0;
        double kept_t = 1e30, min_err = 1e300;
        std::vector<int> lts(cands.size());
        for (size_t k = 0; k < cands.size(); k++) {
            c->P.fmm_order = cands[k].p;
            c->P.fmm_near = cands[k].near;
            batch_invalidate(c);
            double t = 0.0, e = 0.0;
            SV_TRY(sweep_weights(c, B, &lts[k], &t));
            B.m2l_weight = lts[k];
            SV_TRY(plan_forest(c, B, 1));
            SV_TRY(time_accel(c, B, 3, &t));
            SV_TRY(batch_sampled_error(c, B, &e));
            if (e < min_err) {
                min_err = e;
                most_acc = (int)k;
            }
            if (e <= (double)c->P.fmm_tune_err && t < kept_t) {
                kept_t = t;
                kept = (int)k;
            }
        }
        const int k = kept >= 0 ? kept : most_acc;
        c->P.fmm_order = cands[k].p;
        c->P.fmm_near = cands[k].near;
        batch_invalidate(c);
        best_lt = lts[k];
    } else if (B.nfp > 0) {
        SV_TRY(sweep_weights(c, B, &best_lt, &best));
    }
    B.m2l_weight = best_lt;
    SV_TRY(plan_forest(c, B, 1));
    if (B.nfp < B.np) {
        best = 1e30;
        for (int dc : {1024, 2048, 4096, 8192}) {
            B.direct_chunk = dc;
            SV_TRY(build_items(c, B));
            drop_graphs(B);
            double ms = 0;
            SV_TRY(time_accel(c, B, 5, &ms));
            if (ms < best) {
                best = ms;
                best_dc = dc;
            }
        }
        B.direct_chunk = best_dc;
        SV_TRY(build_items(c, B));
        drop_graphs(B);
    }
    double ms = 0;
    SV_TRY(time_accel(c, B, 5, &ms));
    B.tuned_ms = ms;
    const Tuned t{best_lt, best_dc, c->P.fmm_tune_err > 0.0f ? c->P.fmm_order : 0,
                  c->P.fmm_tune_err > 0.0f ? c->P.fmm_near : 0};
    g_tune_cache[key] = t;
    append_cache(cache_path, key, t, ms);
    if (best_ms) *best_ms = ms;
    return SV_OK;
}

sv_status batch_set_tuning(sv_ctx *c, int m2l_weight, int direct_chunk) {
    Batch &B = *c->batch;
    if (m2l_weight < 1 || direct_chunk < kDTile)
        return set_error(c, SV_ERR_INVALID, "M2L weight >= 1 and direct chunk >= %d required", kDTile);
    B.m2l_weight = m2l_weight;
    B.direct_chunk = direct_chunk;
    SV_TRY(build_items(c, B));
    drop_graphs(B);
    B.planned = false;
    return SV_OK;
}

sv_status batch_info(const sv_ctx *c, sv_batch_info *out) {
    const Batch &B = *c->batch;
    memset(out, 0, sizeof(*out));
    if (c->fmm && B.nfp > 0 && B.planned) {
        double m2l = 0, pairs = 0;
        SV_TRY(fmm_counts(const_cast<sv_ctx *>(c), &m2l, &pairs));
        out->fmm_m2l = m2l;
        out->fmm_pairs = pairs;
    }
    out->nplumes = B.np;
    out->fmm_plumes = B.nfp;
    out->slots = B.nv;
    out->fmm_slots = B.nf;
    out->leaf_level = B.fa.spec.L;
    out->m2l_weight = B.m2l_weight;
    out->direct_chunk = B.direct_chunk;
    out->direct_items = B.nitems;
    out->graph_kernels_step = (int32_t)B.step_kernels;
    out->graph_kernels_accel = (int32_t)B.accel_kernels;
    out->tuned_ms = B.tuned_ms;
    out->direct_pairs = B.direct_pairs;
    out->regrows = B.regrows;
    if (B.planned && B.nfp > 0) {
        int ml = 0;
        SV_TRY(fmm_forest_max_leaf(const_cast<sv_ctx *>(c), B.fa, &ml));
        out->max_leaf = ml;
    }
    out->overflow_mask = B.overflow_mask;
    out->m2l_tc = fmm_forest_tc_used(c) ? 1 : 0;
    out->fmm_order = c->P.fmm_order;
    out->fmm_near = c->P.fmm_near;
    if (B.planned && B.nfp > 0) {
        int h[3 * kBLevels];
        SV_CK(const_cast<sv_ctx *>(c), cudaMemcpy(h, B.d_nbox, sizeof(h), cudaMemcpyDeviceToHost));
        for (int l = 0; l < kBLevels; l++) {
            out->level_boxes[l] = h[l];
            out->level_cap[l] = h[kBLevels + l];
            out->level_max[l] = h[2 * kBLevels + l];
        }
    }
    return SV_OK;
}

}  // namespace sv
