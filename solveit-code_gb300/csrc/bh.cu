// bh.cu -- Barnes-Hut treecode on GB300.
//
// Restates BarnesHutForceCalculation::updateAcceleration
// (barnes_hut_force_calculation.cpp:574-715): tree, cell properties
// (computeCellProperties :337-390: net charge, centre of charge weighted by
// |charge|, delta = |centre of charge - geometric centre|) and the walk of
// computeForceFromTree (:417-450) with the acceptance test
// theta * (d - delta) > l  (d = sqrt(r^2 + eps^2), l = cell side, :435) and the
// monopole force q (x - c) / d^3 (:399-408); plus the rotational
// (barnes_hut_force_calculation_rotational.cpp:28-135: target rotated into
// each quadrant, force rotated back, self excluded only in quadrant 0) and
// translational (barnes_hut_force_calculation_translational.cpp:200-280:
// target shifted by each image offset, self excluded only for the centre
// image) variants.
//
// GB300 design:
//   * the octree is tree.cu's level structure built down to single-particle
//     boxes; a box is a leaf of the walk when it holds <= leaf_size particles
//     (the reference stops at one particle per leaf);
//   * cell properties are reduced bottom-up, one kernel per level, in FP64;
//   * node centres and particle positions are stored as FP32 (hi, lo) pairs
//     relative to the root origin, so (target - centre) is formed as
//     (t_hi - c_hi) + (t_lo - c_lo): FP64-like differences with FP32
//     arithmetic only (the walk has no FP64 instruction);
//   * the walk is warp-cooperative and stackless, over the tree threaded the
//     way the reference threads its cells (nextSibling, cell.h:33-35,
//     cell.cpp:171-172): every cell keeps a skip link to the next cell of
//     the depth-first order outside its own subtree (its next sibling, else
//     its parent's skip link).  A warp owns 32 Morton-consecutive targets
//     and walks one cell at a time; each lane keeps one bit per level, set
//     when it rejected the current ancestor at that level, so a lane takes
//     part at a cell when it rejected the cell's parent.  Taking part, it
//     applies its own acceptance test and adds the monopole when it
//     accepts; when some lane rejects, the warp goes down to the first child
//     (or, at a leaf, the rejecting lanes sum the leaf's particles
//     directly), else it follows the skip link.  Each target gets exactly
//     the cells its own walk would accept, the warp visits a cell at most
//     once, and no stack bounds the depth.
#include <cfloat>

#include "sv_internal.cuh"
#include "tree.cuh"

namespace sv {

struct Bh {
    void *arena = nullptr;
    size_t arena_bytes = 0;
    float4 *ph = nullptr, *pl = nullptr;  // particle hi (xyz, q) and lo (xyz, 0)
    int64_t pcap = 0;
    unsigned long long *d_counts = nullptr;  // [0] accepted cells, [1] direct pairs
    unsigned long long *h_counts = nullptr;
    int level_hint = -1;  // deepest level of the last tree
};

namespace {

constexpr int kBhWarps = 4;
constexpr int kBhHalfWarps = 32;  // warps per SM below which the walk takes 16 targets per warp

struct BhLevels {
    const float4 *nh[kMortonBits + 1];  // centre hi (xyz) + net charge
    const float4 *nl[kMortonBits + 1];  // centre lo (xyz) + delta
    const int *child0[kMortonBits + 1];
    const int *start[kMortonBits + 1];
    const int *skip[kMortonBits + 1];   // next cell of the depth-first order outside the subtree, or kEnd
    int deepest;
    int leaf_size;
};

// a cell as (level << 24) | box, and the end of the walk
constexpr int kEnd = -1;
__host__ __device__ __forceinline__ int cell_id(int l, int b) { return (l << 24) | b; }

// Skip links of every cell of levels 0..D, one thread per cell: its next
// sibling (same parent), else the first ancestor's next sibling, else kEnd.
struct SkipArgs {
    const int *parent[kMortonBits + 1];
    int *skip[kMortonBits + 1];
    int nbox[kMortonBits + 1];
    int first[kMortonBits + 2];  // first global cell of each level; first[D + 1] = all cells
    int D;
};

__global__ void skip_links_kernel(SkipArgs a) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= a.first[a.D + 1]) return;
    int l = 0;
    while (l < a.D && g >= a.first[l + 1]) l++;
    const int b0 = g - a.first[l];
    int lv = l, b = b0, out = kEnd;
    for (;;) {
        const bool sib = b + 1 < a.nbox[lv] && (lv == 0 || a.parent[lv][b + 1] == a.parent[lv][b]);
        if (sib) {
            out = cell_id(lv, b + 1);
            break;
        }
        if (lv == 0) break;
        b = a.parent[lv][b];
        lv--;
    }
    a.skip[l][b0] = out;
}

struct BhImages {
    int kind;  // 0 none, 1 rotational, 2 translational offsets
    int count;
    const double *off;
};

__device__ __forceinline__ void split_hilo(double v, float &hi, float &lo) {
    hi = (float)v;
    lo = (float)(v - (double)hi);
}

__global__ void particles_hilo(const double *__restrict__ xs, const double *__restrict__ ys,
                               const double *__restrict__ zs, const float *__restrict__ qs, int n,
                               const double *__restrict__ root, float4 *__restrict__ ph, float4 *__restrict__ pl) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float hx, lx, hy, ly, hz, lz;
    split_hilo(xs[i] - root[0], hx, lx);
    split_hilo(ys[i] - root[1], hy, ly);
    split_hilo(zs[i] - root[2], hz, lz);
    ph[i] = make_float4(hx, hy, hz, qs[i]);
    pl[i] = make_float4(lx, ly, lz, 0.f);
}

// deepest level: properties straight from the particles of each box
__global__ void props_from_particles(int nbox, const int *__restrict__ start, const int4 *__restrict__ coord,
                                     const double *__restrict__ xs, const double *__restrict__ ys,
                                     const double *__restrict__ zs, const float *__restrict__ qs,
                                     const double *__restrict__ root, int level, double *__restrict__ Q,
                                     double *__restrict__ U, double3 *__restrict__ coc, float4 *__restrict__ nh,
                                     float4 *__restrict__ nl) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nbox) return;
    const double side = root[3] / (double)(1ll << level);
    double q = 0, u = 0, cx = 0, cy = 0, cz = 0;
    for (int j = start[b]; j < start[b + 1]; j++) {
        const double qj = qs[j], aq = fabs(qj);
        q += qj;
        u += aq;
        cx += aq * (xs[j] - root[0]);
        cy += aq * (ys[j] - root[1]);
        cz += aq * (zs[j] - root[2]);
    }
    const int4 c = coord[b];
    const double gx = (c.x + 0.5) * side, gy = (c.y + 0.5) * side, gz = (c.z + 0.5) * side;
    if (u != 0.0) {
        cx /= u;
        cy /= u;
        cz /= u;
    } else {
        cx = gx;
        cy = gy;
        cz = gz;
    }
    Q[b] = q;
    U[b] = u;
    coc[b] = make_double3(cx, cy, cz);
    const double dx = cx - gx, dy = cy - gy, dz = cz - gz;
    float hx, lx, hy, ly, hz, lz;
    split_hilo(cx, hx, lx);
    split_hilo(cy, hy, ly);
    split_hilo(cz, hz, lz);
    nh[b] = make_float4(hx, hy, hz, (float)q);
    nl[b] = make_float4(lx, ly, lz, (float)sqrt(dx * dx + dy * dy + dz * dz));
}

// coarser levels from their children (computeCellProperties :358-388):
// centre = sum_c coc_c |Q_c| / sum_c U_c, geometric centre when U = 0
struct PropLevel {
    int nbox;
    const int *child0;
    const int4 *coord;
    double *Q, *U;
    double3 *coc;
    float4 *nh, *nl;
};

__device__ __forceinline__ void props_box(int b, int level, const double *__restrict__ root, const PropLevel &C,
                                          const PropLevel &V) {
    const double side = root[3] / (double)(1ll << level);
    double q = 0, u = 0, tx = 0, ty = 0, tz = 0;
    for (int c = V.child0[b]; c < V.child0[b + 1]; c++) {
        const double qc = C.Q[c], w = fabs(qc);
        q += qc;
        u += C.U[c];
        const double3 p = C.coc[c];
        tx += p.x * w;
        ty += p.y * w;
        tz += p.z * w;
    }
    const int4 cb = V.coord[b];
    const double gx = (cb.x + 0.5) * side, gy = (cb.y + 0.5) * side, gz = (cb.z + 0.5) * side;
    double cx = gx, cy = gy, cz = gz;
    if (u != 0.0) {
        cx = tx / u;
        cy = ty / u;
        cz = tz / u;
    }
    V.Q[b] = q;
    V.U[b] = u;
    V.coc[b] = make_double3(cx, cy, cz);
    const double dx = cx - gx, dy = cy - gy, dz = cz - gz;
    float hx, lx, hy, ly, hz, lz;
    split_hilo(cx, hx, lx);
    split_hilo(cy, hy, ly);
    split_hilo(cz, hz, lz);
    V.nh[b] = make_float4(hx, hy, hz, (float)q);
    V.nl[b] = make_float4(lx, ly, lz, (float)sqrt(dx * dx + dy * dy + dz * dz));
}

// one level from the level below it, one thread per box
__global__ void props_from_children(int level, const double *__restrict__ root, PropLevel C, PropLevel V) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < V.nbox) props_box(b, level, root, C, V);
}

// Levels top .. 0 in one CTA, level by level (coarse levels have few boxes,
// and one launch per level made each of them a launch's latency).
struct PropLevels {
    PropLevel lv[kMortonBits + 1];
};
__global__ void props_coarse_levels(int top, const double *__restrict__ root, PropLevels P) {
    for (int l = top; l >= 0; l--) {
        for (int b = threadIdx.x; b < P.lv[l].nbox; b += blockDim.x) props_box(b, l, root, P.lv[l + 1], P.lv[l]);
        __syncthreads();
    }
}

// TPW targets per warp: 32, or 16 with the two half-warps sharing each
// target (both take the same acceptance decisions, the lower half adds the
// accepted cells, the halves split each opened leaf's particles and add their
// sums at the end): twice the warps for a small plume, each walking the union
// of fewer targets' cells.
template <int TPW>
__global__ void __launch_bounds__(kBhWarps * 32)
bh_walk_kernel(BhLevels T, const float4 *__restrict__ ph, const float4 *__restrict__ pl,
               const double *__restrict__ xs, const double *__restrict__ ys, const double *__restrict__ zs,
               const double *__restrict__ qm, int n, const double *__restrict__ root, float theta, float eps2,
               BhImages im, double *__restrict__ ax, double *__restrict__ ay, double *__restrict__ az,
               unsigned long long *__restrict__ counts) {
    // cell side of every level, from the root cube on the device
    __shared__ float side[kMortonBits + 1];
    if (threadIdx.x <= T.deepest) side[threadIdx.x] = (float)(root[3] / (double)(1ll << threadIdx.x));
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int half = lane / TPW;  // 0, or 1 for the upper half-warp when TPW = 16
    const int i = (blockIdx.x * kBhWarps + wid) * TPW + lane % TPW;
    const bool live = i < n && qm[i] != 0.0;
    const unsigned live_mask = __ballot_sync(0xffffffffu, live);
    if (live_mask == 0) return;
    const int ii = i < n ? i : n - 1;
    const double px = xs[ii], py = ys[ii], pz = zs[ii];
    float sx = 0.f, sy = 0.f, sz = 0.f;
    unsigned long long n_cells = 0, n_pairs = 0;
    for (int g = 0; g < im.count; g++) {
        // target position in this image's frame, and the force rotation back
        double tx = px, ty = py, tz = pz;
        int cb = 1, sb = 0;
        bool self_excl = true;
        if (im.kind == 1) {
            // quadrant g: target rotated by -g*pi/2, force rotated by +g*pi/2
            const int cf = (g == 0) ? 1 : (g == 2 ? -1 : 0);
            const int sf = (g == 1) ? -1 : (g == 3 ? 1 : 0);
            tx = cf * px - sf * py;
            ty = sf * px + cf * py;
            cb = cf;
            sb = -sf;
            self_excl = g == 0;
        } else if (im.kind == 2) {
            tx = px - im.off[3 * g];
            ty = py - im.off[3 * g + 1];
            tz = pz - im.off[3 * g + 2];
            self_excl = im.off[3 * g] == 0.0 && im.off[3 * g + 1] == 0.0 && im.off[3 * g + 2] == 0.0;
        }
        float thx, tlx, thy, tly, thz, tlz;
        split_hilo(tx - root[0], thx, tlx);
        split_hilo(ty - root[1], thy, tly);
        split_hilo(tz - root[2], thz, tlz);
        float fx = 0.f, fy = 0.f, fz = 0.f;
        unsigned want = 0;  // bit l: this lane rejected the current cell's ancestor at level l
        int node = cell_id(0, 0);
        while (node != kEnd) {
            const int lvl = node >> 24, b = node & 0xffffff;
            // taking part: the root for every live target, else the lanes that rejected the parent
            const bool mine = lvl == 0 ? live : ((want >> (lvl - 1)) & 1u) != 0;
            // everything the cell's visit may need, loaded together: one memory
            // latency per cell instead of a chain of three
            const float4 h = T.nh[lvl][b], lo = T.nl[lvl][b];
            const int s0 = T.start[lvl][b], s1 = T.start[lvl][b + 1];
            const int child = lvl < T.deepest ? T.child0[lvl][b] : 0, skip = T.skip[lvl][b];
            bool deeper = false, rej = false;
            if (__any_sync(0xffffffffu, mine)) {
                const float dx = (thx - h.x) + (tlx - lo.x), dy = (thy - h.y) + (tly - lo.y),
                            dz = (thz - h.z) + (tlz - lo.z);
                const float d = sqrtf(fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, eps2))));
                const bool acc = mine && theta * (d - lo.w) > side[lvl];
                if (acc && half == 0) {
                    const float f = h.w / (d * d * d);
                    fx = fmaf(f, dx, fx);
                    fy = fmaf(f, dy, fy);
                    fz = fmaf(f, dz, fz);
                    n_cells++;
                }
                rej = mine && !acc;
                if (__any_sync(0xffffffffu, rej)) {
                    const bool leaf = lvl == T.deepest || (s1 - s0) <= T.leaf_size;
                    if (leaf) {
#pragma unroll 4
                        for (int j = s0 + half; j < s1; j += 32 / TPW) {
                            const float4 qh = ph[j], ql = pl[j];
                            if (rej && !(self_excl && j == i)) {
                                const float ex = (thx - qh.x) + (tlx - ql.x), ey = (thy - qh.y) + (tly - ql.y),
                                            ez = (thz - qh.z) + (tlz - ql.z);
                                const float dd = sqrtf(fmaf(ex, ex, fmaf(ey, ey, fmaf(ez, ez, eps2))));
                                const float f = qh.w / (dd * dd * dd);
                                fx = fmaf(f, ex, fx);
                                fy = fmaf(f, ey, fy);
                                fz = fmaf(f, ez, fz);
                                n_pairs++;
                            }
                        }
                    } else {
                        deeper = true;  // warp-uniform: the cell is internal and some lane rejected it
                    }
                }
            }
            // bit lvl: this lane goes below this cell (it rejected an internal cell)
            want = (deeper && rej) ? (want | (1u << lvl)) : (want & ~(1u << lvl));
            node = deeper ? cell_id(lvl + 1, child) : skip;
        }
        sx += (float)cb * fx - (float)sb * fy;
        sy += (float)sb * fx + (float)cb * fy;
        sz += fz;
    }
    if (TPW == 16) {
        sx += __shfl_xor_sync(0xffffffffu, sx, 16);
        sy += __shfl_xor_sync(0xffffffffu, sy, 16);
        sz += __shfl_xor_sync(0xffffffffu, sz, 16);
    }
    if (half == 0 && live) {
        const double c = qm[i];
        ax[i] = (double)sx * c;
        ay[i] = (double)sy * c;
        az[i] = (double)sz * c;
    } else if (half == 0 && i < n) {
        ax[i] = ay[i] = az[i] = 0.0;
    }
    for (int o = 16; o > 0; o >>= 1) {
        n_cells += __shfl_xor_sync(0xffffffffu, n_cells, o);
        n_pairs += __shfl_xor_sync(0xffffffffu, n_pairs, o);
    }
    if (lane == 0) {
        atomicAdd(&counts[0], n_cells);
        atomicAdd(&counts[1], n_pairs);
    }
}

}  // namespace

sv_status bh_accel(sv_ctx *c) {
    if (c->P.precision != SV_PREC_MIXED)
        return set_error(c, SV_ERR_UNSUPPORTED, "Barnes-Hut runs in mixed precision only");
    if (!c->bh) {
        c->bh = new Bh();
        SV_CK(c, cudaMalloc(&c->bh->d_counts, 2 * sizeof(unsigned long long)));
        SV_CK(c, cudaMallocHost(&c->bh->h_counts, 2 * sizeof(unsigned long long)));
    }
    Bh &B = *c->bh;
    const int n = (int)c->S.n;
    Sorted &S = c->S;
    Tree *Tp = nullptr;
    c->S.resort = false;
    SV_TRY(tree_build(c, kDepthAllSplit, c->P.leaf_size, &Tp));
    Tree &T = *Tp;
    // the splits are exact down to the sorted levels only; a tree reaching
    // them needs the full order
    if (T.n_act > 0 && T.deepest >= S.key_levels && S.key_levels < kMortonBits) {
        c->S.resort = true;
        return SV_OK;
    }
    phase_mark(c, 2);
    phase_mark(c, 3);
    if (T.n_act == 0) {
        SV_CK(c, cudaMemsetAsync(S.ax, 0, sizeof(double) * n, c->stream));
        SV_CK(c, cudaMemsetAsync(S.ay, 0, sizeof(double) * n, c->stream));
        SV_CK(c, cudaMemsetAsync(S.az, 0, sizeof(double) * n, c->stream));
        return SV_OK;
    }
    const int D = T.deepest;
    B.level_hint = D;
    // storage: per level Q, U (double), coc (double3), nh, nl (float4), skip links (int)
    auto rounded = [](size_t sz) { return (sz + 255) & ~(size_t)255; };
    size_t bytes = 0;
    for (int l = 0; l <= D; l++) {
        const size_t nb = T.lv[l].nbox;
        bytes += 2 * rounded(nb * sizeof(double)) + rounded(nb * sizeof(double3)) + 2 * rounded(nb * sizeof(float4)) +
                 rounded(nb * sizeof(int));
    }
    if (B.arena_bytes < bytes) {
        cudaFree(B.arena);
        B.arena = nullptr;
        B.arena_bytes = 0;
        const size_t want = bytes + bytes / 2;  // headroom: a growing tree reallocates rarely
        SV_CK(c, cudaMalloc(&B.arena, want));
        B.arena_bytes = want;
    }
    if (B.pcap < n) {
        cudaFree(B.ph);
        cudaFree(B.pl);
        B.ph = B.pl = nullptr;
        SV_CK(c, cudaMalloc(&B.ph, sizeof(float4) * n));
        SV_CK(c, cudaMalloc(&B.pl, sizeof(float4) * n));
        B.pcap = n;
    }
    char *p = (char *)B.arena;
    auto carve = [&](size_t sz) {
        char *r = p;
        p += rounded(sz);
        return (void *)r;
    };
    double *Q[kMortonBits + 1], *U[kMortonBits + 1];
    double3 *coc[kMortonBits + 1];
    BhLevels L{};
    SkipArgs sk{};
    sk.D = D;
    for (int l = 0; l <= D; l++) {
        const size_t nb = T.lv[l].nbox;
        Q[l] = (double *)carve(nb * sizeof(double));
        U[l] = (double *)carve(nb * sizeof(double));
        coc[l] = (double3 *)carve(nb * sizeof(double3));
        L.nh[l] = (const float4 *)carve(nb * sizeof(float4));
        L.nl[l] = (const float4 *)carve(nb * sizeof(float4));
        L.child0[l] = T.lv[l].child0;
        L.start[l] = T.lv[l].start;
        sk.skip[l] = (int *)carve(nb * sizeof(int));
        L.skip[l] = sk.skip[l];
        sk.parent[l] = T.lv[l].parent;
        sk.nbox[l] = (int)nb;
        sk.first[l + 1] = sk.first[l] + (int)nb;
    }
    skip_links_kernel<<<div_up(sk.first[D + 1], 256), 256, 0, c->stream>>>(sk);
    SV_LAUNCHED(c);
    L.deepest = D;
    L.leaf_size = c->P.leaf_size;
    particles_hilo<<<div_up(T.n_act, 256), 256, 0, c->stream>>>(S.x, S.y, S.z, S.q, T.n_act, S.root, B.ph, B.pl);
    SV_LAUNCHED(c);
    {
        const Level &V = T.lv[D];
        props_from_particles<<<div_up(V.nbox, 128), 128, 0, c->stream>>>(
            V.nbox, V.start, V.coord, S.x, S.y, S.z, S.q, S.root, D, Q[D], U[D], coc[D], (float4 *)L.nh[D],
            (float4 *)L.nl[D]);
        SV_LAUNCHED(c);
    }
    {
        PropLevels pl{};
        for (int l = 0; l <= D; l++)
            pl.lv[l] = PropLevel{T.lv[l].nbox, T.lv[l].child0, T.lv[l].coord, Q[l], U[l], coc[l],
                                 (float4 *)L.nh[l], (float4 *)L.nl[l]};
        // the coarse levels (every level above holding at most kCoarseBoxes boxes) in one launch
        constexpr int kCoarseBoxes = 1024;
        int top = -1;
        while (top + 1 < D && T.lv[top + 1].nbox <= kCoarseBoxes) top++;
        for (int l = D - 1; l > top; l--) {
            props_from_children<<<div_up(T.lv[l].nbox, 128), 128, 0, c->stream>>>(l, S.root, pl.lv[l + 1], pl.lv[l]);
            SV_LAUNCHED(c);
        }
        if (top >= 0) {
            props_coarse_levels<<<1, kCoarseBoxes, 0, c->stream>>>(top, S.root, pl);
            SV_LAUNCHED(c);
        }
    }
    phase_mark(c, 4);
    phase_mark(c, 5);
    BhImages im{0, 1, nullptr};
    double *d_off = nullptr;
    if (c->P.symmetry == SV_SYM_ROTATIONAL) {
        im.kind = 1;
        im.count = 4;
    } else if (c->P.symmetry == SV_SYM_TRANSLATIONAL) {
        static thread_local double h_off[3 * 4096];
        const int cnt = trans_images(c->P, h_off, 4096);
        if (cnt <= 0 || cnt > 4096) return set_error(c, SV_ERR_INVALID, "bad translational image set (%d)", cnt);
        SV_CK(c, cudaMallocAsync(&d_off, sizeof(double) * 3 * cnt, c->stream));
        SV_CK(c, cudaMemcpyAsync(d_off, h_off, sizeof(double) * 3 * cnt, cudaMemcpyHostToDevice, c->stream));
        im.kind = 2;
        im.count = cnt;
        im.off = d_off;
    }
    SV_CK(c, cudaMemsetAsync(B.d_counts, 0, 2 * sizeof(unsigned long long), c->stream));
    // inactive sorted slots (beyond n_act) are never targets (qm = 0)
    // half-warp targets while 32 per warp would leave fewer than kBhHalfWarps warps per SM
    if (div_up(n, 32) < kBhHalfWarps * device_sms())
        bh_walk_kernel<16><<<div_up(n, 16 * kBhWarps), 32 * kBhWarps, 0, c->stream>>>(
            L, B.ph, B.pl, S.x, S.y, S.z, S.qm, T.n_act, S.root, c->P.theta, (float)c->P.softening2, im, S.ax, S.ay,
            S.az, B.d_counts);
    else
        bh_walk_kernel<32><<<div_up(n, 32 * kBhWarps), 32 * kBhWarps, 0, c->stream>>>(
            L, B.ph, B.pl, S.x, S.y, S.z, S.qm, T.n_act, S.root, c->P.theta, (float)c->P.softening2, im, S.ax, S.ay,
            S.az, B.d_counts);
    SV_LAUNCHED(c);
    if (T.n_act < n) {
        SV_CK(c, cudaMemsetAsync(S.ax + T.n_act, 0, sizeof(double) * (n - T.n_act), c->stream));
        SV_CK(c, cudaMemsetAsync(S.ay + T.n_act, 0, sizeof(double) * (n - T.n_act), c->stream));
        SV_CK(c, cudaMemsetAsync(S.az + T.n_act, 0, sizeof(double) * (n - T.n_act), c->stream));
    }
    phase_mark(c, 6);
    if (d_off) SV_CK(c, cudaFreeAsync(d_off, c->stream));
    // the counts reach the host with the stream; bh_counts reads them
    SV_CK(c, cudaMemcpyAsync(B.h_counts, B.d_counts, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                             c->stream));
    c->stats.levels = D;
    c->stats.boxes = 0;
    for (int l = 0; l <= D; l++) c->stats.boxes += T.lv[l].nbox;
    return SV_OK;
}

int bh_sort_levels(const sv_ctx *c) {
    const int h = c->bh ? c->bh->level_hint : -1;
    return h >= 1 ? std::min(kMortonBits, h + 2) : kMortonBits;
}

sv_status bh_counts(sv_ctx *c, double *cells, double *pairs) {
    if (!c->bh) {
        *cells = *pairs = 0;
        return SV_OK;
    }
    SV_CK(c, cudaStreamSynchronize(c->stream));
    *cells = (double)c->bh->h_counts[0];
    *pairs = (double)c->bh->h_counts[1];
    return SV_OK;
}

void bh_free(sv_ctx *c) {
    if (!c->bh) return;
    Bh &B = *c->bh;
    cudaFree(B.arena);
    cudaFree(B.ph);
    cudaFree(B.pl);
    cudaFree(B.d_counts);
    cudaFreeHost(B.h_counts);
    delete c->bh;
    c->bh = nullptr;
}

}  // namespace sv
