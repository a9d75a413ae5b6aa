// fmm.cu -- rotation-based fast multipole method on GB300.
//
// Restates MultipoleMethodForceCalculation::updateAccelerationNoSym
// (multipole_method_force_calculation.cpp:184-522) and its kernels
// (fmm_cpukernel.cpp: p2m_kernel :281-384, m2m_kernel :513-619, m2l_kernel
// :742-909 with rotation() :10-32, l2l_kernel :1050-1126, l2p_kernel
// :1188-1317, p2p_kernel :194-219) on the level-by-level octree of tree.cu:
//
//   P2M   leaf boxes, one warp per box, lanes over particles, then over
//         coefficients (shared-memory transpose).
//   M2M   one warp per parent, lanes over the parent's coefficients, children
//         added in turn (no mutex: one writer per parent).
//   lists per level, one thread per box: the children of the parent's
//         neighbours split into near boxes (|offset| <= ws) and the M2L list
//         (offset class = integer offset target - source).
//   down  one warp per box and level: L2L from the parent, then every M2L of
//         the box's list (phase, folded y-rotation, z-translation, inverse
//         rotation, inverse phase), accumulated in registers, written once.
//   L2P   leaf boxes, lanes over particles: gradient of the local expansion.
//   P2P   leaf boxes, lanes over targets, source chunks staged in shared
//         memory as FP32 offsets from the target box centre (FP64 subtraction
//         once per staged source); a box's short tail chunk of targets spreads
//         each target over a group of lanes that split the sources; per-source-
//         box FP32 partial sums are accumulated with Kahan compensation.
//
// Expansions are kept in box units (coordinates divided by the box side h),
// so the M2L tables depend on the integer offset only; the softened M2L
// distance rho^2 = |offset|^2 + eps^2/h^2 follows fmm_cpukernel.cpp:832.
// ws (well-separation) 1 is the reference's interaction list
// (multipole_method_force_calculation.cpp:2021-2114); ws 2 widens the near
// field to 5x5x5 boxes, which is what brings p = 8 under 1e-5 force error.
#include <cfloat>

#include <algorithm>
#include <string>
#include <vector>

#include "fmm_tables.h"
#include "forest.cuh"
#include "m2l_tc.cuh"
#include "sv_internal.cuh"
#include "tree.cuh"

namespace sv {

struct Fmm {
    int p = 0, ws = 0;
    int trim = 0;  // trimmed near field (sv_params.fmm_near = 2 at ws = 2) for the next evaluation
    FmmTables H;
    int *cls_theta = nullptr;
    float2 *cls_phase = nullptr;
    float *cls_rho2 = nullptr;
    float *dmat = nullptr;
    float *zc = nullptr;
    float *nrm = nullptr;
    float *otab = nullptr;   // rotation-based M2M / L2L tables (oct_layout)
    void *arena = nullptr;
    size_t arena_bytes = 0;
    unsigned long long *d_counts = nullptr;  // [0] M2L translations, [1] P2P pairs, [2] charges differ
    unsigned long long *h_counts = nullptr;
    // caller particles followed by their source-only symmetry images
    double *ex = nullptr, *ey = nullptr, *ez = nullptr, *eq = nullptr, *em = nullptr, *eoff = nullptr;
    int32_t *est = nullptr;
    int64_t ecap = 0;
    int eoff_cap = 0;
    int *has_tgt = nullptr;  // per box of every level: box holds a target
    int64_t tgt_cap = 0;
    float4 *rel = nullptr;   // particle offset from its leaf box centre (FP32) + charge
    int64_t rel_cap = 0;
    double *far = nullptr;   // far-field acceleration (L2P / M2P), 3 x rel_cap, added in the scatter
    int level_hint = -1;     // leaf level of the last evaluation (the next sort orders one level more)
    // forest (batched plumes): tree and per-level arrays carved at reserve time
    Tree *ftree = nullptr;
    void *farena = nullptr;
    size_t farena_bytes = 0;
    float2 *fM[kMortonBits + 1] = {}, *fL[kMortonBits + 1] = {}, *fpart[kMortonBits + 1] = {};
    int fchunks[kMortonBits + 1] = {};
    int *fnbr[kMortonBits + 1] = {}, *fcnt[kMortonBits + 1] = {}, *ftgt[kMortonBits + 1] = {};
    int2 *flst[kMortonBits + 1] = {};
    int *ffd = nullptr, *ffd_cnt = nullptr;  // far-direct lists of the forest's leaf boxes
    float4 *frel = nullptr;
    int64_t frel_cap = 0;
    // the near field runs on its own stream beside the upward and downward passes
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_lists = nullptr, ev_join = nullptr, ev_near[2] = {};
    cudaEvent_t ev_rel = nullptr;  // the second stream's leaf offsets (F.rel) are written
    cudaEvent_t ev_m2l_lists = nullptr;  // single plume: near, interaction and far-direct lists built (second stream)
    M2LTc tc;                // the M2L on the tensor cores (m2l_tc.cu)
};

namespace {

constexpr int kWarps = 4;  // warps per CTA in the per-box kernels

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }

__host__ __device__ constexpr int ncoef(int P) { return P * (P + 1) / 2; }
__device__ __forceinline__ int cidx(int n, int m) { return n * (n + 1) / 2 + m; }
__device__ __forceinline__ void cnm(int c, int &n, int &m) {
    n = 0;
    while ((n + 1) * (n + 2) / 2 <= c) n++;
    m = c - n * (n + 1) / 2;
}

// Regular solid harmonics R_n^m(x), m >= 0, n < P (Cartesian recurrences):
// R_m^m = (x+iy)/(2m) R_{m-1}^{m-1}; R_{m+1}^m = z R_m^m;
// R_n^m = ((2n-1) z R_{n-1}^m - r^2 R_{n-2}^m) / ((n+m)(n-m)).
template <int P>
__device__ __forceinline__ void solid_harmonics(float x, float y, float z, float2 *R) {
    const float r2 = x * x + y * y + z * z;
    R[0] = make_float2(1.f, 0.f);
#pragma unroll
    for (int m = 0; m < P; m++) {
        if (m > 0) {
            const float2 prev = R[cidx(m - 1, m - 1)];
            const float s = 1.f / (2.f * m);
            R[cidx(m, m)] = make_float2((x * prev.x - y * prev.y) * s, (x * prev.y + y * prev.x) * s);
        }
        if (m + 1 < P) R[cidx(m + 1, m)] = cscale(R[cidx(m, m)], z);
#pragma unroll
        for (int n = m + 2; n < P; n++) {
            const float a = (2.f * n - 1.f) * z, d = 1.f / ((n + m) * (n - m));
            const float2 r1 = R[cidx(n - 1, m)], r0 = R[cidx(n - 2, m)];
            R[cidx(n, m)] = make_float2((a * r1.x - r2 * r0.x) * d, (a * r1.y - r2 * r0.y) * d);
        }
    }
}

// Box count of a level: the launch bound nbox, or (forest) the device count.
__device__ __forceinline__ int level_boxes(int nbox, const int *nbd) { return nbd ? min(nbox, *nbd) : nbox; }
// Root record (origin xyz, cube side) of the plume that owns box b.
__device__ __forceinline__ const double *box_root(const double *root, const int *bpid, int b) {
    return bpid ? root + 8 * bpid[b] : root;
}
// First box and stride of the calling warp in a warp-per-box kernel.
#define SV_WARP_BOXES(W) \
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5; \
    const int nb_ = level_boxes(nbox, nbd); \
    for (int b = blockIdx.x * (W) + wid; b < nb_; b += gridDim.x * (W))

// ---------------------------------------------------------------- lists --
// Lists of one box b (coordinates cb, parent par) from its parent's near list
// pnbr: the children of each of the parent's near boxes are classified round
// by round (lanes take the parent's near slots) into the near list (|offset|
// <= WS, written when write_near) and the interaction list (M2L entries
// compacted by ballot).  trim: the trimmed near field of WS = 2, whose
// (2,2,1)- and (2,2,2)-type offsets are interaction-list entries instead
// (fmm_trimmable); the near boxes of a box always have parents at offsets in
// [-1, 1]^3 from its parent, which trimming never removes, so every pair is
// still counted once.  Returns the box's M2L count.
//
// Far-direct lists (fd non-null, the leaf level of a single tree): an
// interaction-list entry whose two boxes hold fewer than fd_thresh particles
// multiplied is cheaper as direct pairs than as an M2L translation; up to
// fd_cap of them per box go to fd (summed by the near field), the rest stay
// M2L entries.
template <int WS>
__device__ __forceinline__ int build_lists_box(int b, int4 cb, int par, const int4 *__restrict__ coord,
                                               const int *__restrict__ pnbr, const int *__restrict__ pchild0,
                                               int *__restrict__ nbr, int2 *__restrict__ m2l,
                                               int *__restrict__ m2l_cnt, int cap, int write_near, int trim,
                                               const int *__restrict__ start = nullptr, int *__restrict__ fd = nullptr,
                                               int *__restrict__ fd_cnt = nullptr, int fd_cap = 0,
                                               int fd_thresh = 0) {
    constexpr int NS1 = 2 * WS + 1, NS = NS1 * NS1 * NS1, R = 2 * WS + 1, SIDE = 2 * R + 1;
    const int lane = threadIdx.x & 31;
    const unsigned lt_mask = (1u << lane) - 1u;
    if (write_near)
        for (int s = lane; s < NS; s += 32) nbr[b * NS + s] = -1;
    __syncwarp();
    const long long nt = fd ? (long long)(start[b + 1] - start[b]) : 0;
    int cnt = 0, dcnt = 0;
    for (int s0 = 0; s0 < NS; s0 += 32) {
        const int s = s0 + lane;
        int c0 = 0, c1 = 0;
        if (s < NS) {
            const int Q = pnbr[par * NS + s];
            if (Q >= 0) {
                c0 = pchild0[Q];
                c1 = pchild0[Q + 1];
            }
        }
        for (int r = 0; r < 8; r++) {
            const int ch = c0 + r;
            bool far = false;
            int cls = 0;
            if (ch < c1) {
                const int4 cc = coord[ch];
                const int ox = cb.x - cc.x, oy = cb.y - cc.y, oz = cb.z - cc.z;
                const int am = max(abs(ox), max(abs(oy), abs(oz)));
                // a consistent tree keeps |offset| <= R; a forest level clamped to
                // its capacity may not, and its result is discarded, but the class
                // index must stay inside the tables
                if (am <= WS && !(trim && fmm_trimmable(ox, oy, oz, WS))) {
                    if (write_near) nbr[b * NS + ((ox + WS) * NS1 + (oy + WS)) * NS1 + (oz + WS)] = ch;
                } else if (am <= R) {
                    far = true;
                    cls = ((ox + R) * SIDE + (oy + R)) * SIDE + (oz + R);
                }
            }
            if (fd) {
                const bool dir = far && (long long)(start[ch + 1] - start[ch]) * nt < (long long)fd_thresh;
                const unsigned bd = __ballot_sync(0xffffffffu, dir);
                if (dir) {
                    const int pos = dcnt + __popc(bd & lt_mask);
                    if (pos < fd_cap) {
                        fd[(size_t)b * fd_cap + pos] = ch;
                        far = false;
                    }
                }
                dcnt += __popc(bd);
            }
            const unsigned bal = __ballot_sync(0xffffffffu, far);
            if (far) {
                const int pos = cnt + __popc(bal & lt_mask);
                if (pos < cap) m2l[(size_t)b * cap + pos] = make_int2(ch, cls);
            }
            cnt += __popc(bal);
            if (!__any_sync(0xffffffffu, ch + 1 < c1)) break;
        }
    }
    if (cnt > cap) cnt = cap;
    if (lane == 0) {
        m2l_cnt[b] = cnt;
        if (fd) fd_cnt[b] = dcnt < fd_cap ? dcnt : fd_cap;
    }
    return cnt;
}

// One level of a forest, one warp per box.
template <int WS>
__global__ void __launch_bounds__(kWarps * 32)
build_lists_kernel(int nbox, const int *__restrict__ nbd, const int *__restrict__ parent,
                   const int4 *__restrict__ coord, const int *__restrict__ pnbr, const int *__restrict__ pchild0,
                   int *__restrict__ nbr, int2 *__restrict__ m2l, int *__restrict__ m2l_cnt, int cap, int trim,
                   unsigned long long *__restrict__ counts, const int *__restrict__ start = nullptr,
                   int *__restrict__ fd = nullptr, int *__restrict__ fd_cnt = nullptr, int fd_cap = 0,
                   int fd_thresh = 0) {
    unsigned long long tot = 0;
    SV_WARP_BOXES(kWarps) {
    const int cnt = build_lists_box<WS>(b, coord[b], parent[b], coord, pnbr, pchild0, nbr, m2l, m2l_cnt, cap, 1,
                                        trim, start, fd, fd_cnt, fd_cap, fd_thresh);
    if (lane == 0) tot += cnt;
    }
    if ((threadIdx.x & 31) == 0 && tot) atomicAdd(&counts[0], tot);
}

// The levels of one tree for the list builders that take all levels in one
// launch: level l's boxes are global indices [first, first + nbox).
struct ListLevel {
    int nbox, first;
    const int4 *coord;
    uint64_t *code;          // box Morton codes at this level (ascending)
    int *nbr;                // near lists [nbox][NS]
    const int *parent;       // box -> parent box at level - 1
    const int *pchild0;      // the parent level's child ranges
    const int *pnbr;         // the parent level's near lists
    int2 *m2l;
    int *m2l_cnt;
    const int *start;        // particle ranges of this level's boxes
    int *fd, *fd_cnt;        // far-direct lists (the leaf level only, else null)
};
struct ListArgs {
    int nlev, total;         // levels 0 .. nlev - 1; boxes of all of them
    int fd_cap, fd_thresh;   // far-direct list capacity per box and pair threshold
    int trim;                // trimmed near field (build_lists_box)
    ListLevel lv[kMortonBits + 1];
};

__device__ __forceinline__ int list_level(const ListArgs &a, int g) {
    int l = 0;
    while (l + 1 < a.nlev && g >= a.lv[l + 1].first) l++;
    return l;
}

__device__ __forceinline__ uint64_t box_code(int x, int y, int z) {
    return morton_spread3((uint32_t)x) | (morton_spread3((uint32_t)y) << 1) | (morton_spread3((uint32_t)z) << 2);
}

// Morton code of every box of every level (a level's boxes are in ascending
// code order)
__global__ void box_codes_kernel(ListArgs a) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= a.total) return;
    const ListLevel &L = a.lv[list_level(a, g)];
    const int b = g - L.first;
    const int4 c = L.coord[b];
    L.code[b] = box_code(c.x, c.y, c.z);
}

// Near lists of every level straight from the boxes (one thread per box and
// slot): the box at target - offset, found by binary search over the level's
// codes, or -1; build_lists_box's layout, without a chain of coarser levels in
// front of it.
template <int WS>
__global__ void near_lists_kernel(ListArgs a) {
    constexpr int NS1 = 2 * WS + 1, NS = NS1 * NS1 * NS1;
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= (int64_t)a.total * NS) return;
    const int g = (int)(t / NS), s = (int)(t - (int64_t)g * NS);
    const int l = list_level(a, g);
    const ListLevel &L = a.lv[l];
    const int b = g - L.first;
    const int ox = s / (NS1 * NS1) - WS, oy = (s / NS1) % NS1 - WS, oz = s % NS1 - WS;
    const int4 cb = L.coord[b];
    const int x = cb.x - ox, y = cb.y - oy, z = cb.z - oz, side = 1 << l;
    int found = -1;
    if (x >= 0 && y >= 0 && z >= 0 && x < side && y < side && z < side && !(a.trim && fmm_trimmable(ox, oy, oz, WS))) {
        const uint64_t key = box_code(x, y, z);
        int lo = 0, hi = L.nbox - 1;
        while (lo <= hi) {
            const int mid = (lo + hi) >> 1;
            const uint64_t cm = L.code[mid];
            if (cm == key) {
                found = mid;
                break;
            }
            if (cm < key) lo = mid + 1;
            else hi = mid - 1;
        }
    }
    L.nbr[(size_t)b * NS + s] = found;
}

// Interaction lists of levels 1 .. nlev - 1, one warp per box, from the near
// lists near_lists_kernel wrote
template <int WS>
__global__ void __launch_bounds__(kWarps * 32) m2l_lists_kernel(ListArgs a, int cap,
                                                                unsigned long long *__restrict__ counts) {
    unsigned long long tot = 0;
    const int lane = threadIdx.x & 31;
    const int first = a.nlev > 1 ? a.lv[1].first : a.total;
    for (int g = first + blockIdx.x * kWarps + (int)(threadIdx.x >> 5); g < a.total; g += gridDim.x * kWarps) {
        const ListLevel &L = a.lv[list_level(a, g)];
        const int b = g - L.first;
        const int cnt = build_lists_box<WS>(b, L.coord[b], L.parent[b], L.coord, L.pnbr, L.pchild0, L.nbr, L.m2l,
                                            L.m2l_cnt, cap, 0, a.trim, L.start, L.fd, L.fd_cnt, a.fd_cap,
                                            a.fd_thresh);
        if (lane == 0) tot += cnt;
    }
    if (lane == 0 && tot) atomicAdd(&counts[0], tot);
}

// Near list of every root: the root itself only (plumes never interact).
__global__ void root_nbr_kernel(int *nbr, int ns, int nroots, const int *__restrict__ nbd) {
    const int nr = level_boxes(nroots, nbd);
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nr * ns; t += gridDim.x * blockDim.x) {
        const int b = t / ns, s = t - b * ns;
        nbr[t] = s == ns / 2 ? b : -1;
    }
}

// ------------------------------------------------------ symmetry images --
// Image g of particle i at slot g*n + i: g = 0 is the particle itself; the
// others are source-only copies (status 2) rotated by g*pi/2 about z
// (rotational variant) or shifted by offset g (translational variant, zero
// offset first).  Sources of status 1 or 2 keep being sources in every image;
// ignored particles (0, -1) stay ignored.
__global__ void expand_images_kernel(const double *__restrict__ x, const double *__restrict__ y,
                                     const double *__restrict__ z, const double *__restrict__ q,
                                     const double *__restrict__ m, const int32_t *__restrict__ st, int64_t n,
                                     int kind, int nimg, const double *__restrict__ off, double *__restrict__ ex,
                                     double *__restrict__ ey, double *__restrict__ ez, double *__restrict__ eq,
                                     double *__restrict__ em, int32_t *__restrict__ est) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= n * nimg) return;
    const int g = (int)(t / n);
    const int64_t i = t - (int64_t)g * n;
    double px = x[i], py = y[i], pz = z[i];
    if (kind == 1) {
        const double x0 = px, y0 = py;
        if (g == 1) { px = -y0; py = x0; }
        else if (g == 2) { px = -x0; py = -y0; }
        else if (g == 3) { px = y0; py = -x0; }
    } else if (kind == 2) {
        px += off[3 * g];
        py += off[3 * g + 1];
        pz += off[3 * g + 2];
    }
    ex[t] = px;
    ey[t] = py;
    ez[t] = pz;
    eq[t] = q[i];
    em[t] = m[i];
    const int32_t w = st[i];
    est[t] = g == 0 ? w : ((w == 1 || w == 2) ? 2 : w);
}

// box holds at least one target (K q/m != 0): leaf level from particles,
// coarser levels from children
__global__ void leaf_targets_kernel(int nbox, const int *__restrict__ nbd, const int *__restrict__ start,
                                    const double *__restrict__ qm, int *__restrict__ flag) {
    const int nb = level_boxes(nbox, nbd);
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += gridDim.x * blockDim.x) {
        int f = 0;
        for (int j = start[b]; j < start[b + 1] && !f; j++) f = qm[j] != 0.0;
        flag[b] = f;
    }
}

__global__ void parent_targets_kernel(int nbox, const int *__restrict__ nbd, const int *__restrict__ child0,
                                      const int *__restrict__ cflag, int *__restrict__ flag) {
    const int nb = level_boxes(nbox, nbd);
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += gridDim.x * blockDim.x) {
        int f = 0;
        for (int c = child0[b]; c < child0[b + 1] && !f; c++) f = cflag[c];
        flag[b] = f;
    }
}

// ------------------------------------------------------------------ P2M --
template <int P>
constexpr int p2m_warps() { return P >= 9 ? 2 : 4; }

template <int P>
__global__ void __launch_bounds__(p2m_warps<P>() * 32)
p2m_kernel(int nbox, const int *__restrict__ nbd, const int *__restrict__ bpid, const int *__restrict__ start,
           const int4 *__restrict__ coord, const double *__restrict__ xs, const double *__restrict__ ys,
           const double *__restrict__ zs, const float *__restrict__ qs, const double *__restrict__ roots, int level,
           const float *__restrict__ nrm, float2 *__restrict__ M) {
    constexpr int NC = ncoef(P), WP = p2m_warps<P>();
    __shared__ float2 buf[WP][32][NC + 1];
    SV_WARP_BOXES(WP) {
    const double *root = box_root(roots, bpid, b);
    const double h = root[3] / (double)(1 << level);
    const int4 cb = coord[b];
    const double cx = root[0] + (cb.x + 0.5) * h, cy = root[1] + (cb.y + 0.5) * h, cz = root[2] + (cb.z + 0.5) * h;
    // the offset in FP64 (positions are large), its scaling in FP32: the FP64
    // pipe runs at 1/64 of the FP32 rate on this GPU
    const float ihf = (float)(1.0 / h);
    float2 a0 = make_float2(0.f, 0.f), a1 = make_float2(0.f, 0.f);
    const int s0 = start[b], s1 = start[b + 1];
    for (int base = s0; base < s1; base += 32) {
        const int i = base + lane;
        float2 R[NC];
        if (i < s1) {
            solid_harmonics<P>((float)(xs[i] - cx) * ihf, (float)(ys[i] - cy) * ihf, (float)(zs[i] - cz) * ihf, R);
            const float q = qs[i];
#pragma unroll
            for (int c = 0; c < NC; c++) buf[wid][lane][c] = make_float2(q * R[c].x, -q * R[c].y);
        } else {
#pragma unroll
            for (int c = 0; c < NC; c++) buf[wid][lane][c] = make_float2(0.f, 0.f);
        }
        __syncwarp();
        const int rows = min(32, s1 - base);
        for (int r = 0; r < rows && lane < NC; r++) {
            a0 = cadd(a0, buf[wid][r][lane]);
            if (lane + 32 < NC) a1 = cadd(a1, buf[wid][r][lane + 32]);
        }
        __syncwarp();
    }
    if (lane < NC) {
        int n, m;
        cnm(lane, n, m);
        M[(size_t)b * NC + lane] = cscale(a0, nrm[n * P + m]);
        if (lane + 32 < NC) {
            cnm(lane + 32, n, m);
            M[(size_t)b * NC + lane + 32] = cscale(a1, nrm[n * P + m]);
        }
    }
    __syncwarp();
    }
}

// ------------------------------------------------------------------ M2M --
// (defined after the rotation helpers below)
// ----------------------------------------------------------- downward --
// M2L of every level in one launch, then L2L level by level.  A level with few
// boxes (the coarse ones, whose lists are long) splits each box's list over
// `chunks` warps; the chunks' partial sums are kept apart and added in order by
// the L2L pass, so the result does not depend on scheduling.
struct M2LLevel {
    int nbox;             // launch bound: boxes, or the forest capacity
    int chunks;           // warps per box
    int warp0;            // first global warp of the level
    int level;
    const int *nbd;       // device box count (forest) or null
    const int *bpid;      // plume of each box (forest) or null
    const int2 *m2l;
    const int *cnt;
    const int *has_tgt;   // boxes without targets need no local expansion
    const float2 *M;      // multipoles of the level
    float2 *out;          // [box][chunk][coefficient]; with one chunk the level's local expansions
};

struct M2LArgs {
    const int *run_if;    // non-null: run only when *run_if != 0 (the tensor-core M2L overflowed its room)
    int nlev, cap, esz, osz, dsz;
    double eps2;
    const double *root;
    const int *cls_theta;
    const float2 *cls_phase;
    const float *cls_rho2;
    const float *dmat;
    const float *zc;
    M2LLevel lv[kMortonBits + 1];
};

struct L2LArgs {
    int nbox, chunks, has_parent;
    const int *nbd;
    const int *parent;
    const int4 *coord;
    const int *has_tgt;
    const float2 *Lp;     // final locals of the parent level
    const float2 *part;   // this level's M2L partials [box][chunk]
    float2 *L;            // this level's locals (may alias part when chunks == 1)
    const float *otab;    // rotation-based translation tables
};

// rows of the coefficients held in slot 1 (the EXTRA lowest coefficients)
template <int P>
__host__ __device__ constexpr int slot1_rows() {
    constexpr int NC = ncoef(P);
    if (NC <= 32) return 1;
    int n = 0;
    while ((n + 1) * (n + 2) / 2 < NC - 32) n++;
    return n + 1;
}

// Rotation / translation rows are RS = p rounded up to 4 floats (16-byte
// rows, zero padded).  In shared memory the coefficients sit in rows of SR =
// RS + 2 complex values: A[n][m] by degree (n-major) for the rotations, B[k][n]
// by order (k-major) for the z-translation; entries outside a row's range stay
// zero, so whole float4 groups can be read without masks.  The 16-byte pad
// puts the rows of up to 8 consecutive degrees in 8 different 16-byte bank
// groups, so the lanes of a quarter warp (which read rows of different
// degrees) do not conflict.  The shared z-translation table keeps rows (k, j)
// of RS floats at k * ZK + j * RS, with the order stride ZK padded by a few
// 16-byte groups (chosen by counting, per order p, the bank groups the lanes
// of each quarter warp hit).
template <int P>
__host__ __device__ constexpr int rot_rs() { return (P + 3) / 4 * 4; }
template <int P>
__host__ __device__ constexpr int sh_rs() { return rot_rs<P>() + 2; }
template <int P>
__host__ __device__ constexpr int z_ks() { return P * rot_rs<P>() + 4 * (P >= 10 ? 7 : (P <= 4 ? 0 : 3)); }

// One output (n, mp) of a folded y-rotation: real part = E row . Re(A_n),
// imaginary part = O row . Im(A_n) (the O row starts with a zero for m = 0).
// G is the number of 4-coefficient groups to visit (a compile-time bound; a
// lane stops at the groups its degree n covers).
template <int P, int G>
__device__ __forceinline__ float2 rot_row(const float *__restrict__ D, int eoff, int ooff, const float2 *A, int n,
                                          int mp) {
    constexpr int RS = rot_rs<P>();
    // group-major blocks: group q of row r at (q * rows + r) float4s from the block start
    const float4 *E = reinterpret_cast<const float4 *>(D + eoff + RS * (n * (n + 1) / 2)) + mp;
    const float4 *O = reinterpret_cast<const float4 *>(D + ooff + RS * (n * (n - 1) / 2)) + (mp > 0 ? mp - 1 : 0);
    const float4 *A4 = reinterpret_cast<const float4 *>(A + n * sh_rs<P>());
    float re = 0.f, im = 0.f;
#pragma unroll
    for (int q = 0; q < G; q++) {
        if (4 * q <= n) {
            const float4 e = E[q * (n + 1)];
            const float4 a0 = A4[2 * q], a1 = A4[2 * q + 1];
            re = fmaf(e.x, a0.x, re);
            re = fmaf(e.y, a0.z, re);
            re = fmaf(e.z, a1.x, re);
            re = fmaf(e.w, a1.z, re);
            if (mp > 0) {
                const float4 o = O[q * n];
                im = fmaf(o.x, a0.y, im);
                im = fmaf(o.y, a0.w, im);
                im = fmaf(o.z, a1.y, im);
                im = fmaf(o.w, a1.w, im);
            }
        }
    }
    return make_float2(re, im);
}

// One output (j, k) of the translation along z:
// L'_j^k = sum_{n >= k} C[k][j][n] rho^-(j+n+1) M'_n^k  (C is zero for n < k)
template <int P>
__device__ __forceinline__ float2 ztrans_row(const float *__restrict__ zc, const float2 *Bk, int j, int k,
                                             float inv_rho) {
    constexpr int RS = rot_rs<P>();
    const float4 *Z = reinterpret_cast<const float4 *>(zc + k * z_ks<P>() + j * RS);
    const float4 *B4 = reinterpret_cast<const float4 *>(Bk + k * sh_rs<P>());
    float ip = inv_rho;
#pragma unroll
    for (int q = 0; q < 2 * P - 2; q++)
        if (q < j) ip *= inv_rho;  // rho^-(j+1)
    float re = 0.f, im = 0.f;
#pragma unroll
    for (int q = 0; q < RS / 4; q++) {
        const float4 z = Z[q];
        const float4 b0 = B4[2 * q], b1 = B4[2 * q + 1];
        const float f0 = z.x * ip;
        ip *= inv_rho;
        const float f1 = z.y * ip;
        ip *= inv_rho;
        const float f2 = z.z * ip;
        ip *= inv_rho;
        const float f3 = z.w * ip;
        ip *= inv_rho;
        re = fmaf(f0, b0.x, fmaf(f1, b0.z, fmaf(f2, b1.x, fmaf(f3, b1.z, re))));
        im = fmaf(f0, b0.y, fmaf(f1, b0.w, fmaf(f2, b1.y, fmaf(f3, b1.w, im))));
    }
    return make_float2(re, im);
}

// Offsets in the octant table (same as oct_layout on the host).
template <int P>
struct OctOff {
    static constexpr int RS = rot_rs<P>(), DSZ = 2 * RS * P * P, ZSZ = P * P * RS;
    static constexpr int rot = 0, zm2m = 2 * DSZ, zl2l = zm2m + ZSZ, ph_m2m = zl2l + ZSZ, ph_l2l = ph_m2m + 16 * P,
                         th_m2m = ph_l2l + 16 * P, th_l2l = th_m2m + 8;
};

// One output (j, k) of a z-shift by a fixed distance: sum_n Z[k][j][n] B[k][n]
template <int P>
__device__ __forceinline__ float2 zshift_row(const float *__restrict__ zt, const float2 *Bk, int j, int k) {
    constexpr int RS = rot_rs<P>();
    const float4 *Z = reinterpret_cast<const float4 *>(zt + ((size_t)k * P + j) * RS);
    const float4 *B4 = reinterpret_cast<const float4 *>(Bk + k * sh_rs<P>());
    float re = 0.f, im = 0.f;
#pragma unroll
    for (int q = 0; q < RS / 4; q++) {
        const float4 z = __ldg(Z + q);
        const float4 b0 = B4[2 * q], b1 = B4[2 * q + 1];
        re = fmaf(z.x, b0.x, fmaf(z.y, b0.z, fmaf(z.z, b1.x, fmaf(z.w, b1.z, re))));
        im = fmaf(z.x, b0.y, fmaf(z.y, b0.w, fmaf(z.z, b1.y, fmaf(z.w, b1.w, im))));
    }
    return make_float2(re, im);
}

// Rotation-based translation of one coefficient vector (GR normalisation,
// compact layout) along an octant direction: phase e^{i m phi}, y-rotation
// that takes the direction to +z, fixed z-shift Z, back-rotation, phase
// e^{-i m phi}; the result is added into the lane's accumulators.  A and B are
// the warp's degree-major / order-major rows, zero outside (n, m <= n).
template <int P>
__device__ __forceinline__ void oct_translate(const float2 *__restrict__ in, const float2 *__restrict__ ph,
                                              const float *__restrict__ D, const float *__restrict__ Z, float2 *A,
                                              float2 *B, const int *cn, const int *cm, const int *cs,
                                              const bool *has, float2 *acc) {
    constexpr int RS = rot_rs<P>(), SR = sh_rs<P>(), G0 = RS / 4, G1 = slot1_rows<P>() / 4 + 1;
    constexpr int ESZ = RS * P * (P + 1) / 2, OSZ = RS * P * (P - 1) / 2;
#pragma unroll
    for (int t = 0; t < 2; t++)
        if (has[t]) A[cn[t] * SR + cm[t]] = cmul(in[cs[t]], ph[cm[t]]);
    __syncwarp();
    if (has[0]) B[cm[0] * SR + cn[0]] = rot_row<P, G0>(D, 0, ESZ, A, cn[0], cm[0]);
    if (has[1]) B[cm[1] * SR + cn[1]] = rot_row<P, G1>(D, 0, ESZ, A, cn[1], cm[1]);
    __syncwarp();
    if (has[0]) A[cn[0] * SR + cm[0]] = zshift_row<P>(Z, B, cn[0], cm[0]);
    if (has[1]) A[cn[1] * SR + cm[1]] = zshift_row<P>(Z, B, cn[1], cm[1]);
    __syncwarp();
    if (has[0]) acc[0] = cadd(acc[0], cmul(rot_row<P, G0>(D, ESZ + OSZ, 2 * ESZ + OSZ, A, cn[0], cm[0]), cconj(ph[cm[0]])));
    if (has[1]) acc[1] = cadd(acc[1], cmul(rot_row<P, G1>(D, ESZ + OSZ, 2 * ESZ + OSZ, A, cn[1], cm[1]), cconj(ph[cm[1]])));
    __syncwarp();
}

// lane slots of the translation kernels: slot 0 of every lane holds one of
// the NC - EXTRA highest coefficients, slot 1 of the first EXTRA lanes one of
// the EXTRA lowest (NC > 32 at p >= 8)
template <int P>
__device__ __forceinline__ void coef_slots(int lane, int *cn, int *cm, int *cs, bool *has) {
    constexpr int NC = ncoef(P), EXTRA = NC > 32 ? NC - 32 : 0;
    cs[0] = lane + EXTRA;
    cs[1] = lane;
    cnm(min(cs[0], NC - 1), cn[0], cm[0]);
    cnm(min(cs[1], NC - 1), cn[1], cm[1]);
    has[0] = cs[0] < NC;
    has[1] = lane < EXTRA;
}

// M2M: one warp per parent box; each child's multipole translated to the
// parent centre by rotation (O(p^3) per child instead of the O(p^4) direct
// R-convolution), child -> parent box units folded into the z-shift table.
template <int P>
__global__ void __launch_bounds__(kWarps * 32)
m2m_kernel(int nbox, const int *__restrict__ nbd, const int *__restrict__ child0, const int4 *__restrict__ ccoord,
           const float2 *__restrict__ Mc, float2 *__restrict__ Mp, const float *__restrict__ otab) {
    constexpr int NC = ncoef(P), SR = sh_rs<P>();
    using O = OctOff<P>;
    __shared__ __align__(16) float2 A[kWarps][P * SR], B[kWarps][P * SR];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int t = lane; t < P * SR; t += 32) A[wid][t] = B[wid][t] = make_float2(0.f, 0.f);
    __syncwarp();
    int cn[2], cm[2], cs[2];
    bool has[2];
    coef_slots<P>(lane, cn, cm, cs, has);
    const int nb = level_boxes(nbox, nbd);
    for (int b = blockIdx.x * kWarps + wid; b < nb; b += gridDim.x * kWarps) {
        float2 acc[2] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
        const int ch1 = child0[b + 1];
        for (int ch = child0[b]; ch < ch1; ch++) {
            const int4 cc = ccoord[ch];
            const int oc = (cc.x & 1) | ((cc.y & 1) << 1) | ((cc.z & 1) << 2);
            const int th = (int)otab[O::th_m2m + oc];
            oct_translate<P>(Mc + (size_t)ch * NC, reinterpret_cast<const float2 *>(otab + O::ph_m2m) + oc * P,
                             otab + O::rot + th * O::DSZ, otab + O::zm2m, A[wid], B[wid], cn, cm, cs, has, acc);
        }
        if (has[0]) Mp[(size_t)b * NC + cs[0]] = acc[0];
        if (has[1]) Mp[(size_t)b * NC + cs[1]] = acc[1];
    }
}

template <int P>
constexpr int m2l_warps() { return P >= 10 ? 2 : 4; }
// CTAs per SM the M2L is compiled for: the most that keep its registers
// unspilled (the kernel waits on dependent loads, so resident warps hide it)
template <int P>
constexpr int m2l_min_ctas() { return P >= 10 ? 1 : (P >= 8 ? 6 : 8); }
// list entries a warp carries through one pass of the M2L loop
template <int P>
constexpr int m2l_inflight() { return 2; }

// The z-translation table (the same for every entry) is staged once per CTA
// in shared memory; the rotation rows of each entry's polar angle are read
// from global memory (L1/L2), one 16-byte row segment per lane and group.
template <int P>
__global__ void __launch_bounds__(m2l_warps<P>() * 32, m2l_min_ctas<P>()) m2l_kernel(M2LArgs a) {
    constexpr int NC = ncoef(P), RS = rot_rs<P>(), SR = sh_rs<P>(), ZK = z_ks<P>(), WP = m2l_warps<P>();
    constexpr int NU = m2l_inflight<P>();
    if (a.run_if && !*a.run_if) return;
    __shared__ __align__(16) float2 A[WP][NU][P * SR], B[WP][NU][P * SR];
    __shared__ __align__(16) float Zsh[P * ZK];
    // the table's rows (k, j), RS floats each, to k * ZK + j * RS
    for (int t = threadIdx.x; t < P * P * (RS / 4); t += blockDim.x) {
        const int row = t / (RS / 4), g = t % (RS / 4), k = row / P, j = row % P;
        reinterpret_cast<float4 *>(Zsh + k * ZK + j * RS)[g] = __ldg(reinterpret_cast<const float4 *>(a.zc) + t);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int t = lane; t < NU * P * SR; t += 32) {
        A[wid][t / (P * SR)][t % (P * SR)] = make_float2(0.f, 0.f);
        B[wid][t / (P * SR)][t % (P * SR)] = make_float2(0.f, 0.f);
    }
    __syncthreads();
    const int gw = blockIdx.x * WP + wid;
    int li = 0;
    while (li + 1 < a.nlev && gw >= a.lv[li + 1].warp0) li++;
    const int chunks = a.lv[li].chunks;
    const int local = gw - a.lv[li].warp0;
    const int b = local / chunks, ch = local - b * chunks;
    if (b >= level_boxes(a.lv[li].nbox, a.lv[li].nbd) || !a.lv[li].has_tgt[b]) return;
    // Lane slots.  Slot 0 of every lane holds one of the NC - EXTRA highest
    // coefficients; slot 1 of the first EXTRA lanes holds one of the EXTRA
    // lowest (cheapest) coefficients, so the second pass is short.
    constexpr int EXTRA = NC > 32 ? NC - 32 : 0;
    const int c0 = lane + EXTRA, c1 = lane;
    int cn[2], cm[2];
    cnm(min(c0, NC - 1), cn[0], cm[0]);
    cnm(min(c1, NC - 1), cn[1], cm[1]);
    const int cs[2] = {c0, c1};
    const bool has[2] = {c0 < NC, lane < EXTRA};
    float2 acc[2] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
    const double h = box_root(a.root, a.lv[li].bpid, b)[3] / (double)(1 << a.lv[li].level);
    const float eh2 = (float)(a.eps2 / (h * h));
    const int cnt = a.lv[li].cnt[b];
    const int per = (cnt + chunks - 1) / chunks;
    const int e0 = ch * per, e1 = min(cnt, e0 + per);
    const int2 *lst = a.lv[li].m2l + (size_t)b * a.cap;
    const float2 *Ml = a.lv[li].M;
    // NU entries in flight per iteration: their loads and the warp
    // synchronisations overlap (entries past the range's end repeat the last
    // one and are not accumulated)
    constexpr int G0 = RS / 4, G1 = slot1_rows<P>() / 4 + 1;
    for (int e = e0; e < e1; e += NU) {
        int src[NU];
        const float2 *ph[NU];
        const float *D[NU];
        float inv_rho[NU];
#pragma unroll
        for (int u = 0; u < NU; u++) {
            const int2 en = lst[min(e + u, e1 - 1)];
            src[u] = en.x;
            ph[u] = a.cls_phase + (size_t)en.y * P;
            D[u] = a.dmat + (size_t)a.cls_theta[en.y] * a.dsz;
            inv_rho[u] = rsqrtf(a.cls_rho2[en.y] + eh2);
        }
        // phase e^{i m phi}, into the degree-major rows
#pragma unroll
        for (int u = 0; u < NU; u++)
#pragma unroll
            for (int t = 0; t < 2; t++)
                if (has[t]) A[wid][u][cn[t] * SR + cm[t]] = cmul(Ml[(size_t)src[u] * NC + cs[t]], ph[u][cm[t]]);
        __syncwarp();
        // forward y-rotation (folded real matrices), into the order-major rows
#pragma unroll
        for (int u = 0; u < NU; u++) {
            if (has[0]) B[wid][u][cm[0] * SR + cn[0]] = rot_row<P, G0>(D[u], 0, a.esz, &A[wid][u][0], cn[0], cm[0]);
            if (has[1]) B[wid][u][cm[1] * SR + cn[1]] = rot_row<P, G1>(D[u], 0, a.esz, &A[wid][u][0], cn[1], cm[1]);
        }
        __syncwarp();
        // translation along z: L'_j^k = sum_n C[k][j][n] rho^-(j+n+1) M'_n^k
#pragma unroll
        for (int u = 0; u < NU; u++) {
            if (has[0]) A[wid][u][cn[0] * SR + cm[0]] = ztrans_row<P>(Zsh, &B[wid][u][0], cn[0], cm[0], inv_rho[u]);
            if (has[1]) A[wid][u][cn[1] * SR + cm[1]] = ztrans_row<P>(Zsh, &B[wid][u][0], cn[1], cm[1], inv_rho[u]);
        }
        __syncwarp();
        // backward y-rotation and phase e^{-i k phi}
#pragma unroll
        for (int u = 0; u < NU; u++) {
            if (e + u >= e1) break;
            if (has[0]) {
                const float2 r =
                    rot_row<P, G0>(D[u], a.esz + a.osz, 2 * a.esz + a.osz, &A[wid][u][0], cn[0], cm[0]);
                acc[0] = cadd(acc[0], cmul(r, cconj(ph[u][cm[0]])));
            }
            if (has[1]) {
                const float2 r =
                    rot_row<P, G1>(D[u], a.esz + a.osz, 2 * a.esz + a.osz, &A[wid][u][0], cn[1], cm[1]);
                acc[1] = cadd(acc[1], cmul(r, cconj(ph[u][cm[1]])));
            }
        }
        __syncwarp();
    }
    float2 *dst = a.lv[li].out + ((size_t)b * chunks + ch) * NC;
    if (has[0]) dst[cs[0]] = acc[0];
    if (has[1]) dst[cs[1]] = acc[1];
}

// L = (sum of the level's M2L partials, in chunk order) + L2L(parent's L),
// the L2L by rotation (O(p^3)), parent -> child box units folded into the
// z-shift table
template <int P>
__global__ void __launch_bounds__(kWarps * 32) l2l_kernel(L2LArgs a) {
    constexpr int NC = ncoef(P), SR = sh_rs<P>();
    using O = OctOff<P>;
    __shared__ __align__(16) float2 A[kWarps][P * SR], B[kWarps][P * SR];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int t = lane; t < P * SR; t += 32) A[wid][t] = B[wid][t] = make_float2(0.f, 0.f);
    __syncwarp();
    int cn[2], cm[2], cs[2];
    bool has[2];
    coef_slots<P>(lane, cn, cm, cs, has);
    const int nb = level_boxes(a.nbox, a.nbd);
    for (int b = blockIdx.x * kWarps + wid; b < nb; b += gridDim.x * kWarps) {
        if (!a.has_tgt[b]) continue;
        float2 acc[2] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
#pragma unroll
        for (int t = 0; t < 2; t++)
            if (has[t])
                for (int ch = 0; ch < a.chunks; ch++)
                    acc[t] = cadd(acc[t], a.part[((size_t)b * a.chunks + ch) * NC + cs[t]]);
        if (a.has_parent) {
            const int4 cb = a.coord[b];
            const int oc = (cb.x & 1) | ((cb.y & 1) << 1) | ((cb.z & 1) << 2);
            const int th = (int)a.otab[O::th_l2l + oc];
            oct_translate<P>(a.Lp + (size_t)a.parent[b] * NC,
                             reinterpret_cast<const float2 *>(a.otab + O::ph_l2l) + oc * P,
                             a.otab + O::rot + th * O::DSZ, a.otab + O::zl2l, A[wid], B[wid], cn, cm, cs, has, acc);
        }
        if (has[0]) a.L[(size_t)b * NC + cs[0]] = acc[0];
        if (has[1]) a.L[(size_t)b * NC + cs[1]] = acc[1];
    }
}

// warps per box for a level of nbox boxes: enough to give every SM a few
// warps even at the coarse levels, at most 16
inline int m2l_chunks(int nbox) {
    const int want = 16 * device_sms();
    int c = nbox > 0 ? (want + nbox - 1) / nbox : 1;
    return c < 1 ? 1 : (c > 16 ? 16 : c);
}

// ------------------------------------------------------------------ L2P --
template <int P>
__global__ void __launch_bounds__(kWarps * 32)
l2p_kernel(int nbox, const int *__restrict__ nbd, const int *__restrict__ bpid, const int *__restrict__ start,
           const float4 *__restrict__ rel, const double *__restrict__ qm, const double *__restrict__ roots, int level,
           const float *__restrict__ nrm, const float2 *__restrict__ Lc, double *__restrict__ ax,
           double *__restrict__ ay, double *__restrict__ az, const int *__restrict__ has_tgt, int accumulate) {
    constexpr int NC = ncoef(P);
    __shared__ float2 lam[kWarps][NC];
    SV_WARP_BOXES(kWarps) {
    const double *root = box_root(roots, bpid, b);
    if (!has_tgt[b]) {
        // boxes of image copies only: no targets, zero acceleration
        if (!accumulate)
            for (int i = start[b] + lane; i < start[b + 1]; i += 32) ax[i] = ay[i] = az[i] = 0.0;
        continue;
    }
    for (int c = lane; c < NC; c += 32) {
        int n, m;
        cnm(c, n, m);
        lam[wid][c] = cscale(Lc[(size_t)b * NC + c], nrm[n * P + m]);
    }
    __syncwarp();
    // Positions relative to the leaf box centre come from box_relative_kernel
    // (FP32, metres); the per-particle work stays on the FP32 pipe, the FP64
    // pipe (1/64 of its rate on this GPU) sees only the stores' conversions.
    const double h = root[3] / (double)(1 << level);
    const float ihf = (float)(1.0 / h), mih2 = (float)(-1.0 / (h * h));
    const int s1 = start[b + 1];
    for (int i = start[b] + lane; i < s1; i += 32) {
        float2 R[ncoef(P - 1) > 0 ? ncoef(P - 1) : 1];
        const float4 r = rel[i];
        solid_harmonics<P - 1>(r.x * ihf, r.y * ihf, r.z * ihf, R);
        float gz = 0.f;
        float2 gm = make_float2(0.f, 0.f);
#pragma unroll
        for (int n = 1; n < P; n++) {
            const float2 *ln = &lam[wid][cidx(n, 0)];
            gz = fmaf(ln[0].x, R[cidx(n - 1, 0)].x, gz);
#pragma unroll
            for (int m = 1; m < n; m++) {
                const float2 v = cmul(ln[m], R[cidx(n - 1, m)]);
                gz = fmaf(2.f, v.x, gz);
            }
#pragma unroll
            for (int m = 1; m <= n; m++) gm = cadd(gm, cmul(ln[m], R[cidx(n - 1, m - 1)]));
#pragma unroll
            for (int t = 0; t + 1 < n; t++) gm = cadd(gm, cscale(cconj(cmul(ln[t], R[cidx(n - 1, t + 1)])), -1.f));
        }
        // a = -grad(phi) * K q / m, grad in box units / h^2 (added to the
        // near field when that ran first)
        const float f = (float)qm[i] * mih2;
        const float vx = f * gm.x, vy = -f * gm.y, vz = f * gz;
        if (accumulate) {
            ax[i] += (double)vx;
            ay[i] += (double)vy;
            az[i] += (double)vz;
        } else {
            ax[i] = (double)vx;
            ay[i] = (double)vy;
            az[i] = (double)vz;
        }
    }
    __syncwarp();
    }
}


// ----------------------------------------------------------- treecode M2P --
// The treecode mode (FmmType::treecode, m2p_kernel fmm_cpukernel.cpp:1399-1533)
// evaluates every far-field multipole directly at the target particles
// instead of translating it into local expansions.  A leaf box's particles
// receive the multipoles of the interaction lists of all its ancestors
// (levels L..2).  With M in the regular-harmonic normalisation of P2M
// (M = sum q conj(R_n^m(d)), R_n^m = r^n P_n^m e^{im phi} / (n+m)!), the
// potential is phi(x) = sum_{n,m} M_n^m S_n^m(x - c) with the irregular
// harmonics S_n^m = (n-m)! r^{-n-1} P_n^m e^{im phi}, and
//   d/dz S_n^m = -S_{n+1}^m,   (d/dx + i d/dy) S_n^m = -S_{n+1}^{m+1}.
// The softened distance r^2 + eps^2/h^2 enters the recurrences, as the
// reference softens r in its M2P and M2L.

// Irregular solid harmonics S_n^m, m >= 0, degrees 0..Q-1:
// S_0^0 = 1/r; S_m^m = (2m-1)(x+iy)/r^2 S_{m-1}^{m-1}; S_{m+1}^m = (2m+1) z/r^2 S_m^m;
// S_n^m = ((2n-1) z S_{n-1}^m - ((n-1)^2 - m^2) S_{n-2}^m) / r^2.
template <int Q>
__device__ __forceinline__ void irregular_harmonics(float x, float y, float z, float r2, float2 *S) {
    const float ir2 = 1.f / r2;
    S[0] = make_float2(rsqrtf(r2), 0.f);
#pragma unroll
    for (int m = 0; m < Q; m++) {
        if (m > 0) {
            const float2 prev = S[cidx(m - 1, m - 1)];
            const float s = (2.f * m - 1.f) * ir2;
            S[cidx(m, m)] = make_float2((x * prev.x - y * prev.y) * s, (x * prev.y + y * prev.x) * s);
        }
        if (m + 1 < Q) S[cidx(m + 1, m)] = cscale(S[cidx(m, m)], (2.f * m + 1.f) * z * ir2);
#pragma unroll
        for (int n = m + 2; n < Q; n++) {
            const float a = (2.f * n - 1.f) * z, d = (float)((n - 1) * (n - 1) - m * m);
            const float2 s1 = S[cidx(n - 1, m)], s0 = S[cidx(n - 2, m)];
            S[cidx(n, m)] = make_float2((a * s1.x - d * s0.x) * ir2, (a * s1.y - d * s0.y) * ir2);
        }
    }
}

struct TreecodeArgs {
    int L, cap, ws, nleaf;
    const int *parent[kMortonBits + 1];
    const int4 *coord[kMortonBits + 1];
    const int2 *m2l[kMortonBits + 1];
    const int *m2l_cnt[kMortonBits + 1];
    const float2 *M[kMortonBits + 1];
    const int *leaf_start;
    const int *has_tgt;
    const double *x, *y, *z, *qm;
    const double *root;
    const float *nrm;
    double eps2;
    double *ax, *ay, *az;
    int accumulate;  // 1: add to ax (the near field ran first), 0: overwrite
};

template <int P>
__global__ void __launch_bounds__(kWarps * 32) m2p_kernel(TreecodeArgs a) {
    constexpr int NC = ncoef(P), NS = ncoef(P + 1);
    __shared__ float2 Mw[kWarps][NC];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int b = blockIdx.x * kWarps + wid;
    if (b >= a.nleaf) return;
    const int s0 = a.leaf_start[b], s1 = a.leaf_start[b + 1];
    if (!a.has_tgt[b]) {
        if (!a.accumulate)
            for (int i = s0 + lane; i < s1; i += 32) a.ax[i] = a.ay[i] = a.az[i] = 0.0;
        return;
    }
    const int R = 2 * a.ws + 1, SIDE = 2 * R + 1;
    for (int tb = s0; tb < s1; tb += 32) {
        const int i = tb + lane;
        const bool valid = i < s1;
        const int ii = valid ? i : s0;
        double gx = 0.0, gy = 0.0, gz = 0.0;
        int box = b;
        for (int l = a.L; l >= 2; l--) {
            const double h = a.root[3] / (double)(1 << l);
            const int4 cb = a.coord[l][box];
            const double ih = 1.0 / h;
            const float dx0 = (float)((a.x[ii] - (a.root[0] + (cb.x + 0.5) * h)) * ih);
            const float dy0 = (float)((a.y[ii] - (a.root[1] + (cb.y + 0.5) * h)) * ih);
            const float dz0 = (float)((a.z[ii] - (a.root[2] + (cb.z + 0.5) * h)) * ih);
            const float e2 = (float)(a.eps2 * ih * ih);
            const int cnt = a.m2l_cnt[l][box];
            const int2 *lst = a.m2l[l] + (size_t)box * a.cap;
            float fx = 0.f, fy = 0.f, fz = 0.f;
            for (int e = 0; e < cnt; e++) {
                const int2 ent = lst[e];
                __syncwarp();
                for (int c = lane; c < NC; c += 32) {
                    int n, m;
                    cnm(c, n, m);
                    Mw[wid][c] = cscale(a.M[l][(size_t)ent.x * NC + c], 1.f / a.nrm[n * P + m]);
                }
                __syncwarp();
                // target ancestor minus source box, in boxes (exact)
                const int oz = ent.y % SIDE - R, oy = (ent.y / SIDE) % SIDE - R, ox = ent.y / (SIDE * SIDE) - R;
                const float dx = dx0 + (float)ox, dy = dy0 + (float)oy, dz = dz0 + (float)oz;
                float2 S[NS];
                irregular_harmonics<P + 1>(dx, dy, dz, fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, e2))), S);
                float2 gp = make_float2(0.f, 0.f);
                float gzz = 0.f;
#pragma unroll
                for (int n = 0; n < P; n++) {
                    const float2 *Mn = &Mw[wid][cidx(n, 0)];
                    const float2 *Sn = &S[cidx(n + 1, 0)];
                    gzz += cmul(Mn[0], Sn[0]).x;
#pragma unroll
                    for (int m = 1; m <= n; m++) gzz += 2.f * cmul(Mn[m], Sn[m]).x;
#pragma unroll
                    for (int m = 0; m <= n; m++) gp = cadd(gp, cmul(Mn[m], Sn[m + 1]));
#pragma unroll
                    for (int k = 1; k <= n; k++) gp = cadd(gp, cscale(cconj(cmul(Mn[k], Sn[k - 1])), -1.f));
                }
                fx -= gp.x;
                fy -= gp.y;
                fz -= gzz;
            }
            const double s = ih * ih;
            gx += (double)fx * s;
            gy += (double)fy * s;
            gz += (double)fz * s;
            box = a.parent[l][box];
        }
        if (valid) {
            // a = -K q/m grad(phi)
            const double c = a.qm[i];
            if (a.accumulate) {
                a.ax[i] += -c * gx;
                a.ay[i] += -c * gy;
                a.az[i] += -c * gz;
            } else {
                a.ax[i] = -c * gx;
                a.ay[i] = -c * gy;
                a.az[i] = -c * gz;
            }
        }
    }
}

// ------------------------------------------------------------------ P2P --
// Each particle once as an FP32 offset from the centre of its own leaf box
// (one FP64 subtraction per particle) with its charge: the P2P kernel then
// forms source offsets from the target box centre as offset + k*h in FP32.
// A charge other than qs[0] sets *mixed (zeroed beforehand), which keeps the
// P2P kernel on its per-source charge path.
__global__ void __launch_bounds__(kWarps * 32)
box_relative_kernel(int nbox, const int *__restrict__ nbd, const int *__restrict__ bpid,
                    const int *__restrict__ start, const int4 *__restrict__ coord, const double *__restrict__ xs,
                    const double *__restrict__ ys, const double *__restrict__ zs, const float *__restrict__ qs,
                    const double *__restrict__ roots, int level, float4 *__restrict__ rel,
                    unsigned long long *__restrict__ mixed) {
    const float q0 = qs[0];
    bool diff = false;
    SV_WARP_BOXES(kWarps) {
    const double *root = box_root(roots, bpid, b);
    const double h = root[3] / (double)(1 << level);
    const int4 cb = coord[b];
    const double cx = root[0] + (cb.x + 0.5) * h, cy = root[1] + (cb.y + 0.5) * h, cz = root[2] + (cb.z + 0.5) * h;
    for (int j = start[b] + lane; j < start[b + 1]; j += 32) {
        const float q = qs[j];
        diff |= q != q0;
        rel[j] = make_float4((float)(xs[j] - cx), (float)(ys[j] - cy), (float)(zs[j] - cz), q);
    }
    }
    if (__any_sync(0xffffffffu, diff) && (threadIdx.x & 31) == 0) *mixed = 1ull;
}

// 16-byte asynchronous copy global -> shared (LDGSTS): the data lands without
// passing through registers; the issuing thread sees it after cp_async_wait_all.
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// s += v with Kahan compensation e (the running sum is s - e)
__device__ __forceinline__ void kahan_add(float &s, float &e, float v) {
    const float y = v - e, t = s + y;
    e = (t - s) - y;
    s = t;
}

// Near field of one leaf box per warp.  The box's non-empty near boxes, then
// its far-direct boxes (interaction-list entries cheaper as pairs, from
// build_lists_box), are compacted into shared memory with a running count of
// their sources; the sources are then streamed 32 at a time across box
// boundaries (each lane walks forward to the box of its staged source), so the
// pair loop runs without per-box padding or per-box overhead.  Sources are
// staged as negated coordinates in structure-of-arrays rows, so one 64-bit
// load gives two consecutive sources and each pair operation is a packed
// FP32x2 instruction (FADD2 / FFMA2 / FMUL2) over two sources; the reciprocal
// square roots stay scalar.  Targets: two per lane while more than 48 remain,
// then one per lane; a chunk of nt < 32 targets gives each target a group of g
// lanes (a power of two, nt * g <= 32) that split the staged sources.  Each
// 32-source chunk's FP32 partial sum is added with Kahan compensation.  The
// result is stored (each particle of a box with targets once; boxes without
// targets are left as they are).  CLAMP: floor r^2 at kMinR2, needed only when
// eps^2 < kMinR2 (a zero-distance pair without softening).  UQ: every particle
// of the tree carries the same charge Q (box_relative_kernel found no other),
// so the pair weight is r^-3 alone, the sums are scaled by the target's own
// charge (= Q) at the end, and padding sources sit far away (r^-3 underflows
// to zero) instead of carrying zero charge.
constexpr int kFarDirectCap = 128;  // far-direct source boxes per leaf box
// source boxes a leaf box's near field can take: its near boxes and its far-direct ones
template <int WS>
constexpr int p2p_nsp() { return ((2 * WS + 1) * (2 * WS + 1) * (2 * WS + 1) + 31) / 32 * 32 + kFarDirectCap; }


template <int WS, bool CLAMP, bool UQ>
__device__ __forceinline__ void
p2p_body(int nbox, const int *__restrict__ nbd, const int *__restrict__ bpid, const int *__restrict__ start,
         const int4 *__restrict__ coord, const int *__restrict__ nbr, const double *__restrict__ qm,
         const double *__restrict__ roots, int level, float eps2, double *__restrict__ ax, double *__restrict__ ay,
         double *__restrict__ az, unsigned long long *__restrict__ counts, const int *__restrict__ has_tgt,
         const float4 *__restrict__ rel, const int *__restrict__ fd, const int *__restrict__ fd_cnt, int fd_cap,
         float (*st)[4][32], float4 (*raw)[2][32], int2 (*nb_rng)[p2p_nsp<WS>()],
         float4 (*nb_off)[p2p_nsp<WS>()]) {
    constexpr int NS1 = 2 * WS + 1, NS = NS1 * NS1 * NS1;
    const float4 pad = UQ ? make_float4(1e18f, 0.f, 0.f, 0.f) : make_float4(0.f, 0.f, 0.f, 0.f);
    const float2 E2 = make_float2(eps2, eps2);
    unsigned long long pairs = 0;
    const unsigned lt_mask = (1u << (threadIdx.x & 31)) - 1u;
    SV_WARP_BOXES(kWarps) {
    if (!has_tgt[b]) continue;
    // a power of two: k * hf is exact
    const float hf = (float)(box_root(roots, bpid, b)[3] / (double)(1 << level));
    const int4 cb = coord[b];
    int nnz = 0, total = 0;
    // the non-empty boxes of a list (count warp-uniform; -1 entries skipped)
    // appended with their running source count and their offset
    auto add_boxes = [&](const int *list, int count) {
        for (int s0 = 0; s0 < count; s0 += 32) {
            const int s = s0 + lane;
            int Q = -1, j0 = 0, cnt = 0;
            if (s < count) {
                Q = list[s];
                if (Q >= 0) {
                    j0 = start[Q];
                    cnt = start[Q + 1] - j0;
                }
            }
            const bool f = cnt > 0;
            const unsigned bal = __ballot_sync(0xffffffffu, f);
            int inc = cnt;
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, inc, o);
                if (lane >= o) inc += t;
            }
            if (f) {
                const int pos = nnz + __popc(bal & lt_mask);
                const int4 cq = coord[Q];
                nb_rng[wid][pos] = make_int2(j0, total + inc);
                nb_off[wid][pos] = make_float4((float)(cq.x - cb.x) * hf, (float)(cq.y - cb.y) * hf,
                                               (float)(cq.z - cb.z) * hf, 0.f);
            }
            nnz += __popc(bal);
            total += __shfl_sync(0xffffffffu, inc, 31);
        }
    };
    add_boxes(nbr + (size_t)b * NS, NS);
    if (fd) add_boxes(fd + (size_t)b * fd_cap, fd_cnt[b]);
    __syncwarp();
    const int t0 = start[b], t1 = start[b + 1];
    // Sources are staged one 32-source chunk ahead: the lane's source of the
    // next chunk is copied into raw[buf] (cp.async) while the current chunk's
    // pairs run.  kb / kbeg: the lane's current source box and its first
    // running index (lanes walk forward through the compacted boxes); kn: the
    // box slot of the copied source, -1 past the end.
    int kb = 0, kbeg = 0, kn = -1;
    auto prefetch = [&](int c0, int buf) {
        const int j = c0 + lane;
        kn = -1;
        if (j < total) {
            int2 rg = nb_rng[wid][kb];
            while (rg.y <= j) {
                kbeg = rg.y;
                rg = nb_rng[wid][++kb];
            }
            cp_async16(&raw[wid][buf][lane], rel + rg.x + (j - kbeg));
            kn = kb;
        }
        cp_async_commit();
    };
    // the copied chunk, moved to its target-box offset, into the staging rows
    auto stage = [&](int buf) {
        cp_async_wait_all();
        float4 v = pad;
        if (kn >= 0) {
            const float4 r = raw[wid][buf][lane];
            const float4 o = nb_off[wid][kn];
            v = make_float4(r.x + o.x, r.y + o.y, r.z + o.z, r.w);
        }
        st[wid][0][lane] = -v.x;
        st[wid][1][lane] = -v.y;
        st[wid][2][lane] = -v.z;
        if (!UQ) st[wid][3][lane] = v.w;
    };
    int tb = t0;
    // two targets per lane while more than 48 remain: each staged source
    // (one shared-memory load) then feeds two pairs.  33-48 targets cost less
    // as one full pass of 32 and a pass that splits the sources of the
    // remaining 1-16 targets over 2-32 lanes each.
    for (; t1 - tb > 48; tb += 64) {
        const int ia = tb + lane, ib = tb + 32 + lane;
        const bool vb = ib < t1;
        const float4 ta = rel[ia], tbv = rel[vb ? ib : ia];
        if (lane == 0) pairs += (unsigned long long)total * (unsigned long long)min(64, t1 - tb);
        const float2 AX = make_float2(ta.x, ta.x), AY = make_float2(ta.y, ta.y), AZ = make_float2(ta.z, ta.z);
        const float2 BX = make_float2(tbv.x, tbv.x), BY = make_float2(tbv.y, tbv.y), BZ = make_float2(tbv.z, tbv.z);
        float sax = 0.f, say = 0.f, saz = 0.f, eax = 0.f, eay = 0.f, eaz = 0.f;
        float sbx = 0.f, sby = 0.f, sbz = 0.f, ebx = 0.f, eby = 0.f, ebz = 0.f;
        kb = kbeg = 0;
        prefetch(0, 0);
        for (int c0 = 0, buf = 0; c0 < total; c0 += 32, buf ^= 1) {
            stage(buf);
            if (c0 + 32 < total) prefetch(c0 + 32, buf ^ 1);
            __syncwarp();
            float2 gax = make_float2(0.f, 0.f), gay = gax, gaz = gax, gbx = gax, gby = gax, gbz = gax;
#pragma unroll 4
            for (int k = 0; k < 32; k += 2) {
                const float2 X = ld2(st[wid][0], k), Y = ld2(st[wid][1], k), Z = ld2(st[wid][2], k);
                const float2 Q = UQ ? make_float2(1.f, 1.f) : ld2(st[wid][3], k);
                pair2<CLAMP, UQ>(X, Y, Z, Q, AX, AY, AZ, E2, gax, gay, gaz);
                pair2<CLAMP, UQ>(X, Y, Z, Q, BX, BY, BZ, E2, gbx, gby, gbz);
            }
            const float fax = gax.x + gax.y, fay = gay.x + gay.y, faz = gaz.x + gaz.y;
            const float fbx = gbx.x + gbx.y, fby = gby.x + gby.y, fbz = gbz.x + gbz.y;
            __syncwarp();
            kahan_add(sax, eax, fax);
            kahan_add(say, eay, fay);
            kahan_add(saz, eaz, faz);
            kahan_add(sbx, ebx, fbx);
            kahan_add(sby, eby, fby);
            kahan_add(sbz, ebz, fbz);
        }
        {
            const double c = UQ ? qm[ia] * (double)ta.w : qm[ia];
            ax[ia] = (double)(sax - eax) * c;
            ay[ia] = (double)(say - eay) * c;
            az[ia] = (double)(saz - eaz) * c;
        }
        if (vb) {
            const double c = UQ ? qm[ib] * (double)tbv.w : qm[ib];
            ax[ib] = (double)(sbx - ebx) * c;
            ay[ib] = (double)(sby - eby) * c;
            az[ib] = (double)(sbz - ebz) * c;
        }
    }
    for (; tb < t1; tb += 32) {
        const int nt = min(32, t1 - tb);
        int lg = 0;
        while ((nt << (lg + 1)) <= 32) lg++;
        const int g = 1 << lg;
        const int tloc = lane >> lg, sub = lane & (g - 1);
        const bool valid = tloc < nt;
        const int i = tb + (valid ? tloc : 0);
        const float4 ti = rel[i];
        const float2 TX = make_float2(ti.x, ti.x), TY = make_float2(ti.y, ti.y), TZ = make_float2(ti.z, ti.z);
        if (lane == 0) pairs += (unsigned long long)total * (unsigned long long)nt;
        float sx = 0.f, sy = 0.f, sz = 0.f, ex = 0.f, ey = 0.f, ez = 0.f;
        kb = kbeg = 0;
        prefetch(0, 0);
        for (int c0 = 0, buf = 0; c0 < total; c0 += 32, buf ^= 1) {
            stage(buf);
            if (c0 + 32 < total) prefetch(c0 + 32, buf ^ 1);
            __syncwarp();
            // g lanes per target, each taking pairs of consecutive sources 2 sub + 2 g i
            // (g = 1: every lane a target and all 32 staged sources; padding adds nothing)
            float2 gx = make_float2(0.f, 0.f), gy = gx, gz = gx;
#pragma unroll 4
            for (int k = 2 * sub; k < 32; k += 2 * g) {
                const float2 X = ld2(st[wid][0], k), Y = ld2(st[wid][1], k), Z = ld2(st[wid][2], k);
                const float2 Q = UQ ? make_float2(1.f, 1.f) : ld2(st[wid][3], k);
                pair2<CLAMP, UQ>(X, Y, Z, Q, TX, TY, TZ, E2, gx, gy, gz);
            }
            const float fx = gx.x + gx.y, fy = gy.x + gy.y, fz = gz.x + gz.y;
            __syncwarp();
            float y = fx - ex, t = sx + y;
            ex = (t - sx) - y;
            sx = t;
            y = fy - ey;
            t = sy + y;
            ey = (t - sy) - y;
            sy = t;
            y = fz - ez;
            t = sz + y;
            ez = (t - sz) - y;
            sz = t;
        }
        sx -= ex;
        sy -= ey;
        sz -= ez;
        // combine the g lanes of each target
        for (int o = g >> 1; o > 0; o >>= 1) {
            sx += __shfl_xor_sync(0xffffffffu, sx, o);
            sy += __shfl_xor_sync(0xffffffffu, sy, o);
            sz += __shfl_xor_sync(0xffffffffu, sz, o);
        }
        if (valid && sub == 0) {
            const double c = UQ ? qm[i] * (double)ti.w : qm[i];
            ax[i] = (double)sx * c;
            ay[i] = (double)sy * c;
            az[i] = (double)sz * c;
        }
    }
    __syncwarp();
    }
    if ((threadIdx.x & 31) == 0 && pairs) atomicAdd(&counts[1], pairs);
}

// counts[2] != 0: box_relative_kernel met two different charges
template <int WS, bool CLAMP>
__global__ void __launch_bounds__(kWarps * 32, 6)
p2p_kernel(int nbox, const int *__restrict__ nbd, const int *__restrict__ bpid, const int *__restrict__ start,
           const int4 *__restrict__ coord, const int *__restrict__ nbr, const double *__restrict__ qm,
           const double *__restrict__ roots, int level, float eps2, double *__restrict__ ax, double *__restrict__ ay,
           double *__restrict__ az, unsigned long long *__restrict__ counts, const int *__restrict__ has_tgt,
           const float4 *__restrict__ rel, const int *__restrict__ fd, const int *__restrict__ fd_cnt, int fd_cap) {
    __shared__ __align__(16) float src[kWarps][4][32];  // staged sources: -x, -y, -z, charge
    __shared__ int2 nb_rng[kWarps][p2p_nsp<WS>()];    // (first source, running source count at the box's end)
    __shared__ float4 nb_off[kWarps][p2p_nsp<WS>()];  // source box centre - target box centre (exact in FP32)
    __shared__ float4 raw[kWarps][2][32];             // next chunk's sources as copied (double buffer)
    if (counts[2] == 0)
        p2p_body<WS, CLAMP, true>(nbox, nbd, bpid, start, coord, nbr, qm, roots, level, eps2, ax, ay, az, counts,
                                  has_tgt, rel, fd, fd_cnt, fd_cap, src, raw, nb_rng, nb_off);
    else
        p2p_body<WS, CLAMP, false>(nbox, nbd, bpid, start, coord, nbr, qm, roots, level, eps2, ax, ay, az, counts,
                                   has_tgt, rel, fd, fd_cnt, fd_cap, src, raw, nb_rng, nb_off);
}

// P2P launch: well-separation and whether r^2 needs the kMinR2 floor
inline void launch_p2p(int ws, float eps2, int grid, cudaStream_t st, int nbox, const int *nbd, const int *bpid,
                       const int *start, const int4 *coord, const int *nbr, const double *qm, const double *roots,
                       int level, double *ax, double *ay, double *az, unsigned long long *counts,
                       const int *has_tgt, const float4 *rel, const int *fd = nullptr,
                       const int *fd_cnt = nullptr, int fd_cap = 0) {
    const bool clamp = !(eps2 >= kMinR2);
#define SV_P2P(W, C) p2p_kernel<W, C><<<grid, kWarps * 32, 0, st>>>(nbox, nbd, bpid, start, coord, nbr, qm, roots, \
                                                                   level, eps2, ax, ay, az, counts, has_tgt, rel,  \
                                                                   fd, fd_cnt, fd_cap)
    if (ws == 1) {
        if (clamp) SV_P2P(1, true);
        else SV_P2P(1, false);
    } else {
        if (clamp) SV_P2P(2, true);
        else SV_P2P(2, false);
    }
#undef SV_P2P
}

template <int P>
sv_status run_fmm(sv_ctx *c, Fmm &F, Tree &T) {
    constexpr int NC = ncoef(P);
    const int L = T.deepest;
    const int ws = F.ws;
    const int ns1 = 2 * ws + 1, ns = ns1 * ns1 * ns1;
    const int cap = ns * 8 - ns;
    Sorted &S = c->S;
    // arena: per level M, Loc, nbr, m2l, cnt, and M2L partials where a box's list is split
    auto rounded = [](size_t sz) { return (sz + 255) & ~(size_t)255; };
    int chunks[kMortonBits + 1];
    size_t bytes = 0;
    for (int l = 0; l <= L; l++) {
        const size_t nb = T.lv[l].nbox;
        chunks[l] = m2l_chunks((int)nb);
        bytes += 2 * rounded(nb * NC * sizeof(float2)) + rounded(nb * ns * sizeof(int)) +
                 rounded(nb * cap * sizeof(int2)) + rounded(nb * sizeof(int));
        if (chunks[l] > 1) bytes += rounded(nb * chunks[l] * NC * sizeof(float2));
    }
    for (int l = 0; l <= L; l++) bytes += rounded((size_t)T.lv[l].nbox * sizeof(uint64_t));  // box codes
    // far-direct lists of the leaf boxes (sv_params.fmm_direct_pairs; 0: 1024 pairs, < 0: none)
    const int fd_thresh = c->P.fmm_direct_pairs == 0 ? 1024 : c->P.fmm_direct_pairs;
    const bool use_fd = fd_thresh > 0 && L >= 2;
    if (use_fd) bytes += rounded((size_t)T.lv[L].nbox * (kFarDirectCap + 1) * sizeof(int));
    if (F.arena_bytes < bytes) {
        cudaFree(F.arena);
        F.arena = nullptr;
        F.arena_bytes = 0;
        const size_t want = bytes + bytes / 2;  // headroom: a growing tree reallocates rarely
        SV_CK(c, cudaMalloc(&F.arena, want));
        F.arena_bytes = want;
    }
    char *p = (char *)F.arena;
    auto carve = [&](size_t sz) {
        char *r = p;
        p += (sz + 255) & ~(size_t)255;
        return (void *)r;
    };
    float2 *Mv[kMortonBits + 1], *Lv[kMortonBits + 1], *part[kMortonBits + 1];
    int *nbr[kMortonBits + 1], *cnt[kMortonBits + 1];
    int2 *lst[kMortonBits + 1];
    for (int l = 0; l <= L; l++) {
        const size_t nb = T.lv[l].nbox;
        Mv[l] = (float2 *)carve(nb * NC * sizeof(float2));
        Lv[l] = (float2 *)carve(nb * NC * sizeof(float2));
        nbr[l] = (int *)carve(nb * ns * sizeof(int));
        lst[l] = (int2 *)carve(nb * cap * sizeof(int2));
        cnt[l] = (int *)carve(nb * sizeof(int));
        part[l] = chunks[l] > 1 ? (float2 *)carve(nb * chunks[l] * NC * sizeof(float2)) : Lv[l];
    }
    // every level's lists in two launches (near lists, then interaction lists)
    ListArgs la{};
    la.nlev = L + 1;
    for (int l = 0; l <= L; l++) {
        ListLevel &q = la.lv[l];
        q.nbox = T.lv[l].nbox;
        q.first = la.total;
        la.total += q.nbox;
        q.coord = T.lv[l].coord;
        q.code = (uint64_t *)carve((size_t)q.nbox * sizeof(uint64_t));
        q.nbr = nbr[l];
        q.parent = T.lv[l].parent;
        q.pchild0 = l > 0 ? T.lv[l - 1].child0 : nullptr;
        q.pnbr = l > 0 ? nbr[l - 1] : nullptr;
        q.m2l = lst[l];
        q.m2l_cnt = cnt[l];
        q.start = T.lv[l].start;
        q.fd = q.fd_cnt = nullptr;
    }
    la.fd_cap = kFarDirectCap;
    la.fd_thresh = fd_thresh;
    la.trim = F.trim;
    if (use_fd) {
        la.lv[L].fd = (int *)carve((size_t)T.lv[L].nbox * kFarDirectCap * sizeof(int));
        la.lv[L].fd_cnt = (int *)carve((size_t)T.lv[L].nbox * sizeof(int));
    }
    phase_mark(c, 2);
    SV_CK(c, cudaMemsetAsync(F.d_counts, 0, 3 * sizeof(unsigned long long), c->stream));
    // which boxes hold targets (all of them unless symmetry images are present)
    int *tgt[kMortonBits + 1];
    {
        int64_t tot = 0;
        for (int l = 0; l <= L; l++) tot += T.lv[l].nbox;
        if (F.tgt_cap < tot) {
            cudaFree(F.has_tgt);
            F.has_tgt = nullptr;
            const int64_t want = tot + tot / 2;  // headroom: a growing tree reallocates rarely
            SV_CK(c, cudaMalloc(&F.has_tgt, sizeof(int) * want));
            F.tgt_cap = want;
        }
        int64_t o = 0;
        for (int l = 0; l <= L; l++) {
            tgt[l] = F.has_tgt + o;
            o += T.lv[l].nbox;
        }
    }
    if (F.rel_cap < c->S.n) {
        cudaFree(F.rel);
        cudaFree(F.far);
        F.rel = nullptr;
        F.far = nullptr;
        SV_CK(c, cudaMalloc(&F.rel, sizeof(float4) * c->S.n));
        SV_CK(c, cudaMalloc(&F.far, 3 * sizeof(double) * c->S.n));
        F.rel_cap = c->S.n;
    }
    double *fx = F.far, *fy = F.far + F.rel_cap, *fz = F.far + 2 * F.rel_cap;
    // Two streams from here on.  The second takes the leaf level's target
    // flags, then the near and interaction lists of every level in two
    // launches (boxes found by binary search over each level's Morton codes),
    // then runs the near field (P2P), which needs only the sorted particles,
    // the leaf boxes and their near lists, and writes the accelerations.  The
    // main stream derives the coarser target flags and runs the upward pass,
    // then M2L / L2L and the far field (L2P or the treecode's M2P, into their
    // own arrays) beside the near field, then waits for it; the scatter to the
    // caller's order adds the two.
    SV_CK(c, cudaEventRecord(F.ev_fork, c->stream));
    SV_CK(c, cudaStreamWaitEvent(F.side, F.ev_fork, 0));
    {
        const Level &V = T.lv[L];
        leaf_targets_kernel<<<div_up(V.nbox, 256), 256, 0, F.side>>>(V.nbox, nullptr, V.start, S.qm, tgt[L]);
        SV_LAUNCHED(c);
        SV_CK(c, cudaEventRecord(F.ev_lists, F.side));
        box_codes_kernel<<<div_up(la.total, 256), 256, 0, F.side>>>(la);
        SV_LAUNCHED(c);
        const int64_t slots = (int64_t)la.total * ns;
        if (ws == 1) near_lists_kernel<1><<<div_up(slots, 256), 256, 0, F.side>>>(la);
        else near_lists_kernel<2><<<div_up(slots, 256), 256, 0, F.side>>>(la);
        SV_LAUNCHED(c);
        if (L > 0) {
            const int g = std::min(div_up(la.total - la.lv[1].first, kWarps), 16 * device_sms());
            if (ws == 1) m2l_lists_kernel<1><<<g, kWarps * 32, 0, F.side>>>(la, cap, F.d_counts);
            else m2l_lists_kernel<2><<<g, kWarps * 32, 0, F.side>>>(la, cap, F.d_counts);
            SV_LAUNCHED(c);
        }
        SV_CK(c, cudaEventRecord(F.ev_m2l_lists, F.side));
        box_relative_kernel<<<div_up(V.nbox, kWarps), kWarps * 32, 0, F.side>>>(
            V.nbox, nullptr, nullptr, V.start, V.coord, S.x, S.y, S.z, S.q, S.root, L, F.rel, F.d_counts + 2);
        SV_LAUNCHED(c);
        SV_CK(c, cudaEventRecord(F.ev_rel, F.side));
        if (c->P.profile_phases) SV_CK(c, cudaEventRecord(F.ev_near[0], F.side));
        launch_p2p(ws, (float)c->P.softening2, div_up(V.nbox, kWarps), F.side, V.nbox, nullptr, nullptr, V.start,
                   V.coord, nbr[L], S.qm, S.root, L, S.ax, S.ay, S.az, F.d_counts, tgt[L], F.rel, la.lv[L].fd,
                   la.lv[L].fd_cnt, kFarDirectCap);
        SV_LAUNCHED(c);
        if (c->P.profile_phases) {
            SV_CK(c, cudaEventRecord(F.ev_near[1], F.side));
            c->near_ev[0] = F.ev_near[0];
            c->near_ev[1] = F.ev_near[1];
        }
        SV_CK(c, cudaEventRecord(F.ev_join, F.side));
    }
    // coarser target flags from the leaf flags
    SV_CK(c, cudaStreamWaitEvent(c->stream, F.ev_lists, 0));
    for (int l = L - 1; l >= 0; l--) {
        parent_targets_kernel<<<div_up(T.lv[l].nbox, 256), 256, 0, c->stream>>>(T.lv[l].nbox, nullptr,
                                                                                T.lv[l].child0, tgt[l + 1], tgt[l]);
        SV_LAUNCHED(c);
    }
    phase_mark(c, 3);
    // upward pass
    {
        const Level &V = T.lv[L];
        p2m_kernel<P><<<div_up(V.nbox, p2m_warps<P>()), p2m_warps<P>() * 32, 0, c->stream>>>(
            V.nbox, nullptr, nullptr, V.start, V.coord, S.x, S.y, S.z, S.q, S.root, L, F.nrm, Mv[L]);
        SV_LAUNCHED(c);
    }
    for (int l = L - 1; l >= 2; l--) {
        const Level &V = T.lv[l];
        m2m_kernel<P><<<div_up(V.nbox, kWarps), kWarps * 32, 0, c->stream>>>(
            V.nbox, nullptr, V.child0, T.lv[l + 1].coord, Mv[l + 1], Mv[l], F.otab);
        SV_LAUNCHED(c);
    }
    SV_CK(c, cudaStreamWaitEvent(c->stream, F.ev_m2l_lists, 0));
    phase_mark(c, 4);
    const bool treecode = c->P.fmm_type == SV_FMM_TREECODE || c->P.fmm_type == SV_FMM_TREECODE_OUTLIERS;
    // downward pass: M2L of all levels in one launch, then L2L level by level
    // (the treecode evaluates multipoles at the particles instead)
    F.tc.launched = false;
    if (!treecode && L >= 2) {
        M2LArgs a{};
        a.cap = cap;
        a.esz = F.H.esz;
        a.osz = F.H.osz;
        a.dsz = F.H.dsz;
        a.eps2 = c->P.softening2;
        a.root = S.root;
        a.cls_theta = F.cls_theta;
        a.cls_phase = F.cls_phase;
        a.cls_rho2 = F.cls_rho2;
        a.dmat = F.dmat;
        a.zc = F.zc;
        int warps = 0;
        for (int l = 2; l <= L; l++) {
            M2LLevel &V = a.lv[a.nlev++];
            V.nbox = T.lv[l].nbox;
            V.chunks = chunks[l];
            V.warp0 = warps;
            V.level = l;
            V.nbd = nullptr;
            V.bpid = nullptr;
            V.m2l = lst[l];
            V.cnt = cnt[l];
            V.has_tgt = tgt[l];
            V.M = Mv[l];
            V.out = part[l];
            warps += V.nbox * V.chunks;
        }
        if (c->P.fmm_m2l_tc >= 0) {
            // the tensor-core M2L; the rotation kernel below runs only if it overflowed its room
            TcArgs ta{};
            ta.nlev = a.nlev;
            ta.cap = cap;
            ta.eps2 = c->P.softening2;
            ta.root = S.root;
            ta.cls_rho2 = F.cls_rho2;
            int64_t boxes = 0;
            for (int k = 0; k < a.nlev; k++) {
                const M2LLevel &V = a.lv[k];
                TcLevel &q = ta.lv[k];
                q.nbox = V.nbox;
                q.level = V.level;
                q.chunks = V.chunks;
                q.warp0 = V.warp0;
                q.first = (int)boxes;
                q.nbd = nullptr;
                q.bpid = nullptr;
                q.m2l = lst[V.level];
                q.cnt = V.cnt;
                q.has_tgt = V.has_tgt;
                q.M = V.M;
                q.out = V.out;
                boxes += V.nbox;
            }
            ta.total_boxes = (int)boxes;
            // room: the last evaluation's translations (read back by then) with a margin, at least 32 per box
            const int64_t last = F.tc.h_ctl && F.tc.p == P && F.tc.ws == ws ? F.tc.h_ctl[0] : 0;
            SV_TRY(m2l_tc_prepare(c, F.tc, P, ws, std::max<int64_t>(last + last / 4, 32 * boxes)));
            ta.ncls = F.tc.ncls;
            SV_TRY(m2l_tc_launch(c, F.tc, ta, warps, c->stream));
            a.run_if = m2l_tc_skip_flag(F.tc);
            F.tc.launched = true;
        }
        m2l_kernel<P><<<div_up(warps, m2l_warps<P>()), m2l_warps<P>() * 32, 0, c->stream>>>(a);
        SV_LAUNCHED(c);
        for (int l = 2; l <= L; l++) {
            const Level &V = T.lv[l];
            L2LArgs b{};
            b.nbox = V.nbox;
            b.chunks = chunks[l];
            b.has_parent = l > 2;
            b.nbd = nullptr;
            b.parent = V.parent;
            b.coord = V.coord;
            b.has_tgt = tgt[l];
            b.Lp = l > 2 ? Lv[l - 1] : nullptr;
            b.part = part[l];
            b.L = Lv[l];
            b.otab = F.otab;
            l2l_kernel<P><<<div_up(V.nbox, kWarps), kWarps * 32, 0, c->stream>>>(b);
            SV_LAUNCHED(c);
        }
    }
    phase_mark(c, 5);
    // far field into its own arrays, beside the near field
    S.far = nullptr;
    {
        const Level &V = T.lv[L];
        if (L >= 2 && treecode) {
            TreecodeArgs ta{};
            ta.L = L;
            ta.cap = cap;
            ta.ws = ws;
            ta.nleaf = V.nbox;
            for (int l = 0; l <= L; l++) {
                ta.parent[l] = T.lv[l].parent;
                ta.coord[l] = T.lv[l].coord;
                ta.m2l[l] = lst[l];
                ta.m2l_cnt[l] = cnt[l];
                ta.M[l] = Mv[l];
            }
            ta.leaf_start = V.start;
            ta.has_tgt = tgt[L];
            ta.x = S.x;
            ta.y = S.y;
            ta.z = S.z;
            ta.qm = S.qm;
            ta.root = S.root;
            ta.nrm = F.nrm;
            ta.eps2 = c->P.softening2;
            ta.ax = fx;
            ta.ay = fy;
            ta.az = fz;
            ta.accumulate = 0;
            m2p_kernel<P><<<div_up(V.nbox, kWarps), kWarps * 32, 0, c->stream>>>(ta);
            SV_LAUNCHED(c);
            S.far = F.far;
        } else if (L >= 2) {
            SV_CK(c, cudaStreamWaitEvent(c->stream, F.ev_rel, 0));  // the leaf offsets of the second stream
            l2p_kernel<P><<<div_up(V.nbox, kWarps), kWarps * 32, 0, c->stream>>>(
                V.nbox, nullptr, nullptr, V.start, F.rel, S.qm, S.root, L, F.nrm, Lv[L], fx, fy, fz, tgt[L], 0);
            SV_LAUNCHED(c);
            S.far = F.far;
        }
        S.far_stride = F.rel_cap;
        phase_mark(c, 6);
    }
    SV_CK(c, cudaStreamWaitEvent(c->stream, F.ev_join, 0));
    SV_CK(c, cudaMemcpyAsync(F.h_counts, F.d_counts, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                             c->stream));
    c->stats.levels = L;
    c->stats.boxes = T.lv[L].nbox;
    return SV_OK;
}


// ------------------------------------------------------------------ forest --
inline int forest_grid(int cap, int per_cta) {
    const int g = div_up(cap > 0 ? cap : 1, per_cta);
    const int gmax = 16 * device_sms();  // grid-stride launches: at most 16 CTAs per SM
    return g < gmax ? g : gmax;
}

template <int P>
sv_status run_fmm_forest(sv_ctx *c, Fmm &F, const ForestArgs &fa) {
    const ForestSpec &f = fa.spec;
    const int L = f.L;
    const int ws = F.ws;
    const int ns1 = 2 * ws + 1, ns = ns1 * ns1 * ns1;
    const int cap = ns * 8 - ns;
    Sorted &S = c->S;
    Tree &T = *F.ftree;
    int *nbd = fa.d_nbox;
    SV_TRY(tree_build_forest(c, T, f, nbd, fa.d_err));
    SV_CK(c, cudaMemsetAsync(F.d_counts, 0, 3 * sizeof(unsigned long long), c->stream));
    // Two streams, as in run_fmm: target flags, lists and the near field on the
    // second (the forest's slots only: the direct plumes' slots belong to
    // another stream), the upward and downward passes on the main one.
    cudaStream_t sd = F.side;
    SV_CK(c, cudaEventRecord(F.ev_fork, c->stream));
    SV_CK(c, cudaStreamWaitEvent(sd, F.ev_fork, 0));
    root_nbr_kernel<<<forest_grid(f.cap[0] * ns, 256), 256, 0, sd>>>(F.fnbr[0], ns, f.cap[0], nbd);
    SV_LAUNCHED(c);
    leaf_targets_kernel<<<forest_grid(f.cap[L], 256), 256, 0, sd>>>(f.cap[L], nbd + L, T.lv[L].start, S.qm,
                                                                  F.ftgt[L]);
    SV_LAUNCHED(c);
    for (int l = L - 1; l >= 0; l--) {
        parent_targets_kernel<<<forest_grid(f.cap[l], 256), 256, 0, sd>>>(f.cap[l], nbd + l, T.lv[l].child0,
                                                                        F.ftgt[l + 1], F.ftgt[l]);
        SV_LAUNCHED(c);
    }
    // far-direct lists at the leaf level (sv_params.fmm_direct_pairs, as the single tree's)
    const int fd_thresh = c->P.fmm_direct_pairs == 0 ? 1024 : c->P.fmm_direct_pairs;
    for (int l = 1; l <= L; l++) {
        const Level &V = T.lv[l];
        const Level &U = T.lv[l - 1];
        const bool fdl = l == L && fd_thresh > 0;
        if (ws == 1)
            build_lists_kernel<1><<<forest_grid(f.cap[l], kWarps), kWarps * 32, 0, sd>>>(
                f.cap[l], nbd + l, V.parent, V.coord, F.fnbr[l - 1], U.child0, F.fnbr[l], F.flst[l], F.fcnt[l], cap,
                F.trim, F.d_counts, V.start, fdl ? F.ffd : nullptr, F.ffd_cnt, kFarDirectCap, fd_thresh);
        else
            build_lists_kernel<2><<<forest_grid(f.cap[l], kWarps), kWarps * 32, 0, sd>>>(
                f.cap[l], nbd + l, V.parent, V.coord, F.fnbr[l - 1], U.child0, F.fnbr[l], F.flst[l], F.fcnt[l], cap,
                F.trim, F.d_counts, V.start, fdl ? F.ffd : nullptr, F.ffd_cnt, kFarDirectCap, fd_thresh);
        SV_LAUNCHED(c);
    }
    SV_CK(c, cudaEventRecord(F.ev_lists, sd));
    {
        const Level &V = T.lv[L];
        const int g = forest_grid(f.cap[L], kWarps);
        SV_CK(c, cudaMemsetAsync(S.ax, 0, sizeof(double) * f.n, sd));
        SV_CK(c, cudaMemsetAsync(S.ay, 0, sizeof(double) * f.n, sd));
        SV_CK(c, cudaMemsetAsync(S.az, 0, sizeof(double) * f.n, sd));
        box_relative_kernel<<<g, kWarps * 32, 0, sd>>>(f.cap[L], nbd + L, V.pid, V.start, V.coord, S.x, S.y, S.z,
                                                       S.q, fa.roots, L, F.frel, F.d_counts + 2);
        SV_LAUNCHED(c);
        launch_p2p(ws, (float)c->P.softening2, g, sd, f.cap[L], nbd + L, V.pid, V.start, V.coord, F.fnbr[L], S.qm,
                   fa.roots, L, S.ax, S.ay, S.az, F.d_counts, F.ftgt[L], F.frel, fd_thresh > 0 ? F.ffd : nullptr,
                   F.ffd_cnt, kFarDirectCap);
        SV_LAUNCHED(c);
        SV_CK(c, cudaEventRecord(F.ev_join, sd));
    }
    {
        const Level &V = T.lv[L];
        p2m_kernel<P><<<forest_grid(f.cap[L], p2m_warps<P>()), p2m_warps<P>() * 32, 0, c->stream>>>(
            f.cap[L], nbd + L, V.pid, V.start, V.coord, S.x, S.y, S.z, S.q, fa.roots, L, F.nrm, F.fM[L]);
        SV_LAUNCHED(c);
    }
    for (int l = L - 1; l >= 2; l--) {
        const Level &V = T.lv[l];
        m2m_kernel<P><<<forest_grid(f.cap[l], kWarps), kWarps * 32, 0, c->stream>>>(
            f.cap[l], nbd + l, V.child0, T.lv[l + 1].coord, F.fM[l + 1], F.fM[l], F.otab);
        SV_LAUNCHED(c);
    }
    SV_CK(c, cudaStreamWaitEvent(c->stream, F.ev_lists, 0));
    {
        M2LArgs a{};
        a.cap = cap;
        a.esz = F.H.esz;
        a.osz = F.H.osz;
        a.dsz = F.H.dsz;
        a.eps2 = c->P.softening2;
        a.root = fa.roots;
        a.cls_theta = F.cls_theta;
        a.cls_phase = F.cls_phase;
        a.cls_rho2 = F.cls_rho2;
        a.dmat = F.dmat;
        a.zc = F.zc;
        long long warps = 0;
        for (int l = 2; l <= L; l++) {
            M2LLevel &V = a.lv[a.nlev++];
            V.nbox = f.cap[l];
            V.chunks = F.fchunks[l];
            V.warp0 = (int)warps;
            V.level = l;
            V.nbd = nbd + l;
            V.bpid = T.lv[l].pid;
            V.m2l = F.flst[l];
            V.cnt = F.fcnt[l];
            V.has_tgt = F.ftgt[l];
            V.M = F.fM[l];
            V.out = F.fpart[l];
            warps += (long long)V.nbox * V.chunks;
        }
        F.tc.launched = false;
        if (c->P.fmm_m2l_tc >= 0 && F.tc.cap > 0 && F.tc.p == P && F.tc.ws == ws) {
            // the tensor-core M2L (room reserved with the forest); the rotation
            // kernel below runs only if the translations overflowed it
            TcArgs ta{};
            ta.nlev = a.nlev;
            ta.cap = cap;
            ta.eps2 = c->P.softening2;
            ta.root = fa.roots;
            ta.cls_rho2 = F.cls_rho2;
            ta.ncls = F.tc.ncls;
            long long boxes = 0;
            for (int k = 0; k < a.nlev; k++) {
                const M2LLevel &V = a.lv[k];
                TcLevel &q = ta.lv[k];
                q.nbox = V.nbox;
                q.level = V.level;
                q.chunks = V.chunks;
                q.warp0 = V.warp0;
                q.first = (int)boxes;
                q.nbd = V.nbd;
                q.bpid = V.bpid;
                q.m2l = F.flst[V.level];
                q.cnt = V.cnt;
                q.has_tgt = V.has_tgt;
                q.M = V.M;
                q.out = V.out;
                boxes += V.nbox;
            }
            ta.total_boxes = (int)boxes;
            SV_TRY(m2l_tc_launch(c, F.tc, ta, (int)warps, c->stream));
            a.run_if = m2l_tc_skip_flag(F.tc);
            F.tc.launched = true;
        }
        m2l_kernel<P><<<(int)((warps + m2l_warps<P>() - 1) / m2l_warps<P>()), m2l_warps<P>() * 32, 0,
                          c->stream>>>(a);
        SV_LAUNCHED(c);
        for (int l = 2; l <= L; l++) {
            const Level &V = T.lv[l];
            L2LArgs b{};
            b.nbox = f.cap[l];
            b.chunks = F.fchunks[l];
            b.has_parent = l > 2;
            b.nbd = nbd + l;
            b.parent = V.parent;
            b.coord = V.coord;
            b.has_tgt = F.ftgt[l];
            b.Lp = l > 2 ? F.fL[l - 1] : nullptr;
            b.part = F.fpart[l];
            b.L = F.fL[l];
            b.otab = F.otab;
            l2l_kernel<P><<<forest_grid(f.cap[l], kWarps), kWarps * 32, 0, c->stream>>>(b);
            SV_LAUNCHED(c);
        }
    }
    SV_CK(c, cudaStreamWaitEvent(c->stream, F.ev_join, 0));
    {
        const Level &V = T.lv[L];
        const int g = forest_grid(f.cap[L], kWarps);
        l2p_kernel<P><<<g, kWarps * 32, 0, c->stream>>>(f.cap[L], nbd + L, V.pid, V.start, F.frel, S.qm, fa.roots,
                                                        L, F.nrm, F.fL[L], S.ax, S.ay, S.az, F.ftgt[L], 1);
        SV_LAUNCHED(c);
    }
    SV_CK(c, cudaMemcpyAsync(F.h_counts, F.d_counts, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                             c->stream));
    return SV_OK;
}

sv_status ensure_tables(sv_ctx *c, Fmm &F, int p, int ws) {
    if (F.p == p && F.ws == ws && F.dmat) return SV_OK;
    std::string err;
    if (!build_fmm_tables(p, ws, F.H, err)) return set_error(c, SV_ERR_INVALID, "FMM tables: %s", err.c_str());
    cudaFree(F.cls_theta); cudaFree(F.cls_phase); cudaFree(F.cls_rho2); cudaFree(F.dmat);
    cudaFree(F.zc); cudaFree(F.nrm); cudaFree(F.otab);
    const FmmTables &H = F.H;
    SV_CK(c, cudaMalloc(&F.cls_theta, sizeof(int) * H.cls_theta.size()));
    SV_CK(c, cudaMalloc(&F.cls_phase, sizeof(float) * H.cls_phase.size()));
    SV_CK(c, cudaMalloc(&F.cls_rho2, sizeof(float) * H.cls_rho2.size()));
    SV_CK(c, cudaMalloc(&F.dmat, sizeof(float) * H.dmat.size()));
    SV_CK(c, cudaMalloc(&F.zc, sizeof(float) * H.zc.size()));
    SV_CK(c, cudaMalloc(&F.nrm, sizeof(float) * H.nrm.size()));
    SV_CK(c, cudaMalloc(&F.otab, sizeof(float) * H.otab.size()));
    SV_CK(c, cudaMemcpy(F.cls_theta, H.cls_theta.data(), sizeof(int) * H.cls_theta.size(), cudaMemcpyHostToDevice));
    SV_CK(c, cudaMemcpy(F.cls_phase, H.cls_phase.data(), sizeof(float) * H.cls_phase.size(), cudaMemcpyHostToDevice));
    SV_CK(c, cudaMemcpy(F.cls_rho2, H.cls_rho2.data(), sizeof(float) * H.cls_rho2.size(), cudaMemcpyHostToDevice));
    SV_CK(c, cudaMemcpy(F.dmat, H.dmat.data(), sizeof(float) * H.dmat.size(), cudaMemcpyHostToDevice));
    SV_CK(c, cudaMemcpy(F.zc, H.zc.data(), sizeof(float) * H.zc.size(), cudaMemcpyHostToDevice));
    SV_CK(c, cudaMemcpy(F.nrm, H.nrm.data(), sizeof(float) * H.nrm.size(), cudaMemcpyHostToDevice));
    SV_CK(c, cudaMemcpy(F.otab, H.otab.data(), sizeof(float) * H.otab.size(), cudaMemcpyHostToDevice));
    F.p = p;
    F.ws = ws;
    return SV_OK;
}

}  // namespace

void fmm_free(sv_ctx *c) {
    if (!c->fmm) return;
    Fmm &F = *c->fmm;
    cudaFree(F.cls_theta); cudaFree(F.cls_phase); cudaFree(F.cls_rho2); cudaFree(F.dmat);
    cudaFree(F.zc); cudaFree(F.nrm); cudaFree(F.otab); cudaFree(F.arena); cudaFree(F.d_counts);
    cudaFree(F.ex); cudaFree(F.ey); cudaFree(F.ez); cudaFree(F.eq); cudaFree(F.em); cudaFree(F.est);
    cudaFree(F.eoff); cudaFree(F.has_tgt); cudaFree(F.rel); cudaFree(F.far);
    cudaFree(F.farena); cudaFree(F.frel);
    m2l_tc_free(F.tc);
    if (F.ftree) {
        tree_release(*F.ftree);
        delete F.ftree;
    }
    cudaFreeHost(F.h_counts);
    if (F.side) cudaStreamDestroy(F.side);
    if (F.ev_fork) cudaEventDestroy(F.ev_fork);
    if (F.ev_join) cudaEventDestroy(F.ev_join);
    if (F.ev_lists) cudaEventDestroy(F.ev_lists);
    if (F.ev_m2l_lists) cudaEventDestroy(F.ev_m2l_lists);
    if (F.ev_rel) cudaEventDestroy(F.ev_rel);
    for (cudaEvent_t e : F.ev_near)
        if (e) cudaEventDestroy(e);
    c->near_ev[0] = c->near_ev[1] = nullptr;
    delete c->fmm;
    c->fmm = nullptr;
}

static sv_status fmm_state(sv_ctx *c) {
    if (!c->fmm) {
        c->fmm = new Fmm();
        Fmm &F = *c->fmm;
        SV_CK(c, cudaMalloc(&F.d_counts, 3 * sizeof(unsigned long long)));
        SV_CK(c, cudaMallocHost(&F.h_counts, 2 * sizeof(unsigned long long)));
        SV_CK(c, cudaStreamCreateWithFlags(&F.side, cudaStreamNonBlocking));
        SV_CK(c, cudaEventCreateWithFlags(&F.ev_fork, cudaEventDisableTiming));
        SV_CK(c, cudaEventCreateWithFlags(&F.ev_join, cudaEventDisableTiming));
        SV_CK(c, cudaEventCreateWithFlags(&F.ev_lists, cudaEventDisableTiming));
        SV_CK(c, cudaEventCreateWithFlags(&F.ev_m2l_lists, cudaEventDisableTiming));
        SV_CK(c, cudaEventCreateWithFlags(&F.ev_rel, cudaEventDisableTiming));
        SV_CK(c, cudaEventCreate(&F.ev_near[0]));
        SV_CK(c, cudaEventCreate(&F.ev_near[1]));
    }
    return SV_OK;
}

sv_status fmm_sort_images(sv_ctx *c, int64_t first, int64_t last) {
    SV_TRY(fmm_state(c));
    Fmm &F = *c->fmm;
    const int64_t n = c->n;
    int kind = 0, nimg = 1;
    std::vector<double> off;
    if (c->P.symmetry == SV_SYM_ROTATIONAL) {
        kind = 1;
        nimg = 4;
    } else if (c->P.symmetry == SV_SYM_TRANSLATIONAL) {
        kind = 2;
        std::vector<double> h(3 * 4096);
        nimg = trans_images(c->P, h.data(), 4096);
        if (nimg <= 0 || nimg > 4096) return set_error(c, SV_ERR_INVALID, "bad translational image set (%d)", nimg);
        // the zero offset (the particles themselves) goes first
        off.reserve(3 * nimg);
        int zero = -1;
        for (int g = 0; g < nimg; g++)
            if (h[3 * g] == 0.0 && h[3 * g + 1] == 0.0 && h[3 * g + 2] == 0.0) zero = g;
        if (zero < 0) return set_error(c, SV_ERR_INVALID, "image set without the zero offset");
        off.insert(off.end(), {0.0, 0.0, 0.0});
        for (int g = 0; g < nimg; g++)
            if (g != zero) off.insert(off.end(), {h[3 * g], h[3 * g + 1], h[3 * g + 2]});
    }
    const int64_t ne = n * nimg;
    if (ne > (int64_t)INT32_MAX) return set_error(c, SV_ERR_CAPACITY, "%lld particles with images", (long long)ne);
    if (F.ecap < ne) {
        cudaFree(F.ex); cudaFree(F.ey); cudaFree(F.ez); cudaFree(F.eq); cudaFree(F.em); cudaFree(F.est);
        F.ex = F.ey = F.ez = F.eq = F.em = nullptr;
        F.est = nullptr;
        SV_CK(c, cudaMalloc(&F.ex, sizeof(double) * ne));
        SV_CK(c, cudaMalloc(&F.ey, sizeof(double) * ne));
        SV_CK(c, cudaMalloc(&F.ez, sizeof(double) * ne));
        SV_CK(c, cudaMalloc(&F.eq, sizeof(double) * ne));
        SV_CK(c, cudaMalloc(&F.em, sizeof(double) * ne));
        SV_CK(c, cudaMalloc(&F.est, sizeof(int32_t) * ne));
        F.ecap = ne;
    }
    if (kind == 2) {
        if (F.eoff_cap < nimg) {
            cudaFree(F.eoff);
            F.eoff = nullptr;
            SV_CK(c, cudaMalloc(&F.eoff, sizeof(double) * 3 * nimg));
            F.eoff_cap = nimg;
        }
        SV_CK(c, cudaMemcpyAsync(F.eoff, off.data(), sizeof(double) * 3 * nimg, cudaMemcpyHostToDevice, c->stream));
        // the host vector must outlive the copy
        SV_CK(c, cudaStreamSynchronize(c->stream));
    }
    expand_images_kernel<<<div_up(ne, 256), 256, 0, c->stream>>>(c->x, c->y, c->z, c->q, c->m, force_status(c), n, kind,
                                                                 nimg, F.eoff, F.ex, F.ey, F.ez, F.eq, F.em, F.est);
    SV_LAUNCHED(c);
    const ParticleView v{F.ex, F.ey, F.ez, F.eq, F.em, F.est, ne, n};
    return sort_view(c, v, first, last);
}

int fmm_sort_levels(const sv_ctx *c) {
    const int h = c->fmm ? c->fmm->level_hint : -1;
    return h >= 2 ? std::min(kMortonBits, h + 1) : kMortonBits;
}

sv_status fmm_accel(sv_ctx *c) {
    if (c->P.precision != SV_PREC_MIXED)
        return set_error(c, SV_ERR_UNSUPPORTED, "FMM runs in mixed precision only");
    const int p = c->P.fmm_order;
    if (p != 4 && p != 6 && p != 8 && p != 10)
        return set_error(c, SV_ERR_UNSUPPORTED, "FMM order %d not instantiated (4, 6, 8, 10)", p);
    SV_TRY(fmm_state(c));
    Fmm &F = *c->fmm;
    SV_TRY(ensure_tables(c, F, p, c->P.fmm_ws));
    F.trim = c->P.fmm_near == 2 && c->P.fmm_ws == 2;
    Tree *T = nullptr;
    c->S.resort = false;
    SV_TRY(tree_build(c, kDepthMeanOccupancy, c->P.fmm_leaf_target, &T));
    // the depth rule's box counts are exact down to the sorted levels only; a
    // leaf level at or below them needs the full order
    if (T->n_act > 0 && T->deepest >= c->S.key_levels && c->S.key_levels < kMortonBits) {
        c->S.resort = true;
        return SV_OK;
    }
    F.level_hint = T->deepest;
    if (T->n_act == 0) {
        SV_CK(c, cudaMemsetAsync(c->S.ax, 0, sizeof(double) * c->S.n, c->stream));
        SV_CK(c, cudaMemsetAsync(c->S.ay, 0, sizeof(double) * c->S.n, c->stream));
        SV_CK(c, cudaMemsetAsync(c->S.az, 0, sizeof(double) * c->S.n, c->stream));
        return SV_OK;
    }
    switch (p) {
    case 4: SV_TRY(run_fmm<4>(c, F, *T)); break;
    case 6: SV_TRY(run_fmm<6>(c, F, *T)); break;
    case 8: SV_TRY(run_fmm<8>(c, F, *T)); break;
    default: SV_TRY(run_fmm<10>(c, F, *T)); break;
    }
    return SV_OK;
}

sv_status fmm_forest_reserve(sv_ctx *c, const ForestArgs &fa) {
    const int p = fa.p;
    if (p != 4 && p != 6 && p != 8 && p != 10)
        return set_error(c, SV_ERR_UNSUPPORTED, "FMM order %d not instantiated (4, 6, 8, 10)", p);
    if (fa.ws != 1 && fa.ws != 2) return set_error(c, SV_ERR_INVALID, "well-separation must be 1 or 2");
    const ForestSpec &f = fa.spec;
    if (f.L < 2 || f.L > kMortonBits) return set_error(c, SV_ERR_INVALID, "forest leaf level %d", f.L);
    SV_TRY(fmm_state(c));
    Fmm &F = *c->fmm;
    SV_TRY(ensure_tables(c, F, p, fa.ws));
    F.trim = c->P.fmm_near == 2 && fa.ws == 2;
    if (!F.ftree) F.ftree = new Tree();
    SV_TRY(tree_forest_reserve(c, *F.ftree, f));
    const int NC = p * (p + 1) / 2;
    const int ns1 = 2 * fa.ws + 1, ns = ns1 * ns1 * ns1, cap = 7 * ns;
    auto rounded = [](size_t sz) { return (sz + 255) & ~(size_t)255; };
    size_t bytes = 0;
    for (int l = 0; l <= f.L; l++) {
        const size_t nb = (size_t)f.cap[l];
        F.fchunks[l] = m2l_chunks((int)nb);
        bytes += 2 * rounded(nb * NC * sizeof(float2)) + rounded(nb * ns * sizeof(int)) +
                 rounded(nb * cap * sizeof(int2)) + 2 * rounded(nb * sizeof(int));
        if (F.fchunks[l] > 1) bytes += rounded(nb * F.fchunks[l] * NC * sizeof(float2));
    }
    bytes += rounded((size_t)f.cap[f.L] * kFarDirectCap * sizeof(int)) + rounded((size_t)f.cap[f.L] * sizeof(int));
    if (F.farena_bytes < bytes) {
        cudaFree(F.farena);
        F.farena = nullptr;
        F.farena_bytes = 0;
        SV_CK(c, cudaMalloc(&F.farena, bytes));
        F.farena_bytes = bytes;
    }
    char *q = (char *)F.farena;
    auto carve = [&](size_t sz) {
        char *r = q;
        q += (sz + 255) & ~(size_t)255;
        return (void *)r;
    };
    for (int l = 0; l <= kMortonBits; l++) {
        F.fM[l] = F.fL[l] = F.fpart[l] = nullptr;
        F.fnbr[l] = F.fcnt[l] = F.ftgt[l] = nullptr;
        F.flst[l] = nullptr;
    }
    for (int l = 0; l <= f.L; l++) {
        const size_t nb = (size_t)f.cap[l];
        F.fM[l] = (float2 *)carve(nb * NC * sizeof(float2));
        F.fL[l] = (float2 *)carve(nb * NC * sizeof(float2));
        F.fnbr[l] = (int *)carve(nb * ns * sizeof(int));
        F.flst[l] = (int2 *)carve(nb * cap * sizeof(int2));
        F.fcnt[l] = (int *)carve(nb * sizeof(int));
        F.ftgt[l] = (int *)carve(nb * sizeof(int));
        F.fpart[l] = F.fchunks[l] > 1 ? (float2 *)carve(nb * F.fchunks[l] * NC * sizeof(float2)) : F.fL[l];
    }
    F.ffd = (int *)carve((size_t)f.cap[f.L] * kFarDirectCap * sizeof(int));
    F.ffd_cnt = (int *)carve((size_t)f.cap[f.L] * sizeof(int));
    if (c->P.fmm_m2l_tc >= 0 && f.L >= 2) {
        // room of the tensor-core M2L: the last run's translations with a
        // margin, at least 32 per box of the M2L levels (a graph keeps the
        // buffers' addresses, so the room only changes here, at plan time)
        int64_t boxes = 0;
        for (int l = 2; l <= f.L; l++) boxes += f.cap[l];
        const int64_t last = F.tc.h_ctl && F.tc.p == p && F.tc.ws == fa.ws ? F.tc.h_ctl[0] : 0;
        SV_TRY(m2l_tc_prepare(c, F.tc, p, fa.ws, std::max<int64_t>(last + last / 4, 32 * boxes)));
    }
    if (F.frel_cap < f.n) {
        cudaFree(F.frel);
        F.frel = nullptr;
        SV_CK(c, cudaMalloc(&F.frel, sizeof(float4) * (size_t)std::max(f.n, 1)));
        F.frel_cap = f.n;
    }
    return SV_OK;
}

sv_status fmm_forest_tc_grow(sv_ctx *c) {
    Fmm &F = *c->fmm;
    const int64_t need = F.tc.h_ctl ? F.tc.h_ctl[0] : 0;  // the true count of the run that overflowed
    // expanding plumes add ~25 % translations per step: four times the count
    // lasts ~6 steps; the room stays within 40 % of the device's memory
    // (beyond it the rotation kernel takes the translations that do not fit)
    size_t free_b = 0, total_b = 0;
    SV_CK(c, cudaMemGetInfo(&free_b, &total_b));
    const int p = F.tc.p;
    const double per_entry = 16.0 + (double)(((size_t)p * (p + 1) * 4 + 15) / 16 * 16);
    const int64_t limit = (int64_t)(0.4 * (double)total_b / per_entry);
    const int64_t want = std::min<int64_t>(4 * need, limit);
    if (want <= F.tc.cap) return SV_OK;
    return m2l_tc_prepare(c, F.tc, p, F.tc.ws, want, true);
}

bool fmm_forest_tc_used(const sv_ctx *c) {
    const Fmm *F = c->fmm;
    return F && F->tc.launched && F->tc.h_ctl && !F->tc.h_ctl[2];
}

bool fmm_forest_tc_overflowed(const sv_ctx *c) {
    const Fmm *F = c->fmm;
    return F && F->tc.launched && F->tc.h_ctl && F->tc.h_ctl[2];
}

__global__ void max_count_kernel(const int4 *__restrict__ coord, const int *__restrict__ nbd, int cap,
                                 int *__restrict__ out) {
    const int nb = level_boxes(cap, nbd);
    int m = 0;
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += gridDim.x * blockDim.x) m = max(m, coord[b].w);
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m) atomicMax(out, m);
}

sv_status fmm_forest_max_leaf(sv_ctx *c, const ForestArgs &fa, int *out) {
    if (!c->fmm || !c->fmm->ftree) {
        *out = 0;
        return SV_OK;
    }
    const int L = fa.spec.L;
    int *d = nullptr;
    SV_CK(c, cudaMallocAsync(&d, sizeof(int), c->stream));
    SV_CK(c, cudaMemsetAsync(d, 0, sizeof(int), c->stream));
    max_count_kernel<<<forest_grid(fa.spec.cap[L], 256), 256, 0, c->stream>>>(c->fmm->ftree->lv[L].coord,
                                                                             fa.d_nbox + L, fa.spec.cap[L], d);
    SV_CK(c, cudaMemcpyAsync(c->h_scalar, d, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    SV_CK(c, cudaFreeAsync(d, c->stream));
    SV_CK(c, cudaStreamSynchronize(c->stream));
    memcpy(out, c->h_scalar, sizeof(int));
    return SV_OK;
}

sv_status fmm_forest_run(sv_ctx *c, const ForestArgs &fa) {
    if (fa.spec.n <= 0) return SV_OK;
    Fmm &F = *c->fmm;
    switch (fa.p) {
    case 4: return run_fmm_forest<4>(c, F, fa);
    case 6: return run_fmm_forest<6>(c, F, fa);
    case 8: return run_fmm_forest<8>(c, F, fa);
    default: return run_fmm_forest<10>(c, F, fa);
    }
}

sv_status fmm_counts(sv_ctx *c, double *m2l, double *pairs) {
    if (!c->fmm) {
        *m2l = *pairs = 0;
        return SV_OK;
    }
    SV_CK(c, cudaStreamSynchronize(c->stream));
    *m2l = (double)c->fmm->h_counts[0];
    *pairs = (double)c->fmm->h_counts[1];
    const M2LTc &tc = c->fmm->tc;
    c->stats.m2l_tc = tc.launched && tc.h_ctl && !tc.h_ctl[2];
    if (tc.launched && tc.h_ctl && tc.h_ctl[3])
        return set_error(c, SV_ERR_TIMEOUT, "tensor-core M2L: a bounded wait on the tensor cores gave up");
    return SV_OK;
}

}  // namespace sv
