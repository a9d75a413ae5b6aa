// tree.cu -- sparse octree over the Morton-sorted plume, built level by level.
//
// Stands in for the reference's two tree builders: the Barnes-Hut pointer
// octree (cell.cpp:7-175, barnes_hut_force_calculation.cpp:224-331, one
// particle per leaf, built serially by insertion) and the FMM's uniform-depth
// Morton boxes (multipole_method_force_calculation.cpp:883-1377: Morton keys,
// counting sort, particleOffset ranges, countNonEmptyBoxes).
//
// Here every level l = 0..deepest is a sorted array of the occupied boxes:
// box b at level l owns the contiguous particle range [start[b], start[b+1])
// of the sorted plume, has integer coordinates (ix, iy, iz) in units of
// S/2^l, a parent at level l-1 and a contiguous range of children at level
// l+1.  All of it comes from one quantity per particle, lvl[i] = the coarsest
// level at which particle i and i-1 fall into different boxes (from the
// highest differing bit of their Morton keys): particle i starts a box at
// every level >= lvl[i].
#include <algorithm>
#include <vector>

#include "sv_internal.cuh"
#include "tree.cuh"

namespace sv {
namespace {

constexpr int kLevels = kMortonBits + 1;  // levels 0..21

__global__ void split_levels(const uint64_t *__restrict__ keys, int n, uint8_t *__restrict__ lvl,
                             int *__restrict__ hist, int *__restrict__ n_act) {
    __shared__ int sh[kLevels + 1];
    if (threadIdx.x <= kLevels) sh[threadIdx.x] = 0;
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const uint64_t k = keys[i];
        const bool act = k != kInactiveKey;
        const bool prev_act = i > 0 && keys[i - 1] != kInactiveKey;
        if (act && !prev_act && i > 0) {
            // cannot happen: inactive keys sort last
        }
        if (!act && (i == 0 || prev_act)) *n_act = i;
        uint8_t l = 0;
        if (act) {
            if (i == 0) {
                l = 0;  // the first particle opens the root box and every box below it
            } else {
                const uint64_t x = k ^ keys[i - 1];
                if (x == 0) {
                    l = kLevels;  // same finest cell: never starts a box
                } else {
                    const int b = 63 - __clzll((long long)x);
                    l = (uint8_t)(kMortonBits - b / 3);
                }
                atomicAdd(&sh[l], 1);
            }
            lvl[i] = l;
        } else {
            lvl[i] = 0xff;
        }
    }
    __syncthreads();
    if (threadIdx.x <= kLevels && sh[threadIdx.x]) atomicAdd(&hist[threadIdx.x], sh[threadIdx.x]);
}

constexpr int kBuildThreads = 1024;  // particles per CTA of the level builder

// Deepest level at which some box still holds more than `leaf` particles, as
// max_i min(lvl[i+1 .. i+leaf]): a window of leaf+1 consecutive particles
// without a box boundary at level <= l means a box of level l with more than
// `leaf` particles.  Slots past the active particles count as boundaries.
// the histogram's counters zeroed and the active count at n (no inactive particle)
__global__ void hist_init(int *__restrict__ hist, int n) {
    const int t = threadIdx.x;
    if (t <= kLevels) hist[t] = 0;
    if (t == kLevels + 1) hist[t] = n;
}

// the histogram into the host's mapped copy (the host waits on the stream, then reads it)
__global__ void hist_publish(const int *__restrict__ hist, int *__restrict__ out) {
    const int t = threadIdx.x;
    if (t < kLevels + 2) out[t] = hist[t];
}

__global__ void window_depth(const uint8_t *__restrict__ lvl, int n, int leaf, int *__restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    int m = 0;
    if (i < n) {
        m = 255;
        for (int k = 1; k <= leaf; k++) {
            const int j = i + k;
            int v = j < n ? (int)lvl[j] : 0;
            if (v == 255) v = 0;
            m = min(m, v);
        }
        if (m == 255) m = 0;
    }
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m > 0) atomicMax(out, m);
}

// Forest variant: keys hold the plume id above 3*mbits Morton bits; a change
// of plume opens a new root (level 0).  Every slot takes part (slots that are
// no source carry zero charge), so there is no inactive tail.
__global__ void split_levels_forest(const uint64_t *__restrict__ keys, int n, int mbits, uint8_t *__restrict__ lvl) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint8_t l = 0;
    if (i > 0) {
        const uint64_t x = keys[i] ^ keys[i - 1];
        if (x == 0) {
            l = kLevels;
        } else {
            const int b = 63 - __clzll((long long)x);
            l = b >= 3 * mbits ? 0 : (uint8_t)(mbits - b / 3);
        }
    }
    lvl[i] = l;
}

struct LevelPtrs {
    int *start[kLevels];
    int *parent[kLevels];
    int *child0[kLevels];
    int4 *coord[kLevels];
    int *pid[kLevels];           // plume of each box (forest) or null
    int nbox[kLevels];
    int cap[kLevels];            // box capacity per level (forest) or 0
    int first_box[kLevels + 1];  // prefix sums of nbox (flattened box index)
};

__device__ __forceinline__ uint32_t compact3(uint64_t x) {
    x &= 0x1249249249249249ull;
    x = (x ^ (x >> 2)) & 0x10c30c30c30c30c3ull;
    x = (x ^ (x >> 4)) & 0x100f00f00f00f00full;
    x = (x ^ (x >> 8)) & 0x1f0000ff0000ffull;
    x = (x ^ (x >> 16)) & 0x1f00000000ffffull;
    x = (x ^ (x >> 32)) & 0x1fffffull;
    return (uint32_t)x;
}

// Per CTA of kBuildThreads particles and per level l <= L: how many of its
// particles start a box at level l (lvl[i] <= l).
__global__ void __launch_bounds__(kBuildThreads)
count_starts(const uint8_t *__restrict__ lvl, int n, int L, int *__restrict__ cnt) {
    __shared__ int wc[kBuildThreads / 32][kLevels];
    const int i = blockIdx.x * kBuildThreads + threadIdx.x;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int my = i < n ? (int)lvl[i] : 255;
    for (int l = 0; l <= L; l++) {
        const unsigned bal = __ballot_sync(0xffffffffu, my <= l);
        if (lane == 0) wc[w][l] = __popc(bal);
    }
    __syncthreads();
    if (threadIdx.x <= L) {
        int s = 0;
        for (int k = 0; k < kBuildThreads / 32; k++) s += wc[k][threadIdx.x];
        cnt[blockIdx.x * kLevels + threadIdx.x] = s;
    }
}

// Exclusive scan over the CTAs of each level (one block per level).  With
// nbox_out: the level's box count, clamped to cap[l] (err set when clamped).
__global__ void __launch_bounds__(1024) scan_counts(int *__restrict__ cnt, int nblk, int *__restrict__ nbox_out,
                                                    const int *__restrict__ cap, int *__restrict__ err) {
    __shared__ int buf[1024];
    __shared__ int carry;
    const int l = blockIdx.x;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < nblk; base += 1024) {
        const int k = base + threadIdx.x;
        const int v = k < nblk ? cnt[k * kLevels + l] : 0;
        buf[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < 1024; o <<= 1) {
            const int t = threadIdx.x >= o ? buf[threadIdx.x - o] : 0;
            __syncthreads();
            buf[threadIdx.x] += t;
            __syncthreads();
        }
        if (k < nblk) cnt[k * kLevels + l] = carry + buf[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry += buf[1023];
        __syncthreads();
    }
    if (nbox_out && threadIdx.x == 0) {
        int t = carry;
        atomicMax(&nbox_out[2 * kLevels + l], t);  // largest count seen, for capacity planning
        if (t > cap[l]) {
            atomicOr(err, 1 << l);
            t = cap[l];
        }
        nbox_out[l] = t;
    }
}

// Every particle that starts a box at level l writes its index as that box's
// start, and the box's integer coordinates from its Morton key.
__global__ void __launch_bounds__(kBuildThreads)
scatter_starts(const uint8_t *__restrict__ lvl, const uint64_t *__restrict__ keys, int n, int L, int mbits,
               const int *__restrict__ off, LevelPtrs P) {
    const uint64_t mmask = mbits >= 21 ? ~0ull : ((1ull << (3 * mbits)) - 1ull);
    __shared__ int wc[kBuildThreads / 32];
    __shared__ int wpre[kBuildThreads / 32];
    const int i = blockIdx.x * kBuildThreads + threadIdx.x;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int my = i < n ? (int)lvl[i] : 255;
    const uint64_t key = i < n ? keys[i] : 0ull;
    const unsigned lt = (1u << lane) - 1u;
    for (int l = 0; l <= L; l++) {
        const bool f = my <= l;
        const unsigned bal = __ballot_sync(0xffffffffu, f);
        if (lane == 0) wc[w] = __popc(bal);
        __syncthreads();
        if (w == 0) {
            const int v = wc[lane];
            int inc = v;
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, inc, o);
                if (lane >= o) inc += t;
            }
            wpre[lane] = inc - v;
        }
        __syncthreads();
        if (f) {
            const int idx = off[blockIdx.x * kLevels + l] + wpre[w] + __popc(bal & lt);
            if (P.cap[l] == 0 || idx < P.cap[l]) {
                P.start[l][idx] = i;
                const uint64_t k = (key & mmask) >> (3 * (mbits - l));
                P.coord[l][idx] = make_int4((int)compact3(k), (int)compact3(k >> 1), (int)compact3(k >> 2), 0);
                if (P.pid[l]) P.pid[l][idx] = (int)(key >> (3 * mbits));
            }
        }
        __syncthreads();
    }
}

__device__ __forceinline__ int upper_bound_i(const int *__restrict__ a, int n, int v) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (a[mid] <= v) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Close every level: particle counts, sentinels, parents and first children
// (both by binary search on the neighbouring level's sorted starts: the starts
// of level l-1 are a subset of those of level l).
__global__ void link_levels(int L, int n_act, int total, LevelPtrs P) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= total) return;
    int l = 0;
    while (t >= P.first_box[l + 1]) l++;
    const int b = t - P.first_box[l];
    const int nb = P.nbox[l];
    const int s = P.start[l][b];
    const int e = b + 1 < nb ? P.start[l][b + 1] : n_act;
    P.coord[l][b].w = e - s;
    if (b == 0) {
        P.start[l][nb] = n_act;
        if (l < L) P.child0[l][nb] = P.nbox[l + 1];
    }
    if (l >= 1) P.parent[l][b] = upper_bound_i(P.start[l - 1], P.nbox[l - 1], s) - 1;
    if (l < L) P.child0[l][b] = upper_bound_i(P.start[l + 1], P.nbox[l + 1], s) - 1;
}

// After a capacity overflow the run is redone by the host with larger
// capacities: empty every level so that the rest of the run (and any further
// captured step) does no work.
__global__ void drop_if_overflow(int L, int *__restrict__ nbox, const int *__restrict__ err) {
    if (*err && threadIdx.x <= L) nbox[threadIdx.x] = 0;
}

// Forest variant of link_levels: box counts live on the device; blockIdx.y
// is the level, boxes are visited grid-stride.
__global__ void link_levels_forest(int L, int n, const int *__restrict__ nbox, LevelPtrs P) {
    const int l = blockIdx.y;
    const int nb = nbox[l];
    const int nb_up = l >= 1 ? nbox[l - 1] : 0, nb_dn = l < L ? nbox[l + 1] : 0;
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += gridDim.x * blockDim.x) {
        const int s = P.start[l][b];
        const int e = b + 1 < nb ? P.start[l][b + 1] : n;
        P.coord[l][b].w = e - s;
        if (b == 0) {
            P.start[l][nb] = n;
            if (l < L) P.child0[l][nb] = nb_dn;
        }
        if (l >= 1) P.parent[l][b] = upper_bound_i(P.start[l - 1], nb_up, s) - 1;
        if (l < L) P.child0[l][b] = upper_bound_i(P.start[l + 1], nb_dn, s) - 1;
    }
}

sv_status arena_reserve(sv_ctx *c, Tree &T, size_t bytes) {
    if (T.arena_bytes >= bytes) return SV_OK;
    cudaFree(T.arena);
    T.arena = nullptr;
    T.arena_bytes = 0;
    const size_t want = bytes + bytes / 2;  // headroom: a growing tree reallocates rarely
    SV_CK(c, cudaMalloc(&T.arena, want));
    T.arena_bytes = want;
    return SV_OK;
}

}  // namespace

void tree_free(sv_ctx *c) {
    if (!c->tree) return;
    Tree &T = *c->tree;
    cudaFree(T.lvl);
    cudaFree(T.hist);
    cudaFree(T.scratch);
    cudaFree(T.arena);
    cudaFreeHost(T.h_hist);
    delete c->tree;
    c->tree = nullptr;
}

// Histogram of split levels and count of active particles (one readback).
static sv_status tree_levels(sv_ctx *c, Tree &T, int leaf_window) {
    const int n = (int)c->S.n;
    if (T.cap < n) {
        cudaFree(T.lvl);
        cudaFree(T.scratch);
        T.lvl = nullptr;
        T.scratch = nullptr;
        const int cap = std::max(n, 1024);
        SV_CK(c, cudaMalloc(&T.lvl, cap));
        SV_CK(c, cudaMalloc(&T.scratch, sizeof(int) * (size_t)kLevels * (cap / kBuildThreads + 1)));
        T.cap = cap;
    }
    hist_init<<<1, 32, 0, c->stream>>>(T.hist, n);
    SV_LAUNCHED(c);
    split_levels<<<div_up(n, 256), 256, 0, c->stream>>>(c->S.keys, n, T.lvl, T.hist, T.hist + kLevels + 1);
    SV_LAUNCHED(c);
    if (leaf_window > 0) {
        SV_CK(c, cudaMemsetAsync(T.hist + kLevels, 0, sizeof(int), c->stream));
        window_depth<<<div_up(n, 256), 256, 0, c->stream>>>(T.lvl, n, leaf_window, T.hist + kLevels);
        SV_LAUNCHED(c);
    }
    // the pinned host copy is mapped: a kernel writes it, no copy engine in the round trip
    if (T.d_h_hist) {
        hist_publish<<<1, 32, 0, c->stream>>>(T.hist, T.d_h_hist);
        SV_LAUNCHED(c);
    } else {
        SV_CK(c, cudaMemcpyAsync(T.h_hist, T.hist, sizeof(int) * (kLevels + 2), cudaMemcpyDeviceToHost, c->stream));
    }
    SV_CK(c, cudaStreamSynchronize(c->stream));
    T.n_act = T.h_hist[kLevels + 1];
    int acc = T.n_act > 0 ? 1 : 0;
    for (int l = 0; l < kLevels; l++) {
        acc += (l > 0) ? T.h_hist[l] : 0;
        T.nbox_level[l] = T.n_act > 0 ? acc : 0;
    }
    return SV_OK;
}

sv_status tree_build(sv_ctx *c, int depth_rule, int param, Tree **out) {
    if (!c->tree) {
        c->tree = new Tree();
        SV_CK(c, cudaMalloc(&c->tree->hist, sizeof(int) * (kLevels + 2)));
        SV_CK(c, cudaMallocHost(&c->tree->h_hist, sizeof(int) * (kLevels + 2)));
        void *dp = nullptr;
        if (cudaHostGetDevicePointer(&dp, c->tree->h_hist, 0) == cudaSuccess) c->tree->d_h_hist = (int *)dp;
        else (void)cudaGetLastError();
    }
    Tree &T = *c->tree;
    *out = &T;
    SV_TRY(tree_levels(c, T, depth_rule == kDepthAllSplit ? param : 0));
    const int na = T.n_act;
    if (na == 0) {
        T.deepest = -1;
        return SV_OK;
    }
    // pick the deepest level
    int L = 0;
    if (depth_rule == kDepthMeanOccupancy) {
        // deepest level whose mean occupancy is still >= param particles per box
        L = 0;
        for (int l = 1; l < kLevels; l++) {
            if ((double)na / T.nbox_level[l] >= (double)param) L = l;
            else break;
        }
        if (L < 2) L = std::min(2, kLevels - 1);
    } else {
        // deepest level needed so that no box holds more than param particles:
        // the first level at which the largest box is small enough; the largest
        // box is bounded by the smallest gap between consecutive starts, which
        // is only known on the device, so use the level of mean occupancy 1/8
        // of param as a safe upper bound and let leaves stop early.
        // first level at which no box exceeds `param` particles (duplicate
        // positions stop at the finest level)
        L = std::min(kLevels - 1, T.h_hist[kLevels]);
        if (L < 1) L = 1;
    }
    T.deepest = L;
    // carve the arena: per level start[nbox+1], parent[nbox], child0[nbox+1], coord[nbox]
    auto rounded = [](size_t sz) { return (sz + 255) & ~(size_t)255; };
    size_t bytes = 0;
    for (int l = 0; l <= L; l++) {
        const size_t nb = (size_t)T.nbox_level[l];
        bytes += rounded(sizeof(int) * (nb + 1)) + rounded(sizeof(int) * nb) + rounded(sizeof(int) * (nb + 1)) +
                 rounded(sizeof(int4) * nb);
    }
    SV_TRY(arena_reserve(c, T, bytes));
    char *p = (char *)T.arena;
    auto carve = [&](size_t sz) {
        char *r = p;
        p += (sz + 255) & ~(size_t)255;
        return (void *)r;
    };
    for (int l = 0; l <= L; l++) {
        Level &V = T.lv[l];
        V.nbox = T.nbox_level[l];
        V.start = (int *)carve(sizeof(int) * (V.nbox + 1));
        V.parent = (int *)carve(sizeof(int) * V.nbox);
        V.child0 = (int *)carve(sizeof(int) * (V.nbox + 1));
        V.coord = (int4 *)carve(sizeof(int4) * V.nbox);
    }
    LevelPtrs P{};
    int total = 0;
    for (int l = 0; l <= L; l++) {
        P.start[l] = T.lv[l].start;
        P.parent[l] = T.lv[l].parent;
        P.child0[l] = T.lv[l].child0;
        P.coord[l] = T.lv[l].coord;
        P.nbox[l] = T.lv[l].nbox;
        P.first_box[l] = total;
        total += T.lv[l].nbox;
    }
    for (int l = L + 1; l <= kLevels; l++) P.first_box[l] = total;
    const int nblk = div_up(na, kBuildThreads);
    count_starts<<<nblk, kBuildThreads, 0, c->stream>>>(T.lvl, na, L, T.scratch);
    SV_LAUNCHED(c);
    scan_counts<<<L + 1, 1024, 0, c->stream>>>(T.scratch, nblk, nullptr, nullptr, nullptr);
    SV_LAUNCHED(c);
    scatter_starts<<<nblk, kBuildThreads, 0, c->stream>>>(T.lvl, c->S.keys, na, L, kMortonBits, T.scratch, P);
    SV_LAUNCHED(c);
    link_levels<<<div_up(total, 256), 256, 0, c->stream>>>(L, na, total, P);
    SV_LAUNCHED(c);
    return SV_OK;
}

void tree_release(Tree &T) {
    cudaFree(T.lvl);
    cudaFree(T.hist);
    cudaFree(T.scratch);
    cudaFree(T.arena);
    cudaFreeHost(T.h_hist);
    T = Tree();
}

sv_status tree_forest_reserve(sv_ctx *c, Tree &T, const ForestSpec &f) {
    const int n = std::max(f.n, 1);
    if (T.cap < n) {
        cudaFree(T.lvl);
        cudaFree(T.scratch);
        T.lvl = nullptr;
        T.scratch = nullptr;
        const int cap = std::max(n, 1024);
        SV_CK(c, cudaMalloc(&T.lvl, cap));
        SV_CK(c, cudaMalloc(&T.scratch, sizeof(int) * (size_t)kLevels * (cap / kBuildThreads + 1)));
        T.cap = cap;
    }
    auto rounded = [](size_t sz) { return (sz + 255) & ~(size_t)255; };
    size_t bytes = 0;
    for (int l = 0; l <= f.L; l++) {
        const size_t nb = (size_t)f.cap[l];
        bytes += 2 * rounded(sizeof(int) * (nb + 1)) + 2 * rounded(sizeof(int) * nb) + rounded(sizeof(int4) * nb);
    }
    SV_TRY(arena_reserve(c, T, bytes));
    char *p = (char *)T.arena;
    auto carve = [&](size_t sz) {
        char *r = p;
        p += (sz + 255) & ~(size_t)255;
        return (void *)r;
    };
    for (int l = 0; l <= f.L; l++) {
        Level &V = T.lv[l];
        V.cap = f.cap[l];
        V.nbox = f.cap[l];
        V.start = (int *)carve(sizeof(int) * (V.cap + 1));
        V.parent = (int *)carve(sizeof(int) * V.cap);
        V.child0 = (int *)carve(sizeof(int) * (V.cap + 1));
        V.coord = (int4 *)carve(sizeof(int4) * V.cap);
        V.pid = (int *)carve(sizeof(int) * V.cap);
    }
    T.deepest = f.L;
    T.n_act = f.n;
    return SV_OK;
}

sv_status tree_build_forest(sv_ctx *c, Tree &T, const ForestSpec &f, int *d_nbox, int *d_err) {
    const int n = f.n, L = f.L;
    if (n <= 0) return SV_OK;
    split_levels_forest<<<div_up(n, 256), 256, 0, c->stream>>>(c->S.keys, n, f.mbits, T.lvl);
    SV_LAUNCHED(c);
    LevelPtrs P{};
    for (int l = 0; l <= L; l++) {
        P.start[l] = T.lv[l].start;
        P.parent[l] = T.lv[l].parent;
        P.child0[l] = T.lv[l].child0;
        P.coord[l] = T.lv[l].coord;
        P.pid[l] = T.lv[l].pid;
        P.cap[l] = T.lv[l].cap;
    }
    const int nblk = div_up(n, kBuildThreads);
    count_starts<<<nblk, kBuildThreads, 0, c->stream>>>(T.lvl, n, L, T.scratch);
    SV_LAUNCHED(c);
    scan_counts<<<L + 1, 1024, 0, c->stream>>>(T.scratch, nblk, d_nbox, d_nbox + kLevels, d_err);
    SV_LAUNCHED(c);
    scatter_starts<<<nblk, kBuildThreads, 0, c->stream>>>(T.lvl, c->S.keys, n, L, f.mbits, T.scratch, P);
    SV_LAUNCHED(c);
    drop_if_overflow<<<1, 32, 0, c->stream>>>(L, d_nbox, d_err);
    SV_LAUNCHED(c);
    int maxcap = 1;
    for (int l = 0; l <= L; l++) maxcap = std::max(maxcap, f.cap[l]);
    link_levels_forest<<<dim3(std::min(div_up(maxcap, 256), 4 * device_sms()), L + 1), 256, 0, c->stream>>>(L, n, d_nbox, P);
    SV_LAUNCHED(c);
    return SV_OK;
}

}  // namespace sv
