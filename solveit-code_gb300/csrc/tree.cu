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
#include <cub/device/device_scan.cuh>
#include <cub/device/device_select.cuh>

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

// flag[i] = particle i (i < n_act) starts a box at level L
__global__ void flag_particles(const uint8_t *__restrict__ lvl, int n_act, int L, int *__restrict__ flag) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n_act) flag[i] = (i == 0 || lvl[i] <= L) ? 1 : 0;
}

// flag[b] = level-(l+1) box b starts a box at level l
__global__ void flag_boxes(const int *__restrict__ start_fine, const uint8_t *__restrict__ lvl, int nfine, int l,
                           int *__restrict__ flag) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < nfine) flag[b] = (b == 0 || lvl[start_fine[b]] <= l) ? 1 : 0;
}

__global__ void iota_kernel(int *__restrict__ a, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = i;
}

// level-l box b: start particle = start of its first child (or itself at the
// leaf level), close the range arrays, parent of the finer boxes.
__global__ void finish_level(const int *__restrict__ sel, int nbox, const int *__restrict__ start_fine,
                             int n_act, int is_leaf_level, int *__restrict__ start, int *__restrict__ child0,
                             int nfine) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < nbox) {
        const int s = sel[b];
        start[b] = is_leaf_level ? s : start_fine[s];
        if (!is_leaf_level) child0[b] = s;
    }
    if (b == 0) {
        start[nbox] = n_act;
        if (!is_leaf_level) child0[nbox] = nfine;
    }
}

__global__ void parents_from_scan(const int *__restrict__ incl, int nfine, int *__restrict__ parent) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < nfine) parent[b] = incl[b] - 1;
}

__device__ __forceinline__ uint32_t compact3(uint64_t x) {
    x &= 0x1249249249249249ull;
    x = (x ^ (x >> 2)) & 0x10c30c30c30c30c3ull;
    x = (x ^ (x >> 4)) & 0x100f00f00f00f00full;
    x = (x ^ (x >> 8)) & 0x1f0000ff0000ffull;
    x = (x ^ (x >> 16)) & 0x1f00000000ffffull;
    x = (x ^ (x >> 32)) & 0x1fffffull;
    return (uint32_t)x;
}

__global__ void box_coords(const int *__restrict__ start, int nbox, const uint64_t *__restrict__ keys, int l,
                           int4 *__restrict__ coord) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nbox) return;
    const uint64_t k = keys[start[b]] >> (3 * (kMortonBits - l));
    coord[b] = make_int4((int)compact3(k), (int)compact3(k >> 1), (int)compact3(k >> 2), start[b + 1] - start[b]);
}

sv_status arena_reserve(sv_ctx *c, Tree &T, size_t bytes) {
    if (T.arena_bytes >= bytes) return SV_OK;
    cudaFree(T.arena);
    T.arena = nullptr;
    T.arena_bytes = 0;
    const size_t want = bytes + bytes / 4;
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
    cudaFree(T.cub_tmp);
    cudaFree(T.arena);
    cudaFreeHost(T.h_hist);
    delete c->tree;
    c->tree = nullptr;
}

// Histogram of split levels and count of active particles (one readback).
static sv_status tree_levels(sv_ctx *c, Tree &T) {
    const int n = (int)c->S.n;
    if (T.cap < n) {
        cudaFree(T.lvl); cudaFree(T.scratch); cudaFree(T.cub_tmp);
        T.lvl = nullptr; T.scratch = nullptr; T.cub_tmp = nullptr;
        const int cap = std::max(n, 1024);
        SV_CK(c, cudaMalloc(&T.lvl, cap));
        SV_CK(c, cudaMalloc(&T.scratch, sizeof(int) * 3 * (size_t)(cap + 1)));
        size_t b1 = 0, b2 = 0, b3 = 0;
        SV_CK(c, cub::DeviceScan::InclusiveSum(nullptr, b1, T.scratch, T.scratch, cap, c->stream));
        SV_CK(c, cub::DeviceSelect::Flagged(nullptr, b2, T.scratch, T.scratch, T.scratch, T.scratch, cap,
                                            c->stream));
        b3 = std::max(b1, b2);
        SV_CK(c, cudaMalloc(&T.cub_tmp, b3));
        T.cub_bytes = b3;
        T.cap = cap;
    }
    SV_CK(c, cudaMemsetAsync(T.hist, 0, sizeof(int) * (kLevels + 2), c->stream));
    // n_act defaults to n (no inactive particle)
    T.h_hist[kLevels + 1] = n;
    SV_CK(c, cudaMemcpyAsync(T.hist + kLevels + 1, T.h_hist + kLevels + 1, sizeof(int), cudaMemcpyHostToDevice,
                             c->stream));
    split_levels<<<div_up(n, 256), 256, 0, c->stream>>>(c->S.keys, n, T.lvl, T.hist, T.hist + kLevels + 1);
    SV_LAUNCHED(c);
    SV_CK(c, cudaMemcpyAsync(T.h_hist, T.hist, sizeof(int) * (kLevels + 2), cudaMemcpyDeviceToHost, c->stream));
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
    }
    Tree &T = *c->tree;
    *out = &T;
    SV_TRY(tree_levels(c, T));
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
        L = kLevels - 1;
        for (int l = 1; l < kLevels; l++) {
            if (T.nbox_level[l] >= na) { L = l; break; }
        }
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
    int *flag = T.scratch;
    int *incl = T.scratch + (T.cap + 1);
    int *sel = T.scratch + 2 * (T.cap + 1);
    int *d_num = T.hist + kLevels;  // reuse a histogram slot as the selection count
    // leaf level from the particles
    {
        Level &V = T.lv[L];
        flag_particles<<<div_up(na, 256), 256, 0, c->stream>>>(T.lvl, na, L, flag);
        SV_LAUNCHED(c);
        iota_kernel<<<div_up(na, 256), 256, 0, c->stream>>>(incl, na);
        SV_LAUNCHED(c);
        size_t tb = T.cub_bytes;
        SV_CK(c, cub::DeviceSelect::Flagged(T.cub_tmp, tb, incl, flag, sel, d_num, na, c->stream));
        c->launches += 2;
        finish_level<<<div_up(V.nbox + 1, 256), 256, 0, c->stream>>>(sel, V.nbox, nullptr, na, 1, V.start,
                                                                      nullptr, 0);
        SV_LAUNCHED(c);
    }
    for (int l = L - 1; l >= 0; l--) {
        Level &V = T.lv[l];
        Level &F = T.lv[l + 1];
        flag_boxes<<<div_up(F.nbox, 256), 256, 0, c->stream>>>(F.start, T.lvl, F.nbox, l, flag);
        SV_LAUNCHED(c);
        size_t tb = T.cub_bytes;
        SV_CK(c, cub::DeviceScan::InclusiveSum(T.cub_tmp, tb, flag, incl, F.nbox, c->stream));
        c->launches += 2;
        parents_from_scan<<<div_up(F.nbox, 256), 256, 0, c->stream>>>(incl, F.nbox, F.parent);
        SV_LAUNCHED(c);
        iota_kernel<<<div_up(F.nbox, 256), 256, 0, c->stream>>>(incl, F.nbox);
        SV_LAUNCHED(c);
        tb = T.cub_bytes;
        SV_CK(c, cub::DeviceSelect::Flagged(T.cub_tmp, tb, incl, flag, sel, d_num, F.nbox, c->stream));
        c->launches += 2;
        finish_level<<<div_up(V.nbox + 1, 256), 256, 0, c->stream>>>(sel, V.nbox, F.start, na, 0, V.start,
                                                                      V.child0, F.nbox);
        SV_LAUNCHED(c);
    }
    for (int l = 0; l <= L; l++) {
        Level &V = T.lv[l];
        box_coords<<<div_up(V.nbox, 256), 256, 0, c->stream>>>(V.start, V.nbox, c->S.keys, l, V.coord);
        SV_LAUNCHED(c);
    }
    return SV_OK;
}

}  // namespace sv
