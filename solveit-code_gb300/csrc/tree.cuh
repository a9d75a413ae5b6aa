// tree.cuh -- level-by-level sparse octree shared by the BH and FMM paths.
#pragma once

#include "sv_internal.cuh"

namespace sv {

constexpr int kDepthMeanOccupancy = 0;  // FMM: deepest level with mean occupancy >= param
constexpr int kDepthAllSplit = 1;       // BH: down to the level where no box holds more than param

struct Level {
    int nbox = 0;
    int *start = nullptr;   // [nbox+1] first sorted particle of each box (start[nbox] = n_act)
    int *parent = nullptr;  // [nbox] box index at level-1 (unused at level 0)
    int *child0 = nullptr;  // [nbox+1] first child at level+1 (child0[nbox] = boxes at level+1)
    int4 *coord = nullptr;  // [nbox] integer box coordinates (x, y, z) and particle count (w)
    int *pid = nullptr;     // [nbox] plume of the box (forest only)
    int cap = 0;            // box capacity (forest only)
};

struct Tree {
    int cap = 0;
    int n_act = 0;          // particles in the tree (status 1 or 2), sorted first
    int deepest = -1;       // deepest level built
    int nbox_level[kMortonBits + 1] = {0};
    Level lv[kMortonBits + 1];
    uint8_t *lvl = nullptr; // per particle: coarsest level at which it starts a box
    int *hist = nullptr;    // device histogram [levels] + n_act
    int *h_hist = nullptr;  // pinned mirror
    int *d_h_hist = nullptr;  // its device address (mapped), null where it has none
    int *scratch = nullptr; // per-CTA, per-level box-start counts of the level builder
    void *arena = nullptr;
    size_t arena_bytes = 0;
};

// Builds levels 0..deepest.  depth_rule kDepthMeanOccupancy uses param as the
// target mean particles per occupied box at the deepest level.
sv_status tree_build(sv_ctx *c, int depth_rule, int param, Tree **out);

// A forest of octrees over many plumes sorted by (plume id, Morton key): the
// first n slots of c->S, keys with the plume id above 3*mbits Morton bits.
// Level 0 holds one root per plume.  The depth L and the per-level box
// capacities are fixed, and box counts stay on the device, so a build issues
// no host synchronisation and can be captured in a CUDA graph.
struct ForestSpec {
    int n = 0;
    int L = 0;
    int mbits = 18;
    int cap[kMortonBits + 1] = {0};
};
// Allocates the forest's arrays for spec (host call, outside any capture).
sv_status tree_forest_reserve(sv_ctx *c, Tree &T, const ForestSpec &f);
// Launches only.  d_nbox is a device array of 3 (kMortonBits + 1) ints: the
// first third receives each level's box count, clamped to the capacity that
// the caller stored in the second third; the last third keeps the largest
// unclamped count seen.  Bit l of *d_err is set when level l overflowed.
sv_status tree_build_forest(sv_ctx *c, Tree &T, const ForestSpec &f, int *d_nbox, int *d_err);
void tree_release(Tree &T);

}  // namespace sv
