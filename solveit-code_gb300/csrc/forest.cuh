// forest.cuh -- FMM over a forest of plumes (one octree root per plume).
//
// Used by the batched path (batch.cu): the first spec.n slots of the context's
// Morton-sorted copy hold every FMM plume, sorted by (plume id, Morton key),
// with each plume's root record (origin xyz, cube side) in roots[8 * pid].
// The depth and all capacities are fixed when the forest is reserved, every
// kernel reads its box count from the device, and a run issues no host
// synchronisation, so it can be captured in a CUDA graph.
#pragma once

#include "tree.cuh"

namespace sv {

struct ForestArgs {
    ForestSpec spec;                 // slots, leaf level, Morton bits, box capacities
    int p = 6, ws = 2;               // expansion order and well-separation
    int nroots = 0;                  // plumes in the forest
    const double *roots = nullptr;   // device [8 * nroots]
    int *d_nbox = nullptr;           // device [3 * (kMortonBits + 1)]: counts, capacities, largest counts
    int *d_err = nullptr;            // device: bit l = level l overflowed its capacity
};

// Allocates the forest's tree and expansion arrays (host call).
sv_status fmm_forest_reserve(sv_ctx *c, const ForestArgs &a);
// Launches the tree build, lists, P2M/M2M, M2L/L2L, L2P and P2P; writes the
// acceleration of slots [0, spec.n) into c->S.a{x,y,z}.
sv_status fmm_forest_run(sv_ctx *c, const ForestArgs &a);
// Largest leaf-box occupancy of the last run (blocking; diagnostics).
sv_status fmm_forest_max_leaf(sv_ctx *c, const ForestArgs &a, int *out);
// The last run's tensor-core M2L found more translations than its room and
// ran the rotation kernel instead (read after the run has completed).
bool fmm_forest_tc_overflowed(const sv_ctx *c);
// Grows that room to four times the last run's translations, within 40 % of
// the device's memory (host call, outside any capture; the buffers move, so
// the caller captures its graphs again).
sv_status fmm_forest_tc_grow(sv_ctx *c);
// The last run's M2L ran on the tensor cores (read after the run has completed).
bool fmm_forest_tc_used(const sv_ctx *c);

}  // namespace sv
