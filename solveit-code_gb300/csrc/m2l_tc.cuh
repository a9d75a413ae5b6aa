// m2l_tc.cuh -- M2L on the tensor cores (tcgen05): interface for fmm.cu.
//
// The M2L translations of all levels are grouped by offset class (the
// integer offset target - source in box units); every class has one dense
// real operator (build_m2l_dense), so a class's translations are one
// contraction D[entries x R] = A[entries x R] . K_class^T with the source
// multipoles as the rows of A.  Each tile of 128 entries of one class is one
// CTA's unit of work: its multipoles are gathered into shared memory, split
// into TF32 high and low parts, and contracted with the class operator's
// high and low parts (three tcgen05.mma passes: lo.hi + hi.lo + hi.hi,
// FP32 accumulation in tensor memory); each entry's translated expansion is
// written as one row of a buffer, and a reduction in the shape of the
// rotation M2L kernel adds a box's rows in list order, so the result does not
// depend on the order in which the tiles ran.
//
// Softening: the rotation M2L takes the distance rho^2 = |offset|^2 +
// eps^2/h^2 (fmm_cpukernel.cpp:832).  Its translation factor rho^-(j+n+1)
// splits into rho^-n on the input degree and rho^-(j+1) on the output degree,
// and both commute with the rotations (which keep the degree), so with t =
// |offset| / rho the softened operator is diag(t^(j+1)) K diag(t^n): the
// gather scales a source's degree-n coefficients by t^n and the epilogue the
// degree-j outputs by t^(j+1).
#pragma once

#include "sv_internal.cuh"

namespace sv {

struct TcLevel {
    int nbox;             // launch bound: boxes, or the forest capacity
    int level;
    int chunks;           // warps per box of the reduction (as the rotation M2L splits lists)
    int warp0;            // first global warp of the level in the reduction
    int first;            // first global box of the level in the class pass
    const int *nbd;       // device box count (forest) or null
    const int *bpid;      // plume of each box (forest) or null
    int2 *m2l;            // the level's lists: (source box, class); the bucket pass writes the row into .x
    const int *cnt;
    const int *has_tgt;
    const float2 *M;      // multipoles of the level
    float2 *out;          // [box][chunk][coefficient], as the rotation M2L writes them
};

struct TcArgs {
    int nlev, cap, ncls, total_boxes;
    double eps2;
    const double *root;
    const float *cls_rho2;
    TcLevel lv[kMortonBits + 1];
};

// Device state of the tensor-core M2L of one context.
struct M2LTc {
    int p = 0, ws = 0, ncls = 0;
    void *ops = nullptr;          // per class: TF32 high and low operator images (shared-memory layout)
    size_t ops_bytes = 0;
    int *ctl = nullptr;           // [0] entries, [1] tiles, [2] overflow, [3] wait timed out, then per class:
                                  // count, entry offset, tile offset, cursor
    int4 *bucket = nullptr;       // per entry in class order: level, source box, t (float bits), -
    int4 *tiles = nullptr;        // per tile of 128 entries: class, first row, row count
    void *rows = nullptr;         // per entry in class order: the translated expansion (NC float2, rows
                                  // padded to 16-byte multiples)
    int64_t cap = 0;              // entries bucket / rows hold
    int *h_ctl = nullptr;         // pinned copy of ctl[0..3]
    bool launched = false;        // the last evaluation launched the tensor-core M2L
};

// Build (once per order / separation) and upload the class operators;
// reserve room for `entries` translations (half as much again when it has to
// grow, unless exact).
sv_status m2l_tc_prepare(sv_ctx *c, M2LTc &T, int p, int ws, int64_t entries, bool exact = false);
// The class pass, the bucket pass, the tensor-core tiles and the reduction,
// all on stream s.  When the translations exceed the reserved room, nothing
// is computed and ctl[2] is set: the caller's rotation M2L launch then runs
// instead (m2l_tc_skip_flag).
sv_status m2l_tc_launch(sv_ctx *c, M2LTc &T, const TcArgs &a, int reduce_warps, cudaStream_t s);
// Flag the rotation M2L kernel reads: it runs only when the flag is set.
inline const int *m2l_tc_skip_flag(const M2LTc &T) { return T.ctl + 2; }
void m2l_tc_free(M2LTc &T);

}  // namespace sv
