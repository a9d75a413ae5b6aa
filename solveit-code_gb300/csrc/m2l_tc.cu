// m2l_tc.cu -- M2L on the tensor cores (tcgen05.mma, TF32 x3, FP32 in TMEM).
//
// Work per evaluation (all on one stream, no host synchronisation):
//   1. class pass    warp per box of every level: histogram of the M2L list
//                    entries over the offset classes (shared-memory counts,
//                    one global add per block and class);
//   2. class scan    one block: per class the first entry and first tile
//                    (128 entries), the totals, and the overflow flag when
//                    the entries exceed the reserved room;
//   3. bucket pass   the same walk again: each entry gets its row in class
//                    order (block-reserved ranges), the bucket record (level,
//                    source box, softening factor t) and, in its list slot,
//                    the row number;
//   4. tiles         persistent CTAs over the tiles: bulk copy (TMA) of the
//                    class operator's TF32 high / low images into shared
//                    memory, gather of the tile's multipoles (scaled by t^n)
//                    split into TF32 high / low, three tcgen05.mma passes of
//                    K / 8 steps into a 128 x N FP32 accumulator in tensor
//                    memory, tcgen05.ld back, scaled by t^(j+1), one row per
//                    entry written;
//   5. reduction     warp per (box, chunk) as the rotation M2L: the rows of a
//                    box's entries added in list order.
// The rotation M2L kernel (fmm.cu) is launched after these and runs only when
// step 2 set the overflow flag; steps 3-5 then do nothing.
//
// Shared-memory operands use the canonical K-major layout without swizzle:
// 8-row x 16-byte core matrices, 128 bytes each, the core matrices of one row
// group consecutive along K (leading-dimension offset 128 B) and row groups
// K * 32 bytes apart (stride-dimension offset).
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "fmm_tables.h"
#include "m2l_tc.cuh"

namespace sv {
namespace {

constexpr int kTile = 128;          // entries per tile (the MMA's M)
constexpr int kTcThreads = 128;     // 4 warps: warp w owns TMEM lanes 32w..32w+31 = tile rows
constexpr int kTmemCols = 128;      // accumulator columns allocated (N <= 112)
constexpr int kCtl = 4;             // leading control words of M2LTc::ctl
constexpr int kMaxCls = 2048;       // classes a block can count in shared memory (ws <= 2: 1331)

template <int P>
struct TcShape {
    static constexpr int NC = P * (P + 1) / 2;      // complex coefficients
    static constexpr int R = P * P;                  // real coefficients (Im c_n^0 left out)
    static constexpr int K = (R + 7) / 8 * 8;        // contraction length (MMA K = 8 for TF32)
    static constexpr int N = (R + 15) / 16 * 16;     // accumulator columns (M = 128 needs N % 16 == 0)
    static constexpr int SBO = K * 32;               // bytes between row groups of 8
    static constexpr int ABYTES = kTile / 8 * SBO;   // one TF32 image of the tile's rows
    static constexpr int BBYTES = N / 8 * SBO;       // one TF32 image of the operator
    static constexpr int SMEM = 2 * ABYTES + 2 * BBYTES + 1024;
};

// real index r of (degree n, order m, part): the float offset in a row of NC
// float2 coefficients and the degree
__host__ __device__ constexpr int real_deg(int r) {
    int n = 0;
    while ((n + 1) * (n + 1) <= r) n++;
    return n;
}
__host__ __device__ constexpr int real_float(int r) {
    const int n = real_deg(r), q = r - n * n;  // q = 0: Re c_n^0; 2m - 1 / 2m: Re / Im c_n^m
    const int m = (q + 1) / 2, im = q > 0 && (q % 2) == 0;
    return 2 * (n * (n + 1) / 2 + m) + im;
}

// byte offset of element (row, k) of a K-major canonical image
template <int P>
__host__ __device__ constexpr int img_off(int row, int k) {
    return (row / 8) * TcShape<P>::SBO + (k / 4) * 128 + (row % 8) * 16 + (k % 4) * 4;
}

// ------------------------------------------------------------ PTX helpers --
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Wait for the phase with the given parity; false after ~1 s without it.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    while (!mbar_try_wait(bar, parity))
        if (global_ns() - t0 > 1000000000ull) return false;
    return true;
}

// bulk copy (TMA) global -> shared, completion counted in bytes on bar
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ uint32_t to_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

// shared-memory matrix descriptor: K-major, no swizzle
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((addr & 0x3FFFFu) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version of tcgen05
    return d;                // base offset 0, relative LBO, no swizzle
}

// instruction descriptor of kind::tf32: F32 accumulator, TF32 A and B, both
// K-major, M x N
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// 16 accumulator columns of the warp's 32 lanes (thread i: lane base + i)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
#pragma unroll
    for (int k = 0; k < 16; k++) v[k] = __uint_as_float(r[k]);
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// ------------------------------------------------------- class / buckets --
__device__ __forceinline__ int tc_level_boxes(const TcLevel &v) { return v.nbd ? min(v.nbox, *v.nbd) : v.nbox; }

// global box g -> (level index, box); -1 past the end
__device__ __forceinline__ int tc_find_level(const TcArgs &a, int g, int &b) {
    int li = 0;
    while (li + 1 < a.nlev && g >= a.lv[li + 1].first) li++;
    b = g - a.lv[li].first;
    return li;
}

// Pass 1 (bucket = false): class histogram.  Pass 3 (bucket = true): rows
// in class order.  A block takes kClsBoxes consecutive boxes: one thread
// reads each box's header (level, target flag, entry count), a block scan
// lays the boxes' entries end to end, and the threads then walk the
// flattened entries (every load independent of the others).  Counts go to a
// shared histogram, then one global add per block and class (pass 1) or one
// global range per block and class, from which each entry takes its row
// (pass 3).  Against one box per warp over ~8x more blocks this is slower
// alone under a profiler but faster inside the force evaluation, where these
// passes share the GPU with the near field: fewer, longer-lived blocks take
// fewer of its SM slots (fmm_n1m, 20 steps: 2.36 against 2.40 ms per step).
constexpr int kClsBoxes = 128;

template <bool BUCKET>
__global__ void __launch_bounds__(kClsBoxes) tc_classes_kernel(TcArgs a, int *__restrict__ ctl,
                                                               int4 *__restrict__ bucket) {
    __shared__ int hist[kMaxCls];
    __shared__ int base[BUCKET ? kMaxCls : 1];
    __shared__ int s_off[kClsBoxes + 1], s_li[kClsBoxes], s_b[kClsBoxes];
    __shared__ float s_eh2[BUCKET ? kClsBoxes : 1];
    __shared__ int s_warp[kClsBoxes / 32];
    int *cls_cnt = ctl + kCtl, *cls_off = cls_cnt + a.ncls, *cursor = cls_off + 2 * a.ncls;
    if (BUCKET && ctl[2]) return;  // overflow: the rotation M2L runs instead
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    for (int k = tid; k < a.ncls; k += kClsBoxes) hist[k] = 0;
    // this thread's box
    const int g = blockIdx.x * kClsBoxes + tid;
    int n = 0, li = 0, b = 0;
    if (g < a.total_boxes) {
        li = tc_find_level(a, g, b);
        const TcLevel &v = a.lv[li];
        if (b < tc_level_boxes(v) && v.has_tgt[b]) {
            n = v.cnt[b];
            if (BUCKET) {
                const double h = (v.bpid ? a.root + 8 * v.bpid[b] : a.root)[3] / (double)(1 << v.level);
                s_eh2[tid] = (float)(a.eps2 / (h * h));
            }
        }
    }
    s_li[tid] = li;
    s_b[tid] = b;
    // exclusive scan of the entry counts over the block
    int inc = n;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += u;
    }
    if (lane == 31) s_warp[wid] = inc;
    __syncthreads();
    int woff = 0;
    for (int w = 0; w < wid; w++) woff += s_warp[w];
    s_off[tid] = woff + inc - n;
    if (tid == kClsBoxes - 1) s_off[kClsBoxes] = woff + inc;
    __syncthreads();
    const int total = s_off[kClsBoxes];
    // the box of flattened entry f: the last box whose first entry is <= f
    auto box_of = [&](int f) {
        int lo = 0, hi = kClsBoxes - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (s_off[mid] <= f) lo = mid;
            else hi = mid - 1;
        }
        return lo;
    };
    for (int f = tid; f < total; f += kClsBoxes) {
        const int i = box_of(f);
        atomicAdd(&hist[a.lv[s_li[i]].m2l[(size_t)s_b[i] * a.cap + (f - s_off[i])].y], 1);
    }
    __syncthreads();
    for (int k = tid; k < a.ncls; k += kClsBoxes) {
        const int h = hist[k];
        if (!BUCKET) {
            if (h) atomicAdd(&cls_cnt[k], h);
        } else {
            base[k] = h ? cls_off[k] + atomicAdd(&cursor[k], h) : 0;
            hist[k] = 0;
        }
    }
    if (!BUCKET) return;
    __syncthreads();
    for (int f = tid; f < total; f += kClsBoxes) {
        const int i = box_of(f);
        int2 *slot = a.lv[s_li[i]].m2l + (size_t)s_b[i] * a.cap + (f - s_off[i]);
        const int2 en = *slot;
        const int row = base[en.y] + atomicAdd(&hist[en.y], 1);
        // t = |offset| / rho with rho^2 = |offset|^2 + eps^2 / h^2
        const float t = rsqrtf(1.0f + s_eh2[i] / a.cls_rho2[en.y]);
        bucket[row] = make_int4(s_li[i], en.x, __float_as_int(t), 0);
        slot->x = row;
    }
}

// Pass 2: per class the first entry and first tile, the totals, the overflow
// flag; cursors cleared for pass 3.  One block of kScanThreads threads, each
// scanning up to two consecutive classes.
constexpr int kScanThreads = 1024;

__global__ void __launch_bounds__(kScanThreads) tc_scan_kernel(int ncls, int64_t cap, int *__restrict__ ctl,
                                                                int4 *__restrict__ tiles) {
    int *cls_cnt = ctl + kCtl, *cls_off = cls_cnt + ncls, *tile_off = cls_off + ncls, *cursor = tile_off + ncls;
    __shared__ int s_e[kScanThreads / 32], s_t[kScanThreads / 32];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int k0 = 2 * tid;
    const int c0 = k0 < ncls ? cls_cnt[k0] : 0, c1 = k0 + 1 < ncls ? cls_cnt[k0 + 1] : 0;
    const int t0 = (c0 + kTile - 1) / kTile, t1 = (c1 + kTile - 1) / kTile;
    int ce = c0 + c1, ct = t0 + t1;  // inclusive scan over the block
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int ue = __shfl_up_sync(0xffffffffu, ce, o), ut = __shfl_up_sync(0xffffffffu, ct, o);
        if (lane >= o) {
            ce += ue;
            ct += ut;
        }
    }
    if (lane == 31) {
        s_e[wid] = ce;
        s_t[wid] = ct;
    }
    __syncthreads();
    if (wid == 0) {
        int we = s_e[lane], wt = s_t[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int ue = __shfl_up_sync(0xffffffffu, we, o), ut = __shfl_up_sync(0xffffffffu, wt, o);
            if (lane >= o) {
                we += ue;
                wt += ut;
            }
        }
        s_e[lane] = we;  // inclusive over warps
        s_t[lane] = wt;
    }
    __syncthreads();
    const int pe = (wid ? s_e[wid - 1] : 0) + ce - (c0 + c1), pt = (wid ? s_t[wid - 1] : 0) + ct - (t0 + t1);
    if (k0 < ncls) {
        cls_off[k0] = pe;
        tile_off[k0] = pt;
        cursor[k0] = 0;
    }
    if (k0 + 1 < ncls) {
        cls_off[k0 + 1] = pe + c0;
        tile_off[k0 + 1] = pt + t0;
        cursor[k0 + 1] = 0;
    }
    if (tid == kScanThreads - 1) {
        const int te = s_e[31], tt = s_t[31];
        ctl[0] = te;
        ctl[1] = tt;
        ctl[2] = (int64_t)te > cap ? 1 : 0;
    }
    // the tile table: per tile its class, first row and row count (room for
    // cap / kTile + ncls tiles, which holds whenever the entries fit)
    if ((int64_t)s_e[31] > cap) return;
#pragma unroll
    for (int q = 0; q < 2; q++) {
        const int k = k0 + q, cnt = q ? c1 : c0;
        const int e = q ? pe + c0 : pe, t = q ? pt + t0 : pt;
        if (k >= ncls) break;
        for (int j = 0; j * kTile < cnt; j++) tiles[t + j] = make_int4(k, e + j * kTile, min(kTile, cnt - j * kTile), 0);
    }
}

// ----------------------------------------------------------------- tiles --
struct TileArgs {
    const float2 *M[kMortonBits + 1];  // multipoles per level index
    const int *ctl;
    int *err;                          // ctl + 3: set when a wait gave up
    const int4 *bucket;
    const int4 *tiles;                 // per tile: class, first row, row count
    const unsigned char *ops;          // per class: high then low operator image
    unsigned char *rows;               // RowShape::RSTRIDE bytes per entry
    int ncls;
};

// Rows of the translated expansions and their shared-memory staging:
// RSTRIDE = the NC float2 coefficients rounded up to 16 bytes (bulk copies
// move 16-byte multiples between 16-byte aligned addresses); the staging
// stride SROW is an odd number of 16-byte groups, so the 8 threads of a
// quarter warp touch 8 different bank groups.  A multipole row starts on an
// 8-byte boundary; its bulk copy starts at the 16-byte boundary below and
// covers up to RSTRIDE bytes (so at most 8 bytes past the row, inside the
// carved arena that holds the multipoles).
template <int P>
struct RowShape {
    static constexpr int NC = P * (P + 1) / 2;
    static constexpr int RB = 8 * NC;
    static constexpr int RSTRIDE = (RB + 15) / 16 * 16;
    static constexpr int SROW = (RSTRIDE / 16) % 2 ? RSTRIDE : RSTRIDE + 16;
    static constexpr int STAGE = kTile * SROW;
    // Shared-memory budget of the tile kernel: 100 KB, so that a tile CTA
    // finds room on an SM beside the near field's blocks (which run at the
    // same time, on the other stream).  With the whole 227 KB (two staging
    // buffers of TMA-copied rows, two operator buffers) the kernel alone is
    // faster (61 against 82 us per launch at fmm_n1m), but it waits for SMs
    // that the near field holds: 2.366 against 2.339 ms per step.
    // Staging buffers that fit beside the operand images: two (the next
    // tile's rows stream in during this one), one, or none (the rows are
    // read from global memory directly and stored without staging).
    static constexpr int OPS = 2 * TcShape<P>::ABYTES + 2 * TcShape<P>::BBYTES + 2048;
    static constexpr int BUDGET = 100 * 1024;
    static constexpr int NSTAGE = OPS + 2 * STAGE <= BUDGET ? 2 : (OPS + STAGE <= BUDGET ? 1 : 0);
    // two operator buffers (the next class's operator streams in during this
    // tile) when they fit beside the rest
    static constexpr int NB = OPS + 2 * TcShape<P>::BBYTES + NSTAGE * STAGE <= BUDGET ? 2 : 1;
    static constexpr int SMEM = 2 * TcShape<P>::ABYTES + NB * 2 * TcShape<P>::BBYTES + NSTAGE * STAGE + 1024;
    static_assert(SMEM <= 227 * 1024, "the operand images must fit in shared memory");
};

__device__ __forceinline__ void mbar_arrive_expect(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_s2g(void *dst, const void *src, uint32_t bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_u32(src)),
                 "r"(bytes)
                 : "memory");
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}
// this thread's bulk stores have finished reading shared memory
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// ... and have completed
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// Issue this thread's bulk copy of its row (bucket record bk, when mine) of
// a tile into the staging buffer, arriving on bar with the bytes it expects.
template <int P>
__device__ __forceinline__ void gather_row(const int4 &bk, bool mine, const TileArgs &a, unsigned char *stage,
                                           uint64_t *bar) {
    using Rw = RowShape<P>;
    if (mine) {
        const uintptr_t src = (uintptr_t)(a.M[bk.x] + (size_t)bk.y * Rw::NC);
        const uintptr_t al = src & ~(uintptr_t)15;
        const uint32_t bytes = (uint32_t)((src - al + Rw::RB + 15) & ~(uintptr_t)15);
        mbar_arrive_expect(bar, bytes);
        bulk_g2s(stage + threadIdx.x * Rw::SROW, (const void *)al, bytes, bar);
    } else {
        mbar_arrive_expect(bar, 0);
    }
}

template <int P>
__global__ void __launch_bounds__(kTcThreads) m2l_tc_tiles_kernel(TileArgs a) {
    using S = TcShape<P>;
    using Rw = RowShape<P>;
    extern __shared__ unsigned char dyn[];
    // 1024-byte aligned: A high, A low, B high, B low, staging buffer(s)
    unsigned char *base = (unsigned char *)(((uintptr_t)dyn + 1023) & ~(uintptr_t)1023);
    unsigned char *a_hi = base, *a_lo = base + S::ABYTES, *b_img = base + 2 * S::ABYTES;
    unsigned char *stage0 = b_img + Rw::NB * 2 * S::BBYTES;
    __shared__ __align__(8) uint64_t bar_b[2], bar_mma, bar_row[2];
    __shared__ uint32_t tmem_slot;
    __shared__ int s_abort;
    if (a.ctl[2]) return;  // overflow: the rotation M2L runs instead
    const int total = a.ctl[1];
    // contiguous tile ranges per CTA: neighbouring tiles share their class
    const int t0 = (int)((int64_t)total * blockIdx.x / gridDim.x);
    const int t1 = (int)((int64_t)total * (blockIdx.x + 1) / gridDim.x);
    if (t0 >= t1) return;
    const int tid = threadIdx.x, warp = tid >> 5;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        mbar_init(&bar_b[0], 1);
        mbar_init(&bar_b[1], 1);
        mbar_init(&bar_mma, 1);
        mbar_init(&bar_row[0], kTcThreads);
        mbar_init(&bar_row[1], kTcThreads);
        s_abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;
    constexpr uint32_t idesc = idesc_tf32(kTile, S::N);
    // phase parities and pending flags (bit k: staging / operator buffer k)
    uint32_t ph_b = 0, ph_mma = 0, ph_rows = 0, rows_pending = 0, b_pending = 0;
    bool aborted = false, mma_pending = false;
    int bcls0 = -1, bcls1 = -1;  // class whose operator each buffer holds (or is loading)
    // tile records (class, first row, row count) one and two tiles ahead, and
    // the bucket record of this thread's row of the current and next tile,
    // are loaded an iteration before they are needed
    const int4 none = make_int4(0, 0, 0, 0);
    int4 rec = a.tiles[t0], rec_n = t0 + 1 < t1 ? a.tiles[t0 + 1] : none;
    int4 bk = tid < rec.z ? a.bucket[rec.y + tid] : none;
    if (Rw::NSTAGE > 0) {
        gather_row<P>(bk, tid < rec.z, a, stage0, &bar_row[0]);
        rows_pending |= 1u;
    }
    for (int t = t0; t < t1; t++) {
        const int sb = Rw::NSTAGE == 2 ? (t - t0) & 1 : 0;
        unsigned char *stage = stage0 + sb * Rw::STAGE;
        const int4 rec_nn = t + 2 < t1 ? a.tiles[t + 2] : none;
        const int4 bk_n = t + 1 < t1 && tid < rec_n.z ? a.bucket[rec_n.y + tid] : none;
        const int cls = rec.x, row0 = rec.y, nrows = rec.z;
        const int ncls_next = t + 1 < t1 ? rec_n.x : cls;
        // prefetch the next tile's rows into the other staging buffer (its
        // previous contents, the rows stored two tiles ago, read out first)
        if (Rw::NSTAGE == 2 && t + 1 < t1) {
            bulk_wait_read();
            gather_row<P>(bk_n, tid < rec_n.z, a, stage0 + (sb ^ 1) * Rw::STAGE, &bar_row[sb ^ 1]);
            rows_pending |= 1u << (sb ^ 1);
        }
        // the class operator: in a buffer already, or loaded now into the
        // buffer that does not hold the next tile's class; the next tile's
        // operator, when it differs, streams into the other buffer
        int bsel = bcls0 == cls ? 0 : (Rw::NB == 2 && bcls1 == cls ? 1 : -1);
        if (bsel < 0) {
            bsel = Rw::NB == 2 && bcls0 == ncls_next ? 1 : 0;
            if (tid == 0) {
                mbar_expect_tx(&bar_b[bsel], 2 * S::BBYTES);
                bulk_g2s(b_img + bsel * 2 * S::BBYTES, a.ops + (size_t)cls * 2 * S::BBYTES, 2 * S::BBYTES,
                         &bar_b[bsel]);
            }
            b_pending |= 1u << bsel;
            if (bsel) bcls1 = cls;
            else bcls0 = cls;
        }
        if (Rw::NB == 2 && ncls_next != cls && (bsel ? bcls0 : bcls1) != ncls_next) {
            const int o = bsel ^ 1;
            if (tid == 0) {
                mbar_expect_tx(&bar_b[o], 2 * S::BBYTES);
                bulk_g2s(b_img + o * 2 * S::BBYTES, a.ops + (size_t)ncls_next * 2 * S::BBYTES, 2 * S::BBYTES,
                         &bar_b[o]);
            }
            b_pending |= 1u << o;
            if (o) bcls1 = ncls_next;
            else bcls0 = ncls_next;
        }
        // this tile's rows have landed
        if (Rw::NSTAGE > 0) {
            if (!__syncthreads_and(mbar_wait_bounded(&bar_row[sb], (ph_rows >> sb) & 1u))) {
                aborted = true;
                break;
            }
            ph_rows ^= 1u << sb;
            rows_pending &= ~(1u << sb);
        }
        // convert: thread r scales row r by t^n, splits it into TF32 high / low
        float tfac = 1.0f;
        if (tid < nrows) {
            tfac = __int_as_float(bk.z);
            const float2 *msrc = a.M[bk.x] + (size_t)bk.y * Rw::NC;
            const float *mv = Rw::NSTAGE > 0
                                  ? reinterpret_cast<const float *>(stage + tid * Rw::SROW + ((uintptr_t)msrc & 15))
                                  : reinterpret_cast<const float *>(msrc);
            float tp[P];
            tp[0] = 1.0f;
#pragma unroll
            for (int n = 1; n < P; n++) tp[n] = tp[n - 1] * tfac;
#pragma unroll
            for (int g = 0; g < S::K / 4; g++) {
                uint32_t hi4[4], lo4[4];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const int r = 4 * g + q;
                    const float x = r < S::R ? mv[real_float(r)] * tp[real_deg(r)] : 0.0f;
                    const uint32_t h = to_tf32(x);
                    hi4[q] = h;
                    lo4[q] = to_tf32(x - __uint_as_float(h));
                }
                const int off = img_off<P>(tid, 4 * g);
                *reinterpret_cast<uint4 *>(a_hi + off) = make_uint4(hi4[0], hi4[1], hi4[2], hi4[3]);
                *reinterpret_cast<uint4 *>(a_lo + off) = make_uint4(lo4[0], lo4[1], lo4[2], lo4[3]);
            }
        }
        fence_proxy_async();
        __syncthreads();
        if (tid == 0) {
            bool ok = true;
            if (b_pending & (1u << bsel)) {
                ok = mbar_wait_bounded(&bar_b[bsel], (ph_b >> bsel) & 1u);
                if (ok) {
                    ph_b ^= 1u << bsel;
                    b_pending &= ~(1u << bsel);
                }
            }
            if (ok) {
                tc_fence_after();
                const uint32_t ah = smem_u32(a_hi), al = smem_u32(a_lo), bh = smem_u32(b_img + bsel * 2 * S::BBYTES),
                               bl = bh + S::BBYTES;
                // lo.hi + hi.lo first (the small terms), then hi.hi
                const uint32_t as[3] = {al, ah, ah}, bs[3] = {bh, bl, bh};
#pragma unroll
                for (int pass = 0; pass < 3; pass++)
#pragma unroll
                    for (int kk = 0; kk < S::K / 8; kk++)
                        mma_tf32(tmem, smem_desc(as[pass] + kk * 256, 128, S::SBO),
                                 smem_desc(bs[pass] + kk * 256, 128, S::SBO), idesc, (pass | kk) != 0);
                mma_commit(&bar_mma);
                mma_pending = true;
            } else {
                s_abort = 1;
            }
        }
        __syncthreads();
        if (s_abort) {
            aborted = true;
            break;
        }
        // every thread waits for the accumulator; the CTA decides together
        if (!__syncthreads_and(mbar_wait_bounded(&bar_mma, ph_mma))) {
            aborted = true;
            break;
        }
        ph_mma ^= 1;
        mma_pending = false;
        tc_fence_after();
        // epilogue: warp w reads lanes 32w.. (its threads' rows), scales the
        // degree-j outputs by t^(j+1), writes the row into its (consumed)
        // staging row and stores it with one bulk copy
        float out[S::N];
#pragma unroll
        for (int c = 0; c < S::N; c += 16) tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + c, out + c);
        tmem_wait_ld();
        if (tid < nrows) {
            float tq[P + 1];
            tq[0] = 1.0f;
#pragma unroll
            for (int n = 1; n <= P; n++) tq[n] = tq[n - 1] * tfac;
            float row[Rw::RSTRIDE / 4];
#pragma unroll
            for (int k = 0; k < Rw::RSTRIDE / 4; k++) row[k] = 0.0f;
#pragma unroll
            for (int j = 0; j < S::R; j++) row[real_float(j)] = out[j] * tq[real_deg(j) + 1];
            unsigned char *dst = a.rows + (size_t)(row0 + tid) * Rw::RSTRIDE;
            float4 *st = reinterpret_cast<float4 *>(Rw::NSTAGE > 0 ? stage + tid * Rw::SROW : dst);
#pragma unroll
            for (int k = 0; k < Rw::RSTRIDE / 16; k++)
                st[k] = make_float4(row[4 * k], row[4 * k + 1], row[4 * k + 2], row[4 * k + 3]);
            if (Rw::NSTAGE > 0) {
                fence_proxy_async();
                bulk_s2g(dst, st, Rw::RSTRIDE);
            }
        }
        if (Rw::NSTAGE == 1 && t + 1 < t1) {
            // one staging buffer: the next tile's rows after this tile's stores
            bulk_wait_read();
            gather_row<P>(bk_n, tid < rec_n.z, a, stage0, &bar_row[0]);
            rows_pending |= 1u;
        }
        rec = rec_n;
        rec_n = rec_nn;
        bk = bk_n;
        tc_fence_before();
        __syncthreads();
    }
    // an abandoned wait may leave bulk copies or the MMA in flight: give them
    // a bounded time to land before the CTA's shared memory and TMEM go away
    if (aborted) {
        if (rows_pending & 1u) (void)mbar_wait_bounded(&bar_row[0], ph_rows & 1u);
        if (rows_pending & 2u) (void)mbar_wait_bounded(&bar_row[1], (ph_rows >> 1) & 1u);
        if (tid == 0) {
            atomicExch(a.err, 1);
            if (b_pending & 1u) (void)mbar_wait_bounded(&bar_b[0], ph_b & 1u);
            if (b_pending & 2u) (void)mbar_wait_bounded(&bar_b[1], (ph_b >> 1) & 1u);
            if (mma_pending) (void)mbar_wait_bounded(&bar_mma, ph_mma);
        }
    }
    bulk_wait_all();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
}

// Pass 5: the rows of a box's entries, added in list order into the M2L
// partials the L2L pass reads (the rotation M2L's warp / chunk layout).
template <int P>
__global__ void __launch_bounds__(128) m2l_tc_reduce_kernel(TcArgs a, const int *__restrict__ ctl,
                                                            const unsigned char *__restrict__ rows) {
    constexpr int NC = P * (P + 1) / 2;
    if (ctl[2]) return;
    const int lane = threadIdx.x & 31;
    const int gw = blockIdx.x * 4 + (threadIdx.x >> 5);
    int li = 0;
    while (li + 1 < a.nlev && gw >= a.lv[li + 1].warp0) li++;
    const TcLevel &v = a.lv[li];
    const int local = gw - v.warp0, b = local / v.chunks, ch = local - b * v.chunks;
    if (b >= tc_level_boxes(v) || !v.has_tgt[b]) return;
    const int cnt = v.cnt[b], per = (cnt + v.chunks - 1) / v.chunks;
    const int e0 = ch * per, e1 = min(cnt, e0 + per);
    const int2 *lst = v.m2l + (size_t)b * a.cap;
    float2 acc0 = make_float2(0.f, 0.f), acc1 = make_float2(0.f, 0.f);
    const int c0 = lane < NC ? lane : 0, c1 = lane + 32;
    // 32 row numbers at a time (one per lane), then their rows four at a
    // time, added in list order
    for (int e = e0; e < e1; e += 32) {
        const int m = min(32, e1 - e);
        const int my = lane < m ? lst[e + lane].x : 0;
        for (int k = 0; k < m; k += 4) {
            float2 x[4], y[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int rr = __shfl_sync(0xffffffffu, my, min(k + u, m - 1));
                const float2 *r = reinterpret_cast<const float2 *>(rows + (size_t)rr * RowShape<P>::RSTRIDE);
                x[u] = r[c0];
                y[u] = c1 < NC ? r[c1] : make_float2(0.f, 0.f);
            }
#pragma unroll
            for (int u = 0; u < 4; u++) {
                if (k + u < m) {
                    acc0.x += x[u].x;
                    acc0.y += x[u].y;
                    acc1.x += y[u].x;
                    acc1.y += y[u].y;
                }
            }
        }
    }
    float2 *dst = v.out + ((size_t)b * v.chunks + ch) * NC;
    if (lane < NC) dst[lane] = acc0;
    if (c1 < NC) dst[c1] = acc1;
}

template <int P>
sv_status launch_tc(sv_ctx *c, M2LTc &T, const TcArgs &a, int reduce_warps, cudaStream_t s) {
    static_assert(TcShape<P>::N <= kTmemCols, "accumulator wider than the TMEM allocation");
    const int blocks = std::max(1, div_up(a.total_boxes, kClsBoxes));
    SV_CK(c, cudaMemsetAsync(T.ctl, 0, sizeof(int) * (kCtl + (size_t)a.ncls), s));
    tc_classes_kernel<false><<<blocks, kClsBoxes, 0, s>>>(a, T.ctl, T.bucket);
    SV_LAUNCHED(c);
    tc_scan_kernel<<<1, kScanThreads, 0, s>>>(a.ncls, T.cap, T.ctl, T.tiles);
    SV_LAUNCHED(c);
    tc_classes_kernel<true><<<blocks, kClsBoxes, 0, s>>>(a, T.ctl, T.bucket);
    SV_LAUNCHED(c);
    TileArgs ta{};
    for (int l = 0; l < a.nlev; l++) ta.M[l] = a.lv[l].M;
    ta.ctl = T.ctl;
    ta.err = T.ctl + 3;
    ta.bucket = T.bucket;
    ta.tiles = T.tiles;
    ta.ops = (const unsigned char *)T.ops;
    ta.rows = (unsigned char *)T.rows;
    ta.ncls = a.ncls;
    static bool attr_set[64] = {};
    int dev = 0;
    SV_CK(c, cudaGetDevice(&dev));
    if (dev >= 0 && dev < 64 && !attr_set[dev]) {
        SV_CK(c, cudaFuncSetAttribute(m2l_tc_tiles_kernel<P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      RowShape<P>::SMEM));
        attr_set[dev] = true;
    }
    // one CTA per SM (with staging, its next tile's rows stream in by bulk
    // copies while the current tile converts, multiplies and stores)
    m2l_tc_tiles_kernel<P><<<device_sms(), kTcThreads, RowShape<P>::SMEM, s>>>(ta);
    SV_LAUNCHED(c);
    m2l_tc_reduce_kernel<P><<<div_up(reduce_warps, 4), 128, 0, s>>>(a, T.ctl, (const unsigned char *)T.rows);
    SV_LAUNCHED(c);
    // entries, tiles, overflow and timeout flags: sizing of the next evaluation, error report
    SV_CK(c, cudaMemcpyAsync(T.h_ctl, T.ctl, sizeof(int) * kCtl, cudaMemcpyDeviceToHost, s));
    return SV_OK;
}

// host TF32 rounding, as cvt.rna.tf32.f32: nearest, ties away from zero
float tf32_host(float x) {
    uint32_t u;
    std::memcpy(&u, &x, 4);
    u = (u + 0x1000u) & ~0x1FFFu;
    float r;
    std::memcpy(&r, &u, 4);
    return r;
}

template <int P>
sv_status build_ops(sv_ctx *c, M2LTc &T, int ws) {
    using S = TcShape<P>;
    std::vector<double> K;
    std::string err;
    if (!build_m2l_dense(P, ws, K, err)) return set_error(c, SV_ERR_INVALID, "M2L operators: %s", err.c_str());
    const int range = 2 * ws + 1, side = 2 * range + 1, ncls = side * side * side;
    std::vector<unsigned char> img((size_t)ncls * 2 * S::BBYTES, 0);
    for (int k = 0; k < ncls; k++) {
        unsigned char *hi = img.data() + (size_t)k * 2 * S::BBYTES, *lo = hi + S::BBYTES;
        for (int j = 0; j < S::R; j++)
            for (int i = 0; i < S::R; i++) {
                const double v = K[((size_t)k * S::R + j) * S::R + i];
                const float h = tf32_host((float)v);
                const float l = tf32_host((float)(v - (double)h));
                std::memcpy(hi + img_off<P>(j, i), &h, 4);
                std::memcpy(lo + img_off<P>(j, i), &l, 4);
            }
    }
    cudaFree(T.ops);
    T.ops = nullptr;
    SV_CK(c, cudaMalloc(&T.ops, img.size()));
    SV_CK(c, cudaMemcpy(T.ops, img.data(), img.size(), cudaMemcpyHostToDevice));
    T.ops_bytes = img.size();
    T.ncls = ncls;
    return SV_OK;
}

}  // namespace

sv_status m2l_tc_prepare(sv_ctx *c, M2LTc &T, int p, int ws, int64_t entries, bool exact) {
    if (T.p != p || T.ws != ws || !T.ops) {
        switch (p) {
        case 4: SV_TRY(build_ops<4>(c, T, ws)); break;
        case 6: SV_TRY(build_ops<6>(c, T, ws)); break;
        case 8: SV_TRY(build_ops<8>(c, T, ws)); break;
        case 10: SV_TRY(build_ops<10>(c, T, ws)); break;
        default: return set_error(c, SV_ERR_UNSUPPORTED, "tensor-core M2L: order %d not instantiated", p);
        }
        if (T.ncls > kMaxCls) return set_error(c, SV_ERR_UNSUPPORTED, "tensor-core M2L: %d classes", T.ncls);
        cudaFree(T.ctl);
        T.ctl = nullptr;
        SV_CK(c, cudaMalloc(&T.ctl, sizeof(int) * (kCtl + 4 * (size_t)T.ncls)));
        if (!T.h_ctl) {
            SV_CK(c, cudaMallocHost(&T.h_ctl, sizeof(int) * kCtl));
            memset(T.h_ctl, 0, sizeof(int) * kCtl);
        }
        T.p = p;
        T.ws = ws;
        T.cap = 0;  // rows depend on the order
    }
    if (entries > T.cap) {
        cudaFree(T.bucket);
        cudaFree(T.rows);
        cudaFree(T.tiles);
        T.bucket = nullptr;
        T.rows = nullptr;
        T.tiles = nullptr;
        T.cap = 0;
        // half as much again: a growing plume's count then reallocates (a
        // device-wide synchronisation in the middle of an evaluation) a few
        // times in a run, not at every step
        const int64_t cap = std::max<int64_t>(exact ? entries : entries + entries / 2, 1 << 16);
        SV_CK(c, cudaMalloc(&T.bucket, sizeof(int4) * (size_t)cap));
        SV_CK(c, cudaMalloc(&T.tiles, sizeof(int4) * (size_t)(cap / kTile + T.ncls + 1)));
        const size_t rstride = ((size_t)p * (p + 1) * 4 + 15) / 16 * 16;  // RowShape<p>::RSTRIDE
        SV_CK(c, cudaMalloc(&T.rows, rstride * (size_t)cap));
        T.cap = cap;
    }
    return SV_OK;
}

sv_status m2l_tc_launch(sv_ctx *c, M2LTc &T, const TcArgs &a, int reduce_warps, cudaStream_t s) {
    switch (T.p) {
    case 4: return launch_tc<4>(c, T, a, reduce_warps, s);
    case 6: return launch_tc<6>(c, T, a, reduce_warps, s);
    case 8: return launch_tc<8>(c, T, a, reduce_warps, s);
    case 10: return launch_tc<10>(c, T, a, reduce_warps, s);
    default: return set_error(c, SV_ERR_UNSUPPORTED, "tensor-core M2L: order %d not instantiated", T.p);
    }
}

void m2l_tc_free(M2LTc &T) {
    cudaFree(T.ops);
    cudaFree(T.ctl);
    cudaFree(T.bucket);
    cudaFree(T.rows);
    cudaFree(T.tiles);
    if (T.h_ctl) cudaFreeHost(T.h_ctl);
    T = M2LTc();
}

}  // namespace sv
