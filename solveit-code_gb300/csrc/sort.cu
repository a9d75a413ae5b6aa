// sort.cu -- Morton ordering of the plume shared by every force method.
//
// The reference sorts particles by Morton index only inside the FMM
// (multipole_method_force_calculation.cpp:883-1083 presortMorton / sort /
// sortParticles, unsortParticles :1184).  Here every method works on a
// Morton-sorted copy so that consecutive targets are close in space; the
// caller's array order is untouched (results are scattered back), as the
// reference requires of updateAcceleration.
#include <cub/device/device_radix_sort.cuh>

#include <algorithm>
#include <cmath>

#include "sv_internal.cuh"

namespace sv {
namespace {

constexpr int kRedThreads = 256;

__device__ __forceinline__ bool is_source(int32_t s) { return s == 1 || s == 2; }

// A double's bits as a signed integer whose order is the double's order
// (non-NaN values); the map is its own inverse.  Min / max on these run on
// the integer pipe: GB300's FP64 pipe issues ~2 operations per clock per SM,
// which made the FP64 fmin / fmax the bound of this reduction.
__device__ __forceinline__ long long ordered_bits(long long b) { return b ^ ((b >> 63) & 0x7fffffffffffffffLL); }

// Per-block min/max of source positions (status 1 or 2), exact.
__global__ void bbox_partial(const double *__restrict__ x, const double *__restrict__ y,
                             const double *__restrict__ z, const int32_t *__restrict__ st,
                             int64_t n, double *__restrict__ out) {
    const long long lo0 = ordered_bits(__double_as_longlong(1e300)), hi0 = ordered_bits(__double_as_longlong(-1e300));
    long long mn[3] = {lo0, lo0, lo0}, mx[3] = {hi0, hi0, hi0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        if (!is_source(st[i])) continue;
        const long long p[3] = {ordered_bits(__double_as_longlong(x[i])), ordered_bits(__double_as_longlong(y[i])),
                                ordered_bits(__double_as_longlong(z[i]))};
#pragma unroll
        for (int d = 0; d < 3; d++) {
            mn[d] = min(mn[d], p[d]);
            mx[d] = max(mx[d], p[d]);
        }
    }
    __shared__ long long sh[6][kRedThreads / 32];
#pragma unroll
    for (int d = 0; d < 3; d++) {
        for (int o = 16; o > 0; o >>= 1) {
            mn[d] = min(mn[d], __shfl_xor_sync(0xffffffffu, mn[d], o));
            mx[d] = max(mx[d], __shfl_xor_sync(0xffffffffu, mx[d], o));
        }
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) {
        for (int d = 0; d < 3; d++) {
            sh[d][w] = mn[d];
            sh[3 + d][w] = mx[d];
        }
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        const int d = threadIdx.x;
        long long v = d < 3 ? lo0 : hi0;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) v = d < 3 ? min(v, sh[d][k]) : max(v, sh[d][k]);
        out[blockIdx.x * 6 + d] = __longlong_as_double(ordered_bits(v));
    }
}

// Final reduction (kRedThreads threads over the block partials); root =
// origin (bbox min), cube side S = scale x the smallest power of two > the
// largest extent, with scale a multiple of 1/8 in [1, 2) (so every box side
// and every box-centre offset S/2^l * k, |k| < 8, is exact in binary floating
// point, FP32 included), bbox max, empty flag, and 2^21 / S for the keys.
__global__ void __launch_bounds__(kRedThreads) bbox_final(const double *__restrict__ part, int nblocks,
                                                          double *__restrict__ root, double scale) {
    __shared__ double sh[6];
    __shared__ double wsh[6][kRedThreads / 32];
    double v[6] = {1e300, 1e300, 1e300, -1e300, -1e300, -1e300};
    for (int k = threadIdx.x; k < nblocks; k += blockDim.x)
        for (int d = 0; d < 6; d++) v[d] = d < 3 ? fmin(v[d], part[k * 6 + d]) : fmax(v[d], part[k * 6 + d]);
    for (int d = 0; d < 6; d++)
        for (int o = 16; o > 0; o >>= 1) {
            const double u = __shfl_xor_sync(0xffffffffu, v[d], o);
            v[d] = d < 3 ? fmin(v[d], u) : fmax(v[d], u);
        }
    if ((threadIdx.x & 31) == 0)
        for (int d = 0; d < 6; d++) wsh[d][threadIdx.x >> 5] = v[d];
    __syncthreads();
    if (threadIdx.x < 6) {
        const int d = threadIdx.x;
        double r = d < 3 ? 1e300 : -1e300;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) r = d < 3 ? fmin(r, wsh[d][k]) : fmax(r, wsh[d][k]);
        sh[d] = r;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double ext = 0.0;
        bool empty = sh[0] > sh[3];
        for (int d = 0; d < 3; d++) ext = fmax(ext, sh[3 + d] - sh[d]);
        if (empty) {
            for (int d = 0; d < 6; d++) sh[d] = 0.0;
            ext = 0.0;
        }
        // guard against a zero extent (single particle) and keep the maximum
        // strictly inside the last cell: S > ext.
        double S = 1e-300;
        if (ext > 0.0) {
            int e;
            frexp(ext, &e);            // ext = f * 2^e, f in [0.5, 1)
            S = ldexp(1.0, e) * scale; // >= 2^e > ext
        } else {
            S = 1e-12;
        }
        root[0] = sh[0];
        root[1] = sh[1];
        root[2] = sh[2];
        root[3] = S;
        root[4] = sh[3];
        root[5] = sh[4];
        root[6] = sh[5];
        root[7] = empty ? 1.0 : 0.0;
        root[8] = (double)(1u << kMortonBits) / S;
    }
}

__device__ __forceinline__ uint64_t spread3(uint32_t v) { return morton_spread3(v); }

__global__ void morton_keys(const double *__restrict__ x, const double *__restrict__ y,
                            const double *__restrict__ z, const int32_t *__restrict__ st,
                            int64_t n, const double *__restrict__ root,
                            uint64_t *__restrict__ keys, uint32_t *__restrict__ idx) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    idx[i] = (uint32_t)i;
    if (!is_source(st[i])) {
        keys[i] = kInactiveKey;
        return;
    }
    const double inv = root[8];  // 2^21 / S, exact (S is a power of two)
    const double p[3] = {x[i] - root[0], y[i] - root[1], z[i] - root[2]};
    uint32_t c[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
        // floor(p * inv) clamped to [0, 2^21 - 1]: one round-down conversion
        // (PTX float-to-integer conversions saturate) and an integer clamp give
        // the same cell as floor, fmax and fmin in FP64, with half the FP64
        // operations of the key
        const int f = __double2int_rd(p[d] * inv);
        c[d] = (uint32_t)min(max(f, 0), (int)((1u << kMortonBits) - 1));
    }
    // bit order within a level: x lowest, then y, then z
    keys[i] = spread3(c[0]) | (spread3(c[1]) << 1) | (spread3(c[2]) << 2);
}

__global__ void gather_sorted(const uint32_t *__restrict__ idx, int64_t n,
                              const double *__restrict__ x, const double *__restrict__ y,
                              const double *__restrict__ z, const double *__restrict__ q,
                              const double *__restrict__ m, const double *__restrict__ qom,
                              const int32_t *__restrict__ st, int64_t first, int64_t last, double kconst,
                              double *__restrict__ xs, double *__restrict__ ys,
                              double *__restrict__ zs, float *__restrict__ qs,
                              double *__restrict__ qm) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= n) return;
    const uint32_t i = idx[s];
    xs[s] = x[i];
    ys[s] = y[i];
    zs[s] = z[i];
    const int32_t w = st[i];
    qs[s] = is_source(w) ? (float)q[i] : 0.0f;
    const bool tgt = (w == 1) && (int64_t)i >= first && (int64_t)i < last && m[i] > 0.0;
    qm[s] = tgt ? kconst * (qom ? qom[i] : q[i] / m[i]) : 0.0;
}

// sorted slots of image copies (index >= n_orig) are sources only and have
// no place in the caller's arrays
__global__ void scatter_accel(const uint32_t *__restrict__ idx, int64_t n, int64_t n_orig,
                              const double *__restrict__ axs, const double *__restrict__ ays,
                              const double *__restrict__ azs, const double *__restrict__ far, int64_t fs,
                              const double *__restrict__ qm, double *__restrict__ ax, double *__restrict__ ay,
                              double *__restrict__ az) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= n) return;
    const uint32_t i = idx[s];
    if ((int64_t)i >= n_orig) return;
    if (qm[s] == 0.0) {
        // not a target of this evaluation (status, range or mass): zero, whatever the
        // methods left in its sorted slot
        ax[i] = ay[i] = az[i] = 0.0;
    } else if (far) {
        ax[i] = axs[s] + far[s];
        ay[i] = ays[s] + far[fs + s];
        az[i] = azs[s] + far[2 * fs + s];
    } else {
        ax[i] = axs[s];
        ay[i] = ays[s];
        az[i] = azs[s];
    }
}

}  // namespace

sv_status ensure_sorted_capacity(sv_ctx *c, int64_t n) {
    Sorted &S = c->S;
    if (S.cap >= n && S.x) return SV_OK;
    cudaFree(S.x); cudaFree(S.y); cudaFree(S.z); cudaFree(S.q); cudaFree(S.qm);
    cudaFree(S.idx); cudaFree(S.keys); cudaFree(S.keys_alt); cudaFree(S.idx_alt);
    cudaFree(S.ax); cudaFree(S.ay); cudaFree(S.az); cudaFree(S.cub_tmp);
    cudaFree(S.root); cudaFree(S.red);
    S = Sorted();
    const int64_t cap = n < 1024 ? 1024 : n;
    SV_CK(c, cudaMalloc(&S.x, cap * sizeof(double)));
    SV_CK(c, cudaMalloc(&S.y, cap * sizeof(double)));
    SV_CK(c, cudaMalloc(&S.z, cap * sizeof(double)));
    SV_CK(c, cudaMalloc(&S.q, cap * sizeof(float)));
    SV_CK(c, cudaMalloc(&S.qm, cap * sizeof(double)));
    SV_CK(c, cudaMalloc(&S.idx, cap * sizeof(uint32_t)));
    SV_CK(c, cudaMalloc(&S.idx_alt, cap * sizeof(uint32_t)));
    SV_CK(c, cudaMalloc(&S.keys, cap * sizeof(uint64_t)));
    SV_CK(c, cudaMalloc(&S.keys_alt, cap * sizeof(uint64_t)));
    SV_CK(c, cudaMalloc(&S.ax, cap * sizeof(double)));
    SV_CK(c, cudaMalloc(&S.ay, cap * sizeof(double)));
    SV_CK(c, cudaMalloc(&S.az, cap * sizeof(double)));
    size_t bytes = 0;
    cub::DoubleBuffer<uint64_t> kb(S.keys, S.keys_alt);
    cub::DoubleBuffer<uint32_t> vb(S.idx, S.idx_alt);
    SV_CK(c, cub::DeviceRadixSort::SortPairs(nullptr, bytes, kb, vb, (int)cap, 0, 64, c->stream));
    S.cub_bytes = bytes;
    SV_CK(c, cudaMalloc(&S.cub_tmp, bytes));
    S.red_blocks = 2 * device_sms();
    SV_CK(c, cudaMalloc(&S.red, (size_t)S.red_blocks * 6 * sizeof(double)));
    SV_CK(c, cudaMalloc(&S.root, 16 * sizeof(double)));
    S.cap = cap;
    return SV_OK;
}

// the FMM's root scale rounded down to a multiple of 1/8 (1 for the other methods)
static double root_scale(const sv_ctx *c) {
    const double s = c->P.fmm_root_scale;
    if (c->P.method != SV_METHOD_FMM || !(s >= 1.0)) return 1.0;
    return std::floor(std::min(s, 1.875) * 8.0) / 8.0;
}

sv_status sort_view(sv_ctx *c, const ParticleView &v, int64_t first, int64_t last) {
    const int64_t n = v.n;
    SV_TRY(ensure_sorted_capacity(c, n));
    Sorted &S = c->S;
    S.n = n;
    S.n_orig = v.n_orig;
    const int nb = div_up(n, 256);
    bbox_partial<<<S.red_blocks, kRedThreads, 0, c->stream>>>(v.x, v.y, v.z, v.status, n, S.red);
    SV_LAUNCHED(c);
    bbox_final<<<1, kRedThreads, 0, c->stream>>>(S.red, S.red_blocks, S.root, root_scale(c));
    SV_LAUNCHED(c);
    morton_keys<<<nb, 256, 0, c->stream>>>(v.x, v.y, v.z, v.status, n, S.root, S.keys, S.idx);
    SV_LAUNCHED(c);
    cub::DoubleBuffer<uint64_t> kb(S.keys, S.keys_alt);
    cub::DoubleBuffer<uint32_t> vb(S.idx, S.idx_alt);
    size_t bytes = S.cub_bytes;
    // levels 1 .. want_levels occupy bits >= 3 (kMortonBits - want_levels); bit 63 marks inactive keys
    const int levels = std::max(1, std::min(kMortonBits, S.want_levels));
    S.want_levels = kMortonBits;
    S.key_levels = levels;
    SV_CK(c, cub::DeviceRadixSort::SortPairs(S.cub_tmp, bytes, kb, vb, (int)n, 3 * (kMortonBits - levels),
                                             3 * kMortonBits + 1, c->stream));
    c->launches += 2 * ((3 * levels + 1 + 7) / 8);  // CUB onesweep: histogram + passes
    if (kb.Current() != S.keys) {
        std::swap(S.keys, S.keys_alt);
    }
    if (vb.Current() != S.idx) {
        std::swap(S.idx, S.idx_alt);
    }
    gather_sorted<<<nb, 256, 0, c->stream>>>(S.idx, n, v.x, v.y, v.z, v.q, v.m, v.qom, v.status, first,
                                             std::min(last, v.n_orig), c->P.k_const, S.x, S.y, S.z, S.q, S.qm);
    SV_LAUNCHED(c);
    return SV_OK;
}

sv_status sort_state(sv_ctx *c, int64_t first, int64_t last) {
    const ParticleView v{c->x, c->y, c->z, c->q, c->m, force_status(c), c->n, c->n, c->qom};
    return sort_view(c, v, first, last);
}

sv_status unsort_accel(sv_ctx *c) {
    const int64_t n = c->S.n;
    scatter_accel<<<div_up(n, 256), 256, 0, c->stream>>>(c->S.idx, n, c->S.n_orig, c->S.ax, c->S.ay, c->S.az,
                                                         c->S.far, c->S.far_stride, c->S.qm, c->ax, c->ay, c->az);
    c->S.far = nullptr;
    SV_LAUNCHED(c);
    return SV_OK;
}

}  // namespace sv
