// direct.cu -- all-pairs Coulomb sum on GB300.
//
// Restates DirectForceFunction::direct (direct_force_method.cpp:153-190) and
// its rotational (direct_force_method_rotational.cpp:48-94) and translational
// (direct_force_method_translational.cpp:320-367) variants:
//     a_i = K q_i / m_i * sum_j q_j (r_i - r_j) / (|r_i - r_j|^2 + eps^2)^{3/2}
// for inbound targets i and sources j with status 1 or 2 (j != i for the plain
// sum; the symmetric variants keep the self image, which contributes 0).
//
// Layout: targets and sources are the Morton-sorted copy (sort.cu).  One CTA
// owns TPB*TPT consecutive targets and loops over source tiles staged in
// shared memory; every warp reads the same source at a time (broadcast).
//
// MIXED: the CTA takes the FP64 position of its first target as origin; both
// targets and the staged sources are converted to FP32 offsets from it (one
// FP64 subtraction per staged source), so close pairs keep full FP32 relative
// precision even at 50 um from the plume origin.  Pairs run on the FP32 pipe
// with rsqrtf (MUFU); each tile's partial sums are added into FP64
// accumulators.  FP64: the same tiling with every operation in FP64; 1/sqrt is
// a FP32 rsqrt seed refined by two Newton steps in FP64.
#include <cfloat>

#include "sv_internal.cuh"

namespace sv {
namespace {

constexpr int kTPB = 128;   // threads per CTA
constexpr int kTPT = 2;     // targets per thread
constexpr int kTile = 256;  // sources per shared-memory tile

struct Images {
    int kind;          // 0 none, 1 rotational (4 quadrants), 2 offsets
    int count;         // images per source
    const double *off; // device, 3*count metres (kind 2)
};

__device__ __forceinline__ void image_of(const Images &im, int g, double &x, double &y, double &z) {
    if (im.kind == 1) {
        // source rotated by g*pi/2 about z (quadrantRotationFunction, auxiliary_functions.h:55-57)
        const double x0 = x, y0 = y;
        if (g == 1) { x = -y0; y = x0; }
        else if (g == 2) { x = -x0; y = -y0; }
        else if (g == 3) { x = y0; y = -x0; }
    } else if (im.kind == 2) {
        // target shifted by -offset == source shifted by +offset
        x += im.off[3 * g];
        y += im.off[3 * g + 1];
        z += im.off[3 * g + 2];
    }
}

// true when any of the CTA's kTPB*kTPT targets has a nonzero K q/m (a target)
__device__ __forceinline__ bool block_has_target(const double *__restrict__ qm, int t0, int n) {
    int any = 0;
#pragma unroll
    for (int k = 0; k < kTPT; k++) {
        const int i = t0 + threadIdx.x + k * kTPB;
        any |= (i < n && qm[i] != 0.0);
    }
    return __syncthreads_or(any) != 0;
}

__global__ void __launch_bounds__(kTPB)
direct_mixed_kernel(const double *__restrict__ xs, const double *__restrict__ ys,
                    const double *__restrict__ zs, const float *__restrict__ qs,
                    const double *__restrict__ qm, int n, int chunk, float eps2, Images im,
                    double *__restrict__ ax, double *__restrict__ ay, double *__restrict__ az,
                    int atomic_out) {
    __shared__ __align__(16) float tile[4][kTile];  // staged sources: -x, -y, -z, charge
    const int t0 = blockIdx.x * (kTPB * kTPT);
    const int j_begin = blockIdx.y * chunk;
    const int j_end = min(n, j_begin + chunk);
    const int o = min(t0, n - 1);
    const double ox = xs[o], oy = ys[o], oz = zs[o];
    if (!block_has_target(qm, t0, n)) return;  // whole CTA of non-targets (target subsets)

    float2 TX[kTPT], TY[kTPT], TZ[kTPT];
    const float2 E2 = make_float2(eps2, eps2);
    double sx[kTPT], sy[kTPT], sz[kTPT];
#pragma unroll
    for (int k = 0; k < kTPT; k++) {
        const int i = t0 + threadIdx.x + k * kTPB;
        const int ii = min(i, n - 1);
        const float tx = (float)(xs[ii] - ox), ty = (float)(ys[ii] - oy), tz = (float)(zs[ii] - oz);
        TX[k] = make_float2(tx, tx);
        TY[k] = make_float2(ty, ty);
        TZ[k] = make_float2(tz, tz);
        sx[k] = sy[k] = sz[k] = 0.0;
    }
    for (int g = 0; g < im.count; g++) {
        for (int jt = j_begin; jt < j_end; jt += kTile) {
            __syncthreads();
            for (int s = threadIdx.x; s < kTile; s += kTPB) {
                const int j = jt + s;
                float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
                if (j < j_end) {
                    double px = xs[j], py = ys[j], pz = zs[j];
                    image_of(im, g, px, py, pz);
                    v = make_float4((float)(px - ox), (float)(py - oy), (float)(pz - oz), qs[j]);
                }
                tile[0][s] = -v.x;
                tile[1][s] = -v.y;
                tile[2][s] = -v.z;
                tile[3][s] = v.w;
            }
            __syncthreads();
            // two sources per packed FP32x2 operation; r^2 floored at kMinR2
            // (self pair with eps = 0: d = 0 -> 0 * finite)
            float2 gx[kTPT], gy[kTPT], gz[kTPT];
#pragma unroll
            for (int k = 0; k < kTPT; k++) gx[k] = gy[k] = gz[k] = make_float2(0.f, 0.f);
#pragma unroll 4
            for (int s = 0; s < kTile; s += 2) {
                const float2 X = ld2(tile[0], s), Y = ld2(tile[1], s), Z = ld2(tile[2], s), Q = ld2(tile[3], s);
#pragma unroll
                for (int k = 0; k < kTPT; k++) pair2<true, false>(X, Y, Z, Q, TX[k], TY[k], TZ[k], E2, gx[k], gy[k], gz[k]);
            }
#pragma unroll
            for (int k = 0; k < kTPT; k++) {
                sx[k] += gx[k].x + gx[k].y;
                sy[k] += gy[k].x + gy[k].y;
                sz[k] += gz[k].x + gz[k].y;
            }
        }
    }
#pragma unroll
    for (int k = 0; k < kTPT; k++) {
        const int i = t0 + threadIdx.x + k * kTPB;
        if (i >= n) continue;
        const double c = qm[i];
        if (c == 0.0) continue;
        if (atomic_out) {
            atomicAdd(&ax[i], sx[k] * c);
            atomicAdd(&ay[i], sy[k] * c);
            atomicAdd(&az[i], sz[k] * c);
        } else {
            ax[i] = sx[k] * c;
            ay[i] = sy[k] * c;
            az[i] = sz[k] * c;
        }
    }
}

// 1/sqrt(r2) in FP64: FP32 seed, two Newton-Raphson steps y <- y(3 - r2 y^2)/2
// (each step doubles the number of correct bits: ~23 -> ~46 -> full FP64).
__device__ __forceinline__ double rsqrt_f64(double r2) {
    double y = (double)rsqrtf(fmaxf((float)r2, FLT_MIN));
    double h = 0.5 * r2;
    y = y * fma(-h * y, y, 1.5);
    y = y * fma(-h * y, y, 1.5);
    return y;
}

__global__ void __launch_bounds__(kTPB)
direct_fp64_kernel(const double *__restrict__ xs, const double *__restrict__ ys,
                   const double *__restrict__ zs, const float *__restrict__ qs,
                   const double *__restrict__ qm, int n, int chunk, double eps2, Images im,
                   double *__restrict__ ax, double *__restrict__ ay, double *__restrict__ az,
                   int atomic_out) {
    __shared__ dbl4_t tile[kTile];
    const int t0 = blockIdx.x * (kTPB * kTPT);
    const int j_begin = blockIdx.y * chunk;
    const int j_end = min(n, j_begin + chunk);
    double tx[kTPT], ty[kTPT], tz[kTPT], sx[kTPT], sy[kTPT], sz[kTPT];
    if (!block_has_target(qm, t0, n)) return;
#pragma unroll
    for (int k = 0; k < kTPT; k++) {
        const int ii = min(t0 + (int)threadIdx.x + k * kTPB, n - 1);
        tx[k] = xs[ii];
        ty[k] = ys[ii];
        tz[k] = zs[ii];
        sx[k] = sy[k] = sz[k] = 0.0;
    }
    for (int g = 0; g < im.count; g++) {
        for (int jt = j_begin; jt < j_end; jt += kTile) {
            __syncthreads();
            for (int s = threadIdx.x; s < kTile; s += kTPB) {
                const int j = jt + s;
                dbl4_t v = dbl4(0.0, 0.0, 0.0, 0.0);
                if (j < j_end) {
                    double px = xs[j], py = ys[j], pz = zs[j];
                    image_of(im, g, px, py, pz);
                    v = dbl4(px, py, pz, (double)qs[j]);
                } else {
                    v = dbl4(xs[j_begin] + 1.0, 0.0, 0.0, 0.0);  // far, zero charge
                }
                tile[s] = v;
            }
            __syncthreads();
#pragma unroll 2
            for (int s = 0; s < kTile; s++) {
                const dbl4_t v = tile[s];
#pragma unroll
                for (int k = 0; k < kTPT; k++) {
                    const double dx = tx[k] - v.x, dy = ty[k] - v.y, dz = tz[k] - v.z;
                    const double r2 = fma(dx, dx, fma(dy, dy, fma(dz, dz, eps2)));
                    const double inv = rsqrt_f64(r2);
                    const double w = v.w * inv * inv * inv;
                    sx[k] = fma(dx, w, sx[k]);
                    sy[k] = fma(dy, w, sy[k]);
                    sz[k] = fma(dz, w, sz[k]);
                }
            }
        }
    }
#pragma unroll
    for (int k = 0; k < kTPT; k++) {
        const int i = t0 + threadIdx.x + k * kTPB;
        if (i >= n) continue;
        const double c = qm[i];
        if (c == 0.0) continue;
        if (atomic_out) {
            atomicAdd(&ax[i], sx[k] * c);
            atomicAdd(&ay[i], sy[k] * c);
            atomicAdd(&az[i], sz[k] * c);
        } else {
            ax[i] = sx[k] * c;
            ay[i] = sy[k] * c;
            az[i] = sz[k] * c;
        }
    }
}

}  // namespace

sv_status direct_accel(sv_ctx *c) {
    const int n = (int)c->S.n;
    Sorted &S = c->S;
    Images im{0, 1, nullptr};
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
    const int tblocks = div_up(n, kTPB * kTPT);
    // split the source range so that the grid fills the GPU ~8 CTAs per SM deep
    int splits = div_up(8 * device_sms(), tblocks);
    const int max_splits = div_up(n, kTile);
    if (splits > max_splits) splits = max_splits;
    if (splits < 1) splits = 1;
    int chunk = div_up(div_up(n, splits), kTile) * kTile;
    splits = div_up(n, chunk);
    const int atomic_out = splits > 1;
    if (atomic_out) {
        SV_CK(c, cudaMemsetAsync(S.ax, 0, sizeof(double) * n, c->stream));
        SV_CK(c, cudaMemsetAsync(S.ay, 0, sizeof(double) * n, c->stream));
        SV_CK(c, cudaMemsetAsync(S.az, 0, sizeof(double) * n, c->stream));
    }
    for (int k = 2; k <= 6; k++) phase_mark(c, k);
    dim3 grid(tblocks, splits);
    if (c->P.precision == SV_PREC_FP64) {
        direct_fp64_kernel<<<grid, kTPB, 0, c->stream>>>(S.x, S.y, S.z, S.q, S.qm, n, chunk, c->P.softening2,
                                                         im, S.ax, S.ay, S.az, atomic_out);
    } else {
        direct_mixed_kernel<<<grid, kTPB, 0, c->stream>>>(S.x, S.y, S.z, S.q, S.qm, n, chunk,
                                                          (float)c->P.softening2, im, S.ax, S.ay, S.az,
                                                          atomic_out);
    }
    SV_LAUNCHED(c);
    if (d_off) SV_CK(c, cudaFreeAsync(d_off, c->stream));
    const double pairs = (double)n * (double)n * (double)im.count;
    c->stats.pair_interactions = pairs;
    c->stats.cell_interactions = 0;
    c->stats.flops_algorithmic = 20.0 * pairs;
    return SV_OK;
}

cudaError_t launch_direct_mixed_sorted(const double *xs, const double *ys, const double *zs, const float *qs,
                                       const double *qm, int n, float eps2, double *ax, double *ay, double *az,
                                       cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    const int tblocks = div_up(n, kTPB * kTPT);
    int splits = div_up(8 * device_sms(), tblocks);
    const int max_splits = div_up(n, kTile);
    if (splits > max_splits) splits = max_splits;
    if (splits < 1) splits = 1;
    const int chunk = div_up(div_up(n, splits), kTile) * kTile;
    splits = div_up(n, chunk);
    const int atomic_out = splits > 1;
    cudaError_t e = cudaSuccess;
    if (atomic_out) {
        e = cudaMemsetAsync(ax, 0, sizeof(double) * n, stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(ay, 0, sizeof(double) * n, stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(az, 0, sizeof(double) * n, stream);
        if (e != cudaSuccess) return e;
    }
    Images im{0, 1, nullptr};
    direct_mixed_kernel<<<dim3(tblocks, splits), kTPB, 0, stream>>>(xs, ys, zs, qs, qm, n, chunk, eps2, im, ax, ay,
                                                                    az, atomic_out);
    return cudaGetLastError();
}

}  // namespace sv
