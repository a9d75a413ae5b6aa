// adjoint.cu -- hand-written adjoint of the leapfrog DKD step and the direct sum.
//
// No counterpart in the reference (its integrator only runs forward,
// integration_schemes.cpp:856-891).  Forward step s (t_s = t0 + s dt),
// as sv_leapfrog runs it:
//     x_h     = x_s + h1 v_s                    h1 = clamp(t_s + dt/2 - t_inj, 0, dt/2)
//     a       = F(x_h) + c E                    c = (e/amu) q/m, F = direct sum
//     v_{s+1} = v_s + k a                       k  = clamp(t_s + dt - t_inj, 0, dt), status 1
//     x_{s+1} = x_h + h2 v_{s+1}                h2 = clamp(t_s + dt - t_inj, 0, dt/2)
// F and k act on the injection window t_inj <= t_s + dt/2 only (targets and
// sources); crash, boundary and folding steps are not differentiated (the
// adjoint refuses a context that has them on).
// Reverse step with adjoints (lx, lv) of (x_{s+1}, v_{s+1}):
//     lv += h2 lx;   lh = lx;   la = k lv;   lE += sum_i c_i la_i
//     lh += J(x_h)^T la;        lx = lh;     lv += h1 lh
// with the Jacobian-transpose product of the softened Coulomb sum
//     (J^T la)_k = sum_j G(x_k - x_j) (q_j u_k - q_k u_j),  u = K q/m la,
//     G(d) = I / s^3 - 3 d d^T / s^5,  s^2 = |d|^2 + eps^2,
// a pair kernel with the same tiling and precision modes as the direct sum.
// The forward pass keeps the state every `checkpoint_every` steps; the
// backward pass re-runs each segment from its checkpoint, keeping the segment's
// x_h, and walks it in reverse.
#include <cfloat>

#include "sv_internal.cuh"

namespace sv {

struct Adj {
    int nsteps = 0, every = 0, nck = 0;
    double dt = 0, t0 = 0;
    int64_t n = 0, cap = 0;
    int seg_cap = 0;
    double *ck = nullptr;     // nck x 6 x n: x, y, z, vx, vy, vz
    double *xh = nullptr;     // every x 3 x n: x_h of a segment
    double *lam = nullptr;    // 12 x n: lx(3) lv(3) la(3) tmp(3)
    double *fin = nullptr;    // 6 x n: final state, restored after the backward pass
    double *lE = nullptr;     // 4: dL/dE, then max |u| scratch
    bool forward_done = false;
};

namespace {

constexpr int kTPB = 128;
constexpr int kTPT = 2;
constexpr int kTile = 128;

__device__ __forceinline__ double clampd(double v, double hi) { return fmin(fmax(v, 0.0), hi); }

// (1)-(4): lv += h2 lx; lh = lx (in place); la = k lv; lE += c la
__global__ void adj_prep(double *__restrict__ lx, double *__restrict__ ly, double *__restrict__ lz,
                         double *__restrict__ lvx, double *__restrict__ lvy, double *__restrict__ lvz,
                         double *__restrict__ lax, double *__restrict__ lay, double *__restrict__ laz,
                         const double *__restrict__ q, const double *__restrict__ m, const int32_t *__restrict__ st,
                         const int32_t *__restrict__ wst, const double *__restrict__ t_inj, int64_t n, double ts,
                         double dt, double eoa, double *__restrict__ lE) {
    double e0 = 0, e1 = 0, e2 = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t w = st[i];
        const double h = 0.5 * dt;
        const double h2 = (w == 1 || w == 2) ? clampd(ts + dt - t_inj[i], h) : 0.0;
        // kicked: inbound and injected by the step's mid time (the window of the force)
        const double k = (wst[i] == 1) ? clampd(ts + dt - t_inj[i], dt) : 0.0;
        double vx = lvx[i] + h2 * lx[i], vy = lvy[i] + h2 * ly[i], vz = lvz[i] + h2 * lz[i];
        lvx[i] = vx;
        lvy[i] = vy;
        lvz[i] = vz;
        lax[i] = k * vx;
        lay[i] = k * vy;
        laz[i] = k * vz;
        const double c = (w == 1 && m[i] > 0.0) ? eoa * q[i] / m[i] : 0.0;
        e0 += c * k * vx;
        e1 += c * k * vy;
        e2 += c * k * vz;
    }
    for (int o = 16; o > 0; o >>= 1) {
        e0 += __shfl_xor_sync(0xffffffffu, e0, o);
        e1 += __shfl_xor_sync(0xffffffffu, e1, o);
        e2 += __shfl_xor_sync(0xffffffffu, e2, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&lE[0], e0);
        atomicAdd(&lE[1], e1);
        atomicAdd(&lE[2], e2);
    }
}

// u = K q/m la in sorted order (S.qm is K q/m for targets, 0 otherwise), and
// max |u| (non-negative doubles order like their bit patterns)
__global__ void adj_gather_u(const uint32_t *__restrict__ idx, int n, const double *__restrict__ qm,
                             const double *__restrict__ lax, const double *__restrict__ lay,
                             const double *__restrict__ laz, double *__restrict__ ux, double *__restrict__ uy,
                             double *__restrict__ uz, unsigned long long *__restrict__ umax) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    double a = 0.0;
    if (s < n) {
        const uint32_t i = idx[s];
        const double k = qm[s];
        const double u0 = k * lax[i], u1 = k * lay[i], u2 = k * laz[i];
        ux[s] = u0;
        uy[s] = u1;
        uz[s] = u2;
        a = fmax(fabs(u0), fmax(fabs(u1), fabs(u2)));
        if (!(a <= DBL_MAX)) a = 0.0;  // a non-finite adjoint propagates through the sum itself
    }
    for (int o = 16; o > 0; o >>= 1) a = fmax(a, __shfl_xor_sync(0xffffffffu, a, o));
    if ((threadIdx.x & 31) == 0 && a > 0.0) atomicMax(umax, (unsigned long long)__double_as_longlong(a));
}

// lh += (J^T la) (sorted result scattered to caller order), then lx = lh, lv += h1 lh
__global__ void adj_post(const uint32_t *__restrict__ idx, int64_t ns, int64_t n_orig,
                         const double *__restrict__ jx, const double *__restrict__ jy, const double *__restrict__ jz,
                         double *__restrict__ lx, double *__restrict__ ly, double *__restrict__ lz) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= ns) return;
    const uint32_t i = idx[s];
    if ((int64_t)i >= n_orig) return;
    lx[i] += jx[s];
    ly[i] += jy[s];
    lz[i] += jz[s];
}

__global__ void adj_drift_back(double *__restrict__ lx, double *__restrict__ ly, double *__restrict__ lz,
                               double *__restrict__ lvx, double *__restrict__ lvy, double *__restrict__ lvz,
                               const int32_t *__restrict__ st, const double *__restrict__ t_inj, int64_t n, double ts,
                               double dt) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t w = st[i];
        const double h = 0.5 * dt;
        const double h1 = (w == 1 || w == 2) ? clampd(ts + h - t_inj[i], h) : 0.0;
        lvx[i] += h1 * lx[i];
        lvy[i] += h1 * ly[i];
        lvz[i] += h1 * lz[i];
    }
}

__device__ __forceinline__ double rsqrt_newton(double r2) {
    double y = (double)rsqrtf(fmaxf((float)r2, FLT_MIN));
    const double hh = 0.5 * r2;
    y = y * fma(-hh * y, y, 1.5);
    y = y * fma(-hh * y, y, 1.5);
    return y;
}

struct alignas(32) JSrc64 {
    double x, y, z, q, ux, uy, uz, pad;
};

// Jacobian-transpose pair sum in FP64 on the Morton-sorted copy.
__global__ void __launch_bounds__(kTPB)
jtv_fp64_kernel(const double *__restrict__ xs, const double *__restrict__ ys, const double *__restrict__ zs,
                const float *__restrict__ qs, const double *__restrict__ ux, const double *__restrict__ uy,
                const double *__restrict__ uz, int n, int chunk, double eps2, double *__restrict__ ox,
                double *__restrict__ oy, double *__restrict__ oz, int atomic_out) {
    __shared__ JSrc64 tile[kTile];
    const int t0 = blockIdx.x * (kTPB * kTPT);
    const int j_begin = blockIdx.y * chunk;
    const int j_end = min(n, j_begin + chunk);
    double tx[kTPT], ty[kTPT], tz[kTPT], tq[kTPT], tux[kTPT], tuy[kTPT], tuz[kTPT];
    double sx[kTPT], sy[kTPT], sz[kTPT];
#pragma unroll
    for (int k = 0; k < kTPT; k++) {
        const int ii = min(t0 + (int)threadIdx.x + k * kTPB, n - 1);
        tx[k] = xs[ii];
        ty[k] = ys[ii];
        tz[k] = zs[ii];
        tq[k] = qs[ii];
        tux[k] = ux[ii];
        tuy[k] = uy[ii];
        tuz[k] = uz[ii];
        sx[k] = sy[k] = sz[k] = 0.0;
    }
    for (int jt = j_begin; jt < j_end; jt += kTile) {
        __syncthreads();
        for (int s = threadIdx.x; s < kTile; s += kTPB) {
            const int j = jt + s;
            JSrc64 v{};
            if (j < j_end) {
                v.x = xs[j];
                v.y = ys[j];
                v.z = zs[j];
                v.q = qs[j];
                v.ux = ux[j];
                v.uy = uy[j];
                v.uz = uz[j];
            }
            tile[s] = v;
        }
        __syncthreads();
        const int lim = min(kTile, j_end - jt);
        for (int s = 0; s < lim; s++) {
            const JSrc64 v = tile[s];
#pragma unroll
            for (int k = 0; k < kTPT; k++) {
                const double dx = tx[k] - v.x, dy = ty[k] - v.y, dz = tz[k] - v.z;
                const double r2 = dx * dx + dy * dy + dz * dz + eps2;
                const double inv = rsqrt_newton(r2);
                const double inv2 = inv * inv, inv3 = inv * inv2;
                const double wx = v.q * tux[k] - tq[k] * v.ux;
                const double wy = v.q * tuy[k] - tq[k] * v.uy;
                const double wz = v.q * tuz[k] - tq[k] * v.uz;
                const double dw = 3.0 * ((dx * wx + dy * wy + dz * wz) * inv2) * inv3;
                sx[k] += wx * inv3 - dw * dx;
                sy[k] += wy * inv3 - dw * dy;
                sz[k] += wz * inv3 - dw * dz;
            }
        }
    }
#pragma unroll
    for (int k = 0; k < kTPT; k++) {
        const int i = t0 + threadIdx.x + k * kTPB;
        if (i >= n) continue;
        if (atomic_out) {
            atomicAdd(&ox[i], sx[k]);
            atomicAdd(&oy[i], sy[k]);
            atomicAdd(&oz[i], sz[k]);
        } else {
            ox[i] = sx[k];
            oy[i] = sy[k];
            oz[i] = sz[k];
        }
    }
}

// Source of the mixed kernel: coordinates and u as FP32 hi/lo pairs.
struct alignas(16) JSrc32 {
    float xh, yh, zh, q;
    float xl, yl, zl, p0;
    float uxh, uyh, uzh, p1;
    float uxl, uyl, uzl, p2;
};

__device__ __forceinline__ void split_hl(double v, float &h, float &l) {
    h = (float)v;
    l = (float)(v - (double)h);
}

// Jacobian-transpose pair sum, mixed precision.  The adjoint amplifies the
// error of close pairs over a rollout (a pair at a few softening lengths
// dominates J), so the pair arithmetic is FP32 on hi/lo splits:
//   d = (x_k,hi - x_j,hi) + (x_k,lo - x_j,lo)
// with both coordinates taken relative to the CTA's first target (the hi
// difference of a close pair is exact by Sterbenz's lemma), and
//   w = (q_j u_k,hi - q_k u_j,hi) + (q_j u_k,lo - q_k u_j,lo)
// so a small difference of two large, nearly equal adjoints keeps its digits.
// Units: coordinates in 2^-30 m (1/s^3 in metres overflows FP32), u scaled by
// a power of two su from max|u|; both are exact and undone in FP64 at the end.
// rsqrtf is refined by one Newton step.  Tiles accumulate in FP32, FP64 across
// tiles.
__global__ void __launch_bounds__(kTPB)
jtv_mixed_kernel(const double *__restrict__ xs, const double *__restrict__ ys, const double *__restrict__ zs,
                 const float *__restrict__ qs, const double *__restrict__ ux, const double *__restrict__ uy,
                 const double *__restrict__ uz, const double *__restrict__ umax, int n, int chunk, double eps2,
                 double *__restrict__ ox, double *__restrict__ oy, double *__restrict__ oz, int atomic_out) {
    __shared__ JSrc32 tile[kTile];
    const int t0 = blockIdx.x * (kTPB * kTPT);
    const int j_begin = blockIdx.y * chunk;
    const int j_end = min(n, j_begin + chunk);
    const int o = min(t0, n - 1);
    const double bx = xs[o], by = ys[o], bz = zs[o];
    const double sc = 1073741824.0;  // 2^30
    int ue = 0;
    const double um = *umax;
    if (um > 0.0) frexp(um, &ue);
    const double su = ldexp(1.0, -ue);
    const double back = sc * sc * sc / su;
    const float e2 = (float)(eps2 * sc * sc);
    const float min_r2 = (float)(kMinR2 * sc * sc);
    float txh[kTPT], tyh[kTPT], tzh[kTPT], txl[kTPT], tyl[kTPT], tzl[kTPT], tq[kTPT];
    float tuxh[kTPT], tuyh[kTPT], tuzh[kTPT], tuxl[kTPT], tuyl[kTPT], tuzl[kTPT];
    double sx[kTPT], sy[kTPT], sz[kTPT];
#pragma unroll
    for (int k = 0; k < kTPT; k++) {
        const int ii = min(t0 + (int)threadIdx.x + k * kTPB, n - 1);
        split_hl((xs[ii] - bx) * sc, txh[k], txl[k]);
        split_hl((ys[ii] - by) * sc, tyh[k], tyl[k]);
        split_hl((zs[ii] - bz) * sc, tzh[k], tzl[k]);
        tq[k] = qs[ii];
        split_hl(ux[ii] * su, tuxh[k], tuxl[k]);
        split_hl(uy[ii] * su, tuyh[k], tuyl[k]);
        split_hl(uz[ii] * su, tuzh[k], tuzl[k]);
        sx[k] = sy[k] = sz[k] = 0.0;
    }
    for (int jt = j_begin; jt < j_end; jt += kTile) {
        __syncthreads();
        for (int s = threadIdx.x; s < kTile; s += kTPB) {
            const int j = jt + s;
            JSrc32 v{};
            if (j < j_end) {
                split_hl((xs[j] - bx) * sc, v.xh, v.xl);
                split_hl((ys[j] - by) * sc, v.yh, v.yl);
                split_hl((zs[j] - bz) * sc, v.zh, v.zl);
                v.q = qs[j];
                split_hl(ux[j] * su, v.uxh, v.uxl);
                split_hl(uy[j] * su, v.uyh, v.uyl);
                split_hl(uz[j] * su, v.uzh, v.uzl);
            }
            tile[s] = v;
        }
        __syncthreads();
        float fx[kTPT], fy[kTPT], fz[kTPT];
#pragma unroll
        for (int k = 0; k < kTPT; k++) fx[k] = fy[k] = fz[k] = 0.0f;
        const int lim = min(kTile, j_end - jt);
        for (int s = 0; s < lim; s++) {
            const JSrc32 v = tile[s];
#pragma unroll
            for (int k = 0; k < kTPT; k++) {
                const float dx = (txh[k] - v.xh) + (txl[k] - v.xl);
                const float dy = (tyh[k] - v.yh) + (tyl[k] - v.yl);
                const float dz = (tzh[k] - v.zh) + (tzl[k] - v.zl);
                float r2 = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, e2)));
                r2 = fmaxf(r2, min_r2);
                float inv = rsqrtf(r2);
                inv = inv * fmaf(-0.5f * r2 * inv, inv, 1.5f);
                const float inv2 = inv * inv, inv3 = inv * inv2;
                const float wx = fmaf(-tq[k], v.uxh, v.q * tuxh[k]) + fmaf(-tq[k], v.uxl, v.q * tuxl[k]);
                const float wy = fmaf(-tq[k], v.uyh, v.q * tuyh[k]) + fmaf(-tq[k], v.uyl, v.q * tuyl[k]);
                const float wz = fmaf(-tq[k], v.uzh, v.q * tuzh[k]) + fmaf(-tq[k], v.uzl, v.q * tuzl[k]);
                const float dw = 3.0f * (fmaf(dx, wx, fmaf(dy, wy, dz * wz)) * inv2) * inv3;
                fx[k] = fmaf(-dw, dx, fmaf(wx, inv3, fx[k]));
                fy[k] = fmaf(-dw, dy, fmaf(wy, inv3, fy[k]));
                fz[k] = fmaf(-dw, dz, fmaf(wz, inv3, fz[k]));
            }
        }
#pragma unroll
        for (int k = 0; k < kTPT; k++) {
            sx[k] += (double)fx[k];
            sy[k] += (double)fy[k];
            sz[k] += (double)fz[k];
        }
    }
#pragma unroll
    for (int k = 0; k < kTPT; k++) {
        const int i = t0 + threadIdx.x + k * kTPB;
        if (i >= n) continue;
        if (atomic_out) {
            atomicAdd(&ox[i], sx[k] * back);
            atomicAdd(&oy[i], sy[k] * back);
            atomicAdd(&oz[i], sz[k] * back);
        } else {
            ox[i] = sx[k] * back;
            oy[i] = sy[k] * back;
            oz[i] = sz[k] * back;
        }
    }
}

__global__ void deinterleave(const double *__restrict__ a3, int64_t n, double *__restrict__ x,
                             double *__restrict__ y, double *__restrict__ z) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    x[i] = a3[3 * i];
    y[i] = a3[3 * i + 1];
    z[i] = a3[3 * i + 2];
}

__global__ void interleave(const double *__restrict__ x, const double *__restrict__ y,
                           const double *__restrict__ z, int64_t n, double *__restrict__ a3) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    a3[3 * i] = x[i];
    a3[3 * i + 1] = y[i];
    a3[3 * i + 2] = z[i];
}

int grid_of(int64_t n) { return (int)((n + 255) / 256 > 0 ? (n + 255) / 256 : 1); }
int stream_grid(int64_t n) {
    const int64_t b = (n + 255) / 256;
    return (int)(b < 1 ? 1 : (b > 16 * device_sms() ? 16 * device_sms() : b));
}

sv_status copy_state(sv_ctx *c, double *dst) {
    const size_t b = sizeof(double) * c->n;
    double *src[6] = {c->x, c->y, c->z, c->vx, c->vy, c->vz};
    for (int k = 0; k < 6; k++) SV_CK(c, cudaMemcpyAsync(dst + k * c->n, src[k], b, cudaMemcpyDeviceToDevice, c->stream));
    return SV_OK;
}

sv_status load_state(sv_ctx *c, const double *src) {
    const size_t b = sizeof(double) * c->n;
    double *dst[6] = {c->x, c->y, c->z, c->vx, c->vy, c->vz};
    for (int k = 0; k < 6; k++) SV_CK(c, cudaMemcpyAsync(dst[k], src + k * c->n, b, cudaMemcpyDeviceToDevice, c->stream));
    return SV_OK;
}

// J(x)^T la for the positions currently in c->x, over the particles of
// c->wstatus (the step's window): result added into (lx, ly, lz)
sv_status jtv_add(sv_ctx *c, const double *lax, const double *lay, const double *laz, double *lx, double *ly,
                  double *lz) {
    c->fstatus = c->wstatus;
    const sv_status st = sort_state(c, 0, c->n);
    c->fstatus = nullptr;
    SV_TRY(st);
    Sorted &S = c->S;
    const int n = (int)S.n;
    Adj &A = *c->adj;
    double *ux = A.lam + 9 * A.n, *uy = ux + A.n, *uz = uy + A.n;  // tmp block
    unsigned long long *umax = reinterpret_cast<unsigned long long *>(A.lE + 3);
    SV_CK(c, cudaMemsetAsync(umax, 0, sizeof(*umax), c->stream));
    adj_gather_u<<<grid_of(n), 256, 0, c->stream>>>(S.idx, n, S.qm, lax, lay, laz, ux, uy, uz, umax);
    SV_LAUNCHED(c);
    const int tblocks = div_up(n, kTPB * kTPT);
    int splits = div_up(8 * device_sms(), tblocks);
    const int max_splits = div_up(n, kTile);
    if (splits > max_splits) splits = max_splits;
    if (splits < 1) splits = 1;
    const int chunk = div_up(div_up(n, splits), kTile) * kTile;
    splits = div_up(n, chunk);
    const int atomic_out = splits > 1;
    if (atomic_out) {
        SV_CK(c, cudaMemsetAsync(S.ax, 0, sizeof(double) * n, c->stream));
        SV_CK(c, cudaMemsetAsync(S.ay, 0, sizeof(double) * n, c->stream));
        SV_CK(c, cudaMemsetAsync(S.az, 0, sizeof(double) * n, c->stream));
    }
    const dim3 grid(tblocks, splits);
    if (c->P.precision == SV_PREC_FP64)
        jtv_fp64_kernel<<<grid, kTPB, 0, c->stream>>>(S.x, S.y, S.z, S.q, ux, uy, uz, n, chunk, c->P.softening2, S.ax,
                                                      S.ay, S.az, atomic_out);
    else
        jtv_mixed_kernel<<<grid, kTPB, 0, c->stream>>>(S.x, S.y, S.z, S.q, ux, uy, uz, A.lE + 3, n, chunk,
                                                       c->P.softening2, S.ax, S.ay, S.az, atomic_out);
    SV_LAUNCHED(c);
    adj_post<<<grid_of(n), 256, 0, c->stream>>>(S.idx, n, S.n_orig, S.ax, S.ay, S.az, lx, ly, lz);
    SV_LAUNCHED(c);
    return SV_OK;
}

}  // namespace

void adjoint_free(sv_ctx *c) {
    if (!c->adj) return;
    Adj &A = *c->adj;
    cudaFree(A.ck);
    cudaFree(A.xh);
    cudaFree(A.lam);
    cudaFree(A.fin);
    cudaFree(A.lE);
    delete c->adj;
    c->adj = nullptr;
}

}  // namespace sv

using namespace sv;

extern "C" sv_status sv_adjoint_forward(sv_ctx *c, int32_t nsteps, double dt, double t0, int32_t checkpoint_every) {
    if (!c) return SV_ERR_INVALID;
    if (!c->have_state) return set_error(c, SV_ERR_STATE, "no state uploaded");
    if (nsteps < 0 || !(dt > 0.0) || checkpoint_every < 1)
        return set_error(c, SV_ERR_INVALID, "nsteps >= 0, dt > 0, checkpoint_every >= 1 required");
    if (c->batch) return set_error(c, SV_ERR_UNSUPPORTED, "the adjoint runs on single-plume contexts");
    if (c->P.method != SV_METHOD_DIRECT || c->P.symmetry != SV_SYM_NONE)
        return set_error(c, SV_ERR_UNSUPPORTED, "the adjoint covers the direct sum without symmetry images");
    if (c->B.crash != SV_CRASH_NONE || c->B.bc != SV_BC_NONE || c->B.fold)
        return set_error(c, SV_ERR_UNSUPPORTED, "the adjoint covers drifts without crash, boundary or folding steps");
    if (c->sub.on) return set_error(c, SV_ERR_UNSUPPORTED, "the adjoint covers the single-rate leapfrog");
    if (c->en.on) return set_error(c, SV_ERR_UNSUPPORTED, "the adjoint runs without the energy bookkeeping");
    if (c->field.nt > 0)
        return set_error(c, SV_ERR_UNSUPPORTED, "the adjoint covers the uniform field only (no emitter field map)");
    SV_CK(c, cudaSetDevice(c->device));
    if (!c->adj) c->adj = new Adj();
    Adj &A = *c->adj;
    const int64_t n = c->n;
    const int nck = (nsteps + checkpoint_every - 1) / checkpoint_every + 1;
    const int seg = checkpoint_every < nsteps ? checkpoint_every : (nsteps > 0 ? nsteps : 1);
    if (A.cap < n || A.nck < nck || A.seg_cap < seg) {
        cudaFree(A.ck); cudaFree(A.xh); cudaFree(A.lam); cudaFree(A.fin); cudaFree(A.lE);
        A.ck = A.xh = A.lam = A.fin = A.lE = nullptr;
        const int64_t cap = n > 1 ? n : 1;
        SV_CK(c, cudaMalloc(&A.ck, sizeof(double) * 6 * cap * nck));
        SV_CK(c, cudaMalloc(&A.xh, sizeof(double) * 3 * cap * seg));
        SV_CK(c, cudaMalloc(&A.lam, sizeof(double) * 12 * cap));
        SV_CK(c, cudaMalloc(&A.fin, sizeof(double) * 6 * cap));
        SV_CK(c, cudaMalloc(&A.lE, sizeof(double) * 4));  // lE[3]: max |u| of a step
        A.cap = cap;
        A.nck = nck;
        A.seg_cap = seg;
    }
    A.n = n;
    A.nsteps = nsteps;
    A.every = checkpoint_every;
    A.dt = dt;
    A.t0 = t0;
    for (int s = 0; s < nsteps; s++) {
        if (s % checkpoint_every == 0) SV_TRY(copy_state(c, A.ck + (size_t)(s / checkpoint_every) * 6 * n));
        SV_TRY(leapfrog_step(c, t0 + dt * s, dt, nullptr));
    }
    A.forward_done = true;
    return SV_OK;
}

extern "C" sv_status sv_adjoint_backward(sv_ctx *c, const double *dl_dx3, const double *dl_dv3, double *dl_dx0,
                                         double *dl_dv0, double *dl_defield) {
    if (!c || !dl_dx3 || !dl_dv3) return SV_ERR_INVALID;
    if (!c->adj || !c->adj->forward_done) return set_error(c, SV_ERR_STATE, "sv_adjoint_forward must run first");
    SV_CK(c, cudaSetDevice(c->device));
    Adj &A = *c->adj;
    const int64_t n = A.n;
    if (n != c->n) return set_error(c, SV_ERR_STATE, "state changed since sv_adjoint_forward");
    double *lx = A.lam, *ly = lx + n, *lz = ly + n, *lvx = lz + n, *lvy = lvx + n, *lvz = lvy + n;
    double *lax = lvz + n, *lay = lax + n, *laz = lay + n;
    // final adjoints from the caller (host, 3n interleaved); staging in the tmp block
    double *tmp = A.lam + 9 * n;
    SV_CK(c, cudaMemcpyAsync(tmp, dl_dx3, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, c->stream));
    deinterleave<<<grid_of(n), 256, 0, c->stream>>>(tmp, n, lx, ly, lz);
    SV_LAUNCHED(c);
    SV_CK(c, cudaMemcpyAsync(tmp, dl_dv3, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, c->stream));
    deinterleave<<<grid_of(n), 256, 0, c->stream>>>(tmp, n, lvx, lvy, lvz);
    SV_LAUNCHED(c);
    SV_CK(c, cudaMemsetAsync(A.lE, 0, sizeof(double) * 3, c->stream));
    SV_TRY(copy_state(c, A.fin));
    const double dt = A.dt;
    for (int k = (A.nsteps - 1) / A.every; k >= 0 && A.nsteps > 0; k--) {
        const int s0 = k * A.every;
        const int s1 = s0 + A.every < A.nsteps ? s0 + A.every : A.nsteps;
        // recompute the segment from its checkpoint, keeping every x_h
        SV_TRY(load_state(c, A.ck + (size_t)k * 6 * n));
        for (int s = s0; s < s1; s++)
            SV_TRY(leapfrog_step(c, A.t0 + dt * s, dt, A.xh + (size_t)(s - s0) * 3 * n));
        for (int s = s1 - 1; s >= s0; s--) {
            const double ts = A.t0 + dt * s;
            const double *xh = A.xh + (size_t)(s - s0) * 3 * n;
            SV_CK(c, cudaMemcpyAsync(c->x, xh, sizeof(double) * n, cudaMemcpyDeviceToDevice, c->stream));
            SV_CK(c, cudaMemcpyAsync(c->y, xh + n, sizeof(double) * n, cudaMemcpyDeviceToDevice, c->stream));
            SV_CK(c, cudaMemcpyAsync(c->z, xh + 2 * n, sizeof(double) * n, cudaMemcpyDeviceToDevice, c->stream));
            SV_TRY(window_status(c, ts + 0.5 * dt));
            adj_prep<<<stream_grid(n), 256, 0, c->stream>>>(lx, ly, lz, lvx, lvy, lvz, lax, lay, laz, c->q, c->m,
                                                            c->status, c->wstatus, c->t_inj, n, ts, dt,
                                                            c->P.e_over_amu, A.lE);
            SV_LAUNCHED(c);
            SV_TRY(jtv_add(c, lax, lay, laz, lx, ly, lz));
            adj_drift_back<<<stream_grid(n), 256, 0, c->stream>>>(lx, ly, lz, lvx, lvy, lvz, c->status, c->t_inj, n,
                                                                  ts, dt);
            SV_LAUNCHED(c);
        }
    }
    SV_TRY(load_state(c, A.fin));
    if (dl_dx0) {
        interleave<<<grid_of(n), 256, 0, c->stream>>>(lx, ly, lz, n, tmp);
        SV_LAUNCHED(c);
        SV_CK(c, cudaMemcpyAsync(dl_dx0, tmp, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, c->stream));
        SV_CK(c, cudaStreamSynchronize(c->stream));
    }
    if (dl_dv0) {
        interleave<<<grid_of(n), 256, 0, c->stream>>>(lvx, lvy, lvz, n, tmp);
        SV_LAUNCHED(c);
        SV_CK(c, cudaMemcpyAsync(dl_dv0, tmp, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, c->stream));
        SV_CK(c, cudaStreamSynchronize(c->stream));
    }
    if (dl_defield) {
        SV_CK(c, cudaMemcpyAsync(c->h_scalar, A.lE, sizeof(double) * 3, cudaMemcpyDeviceToHost, c->stream));
        SV_CK(c, cudaStreamSynchronize(c->stream));
        for (int d = 0; d < 3; d++) dl_defield[d] = c->h_scalar[d];
    }
    SV_CK(c, cudaStreamSynchronize(c->stream));
    return SV_OK;
}
