// integrate.cu -- FP64 leapfrog pieces and the energy diagnostic.
//
// drift: ChargedParticles::propagatePositionNew (particles.cpp:693-739)
//        x += v * clamp(t_start + h - t_inj, 0, h) for status 1 or 2.
// kick:  computeBackgroundAcceleration (particles.cpp:496-520) with a uniform
//        field + propagateVelocityNew (particles.cpp:763-786)
//        v += (a + (e/amu)(q/m) E) * clamp(t_start + dt - t_inj, 0, dt) for
//        status 1.
// Both are HBM-bound streams (drift 56 B, kick 88 B per particle).
// energy: computeChargedKineticEnergy / computeChargedElectricPotentialEnergy
//        (particles.cpp:535-578), FP64, all particles, potential halved.
#include "sv_internal.cuh"

namespace sv {
namespace {

__global__ void drift_kernel(double *__restrict__ x, double *__restrict__ y, double *__restrict__ z,
                             const double *__restrict__ vx, const double *__restrict__ vy,
                             const double *__restrict__ vz, const int32_t *__restrict__ st,
                             const double *__restrict__ t_inj, int64_t n, double t_start, double h,
                             const double *__restrict__ tb) {
    if (tb) t_start += tb[0] + tb[1] * tb[2];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t w = st[i];
        if (!(w == 1 || w == 2)) continue;
        const double s = fmin(fmax(t_start + h - t_inj[i], 0.0), h);
        x[i] += vx[i] * s;
        y[i] += vy[i] * s;
        z[i] += vz[i] * s;
    }
}

__global__ void kick_kernel(double *__restrict__ vx, double *__restrict__ vy, double *__restrict__ vz,
                            const double *__restrict__ ax, const double *__restrict__ ay,
                            const double *__restrict__ az, const double *__restrict__ qom,
                            const int32_t *__restrict__ st,
                            const double *__restrict__ t_inj, int64_t n, double t_start, double dt,
                            double eoa, double ex, double ey, double ez, const double *__restrict__ tb) {
    if (tb) t_start += tb[0] + tb[1] * tb[2];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        if (st[i] != 1) continue;
        const double f = eoa * qom[i];
        const double s = fmin(fmax(t_start + dt - t_inj[i], 0.0), dt);
        vx[i] += (ax[i] + ex * f) * s;
        vy[i] += (ay[i] + ey * f) * s;
        vz[i] += (az[i] + ez * f) * s;
    }
}

constexpr int kETile = 256;

// Potential energy: per target sum_j q_i q_j / sqrt(r^2 + eps^2), FP64, with
// each CTA accumulating its partial into one double (atomicAdd).
__global__ void potential_kernel(const double *__restrict__ x, const double *__restrict__ y,
                                 const double *__restrict__ z, const double *__restrict__ q, int64_t n,
                                 double eps2, double *__restrict__ out) {
    __shared__ dbl4_t tile[kETile];
    __shared__ double red[8];
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const bool live = i < n;
    const double xi = live ? x[i] : 0.0, yi = live ? y[i] : 0.0, zi = live ? z[i] : 0.0;
    const double qi = live ? q[i] : 0.0;
    double s = 0.0;
    for (int64_t jt = 0; jt < n; jt += kETile) {
        __syncthreads();
        for (int k = threadIdx.x; k < kETile; k += blockDim.x) {
            const int64_t j = jt + k;
            tile[k] = j < n ? dbl4(x[j], y[j], z[j], q[j]) : dbl4(0, 0, 0, 0);
        }
        __syncthreads();
        const int lim = (int)min((int64_t)kETile, n - jt);
        for (int k = 0; k < lim; k++) {
            if (jt + k == i) continue;
            const dbl4_t v = tile[k];
            const double dx = xi - v.x, dy = yi - v.y, dz = zi - v.z;
            s += v.w / sqrt(dx * dx + dy * dy + dz * dz + eps2);
        }
    }
    s *= qi;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
        atomicAdd(out, t);
    }
}

__global__ void kinetic_kernel(const double *__restrict__ vx, const double *__restrict__ vy,
                               const double *__restrict__ vz, const double *__restrict__ m, int64_t n,
                               double *__restrict__ out) {
    __shared__ double red[8];
    double s = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        s += m[i] * (vx[i] * vx[i] + vy[i] * vy[i] + vz[i] * vz[i]);
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
        atomicAdd(out, t);
    }
}

int stream_grid(int64_t n) {
    int64_t b = (n + 255) / 256;
    const int64_t cap = 16LL * kNumSMs;
    return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

}  // namespace

sv_status drift(sv_ctx *c, double t_start, double h, const double *tb) {
    drift_kernel<<<stream_grid(c->n), 256, 0, c->stream>>>(c->x, c->y, c->z, c->vx, c->vy, c->vz, c->status,
                                                           c->t_inj, c->n, t_start, h, tb);
    SV_LAUNCHED(c);
    return SV_OK;
}

sv_status kick(sv_ctx *c, double t_start, double dt, const double *tb) {
    kick_kernel<<<stream_grid(c->n), 256, 0, c->stream>>>(
        c->vx, c->vy, c->vz, c->ax, c->ay, c->az, c->qom, c->status, c->t_inj, c->n, t_start, dt,
        c->P.e_over_amu, c->P.efield[0], c->P.efield[1], c->P.efield[2], tb);
    SV_LAUNCHED(c);
    return SV_OK;
}

sv_status energy(sv_ctx *c, double *ke, double *pe) {
    // constants as the reference evaluates them (particles.cpp:540-566)
    const float e = 1.6021766e-19f, amu = 1.66053904e-27f, eps0 = 8.85419e-12f;
    const long double pi = 3.14159265358979323846264338328L;
    const double kc = (double)(float)(1 / (4.0 * pi * eps0));
    SV_CK(c, cudaMemsetAsync(c->d_scalar, 0, 2 * sizeof(double), c->stream));
    kinetic_kernel<<<stream_grid(c->n), 256, 0, c->stream>>>(c->vx, c->vy, c->vz, c->m, c->n, c->d_scalar);
    SV_LAUNCHED(c);
    potential_kernel<<<div_up(c->n, 256), 256, 0, c->stream>>>(c->x, c->y, c->z, c->q, c->n,
                                                                c->P.softening2, c->d_scalar + 1);
    SV_LAUNCHED(c);
    SV_CK(c, cudaMemcpyAsync(c->h_scalar, c->d_scalar, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    SV_CK(c, cudaStreamSynchronize(c->stream));
    *ke = 0.5 * (double)amu * c->h_scalar[0];
    *pe = 0.5 * c->h_scalar[1] * (double)e * (double)e * kc;
    return SV_OK;
}

}  // namespace sv
