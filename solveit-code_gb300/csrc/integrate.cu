// integrate.cu -- FP64 leapfrog pieces and the energy diagnostic.
//
// drift: ParticleSystem::propagatePositionNew (particles.cpp:33-40):
//        ChargedParticles::propagatePositionNew (particles.cpp:693-739),
//        x += v * clamp(t_start + h - t_inj, 0, h) for status 1 or 2, with the
//        extractor-grid crash test (structures.h:467-517); then
//        enforceSymmetryConditions (particles.cpp:199-333) and
//        enforceBoundaryConditions (particles.cpp:73-177).  Only particles
//        inside the injection window (t_inj <= t_start + h: LeapfrogDKD::
//        driftNew and findMostRecentInjected, integration_schemes.cpp:705-723,
//        particles.cpp:1328-1366) are touched.
// kick:  computeBackgroundAcceleration (particles.cpp:496-520) with a uniform
//        field + propagateVelocityNew (particles.cpp:763-786)
//        v += (a + (e/amu)(q/m) E) * clamp(t_start + dt - t_inj, 0, dt) for
//        windowed status 1.
// Both are HBM-bound streams (drift 60 B, kick 92 B per particle).
// energy: computeChargedKineticEnergy / computeChargedElectricPotentialEnergy
//        (particles.cpp:535-578), FP64, all particles, potential halved.
#include "sv_internal.cuh"

#include <algorithm>
#include <numeric>
#include <vector>

namespace sv {
namespace {

struct DriftArgs {
    double *x, *y, *z, *vx, *vy, *vz;
    int32_t *st;
    const double *t_inj;
    const int32_t *species;
    int32_t *window;  // status for the force and kick of the step, or null
    int64_t n;
    double t_start, h;
    const double *tb;
    long long seq_base;
    // crash (extractor grid), boundary conditions, folding
    int crash, bc, fold;    // fold: 0 none, 1 rotational, 2 translational, 3 per particle from pfold
    const int8_t *pfold;
    double cz, cw, cr;
    double bsx, bsy, bsz, bsr, bt;
    double Lx, Ly, Lz;
    int ax, ay, az;
    // event log
    sv_event *ev;
    unsigned long long *ev_key, *ev_count;
    long long ev_cap;
};

// std::max / std::min as the reference calls them (a NaN operand falls through the same way)
__device__ __forceinline__ double ref_max(double a, double b) { return a < b ? b : a; }
__device__ __forceinline__ double ref_min(double a, double b) { return b < a ? b : a; }

// CrashParameters::checkExtractorGridCrash (structures.h:467-517): does the
// drift segment (r0, z0) -> (r1, z1) of the (r, z) plane cross the bottom,
// top or inner side of the grid?  *zc receives the z of the crossing.
__device__ bool extractor_crash(double x0, double y0, double z0, double x1, double y1, double z1, double zd,
                                double zw, double rd, double *zc) {
    const double ri = sqrt(x0 * x0 + y0 * y0), rf = sqrt(x1 * x1 + y1 * y1);
    const double m = (z1 - z0) / (rf - ri);
    const double b = z0 - m * ri;
    const double rmin = ref_min(ri, rf), rmax = ref_max(ri, rf);
    const double zmin = ref_min(z0, z1), zmax = ref_max(z0, z1);
    if (zd >= zmin && zd <= zmax) {
        const double tr = (zd - b) / m;
        if (tr >= ref_max(rmin, rd) && tr <= rmax) {
            *zc = zd;
            return true;
        }
    }
    const double zt = zd + zw;
    if (zt >= zmin && zt <= zmax) {
        const double tr = (zt - b) / m;
        if (tr >= ref_max(rmin, rd) && tr <= rmax) {
            *zc = zt;
            return true;
        }
    }
    if (rd >= rmin && rd <= rmax) {
        const double tz = m * rd + b;
        if (tz >= ref_max(zmin, zd) && tz <= ref_min(zmax, zt)) {
            *zc = tz;
            return true;
        }
    }
    return false;
}

// ParticleSystem::translateToSymmetryDomain, one axis (particles.cpp:278-333)
__device__ __forceinline__ double wrap_axis(double p, double L) {
    double t = p + L / 2;
    if (t >= 0) return fmod(t, L) - L / 2;
    t = fmod(t, L);
    return t < 0 ? t + L / 2 : t - L / 2;
}

// phase 0 crash, 1 spatial, 2 temporal: the reference writes each kind of
// event in its own pass over the particles
__device__ void record_event(const DriftArgs &a, long long seq, int phase, int64_t i, double t, double x, double y,
                             double z, double vx, double vy, double vz, int32_t status) {
    const unsigned long long slot = atomicAdd(a.ev_count, 1ull);
    if ((long long)slot >= a.ev_cap) return;
    sv_event e;
    e.time = (float)t;
    e.x = (float)x;
    e.y = (float)y;
    e.z = (float)z;
    e.vx = (float)vx;
    e.vy = (float)vy;
    e.vz = (float)vz;
    e.index = (int32_t)i;
    e.species = a.species ? (uint32_t)a.species[i] : 0xffffffffu;
    e.status = status;
    a.ev[slot] = e;
    a.ev_key[slot] = ((unsigned long long)seq << 34) | ((unsigned long long)phase << 32) | (unsigned long long)(uint32_t)i;
}

// FULL = false: no crash test, folding or boundary conditions (the common
// case), compiled without their code so the streaming loop keeps few registers
template <bool FULL>
__global__ void drift_kernel(DriftArgs a) {
    double t_start = a.t_start;
    long long seq = a.seq_base;
    if (a.tb) {
        t_start += a.tb[0] + a.tb[1] * a.tb[2];
        seq += (long long)a.tb[3] + 2 * (long long)a.tb[2];
    }
    const double h = a.h, T = t_start + h;
    // the arrays are distinct: restrict-qualified copies let the loads and
    // stores of one particle be scheduled freely
    double *__restrict__ px = a.x, *__restrict__ py = a.y, *__restrict__ pz = a.z;
    double *__restrict__ pvx = a.vx, *__restrict__ pvy = a.vy;
    const double *__restrict__ pvz = a.vz, *__restrict__ tinj = a.t_inj;
    int32_t *__restrict__ pst = a.st, *__restrict__ win = a.window;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < a.n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double ti = tinj[i];
        if (!(ti <= T)) {  // not injected by the end of this half step: outside the window
            if (win) win[i] = 0;
            continue;
        }
        int32_t w = pst[i];
        if (!FULL) {
            if (w == 1 || w == 2) {
                const double s = fmin(fmax(T - ti, 0.0), h);
                px[i] += pvx[i] * s;
                py[i] += pvy[i] * s;
                pz[i] += pvz[i] * s;
            }
            if (win) win[i] = w;
            continue;
        }
        const int32_t w0 = w;
        double x = px[i], y = py[i], z = pz[i];
        double vx = pvx[i], vy = pvy[i], vz = pvz[i];
        const double x0 = x, y0 = y, z0 = z, vx0 = vx, vy0 = vy;
        if (w == 1 || w == 2) {
            const double s = fmin(fmax(T - ti, 0.0), h);
            x += vx * s;
            y += vy * s;
            z += vz * s;
            double zc;
            if (FULL && a.crash == SV_CRASH_EXTRACTOR_GRID &&
                extractor_crash(x0, y0, z0, x, y, z, a.cz, a.cw, a.cr, &zc)) {
                w = -1;
                z = zc;
                const double td = (zc - z0) / vz;
                x = x0 + td * vx;
                y = y0 + td * vy;
                record_event(a, seq, 0, i, t_start + td, x, y, z, vx, vy, vz, w);
            }
        }
        const int fold = !FULL ? 0 : a.fold == 3 ? a.pfold[i] : a.fold;
        if (fold == 1) {
            // ParticleSystem::rotateToFirstQuadrant (particles.cpp:225-264)
            if (x < 0 && y < 0) {
                x = -x; y = -y; vx = -vx; vy = -vy;
            } else if (x < 0) {
                const double tx = y, ty = -x, tvx = vy, tvy = -vx;
                x = tx; y = ty; vx = tvx; vy = tvy;
            } else if (y < 0) {
                const double tx = -y, ty = x, tvx = -vy, tvy = vx;
                x = tx; y = ty; vx = tvx; vy = tvy;
            }
        } else if (fold == 2) {
            if (a.ax) x = wrap_axis(x, a.Lx);
            if (a.ay) y = wrap_axis(y, a.Ly);
            if (a.az) z = wrap_axis(z, a.Lz);
        }
        if (FULL && w == 1 && (a.bc == SV_BC_SPACE || a.bc == SV_BC_SPACE_AND_TIME)) {
            // checkOutOfSpatialBounds (particles.cpp:117-139)
            const bool out = (a.bsx != 0 && fabs(x) > a.bsx) || (a.bsy != 0 && fabs(y) > a.bsy) ||
                             (a.bsz != 0 && fabs(z) > a.bsz) || (a.bsr != 0 && sqrt(x * x + y * y) > a.bsr);
            if (out) {
                w = 0;
                record_event(a, seq, 1, i, T, x, y, z, vx, vy, vz, w);
            }
        }
        if (FULL && w == 1 && (a.bc == SV_BC_TIME || a.bc == SV_BC_SPACE_AND_TIME)) {
            // checkOutOfTemporalBounds (particles.cpp:163-168)
            if (T - ti > a.bt) {
                w = 0;
                record_event(a, seq, 2, i, T, x, y, z, vx, vy, vz, w);
            }
        }
        if (x != x0 || y != y0 || z != z0) {
            px[i] = x;
            py[i] = y;
            pz[i] = z;
        }
        if (vx != vx0 || vy != vy0) {
            pvx[i] = vx;
            pvy[i] = vy;
        }
        if (w != w0) pst[i] = w;
        if (win) win[i] = w;
    }
}

// With an emitter field map (FIELD: M.nt > 0) the field at the particle is
// added to the uniform one: computeBackgroundAcceleration (particles.cpp:496-520).
template <bool FIELD>
__global__ void kick_kernel(double *__restrict__ vx, double *__restrict__ vy, double *__restrict__ vz,
                            const double *__restrict__ ax, const double *__restrict__ ay,
                            const double *__restrict__ az, const double *__restrict__ qom,
                            const int32_t *__restrict__ st,
                            const double *__restrict__ t_inj, int64_t n, double t_start, double dt,
                            double eoa, double ex, double ey, double ez, const double *__restrict__ tb,
                            const double *__restrict__ x, const double *__restrict__ y,
                            const double *__restrict__ z, FieldMesh M, float *__restrict__ e2,
                            float *__restrict__ e1) {
    if (tb) t_start += tb[0] + tb[1] * tb[2];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        if (st[i] != 1) continue;
        const double f = eoa * qom[i];
        const double s = fmin(fmax(t_start + dt - t_inj[i], 0.0), dt);
        double fx = ex, fy = ey, fz = ez;
        if (FIELD) {
            int t = M.cache[i];
            double gx, gy, gz;
            field_at(M, x[i], y[i], z[i], &t, &gx, &gy, &gz);
            M.cache[i] = t;
            fx += gx;
            fy += gy;
            fz += gz;
        }
        // the snapshot records' fields: the force's acceleration (turned into
        // E1 = (amu/e)(m/q) a when a snapshot is packed) and E2
        e1[3 * i] = (float)ax[i];
        e1[3 * i + 1] = (float)ay[i];
        e1[3 * i + 2] = (float)az[i];
        e2[3 * i] = (float)fx;  // Efield2 of the snapshot records (particles.cpp:512)
        e2[3 * i + 1] = (float)fy;
        e2[3 * i + 2] = (float)fz;
        vx[i] += (ax[i] + fx * f) * s;
        vy[i] += (ay[i] + fy * f) * s;
        vz[i] += (az[i] + fz * f) * s;
    }
}

__global__ void window_kernel(const int32_t *__restrict__ st, const double *__restrict__ t_inj, int64_t n, double T,
                              int32_t *__restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        out[i] = t_inj[i] <= T ? st[i] : 0;
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
    const int64_t cap = 16LL * device_sms();
    return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

}  // namespace

sv_status events_reserve(sv_ctx *c) {
    const int64_t want = std::max<int64_t>(65536, c->n);
    if (c->d_events && c->ev_cap >= want) return SV_OK;
    events_free(c);
    SV_CK(c, cudaMalloc(&c->d_events, sizeof(sv_event) * want));
    SV_CK(c, cudaMalloc(&c->d_ev_key, sizeof(unsigned long long) * want));
    SV_CK(c, cudaMalloc(&c->d_ev_count, sizeof(unsigned long long)));
    SV_CK(c, cudaMemsetAsync(c->d_ev_count, 0, sizeof(unsigned long long), c->stream));
    c->ev_cap = want;
    return SV_OK;
}

void events_free(sv_ctx *c) {
    cudaFree(c->d_events);
    cudaFree(c->d_ev_key);
    cudaFree(c->d_ev_count);
    c->d_events = nullptr;
    c->d_ev_key = nullptr;
    c->d_ev_count = nullptr;
    c->ev_cap = 0;
}

sv_status drift(sv_ctx *c, double t_start, double h, int32_t *window, const double *tb, long long seq_base) {
    const sv_boundary &B = c->B;
    DriftArgs a{};
    a.x = c->x; a.y = c->y; a.z = c->z;
    a.vx = c->vx; a.vy = c->vy; a.vz = c->vz;
    a.st = c->status;
    a.t_inj = c->t_inj;
    a.species = c->species;
    a.window = window;
    a.n = c->n;
    a.t_start = t_start;
    a.h = h;
    a.tb = tb;
    a.seq_base = tb ? seq_base : c->ev_seq;
    a.crash = B.crash;
    a.bc = B.bc;
    a.fold = !B.fold ? 0 : c->pfold ? 3 : c->P.symmetry == SV_SYM_ROTATIONAL ? 1
                              : c->P.symmetry == SV_SYM_TRANSLATIONAL ? 2 : 0;
    a.pfold = c->pfold;
    a.cz = B.crash_z; a.cw = B.crash_width; a.cr = B.crash_r;
    a.bsx = B.bc_space[0]; a.bsy = B.bc_space[1]; a.bsz = B.bc_space[2]; a.bsr = B.bc_space[3];
    a.bt = B.bc_time;
    a.Lx = c->P.domain_size[0]; a.Ly = c->P.domain_size[1]; a.Lz = c->P.domain_size[2];
    a.ax = c->P.sym_axes[0]; a.ay = c->P.sym_axes[1]; a.az = c->P.sym_axes[2];
    a.ev = c->d_events;
    a.ev_key = c->d_ev_key;
    a.ev_count = c->d_ev_count;
    a.ev_cap = c->ev_cap;
    if (a.crash != SV_CRASH_NONE || a.bc != SV_BC_NONE || a.fold != 0)
        drift_kernel<true><<<stream_grid(c->n), 256, 0, c->stream>>>(a);
    else
        drift_kernel<false><<<stream_grid(c->n), 256, 0, c->stream>>>(a);
    SV_LAUNCHED(c);
    if (!tb) c->ev_seq++;
    return SV_OK;
}

sv_status kick(sv_ctx *c, double t_start, double dt, const int32_t *st, const double *tb) {
    auto k = c->field.nt > 0 ? kick_kernel<true> : kick_kernel<false>;
    k<<<stream_grid(c->n), 256, 0, c->stream>>>(c->vx, c->vy, c->vz, c->ax, c->ay, c->az, c->qom, st, c->t_inj,
                                                c->n, t_start, dt, c->P.e_over_amu, c->P.efield[0], c->P.efield[1],
                                                c->P.efield[2], tb, c->x, c->y, c->z, c->field, c->e2, c->e1);
    SV_LAUNCHED(c);
    return SV_OK;
}

sv_status window_status(sv_ctx *c, double t_window) {
    window_kernel<<<stream_grid(c->n), 256, 0, c->stream>>>(c->status, c->t_inj, c->n, t_window, c->wstatus);
    SV_LAUNCHED(c);
    return SV_OK;
}

sv_status leapfrog_step(sv_ctx *c, double ts, double dt, double *save_xh) {
    const double h = 0.5 * dt;
    if (c->B.crash != SV_CRASH_NONE || c->B.bc != SV_BC_NONE) SV_TRY(events_reserve(c));
    SV_TRY(field_prepare(c));
    SV_TRY(energy_inject(c, ts + h));
    SV_TRY(drift(c, ts, h, c->wstatus));
    SV_TRY(energy_first(c, ts + h));
    if (save_xh) {
        const size_t b = sizeof(double) * c->n;
        SV_CK(c, cudaMemcpyAsync(save_xh, c->x, b, cudaMemcpyDeviceToDevice, c->stream));
        SV_CK(c, cudaMemcpyAsync(save_xh + c->n, c->y, b, cudaMemcpyDeviceToDevice, c->stream));
        SV_CK(c, cudaMemcpyAsync(save_xh + 2 * c->n, c->z, b, cudaMemcpyDeviceToDevice, c->stream));
    }
    c->fstatus = c->wstatus;
    const sv_status s = compute_accel_device(c, 0, c->n);
    c->fstatus = nullptr;
    SV_TRY(s);
    SV_TRY(kick(c, ts, dt, c->wstatus));
    SV_TRY(energy_inject(c, ts + dt));
    SV_TRY(drift(c, ts + h, h, nullptr));
    SV_TRY(energy_first(c, ts + dt));
    return energy_interval(c, ts, dt);
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
