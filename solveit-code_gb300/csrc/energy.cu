// energy.cu -- the energy bookkeeping of the reference's integrator on the
// device: Integrator::initializeEnergyData / updateEnergyInjectionData /
// updateEnergyIntervalData (integration_schemes.cpp:757-835) with
// ParticleSystem's kinetic, potential and field energies (particles.cpp:
// 526-638).
//
// The reference keeps an index window [firstParticle, lastParticle): last
// follows the injection times (findMostRecentInjected), first moves past the
// particles that are neither inbound nor source-only (resetFirstChargedParticle,
// particles.cpp:183-194).  Here the window is {i >= first : t_inj[i] <= t},
// first a device word moved by the same rule after every drift.
//   potential: each particle of a pass is a target of a direct sum over the
//     window (its own index excluded): FP32 pairs on positions split into
//     FP32 hi + lo parts (the difference of two hi parts is exact for close
//     pairs), Kahan-compensated per thread, FP64 across blocks;
//   field energy: the work of the emitter's field along z at the start's
//     (x, y), then along (x, y) at the end's z, left-point samples at
//     FP32-rounded points as the reference passes them to Efield.
#include <cub/cub.cuh>
#include <thrust/iterator/counting_iterator.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "sv_internal.cuh"

namespace sv {
namespace {

constexpr int kPotT = 256;  // targets (threads) per block of the potential kernel

// constants as the reference evaluates them (constants.h:28-47, particles.cpp:540-566)
constexpr float kElemCharge = 1.6021766e-19f;
constexpr float kAmu = 1.66053904e-27f;
constexpr float kEps0 = 8.85419e-12f;

double pe_coef() {
    const long double pi = 3.14159265358979323846264338328L;
    const float ke = (float)(1 / (4.0 * pi * kEps0));
    const float q2 = kElemCharge * kElemCharge;
    return (double)q2 * (double)ke;
}

// work of the field (V) from a to b: along z at a's (x, y), then along (x, y) at b's z
__device__ double path_work(const FieldMesh &M, int *walk, double ax, double ay, double az, double bx, double by,
                            double bz, int steps) {
    const double dx = bx - ax, dy = by - ay, dz = bz - az;
    double tz = 0.0, tr = 0.0, ex, ey, ez;
    int t = *walk;
    for (int k = 0; k < steps; k++) {
        const double pz = az + k * dz / steps;
        field_at(M, (double)(float)ax, (double)(float)ay, (double)(float)pz, &t, &ex, &ey, &ez);
        tz += ez * dz / steps;
    }
    for (int k = 0; k < steps; k++) {
        const double px = ax + k * dx / steps, py = ay + k * dy / steps;
        field_at(M, (double)(float)px, (double)(float)py, (double)(float)bz, &t, &ex, &ey, &ez);
        tr += ex * dx / steps + ey * dy / steps;
    }
    *walk = t;
    return tz + tr;
}

// initializeEnergyData: kinetic energy, field energy from the reference
// position, path start = the particle
__global__ void init_kernel(int64_t n, const double *__restrict__ x, const double *__restrict__ y,
                            const double *__restrict__ z, const double *__restrict__ vx,
                            const double *__restrict__ vy, const double *__restrict__ vz,
                            const double *__restrict__ q, const double *__restrict__ m, FieldMesh M, int steps,
                            double zref, int *__restrict__ walk, double *__restrict__ fe,
                            double *__restrict__ ke_inj, double *__restrict__ ix, double *__restrict__ iy,
                            double *__restrict__ iz) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    ke_inj[i] = 0.5 * (double)kAmu * m[i] * (vx[i] * vx[i] + vy[i] * vy[i] + vz[i] * vz[i]);
    double w = 0.0;
    if (M.nt > 0) {
        int t = -1;
        w = path_work(M, &t, 0.0, 0.0, zref, x[i], y[i], z[i], steps);
        walk[i] = t;
    }
    fe[i] = -(double)kElemCharge * q[i] * w;
    ix[i] = x[i];
    iy[i] = y[i];
    iz[i] = z[i];
}

// the particles injected since the previous pass: t_prev < t_inj <= t
struct InjectedSel {
    const double *t_inj;
    double t, t_prev;
    int have_prev;
    __device__ bool operator()(const int &i) const {
        const double ti = t_inj[i];
        return ti <= t && !(have_prev && ti <= t_prev);
    }
};

// the window: index >= first, t_inj <= t
struct WindowSel {
    const double *t_inj;
    const unsigned long long *first;
    double t;
    __device__ bool operator()(const int &i) const { return (unsigned long long)i >= first[0] && t_inj[i] <= t; }
};

// positions as FP32 hi + lo, charge of the window's members (0 for the rest),
// index bits for the self-pair test
__global__ void split_kernel(int64_t n, const double *__restrict__ x, const double *__restrict__ y,
                             const double *__restrict__ z, const double *__restrict__ q,
                             const double *__restrict__ t_inj, const unsigned long long *__restrict__ first,
                             double t, float4 *__restrict__ ph, float4 *__restrict__ pl) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const bool in = (unsigned long long)i >= first[0] && t_inj[i] <= t;
    const float hx = (float)x[i], hy = (float)y[i], hz = (float)z[i];
    ph[i] = make_float4(hx, hy, hz, in ? (float)q[i] : 0.f);
    pl[i] = make_float4((float)(x[i] - (double)hx), (float)(y[i] - (double)hy), (float)(z[i] - (double)hz),
                        __int_as_float((int)i));
}

__device__ __forceinline__ void kahan(float &s, float &c, float v) {
    const float y = v - c, t = s + y;
    c = (t - s) - y;
    s = t;
}

// pot[k] += sum over window sources j != list[k] of q_j / sqrt(r^2 + eps2),
// the sources [first, n) split over gridDim.y blocks
__global__ void __launch_bounds__(kPotT)
potential_kernel(const int *__restrict__ list, const int *__restrict__ cnt, const float4 *__restrict__ ph,
                 const float4 *__restrict__ pl, const unsigned long long *__restrict__ first, int64_t n, float eps2,
                 double *__restrict__ pot) {
    __shared__ float4 sh[kPotT], sl[kPotT];
    const int nt = *cnt;
    const int k = blockIdx.x * kPotT + threadIdx.x;
    const int i = list[min(k, nt - 1)];
    const float4 th = ph[i], tl = pl[i];
    const int64_t j0 = (int64_t)first[0];
    const int64_t per = (n - j0 + gridDim.y - 1) / gridDim.y;
    const int64_t s0 = j0 + per * blockIdx.y, s1 = min(n, s0 + per);
    float s = 0.f, c = 0.f;
    for (int64_t t0 = s0; t0 < s1; t0 += kPotT) {
        __syncthreads();
        const int64_t j = t0 + threadIdx.x;
        sh[threadIdx.x] = j < s1 ? ph[j] : make_float4(0.f, 0.f, 0.f, 0.f);
        sl[threadIdx.x] = j < s1 ? pl[j] : make_float4(0.f, 0.f, 0.f, __int_as_float(-1));
        __syncthreads();
        float part = 0.f;
#pragma unroll 8
        for (int u = 0; u < kPotT; u++) {
            const float4 a = sh[u], b = sl[u];
            const float dx = (th.x - a.x) + (tl.x - b.x);
            const float dy = (th.y - a.y) + (tl.y - b.y);
            const float dz = (th.z - a.z) + (tl.z - b.z);
            const float r2 = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, eps2)));
            const float w = __float_as_int(b.w) == i ? 0.f : a.w;
            part = fmaf(w, rsqrt_ftz(fmaxf(r2, kMinR2)), part);
        }
        kahan(s, c, part);
    }
    if (k < nt) atomicAdd(&pot[k], (double)(s - c));
}

// block sums of three per-entry values into acc[0..2]
__device__ void add3(double a, double b, double cc, double *acc) {
    __shared__ double red[3][8];
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
        cc += __shfl_xor_sync(0xffffffffu, cc, o);
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        red[0][w] = a;
        red[1][w] = b;
        red[2][w] = cc;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double t = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) t += red[threadIdx.x][k];
        atomicAdd(&acc[threadIdx.x], t);
    }
}

// updateEnergyInjectionData: KE_inj += ke_inj, PE_inj += q pot, FE_inj += fe
__global__ void inject_sums(const int *__restrict__ list, const int *__restrict__ cnt,
                            const double *__restrict__ ke_inj, const double *__restrict__ q,
                            const double *__restrict__ pot, const double *__restrict__ fe, double *__restrict__ acc) {
    const int nt = *cnt;
    double a = 0.0, b = 0.0, cc = 0.0;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nt; k += gridDim.x * blockDim.x) {
        const int i = list[k];
        a += ke_inj[i];
        b += q[i] * pot[k];
        cc += fe[i];
    }
    add3(a, b, cc, acc);
}

// updateEnergyIntervalData, per window particle: the field energy of the path
// moved since the last update (samples per leg as the reference counts them,
// in FP32), then the path restarts at the particle
__global__ void interval_fe(const int *__restrict__ list, const int *__restrict__ cnt, const double *__restrict__ x,
                            const double *__restrict__ y, const double *__restrict__ z, const double *__restrict__ q,
                            const double *__restrict__ t_inj, FieldMesh M, float tpos, float dtf, int interval,
                            int steps, int *__restrict__ walk, double *__restrict__ fe, double *__restrict__ ix,
                            double *__restrict__ iy, double *__restrict__ iz) {
    const int nt = *cnt;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nt) return;
    const int i = list[k];
    if (M.nt > 0) {
        const float tt = fminf(__fmul_rn(dtf, (float)interval), __fsub_rn(tpos, (float)t_inj[i]));
        const int ns = (int)fmaxf(__fdiv_rn(__fmul_rn(tt, (float)steps), dtf), 2.0f);
        int t = walk[i];
        const double w = path_work(M, &t, ix[i], iy[i], iz[i], x[i], y[i], z[i], ns);
        walk[i] = t;
        fe[i] += -(double)kElemCharge * q[i] * w;
    }
    ix[i] = x[i];
    iy[i] = y[i];
    iz[i] = z[i];
}

// KE, q pot, FE of the window into acc[3..5]
__global__ void interval_sums(const int *__restrict__ list, const int *__restrict__ cnt,
                              const double *__restrict__ vx, const double *__restrict__ vy,
                              const double *__restrict__ vz, const double *__restrict__ m,
                              const double *__restrict__ q, const double *__restrict__ pot,
                              const double *__restrict__ fe, double *__restrict__ acc) {
    const int nt = *cnt;
    double a = 0.0, b = 0.0, cc = 0.0;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nt; k += gridDim.x * blockDim.x) {
        const int i = list[k];
        a += 0.5 * (double)kAmu * m[i] * (vx[i] * vx[i] + vy[i] * vy[i] + vz[i] * vz[i]);
        b += q[i] * pot[k];
        cc += fe[i];
    }
    add3(a, b, cc, acc + 3);
}

// resetFirstChargedParticle: the smallest index >= first that is injected
// and inbound or source-only becomes first (first stays if there is none)
__global__ void first_candidate(int64_t n, const int32_t *__restrict__ st, const double *__restrict__ t_inj,
                                double t, unsigned long long *__restrict__ first) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const unsigned long long f = first[0];
    unsigned long long cand = ~0ull;
    if (i < n && (unsigned long long)i >= f && (st[i] == 1 || st[i] == 2) && t_inj[i] <= t)
        cand = (unsigned long long)i;
    for (int o = 16; o > 0; o >>= 1) cand = min(cand, __shfl_xor_sync(0xffffffffu, cand, o));
    if ((threadIdx.x & 31) == 0 && cand != ~0ull) atomicMin(&first[1], cand);
}

__global__ void first_commit(unsigned long long *first) {
    if (first[1] != ~0ull) first[0] = first[1];
    first[1] = ~0ull;
}

}  // namespace
}  // namespace sv

namespace sv {
namespace {

sv_status energy_reserve(sv_ctx *c) {
    EnergyBook &E = c->en;
    if (E.cap >= c->n && E.d_acc) return SV_OK;
    const int64_t keep_rec = E.nrec;
    sv_energy_record *recs = E.recs;
    const int64_t rec_cap = E.rec_cap;
    E.recs = nullptr;
    const int on = E.on, is = E.init_steps, st = E.steps, iv = E.interval;
    energy_free(c);
    E.on = on;
    E.init_steps = is;
    E.steps = st;
    E.interval = iv;
    E.recs = recs;
    E.nrec = keep_rec;
    E.rec_cap = rec_cap;
    const int64_t cap = std::max<int64_t>(c->n, 1);
    SV_CK(c, cudaMalloc(&E.fe, sizeof(double) * cap));
    SV_CK(c, cudaMalloc(&E.ke_inj, sizeof(double) * cap));
    SV_CK(c, cudaMalloc(&E.ix, sizeof(double) * cap));
    SV_CK(c, cudaMalloc(&E.iy, sizeof(double) * cap));
    SV_CK(c, cudaMalloc(&E.iz, sizeof(double) * cap));
    SV_CK(c, cudaMalloc(&E.ph, sizeof(float4) * cap));
    SV_CK(c, cudaMalloc(&E.pl, sizeof(float4) * cap));
    SV_CK(c, cudaMalloc(&E.list, sizeof(int) * cap));
    SV_CK(c, cudaMalloc(&E.pot, sizeof(double) * cap));
    SV_CK(c, cudaMalloc(&E.walk, sizeof(int) * cap));
    SV_CK(c, cudaMalloc(&E.d_first, 2 * sizeof(unsigned long long)));
    SV_CK(c, cudaMalloc(&E.d_cnt, sizeof(int)));
    SV_CK(c, cudaMalloc(&E.d_acc, 6 * sizeof(double)));
    E.cap = cap;
    return SV_OK;
}

// compact the particles sel picks into E.list; returns their count (synchronises)
template <class Sel>
sv_status select(sv_ctx *c, Sel sel, int *count) {
    EnergyBook &E = c->en;
    const int n = (int)c->n;
    size_t need = 0;
    SV_CK(c, cub::DeviceSelect::If(nullptr, need, thrust::counting_iterator<int>(0), E.list, E.d_cnt, n, sel,
                                   c->stream));
    if (need > E.scan_bytes) {
        cudaFree(E.scan_tmp);
        E.scan_tmp = nullptr;
        SV_CK(c, cudaMalloc(&E.scan_tmp, need));
        E.scan_bytes = need;
    }
    SV_CK(c, cub::DeviceSelect::If(E.scan_tmp, need, thrust::counting_iterator<int>(0), E.list, E.d_cnt, n, sel,
                                   c->stream));
    SV_CK(c, cudaMemcpyAsync(count, E.d_cnt, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    SV_CK(c, cudaStreamSynchronize(c->stream));
    return SV_OK;
}

// E.pot[k] = sum over the window at time t of q_j / r for the cnt listed particles
sv_status window_potential(sv_ctx *c, double t, int cnt) {
    EnergyBook &E = c->en;
    const int64_t n = c->n;
    split_kernel<<<div_up(n, 256), 256, 0, c->stream>>>(n, c->x, c->y, c->z, c->q, c->t_inj, E.d_first, t, E.ph,
                                                         E.pl);
    SV_LAUNCHED(c);
    SV_CK(c, cudaMemsetAsync(E.pot, 0, sizeof(double) * cnt, c->stream));
    const int gx = div_up(cnt, kPotT);
    const int gy = std::max(1, std::min(div_up(n, kPotT), div_up(4 * device_sms(), gx)));
    potential_kernel<<<dim3(gx, gy), kPotT, 0, c->stream>>>(E.list, E.d_cnt, E.ph, E.pl, E.d_first, n,
                                                            (float)c->P.softening2, E.pot);
    SV_LAUNCHED(c);
    return SV_OK;
}

int sums_grid(int cnt) { return std::max(1, std::min(div_up(cnt, 256), 4 * device_sms())); }

}  // namespace

sv_status energy_inject(sv_ctx *c, double t_end) {
    EnergyBook &E = c->en;
    if (!E.on || c->n == 0) return SV_OK;
    if (E.need_init) {
        SV_TRY(energy_reserve(c));
        SV_TRY(field_prepare(c));
        const FieldMesh &M = c->field;
        const double zref = M.nt > 0 ? (double)((float)M.zmax * (float)M.r0) : 0.0;
        SV_CK(c, cudaMemsetAsync(E.walk, 0xff, sizeof(int) * c->n, c->stream));
        init_kernel<<<div_up(c->n, 128), 128, 0, c->stream>>>(c->n, c->x, c->y, c->z, c->vx, c->vy, c->vz, c->q,
                                                              c->m, M, E.init_steps, zref, E.walk, E.fe, E.ke_inj,
                                                              E.ix, E.iy, E.iz);
        SV_LAUNCHED(c);
        const unsigned long long f0[2] = {0ull, ~0ull};
        SV_CK(c, cudaMemcpyAsync(E.d_first, f0, sizeof(f0), cudaMemcpyHostToDevice, c->stream));
        SV_CK(c, cudaMemsetAsync(E.d_acc, 0, 6 * sizeof(double), c->stream));
        E.have_prev = false;
        E.need_init = false;
    }
    int cnt = 0;
    SV_TRY(select(c, InjectedSel{c->t_inj, t_end, E.t_prev, E.have_prev ? 1 : 0}, &cnt));
    E.t_prev = E.have_prev ? std::max(E.t_prev, t_end) : t_end;
    E.have_prev = true;
    if (cnt == 0) return SV_OK;
    SV_TRY(window_potential(c, t_end, cnt));
    inject_sums<<<sums_grid(cnt), 256, 0, c->stream>>>(E.list, E.d_cnt, E.ke_inj, c->q, E.pot, E.fe, E.d_acc);
    SV_LAUNCHED(c);
    return SV_OK;
}

sv_status energy_first(sv_ctx *c, double t_end) {
    EnergyBook &E = c->en;
    if (!E.on || c->n == 0) return SV_OK;
    first_candidate<<<div_up(c->n, 256), 256, 0, c->stream>>>(c->n, c->status, c->t_inj, t_end, E.d_first);
    SV_LAUNCHED(c);
    first_commit<<<1, 1, 0, c->stream>>>(E.d_first);
    SV_LAUNCHED(c);
    return SV_OK;
}

// one record (KE_inj, PE_inj, FE_inj, KE, PE, FE)
static sv_status push_record(sv_ctx *c, const sv_energy_record &r) {
    EnergyBook &E = c->en;
    if (E.nrec == E.rec_cap) {
        const int64_t cap = std::max<int64_t>(64, 2 * E.rec_cap);
        sv_energy_record *m = (sv_energy_record *)std::realloc(E.recs, sizeof(sv_energy_record) * cap);
        if (!m) return set_error(c, SV_ERR_CAPACITY, "no host memory for energy records");
        E.recs = m;
        E.rec_cap = cap;
    }
    E.recs[E.nrec++] = r;
    return SV_OK;
}

sv_status energy_interval(sv_ctx *c, double ts, double dt) {
    EnergyBook &E = c->en;
    if (!E.on) return SV_OK;
    const long long iter = std::llround(ts / dt) + 1;
    if (iter % E.interval != 0) return SV_OK;
    if (c->n == 0) return push_record(c, sv_energy_record{0.f, 0.f, 0.f, 0.f, 0.f, 0.f});  // an empty window
    const double t_end = ts + dt;
    int cnt = 0;
    SV_TRY(select(c, WindowSel{c->t_inj, E.d_first, t_end}, &cnt));
    SV_CK(c, cudaMemsetAsync(E.d_acc + 3, 0, 3 * sizeof(double), c->stream));
    if (cnt > 0) {
        // the reference's clock after the step's two drifts, in FP32
        // (host code is built without contraction into fused multiply-adds)
        const float dtf = (float)dt, hf = dtf / 2;
        const float t0f = dtf * (float)(iter - 1);
        const float tpos = (t0f + hf) + hf;
        interval_fe<<<div_up(cnt, 128), 128, 0, c->stream>>>(E.list, E.d_cnt, c->x, c->y, c->z, c->q, c->t_inj,
                                                             c->field, tpos, dtf, E.interval, E.steps, E.walk, E.fe,
                                                             E.ix, E.iy, E.iz);
        SV_LAUNCHED(c);
        SV_TRY(window_potential(c, t_end, cnt));
        interval_sums<<<sums_grid(cnt), 256, 0, c->stream>>>(E.list, E.d_cnt, c->vx, c->vy, c->vz, c->m, c->q,
                                                             E.pot, E.fe, E.d_acc);
        SV_LAUNCHED(c);
    }
    double acc[6];
    SV_CK(c, cudaMemcpyAsync(acc, E.d_acc, sizeof(acc), cudaMemcpyDeviceToHost, c->stream));
    SV_CK(c, cudaStreamSynchronize(c->stream));
    const double pc = pe_coef();
    return push_record(c, sv_energy_record{(float)acc[0], (float)(acc[1] * pc), (float)acc[2], (float)acc[3],
                                           (float)(0.5 * acc[4] * pc), (float)acc[5]});
}

void energy_rearm(sv_ctx *c) {
    c->en.need_init = true;
    c->en.have_prev = false;
    c->en.nrec = 0;
}

void energy_free(sv_ctx *c) {
    EnergyBook &E = c->en;
    cudaFree(E.fe); cudaFree(E.ke_inj); cudaFree(E.ix); cudaFree(E.iy); cudaFree(E.iz);
    cudaFree(E.ph); cudaFree(E.pl); cudaFree(E.list); cudaFree(E.pot); cudaFree(E.walk);
    cudaFree(E.scan_tmp); cudaFree(E.d_first); cudaFree(E.d_cnt); cudaFree(E.d_acc);
    std::free(E.recs);
    E = EnergyBook{};
}

}  // namespace sv

using namespace sv;

extern "C" sv_status sv_set_energy(sv_ctx *c, int32_t enable, int32_t init_steps, int32_t steps, int32_t interval) {
    if (!c) return SV_ERR_INVALID;
    if (!enable) {
        SV_CK(c, cudaSetDevice(c->device));
        energy_free(c);
        return SV_OK;
    }
    if (init_steps < 0 || steps < 0 || interval < 1)
        return set_error(c, SV_ERR_INVALID, "init_steps, steps >= 0 and interval >= 1 required");
    if (c->batch) return set_error(c, SV_ERR_UNSUPPORTED, "energy bookkeeping of a batch");
    EnergyBook &E = c->en;
    E.on = 1;
    E.init_steps = init_steps;
    E.steps = steps;
    E.interval = interval;
    E.need_init = true;
    E.have_prev = false;
    return SV_OK;
}

extern "C" sv_status sv_get_energy_records(sv_ctx *c, sv_energy_record *out, int64_t cap, int64_t *count) {
    if (!c || !count || cap < 0) return SV_ERR_INVALID;
    EnergyBook &E = c->en;
    if (!out) {
        *count = E.nrec;
        return SV_OK;
    }
    const int64_t k = std::min<int64_t>(cap, E.nrec);
    if (k > 0) std::memcpy(out, E.recs, sizeof(sv_energy_record) * k);
    if (k < E.nrec) std::memmove(E.recs, E.recs + k, sizeof(sv_energy_record) * (E.nrec - k));
    E.nrec -= k;
    *count = k;
    return SV_OK;
}
