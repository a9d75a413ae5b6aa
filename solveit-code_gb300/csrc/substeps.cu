// substeps.cu -- multi-rate leapfrog (LeapfrogDKDSubsteps,
// integration_schemes.cpp:899-1528) on the device.
//
// Level l steps with dt_l = dt / 3^l (level 0 = the main step).  A particle's
// level comes from the substep regions: the finer levels cover regions of
// space (|x|, |y|, |z|, r below a limit) or of time since injection where
// particles take the shorter step.  A step of level l < L (L = finest level)
// is drift(l+1), kick(l+1), drift(l+1) for its drift halves, and its kick is
// the same sequence with the kick's "top level" kept; only level L drifts
// (all particles, dt_L / 2) and kicks:
//   setParticleStatus: particles at a level >= top are targets (status 1),
//                      coarser ones sources only (status 2);
//   force (the context's method) + background field, then each target kicked
//   by its own level's dt (variableTimestepKick);
// after the second drift half of a level l < L, particles at levels l and
// l + 1 are re-assigned (crossoverParticles / checkConditions) from the
// region limits of the levels L .. l.
// The level table is resolved on the host exactly as setSubstepTimes
// (integration_schemes.cpp:1361-1427) resolves it, in FP32; the time
// stepping itself runs in FP64.
#include <algorithm>
#include <vector>

#include "sv_internal.cuh"

namespace sv {

namespace {

// BoundaryConditionParameters (structures.h:290-403) in the reference's FP32
struct RefBC {
    int type = SV_BC_NONE;
    float t = 0.0f;
    float s[4] = {0, 0, 0, 0};
};
struct RefSub {
    float dt = 0.0f;
    RefBC bc;
};

void most_stringent(RefBC &b) {
    switch (b.type) {
    case SV_BC_NONE:
        b.t = 0.0f;
        for (float &v : b.s) v = 0.0f;
        break;
    case SV_BC_SPACE: b.t = 0.0f; break;
    case SV_BC_TIME:
        for (float &v : b.s) v = 0.0f;
        break;
    default: break;
    }
    b.type = SV_BC_SPACE_AND_TIME;
}

void choose_min(RefBC &a, const RefBC &b) {
    a.t = (a.t == 0 && b.t == 0) ? 0.0f : std::min(a.t, b.t);
    for (int k = 0; k < 4; k++) a.s[k] = (a.s[k] == 0 && b.s[k] == 0) ? 0.0f : std::min(a.s[k], b.s[k]);
}

void choose_max(RefBC &a, const RefBC &b) {
    a.t = (a.t == 0 || b.t == 0) ? 0.0f : std::max(a.t, b.t);
    for (int k = 0; k < 4; k++) a.s[k] = (a.s[k] == 0 || b.s[k] == 0) ? 0.0f : std::max(a.s[k], b.s[k]);
}

// the reference's two-level region scan of checkSpatialConditions /
// checkTemporalConditions for one coordinate: from the finest level down to
// `level`, the first level whose limit admits the value, then further down
// while the limit stays the same
__device__ int scan_levels(const SubTable &T, int level, double value, int comp, double t_since) {
    int possible = -1;
    double boundary = 0.0;
    for (int i = T.L; i >= level; i--) {
        const double lim = comp < 4 ? T.bs[i][comp] : T.bt[i];
        if (possible == -1) {
            const bool in = comp < 4 ? (fabs(value) < lim || lim == 0.0) : (t_since < lim || lim == 0.0);
            if (in) {
                possible = i;
                boundary = lim;
            }
        } else {
            if (boundary == lim)
                possible--;
            else
                break;
        }
    }
    return possible;
}

// LeapfrogDKDSubsteps::setParticleStatus (integration_schemes.cpp:1216-1236)
// on the particles injected by T, and the windowed status of the kick
__global__ void substep_status_kernel(int32_t *__restrict__ st, int32_t *__restrict__ win,
                                      const int8_t *__restrict__ lev, const double *__restrict__ t_inj, int64_t n,
                                      double T, int top) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        if (!(t_inj[i] <= T)) {
            win[i] = 0;
            continue;
        }
        int32_t w = st[i];
        if (w != 0 && w != -1) {
            w = lev[i] >= top ? 1 : 2;
            st[i] = w;
        }
        win[i] = w;
    }
}

// variableTimestepKick (integration_schemes.cpp:1241-1262) with the
// background field (computeBackgroundAcceleration)
__global__ void substep_kick_kernel(double *__restrict__ vx, double *__restrict__ vy, double *__restrict__ vz,
                                    const double *__restrict__ ax, const double *__restrict__ ay,
                                    const double *__restrict__ az, const double *__restrict__ qom,
                                    const int32_t *__restrict__ win, const int8_t *__restrict__ lev,
                                    const double *__restrict__ t_inj, int64_t n, double t_vel, SubTable T,
                                    double eoa, double ex, double ey, double ez, const double *__restrict__ x,
                                    const double *__restrict__ y, const double *__restrict__ z, FieldMesh M,
                                    float *__restrict__ e2, float *__restrict__ e1) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        if (win[i] != 1) continue;
        const int l = lev[i];
        const double dt = T.dt[l];
        const double s = fmin(fmax(t_vel + dt - t_inj[i], 0.0), dt);
        const double f = eoa * qom[i];
        double fx = ex, fy = ey, fz = ez;
        if (M.nt > 0) {
            int t = M.cache[i];
            double gx, gy, gz;
            field_at(M, x[i], y[i], z[i], &t, &gx, &gy, &gz);
            M.cache[i] = t;
            fx += gx;
            fy += gy;
            fz += gz;
        }
        // the snapshot records' fields (E1 formed from the acceleration when packed)
        e1[3 * i] = (float)ax[i];
        e1[3 * i + 1] = (float)ay[i];
        e1[3 * i + 2] = (float)az[i];
        e2[3 * i] = (float)fx;
        e2[3 * i + 1] = (float)fy;
        e2[3 * i + 2] = (float)fz;
        vx[i] += (ax[i] + fx * f) * s;
        vy[i] += (ay[i] + fy * f) * s;
        vz[i] += (az[i] + fz * f) * s;
    }
}

// crossoverParticles / checkConditions (integration_schemes.cpp:932-1111)
__global__ void crossover_kernel(int8_t *__restrict__ lev, const double *__restrict__ x,
                                 const double *__restrict__ y, const double *__restrict__ z,
                                 const double *__restrict__ t_inj, int64_t n, double t_pos, int level, SubTable T) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        if (!(t_inj[i] <= t_pos)) continue;
        const int l0 = lev[i];
        if (l0 != level && l0 != level + 1) continue;
        const int type = T.type[level + 1];
        const double r = sqrt(x[i] * x[i] + y[i] * y[i]);
        const double ts = t_pos - t_inj[i];
        int out = l0;
        if (type == SV_BC_SPACE || type == SV_BC_SPACE_AND_TIME) {
            out = scan_levels(T, level, x[i], 0, 0.0);
            out = max(out, scan_levels(T, level, y[i], 1, 0.0));
            out = max(out, scan_levels(T, level, z[i], 2, 0.0));
            out = max(out, scan_levels(T, level, r, 3, 0.0));
        }
        if (type == SV_BC_TIME) out = scan_levels(T, level, 0.0, 4, ts);
        if (type == SV_BC_SPACE_AND_TIME) out = max(out, scan_levels(T, level, 0.0, 4, ts));
        // no level of the scan admits the particle: the reference stores -1 and
        // indexes its level table with it; here the particle takes the
        // coarsest level scanned
        lev[i] = (int8_t)(out < 0 ? level : out);
    }
}

__global__ void fill_levels(int8_t *p, int64_t n, int8_t v) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = v;
}

int grid_n(int64_t n) {
    const int64_t b = (n + 255) / 256;
    return (int)(b < 1 ? 1 : (b > 16 * device_sms() ? 16 * device_sms() : b));
}

struct Runner {
    sv_ctx *c;
    const SubTable &T;
    double t_pos, t_vel;

    sv_status drift(int level, bool toggle) {
        if (level != T.L) {
            SV_TRY(drift(level + 1, false));
            SV_TRY(kick(level + 1, level + 1));
            SV_TRY(drift(level + 1, true));
            if (toggle) {
                crossover_kernel<<<grid_n(c->n), 256, 0, c->stream>>>(c->sub_level, c->x, c->y, c->z, c->t_inj,
                                                                      c->n, t_pos, level, T);
                SV_LAUNCHED(c);
            }
            return SV_OK;
        }
        const double h = 0.5 * T.dt[T.L];
        SV_TRY(sv::drift(c, t_pos, h, nullptr));
        t_pos += h;
        return SV_OK;
    }

    sv_status kick(int level, int top) {
        if (level != T.L) {
            SV_TRY(drift(level + 1, false));
            SV_TRY(kick(level + 1, top));
            SV_TRY(drift(level + 1, true));
            return SV_OK;
        }
        substep_status_kernel<<<grid_n(c->n), 256, 0, c->stream>>>(c->status, c->wstatus, c->sub_level, c->t_inj,
                                                                   c->n, t_pos, top);
        SV_LAUNCHED(c);
        c->fstatus = c->wstatus;
        const sv_status s = compute_accel_device(c, 0, c->n);
        c->fstatus = nullptr;
        SV_TRY(s);
        substep_kick_kernel<<<grid_n(c->n), 256, 0, c->stream>>>(
            c->vx, c->vy, c->vz, c->ax, c->ay, c->az, c->qom, c->wstatus, c->sub_level, c->t_inj, c->n, t_vel, T,
            c->P.e_over_amu, c->P.efield[0], c->P.efield[1], c->P.efield[2], c->x, c->y, c->z, c->field, c->e2, c->e1);
        SV_LAUNCHED(c);
        t_vel += T.dt[T.L];
        return SV_OK;
    }
};

}  // namespace

sv_status substeps_reset_levels(sv_ctx *c) {
    if (!c->sub.on) return SV_OK;
    const int64_t want = c->n > 1 ? c->n : 1;
    if (c->sub_cap < want) {
        cudaFree(c->sub_level);
        c->sub_level = nullptr;
        c->sub_cap = 0;
        SV_CK(c, cudaMalloc(&c->sub_level, want));
        c->sub_cap = want;
    }
    // initializeParticleLevels (integration_schemes.cpp:1450-1458): every particle at the finest level
    fill_levels<<<grid_n(want), 256, 0, c->stream>>>(c->sub_level, want, (int8_t)c->sub.L);
    SV_LAUNCHED(c);
    return SV_OK;
}

void substeps_free(sv_ctx *c) {
    cudaFree(c->sub_level);
    c->sub_level = nullptr;
    c->sub_cap = 0;
    c->sub = SubTable{};
}

sv_status substeps_run(sv_ctx *c, int32_t nsteps, double dt, double t0) {
    const SubTable &T = c->sub;
    if (!(dt == T.dt[0]))
        return set_error(c, SV_ERR_INVALID, "the substep table was set for a step of %.9g s, not %.9g s", T.dt[0], dt);
    if (c->B.crash != SV_CRASH_NONE || c->B.bc != SV_BC_NONE) SV_TRY(events_reserve(c));
    SV_TRY(field_prepare(c));
    for (int it = 0; it < nsteps; it++) {
        // LeapfrogDKDSubsteps::runSimulation (integration_schemes.cpp:1494-1526)
        Runner r{c, T, t0 + dt * it, t0 + dt * it};
        SV_TRY(r.drift(0, false));
        SV_TRY(r.kick(0, 0));
        SV_TRY(r.drift(0, true));
    }
    return SV_OK;
}

}  // namespace sv

using namespace sv;

extern "C" sv_status sv_set_substeps(sv_ctx *c, double time_step, int32_t n, const sv_substep *subs) {
    if (!c) return SV_ERR_INVALID;
    SV_CK(c, cudaSetDevice(c->device));
    if (n == 0) {
        substeps_free(c);
        return SV_OK;
    }
    if (n < 0 || !subs || !(time_step > 0.0)) return set_error(c, SV_ERR_INVALID, "substeps: n > 0, table, step > 0");
    if (c->batch) return set_error(c, SV_ERR_UNSUPPORTED, "substeps run on single-plume contexts");
    std::vector<RefSub> in(n);
    for (int i = 0; i < n; i++) {
        if (!(subs[i].dt > 0.0) || subs[i].bc < SV_BC_NONE || subs[i].bc > SV_BC_SPACE_AND_TIME)
            return set_error(c, SV_ERR_INVALID, "substep %d: dt > 0 and a boundary kind required", i);
        in[i].dt = (float)subs[i].dt;
        in[i].bc.type = subs[i].bc;
        in[i].bc.t = (float)subs[i].bc_time;
        for (int k = 0; k < 4; k++) in[i].bc.s[k] = (float)subs[i].bc_space[k];
    }
    // setSubstepTimes (integration_schemes.cpp:1361-1412), in the reference's FP32
    std::sort(in.begin(), in.end(), [](const RefSub &a, const RefSub &b) { return a.dt < b.dt; });
    const float step = (float)time_step;
    float temp_dt = step;
    int L = 0;
    while (temp_dt > in[0].dt) {
        temp_dt /= 3.0;
        L++;
    }
    if (L >= kMaxSubLevels) return set_error(c, SV_ERR_UNSUPPORTED, "%d substep levels (at most %d)", L + 1,
                                             kMaxSubLevels);
    std::vector<RefSub> lv(L + 1);
    if (L != 0) lv[L] = in[0];
    for (int i = 0; i <= L; i++) most_stringent(lv[i].bc);
    for (int i = 1; i < n; i++) {
        int ind = 0;
        temp_dt = step;
        while (temp_dt > in[i].dt) {
            temp_dt /= 3.0;
            ind++;
        }
        if (lv[ind].dt == 0) {
            lv[ind].dt = temp_dt;
            if (ind != 0) lv[ind].bc = in[i].bc;
        } else {
            choose_min(lv[ind].bc, in[i].bc);
        }
    }
    lv[0].dt = step;
    for (int i = 1; i <= L; i++) lv[i].dt = lv[i - 1].dt / 3.0;
    for (int i = L - 1; i >= 0; i--) choose_max(lv[i].bc, lv[i + 1].bc);
    SubTable T;
    T.on = 1;
    T.L = L;
    for (int i = 0; i <= L; i++) {
        // the steps in FP64 from the caller's step; the regions as the reference resolved them
        T.dt[i] = i == 0 ? time_step : T.dt[i - 1] / 3.0;
        T.type[i] = lv[i].bc.type;
        T.bt[i] = lv[i].bc.t;
        for (int k = 0; k < 4; k++) T.bs[i][k] = lv[i].bc.s[k];
    }
    c->sub = T;
    if (c->have_state) SV_TRY(substeps_reset_levels(c));
    return SV_OK;
}

extern "C" sv_status sv_get_substep_levels(sv_ctx *c, int8_t *levels) {
    if (!c || !levels) return SV_ERR_INVALID;
    if (!c->sub.on) return set_error(c, SV_ERR_STATE, "no substep table set");
    if (c->n == 0) return SV_OK;
    SV_CK(c, cudaSetDevice(c->device));
    SV_CK(c, cudaMemcpyAsync(levels, c->sub_level, c->n, cudaMemcpyDeviceToHost, c->stream));
    SV_CK(c, cudaStreamSynchronize(c->stream));
    return SV_OK;
}
