// snapshot.cu -- the state records of the reference's snapshot files
// (Integrator::saveData, integration_schemes.cpp:266-331), packed on the
// device: one record per active particle (status 1 or 2) with index in
// [first, last), or per particle (saveFullCurrentConditions, :197-258), in
// index order (a flag scan gives each record its place).
//   original:    x, y, z, vx, vy, vz, E1[3], E2[3] (float), species (u32),
//                index (i32), lastParticle (i32)                    60 bytes
//   newOriginal: header 0xffffffff (u32), lastParticle (i32), currentTime
//                (float); then index (i32), species (u32), x, y, z, vx, vy,
//                vz, E1[3], E2[3] (float)                            56 bytes
// E1 and E2 are the particle-particle field, (amu/e)(m/q) a
// (Integrator::updateAcceleration, :336-367), and the background field
// (particles.cpp:512) at the particle's last kick as a target: the reference
// recomputes E1 after every force for particles whose acceleration that force
// did not touch, which leaves them their value of the last kick too.
#include <cub/cub.cuh>

#include "sv_internal.cuh"

namespace sv {
namespace {

// saveData keeps status 1 and 2 in [first, last); saveFullCurrentConditions
// (integration_schemes.cpp:197-258) every particle
__global__ void active_flags(const int32_t *__restrict__ st, int64_t n, int64_t first, int64_t last, int full,
                             int *__restrict__ flag) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int32_t w = st[i];
    flag[i] = (full || (i >= first && i < last && (w == 1 || w == 2))) ? 1 : 0;
}

__global__ void pack_records(const int *__restrict__ flag, const int *__restrict__ pos, int64_t n,
                             const double *__restrict__ x, const double *__restrict__ y, const double *__restrict__ z,
                             const double *__restrict__ vx, const double *__restrict__ vy,
                             const double *__restrict__ vz, const double *__restrict__ q,
                             const double *__restrict__ m, double amu_over_e, const int32_t *__restrict__ species,
                             const float *__restrict__ a1, const float *__restrict__ e2, int fmt,
                             int32_t last_particle, unsigned char *__restrict__ out) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n || !flag[i]) return;
    // E1 = (amu/e) (m/q) a (Integrator::updateAcceleration, integration_schemes.cpp:350-356)
    const double k = q[i] != 0.0 ? amu_over_e * m[i] / q[i] : 0.0;
    const float f[12] = {(float)x[i],    (float)y[i],    (float)z[i],    (float)vx[i],
                         (float)vy[i],   (float)vz[i],   (float)(k * a1[3 * i]),      (float)(k * a1[3 * i + 1]),
                         (float)(k * a1[3 * i + 2]),  e2[3 * i],      e2[3 * i + 1],  e2[3 * i + 2]};
    const uint32_t sp = species[i] < 0 ? 0xffffffffu : (uint32_t)species[i];
    const int32_t idx = (int32_t)i;
    if (fmt == SV_SNAPSHOT_ORIGINAL) {
        unsigned char *r = out + (size_t)pos[i] * 60;
        memcpy(r, f, 48);
        memcpy(r + 48, &sp, 4);
        memcpy(r + 52, &idx, 4);
        memcpy(r + 56, &last_particle, 4);
    } else {
        unsigned char *r = out + 12 + (size_t)pos[i] * 56;
        memcpy(r, &idx, 4);
        memcpy(r + 4, &sp, 4);
        memcpy(r + 8, f, 48);
    }
}

}  // namespace
}  // namespace sv

using namespace sv;

extern "C" sv_status sv_snapshot(sv_ctx *c, int32_t format, int64_t first, int64_t last, float current_time,
                                 void *out, int64_t cap_bytes, int64_t *bytes) {
    if (!c || !bytes || cap_bytes < 0) return SV_ERR_INVALID;
    const int full = (format & SV_SNAPSHOT_FULL) ? 1 : 0;
    format &= ~SV_SNAPSHOT_FULL;
    if (format != SV_SNAPSHOT_ORIGINAL && format != SV_SNAPSHOT_NEW_ORIGINAL)
        return set_error(c, SV_ERR_INVALID, "unknown snapshot format %d", format);
    if (!c->have_state) return set_error(c, SV_ERR_STATE, "no state uploaded");
    if (c->batch) return set_error(c, SV_ERR_UNSUPPORTED, "snapshots of a batch: download the state");
    const int64_t n = c->n;
    if (first < 0) first = 0;
    if (last < 0 || last > n) last = n;
    const int32_t last_particle = (int32_t)last;
    const size_t head = format == SV_SNAPSHOT_NEW_ORIGINAL ? 12 : 0, rec = format == SV_SNAPSHOT_NEW_ORIGINAL ? 56 : 60;
    SV_CK(c, cudaSetDevice(c->device));
    int64_t count = 0;
    unsigned char *d_out = nullptr;
    int *flag = nullptr;
    if (n > 0) {
        // flags and their exclusive scan, then the records
        size_t tmp = 0;
        SV_CK(c, cub::DeviceScan::ExclusiveSum(nullptr, tmp, (int *)nullptr, (int *)nullptr, (int)n, c->stream));
        const size_t tmp_al = (tmp + 255) / 256 * 256;
        void *stg = nullptr;
        SV_CK(c, cudaMalloc(&stg, tmp_al + sizeof(int) * 2 * (size_t)n));
        void *cub_tmp = stg;  // the allocation's 256-byte alignment first
        flag = (int *)((char *)stg + tmp_al);
        int *pos = flag + n;
        cudaError_t e = cudaSuccess;
        active_flags<<<div_up(n, 256), 256, 0, c->stream>>>(c->status, n, first, last, full, flag);
        c->launches++;
        if ((e = cudaGetLastError()) == cudaSuccess)
            e = cub::DeviceScan::ExclusiveSum(cub_tmp, tmp, flag, pos, (int)n, c->stream);
        int hpos = 0, hflag = 0;
        if (e == cudaSuccess) e = cudaMemcpyAsync(&hpos, pos + n - 1, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&hflag, flag + n - 1, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        count = hpos + hflag;
        const size_t total = head + rec * (size_t)count;
        if (e == cudaSuccess && out && (int64_t)total <= cap_bytes && count > 0) {
            e = cudaMalloc(&d_out, total);
            if (e == cudaSuccess) {
                pack_records<<<div_up(n, 256), 256, 0, c->stream>>>(
                    flag, pos, n, c->x, c->y, c->z, c->vx, c->vy, c->vz, c->q, c->m, 1.0 / c->P.e_over_amu,
                    c->species, c->e1, c->e2, format, last_particle, d_out);
                c->launches++;
                e = cudaGetLastError();
            }
            if (e == cudaSuccess)
                e = cudaMemcpyAsync((unsigned char *)out + head, d_out + head, rec * (size_t)count,
                                    cudaMemcpyDeviceToHost, c->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        }
        cudaFree(d_out);
        cudaFree(stg);
        SV_CK(c, e);
    }
    const size_t total = head + rec * (size_t)count;
    *bytes = (int64_t)total;
    if (!out) return SV_OK;
    if ((int64_t)total > cap_bytes) return set_error(c, SV_ERR_CAPACITY, "snapshot needs %zu bytes", total);
    if (format == SV_SNAPSHOT_NEW_ORIGINAL) {
        const uint32_t tag = 0xffffffffu;
        memcpy(out, &tag, 4);
        memcpy((unsigned char *)out + 4, &last_particle, 4);
        memcpy((unsigned char *)out + 8, &current_time, 4);
    }
    return SV_OK;
}
