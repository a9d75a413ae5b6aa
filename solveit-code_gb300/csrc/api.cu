// api.cu -- the C ABI (include/solveit_gpu.h): context, state transfer,
// dispatch of force methods, leapfrog, diagnostics.
#include <cmath>
#include <cstdarg>
#include <vector>
#include <algorithm>
#include <atomic>

#include "sv_internal.cuh"

namespace sv {

int device_sms() {
    constexpr int kMaxDevices = 64;
    static std::atomic<int> cache[kMaxDevices];  // 0: not queried yet
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) dev = -1;
    if (dev >= 0) {
        const int v = cache[dev].load(std::memory_order_relaxed);
        if (v > 0) return v;
    }
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev < 0 ? 0 : dev) != cudaSuccess || sms < 1)
        sms = 1;  // no device answers: launches stay valid, only smaller
    if (dev >= 0) cache[dev].store(sms, std::memory_order_relaxed);
    return sms;
}

sv_status set_error(sv_ctx *c, sv_status s, const char *fmt, ...) {
    if (c) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(c->err, sizeof(c->err), fmt, ap);
        va_end(ap);
    }
    return s;
}

sv_status cuda_error(sv_ctx *c, cudaError_t e, const char *what, const char *file, int line) {
    return set_error(c, e == cudaErrorMemoryAllocation ? SV_ERR_ALLOC : SV_ERR_CUDA, "%s failed: %s (%s:%d)",
                     what, cudaGetErrorString(e), file, line);
}

// Image offsets of the reference's finite periodic lattice: the Grid's
// canonical points (lattice_point.h:65-131: generated pass by pass, sorted by
// descending norm) expanded by the sign / axis-permutation loops of
// directKernelTranslationCalculation (direct_force_method_translational.cpp:
// 35-306).  Returned in that summation order, as metres.
int trans_images(const sv_params &P, double *out, int max_out) {
    int box = 1;
    for (int l = 0; l < P.sym_levels; l++) box *= 3;
    const int n = box / 2;
    const int ax[3] = {P.sym_axes[0] != 0, P.sym_axes[1] != 0, P.sym_axes[2] != 0};
    const int dsum = ax[0] + ax[1] + ax[2];
    struct Pt { int v[3]; int norm() const { return v[0] * v[0] + v[1] * v[1] + v[2] * v[2]; } };
    std::vector<Pt> pts;
    int t[3] = {ax[0], ax[1], ax[2]};
    for (int pass = 0; pass < dsum; pass++) {
        for (int i = t[0];; i++) {
            for (int j = t[1];; j++) {
                for (int k = t[2];; k++) {
                    pts.push_back(Pt{{i, j, k}});
                    if (!(t[2] != 0 && k + 1 <= n)) break;
                }
                if (!(t[1] != 0 && j + 1 <= n)) break;
            }
            if (!(t[0] != 0 && i + 1 <= n)) break;
        }
        if (t[0] == 0) {
            if (t[1] == 0) t[2] = 0; else t[1] = 0;
        } else {
            t[0] = 0;
        }
    }
    pts.push_back(Pt{{0, 0, 0}});
    std::stable_sort(pts.begin(), pts.end(), [](const Pt &a, const Pt &b) { return a.norm() > b.norm(); });
    auto oe = [](int i) { return (i & 1) ? -1 : 1; };
    int cnt = 0;
    auto emit = [&](int x, int y, int z) {
        if (cnt < max_out) {
            out[3 * cnt + 0] = x * P.domain_size[0];
            out[3 * cnt + 1] = y * P.domain_size[1];
            out[3 * cnt + 2] = z * P.domain_size[2];
        }
        cnt++;
    };
    for (const Pt &p : pts) {
        const int px = p.v[0], py = p.v[1], pz = p.v[2];
        const int nz = (px != 0) + (py != 0) + (pz != 0);
        const int ni = 1 + (px != 0), nj = 1 + (py != 0), nk = 1 + (pz != 0);
        if (dsum == 3 && nz == 3) {
            for (int i = 0; i < 2; i++)
                for (int j = 0; j < 2; j++)
                    for (int k = 0; k < 2; k++) emit(oe(i) * px, oe(j) * py, oe(k) * pz);
        } else if (dsum == 3 && nz == 2) {
            for (int jj = 0; jj < 3; jj++)
                for (int i = 0; i < ni; i++)
                    for (int j = 0; j < nj; j++)
                        for (int k = 0; k < nk; k++)
                            emit((jj != 0) * oe(i) * px + (px == 0) * ((jj == 1) * oe(j) * py + (jj == 2) * oe(k) * pz),
                                 (jj != 1) * oe(j) * py + (py == 0) * ((jj == 0) * oe(i) * px + (jj == 2) * oe(k) * pz),
                                 (jj != 2) * oe(k) * pz + (pz == 0) * ((jj == 0) * oe(i) * px + (jj == 1) * oe(j) * py));
        } else if (dsum == 3 && nz == 1) {
            for (int jj = 0; jj < 3; jj++)
                for (int i = 0; i < ni; i++)
                    for (int j = 0; j < nj; j++)
                        for (int k = 0; k < nk; k++)
                            emit((jj == 0) * oe(i) * px + (jj == 1) * oe(j) * py + (jj == 2) * oe(k) * pz,
                                 (jj == 0) * oe(j) * py + (jj == 1) * oe(k) * pz + (jj == 2) * oe(i) * px,
                                 (jj == 0) * oe(k) * pz + (jj == 1) * oe(i) * px + (jj == 2) * oe(j) * py);
        } else if (dsum == 2 && nz == 2) {
            for (int i = 0; i < ni; i++)
                for (int j = 0; j < nj; j++)
                    for (int k = 0; k < nk; k++) emit(oe(i) * px, oe(j) * py, oe(k) * pz);
        } else if (dsum == 2 && nz == 1) {
            for (int jj = 0; jj < 2; jj++)
                for (int i = 0; i < ni; i++)
                    for (int j = 0; j < nj; j++)
                        for (int k = 0; k < nk; k++)
                            emit(ax[0] * ((jj == 0) * oe(i) * px + (jj == 1) * (oe(j) * py + oe(k) * pz)),
                                 ax[1] * ((jj == 0) * oe(j) * py + (jj == 1) * (oe(i) * px + oe(k) * pz)),
                                 ax[2] * ((jj == 0) * oe(k) * pz + (jj == 1) * (oe(i) * px + oe(j) * py)));
        } else if (dsum == 1 && nz == 1) {
            for (int i = 0; i < ni; i++)
                for (int j = 0; j < nj; j++)
                    for (int k = 0; k < nk; k++) emit(oe(i) * px, oe(j) * py, oe(k) * pz);
        } else {
            emit(0, 0, 0);
        }
    }
    return cnt;
}

namespace {

template <typename T>
sv_status dev_alloc(sv_ctx *c, T **p, int64_t count) {
    cudaFree(*p);
    *p = nullptr;
    SV_CK(c, cudaMalloc(p, sizeof(T) * (size_t)(count > 0 ? count : 1)));
    return SV_OK;
}

void free_state(sv_ctx *c) {
    cudaFree(c->x); cudaFree(c->y); cudaFree(c->z);
    cudaFree(c->vx); cudaFree(c->vy); cudaFree(c->vz);
    cudaFree(c->q); cudaFree(c->m); cudaFree(c->t_inj); cudaFree(c->status); cudaFree(c->qom);
    cudaFree(c->species); cudaFree(c->wstatus); cudaFree(c->e2); cudaFree(c->e1); cudaFree(c->rstatus);
    cudaFree(c->ax); cudaFree(c->ay); cudaFree(c->az);
    c->x = c->y = c->z = c->vx = c->vy = c->vz = c->q = c->m = c->t_inj = c->qom = nullptr;
    c->ax = c->ay = c->az = nullptr;
    c->status = c->species = c->wstatus = c->rstatus = nullptr;
    c->e2 = c->e1 = nullptr;
    c->cap = 0;
}

sv_status ensure_capacity(sv_ctx *c, int64_t n) {
    if (n <= c->cap && c->x) return SV_OK;
    free_state(c);
    const int64_t cap = std::max<int64_t>(n, 1024);
    SV_TRY(dev_alloc(c, &c->x, cap)); SV_TRY(dev_alloc(c, &c->y, cap)); SV_TRY(dev_alloc(c, &c->z, cap));
    SV_TRY(dev_alloc(c, &c->vx, cap)); SV_TRY(dev_alloc(c, &c->vy, cap)); SV_TRY(dev_alloc(c, &c->vz, cap));
    SV_TRY(dev_alloc(c, &c->q, cap)); SV_TRY(dev_alloc(c, &c->m, cap)); SV_TRY(dev_alloc(c, &c->t_inj, cap));
    SV_TRY(dev_alloc(c, &c->qom, cap));
    SV_TRY(dev_alloc(c, &c->status, cap));
    SV_TRY(dev_alloc(c, &c->species, cap)); SV_TRY(dev_alloc(c, &c->wstatus, cap));
    SV_TRY(dev_alloc(c, &c->rstatus, cap));
    SV_TRY(dev_alloc(c, &c->e2, 3 * cap)); SV_TRY(dev_alloc(c, &c->e1, 3 * cap));
    SV_TRY(dev_alloc(c, &c->ax, cap)); SV_TRY(dev_alloc(c, &c->ay, cap)); SV_TRY(dev_alloc(c, &c->az, cap));
    c->cap = cap;
    return SV_OK;
}

__device__ double species_mass(int s);

// q/m, and the species code of the mass (ParticleSpeciesFunction::getMass,
// particles.h:65-87, inverted; the codes' masses are distinct) for the event records
__global__ void charge_over_mass(const double *__restrict__ q, const double *__restrict__ m, int64_t n,
                                 double *__restrict__ qom, int32_t *__restrict__ species) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double mi = m[i];
    qom[i] = mi > 0.0 ? q[i] / mi : 0.0;
    int32_t code = -1;
    for (int k = 0; k < 8; k++)
        if (k != 3 && mi == species_mass(k)) code = k;
    species[i] = code;
}

__global__ void unpack_fp64(const double *__restrict__ x3, const double *__restrict__ v3,
                            const double *__restrict__ q, const double *__restrict__ m,
                            const int32_t *__restrict__ st, const double *__restrict__ tinj, int64_t n,
                            int has_v, int has_t, double *__restrict__ x, double *__restrict__ y,
                            double *__restrict__ z, double *__restrict__ vx, double *__restrict__ vy,
                            double *__restrict__ vz, double *__restrict__ qo, double *__restrict__ mo,
                            int32_t *__restrict__ so, double *__restrict__ to) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    x[i] = x3[3 * i]; y[i] = x3[3 * i + 1]; z[i] = x3[3 * i + 2];
    vx[i] = has_v ? v3[3 * i] : 0.0; vy[i] = has_v ? v3[3 * i + 1] : 0.0; vz[i] = has_v ? v3[3 * i + 2] : 0.0;
    qo[i] = q[i]; mo[i] = m[i]; so[i] = st[i];
    to[i] = has_t ? tinj[i] : 0.0;
}

// The same unpacking, reading the caller's arrays in place in mapped host
// memory (over NVLink-C2C on a Grace-Blackwell node): each thread takes
// consecutive doubles of the interleaved x3 / v3 arrays, so a warp's loads are
// one contiguous run across the link.
__global__ void unpack_mapped(const double *__restrict__ x3, const double *__restrict__ v3,
                              const double *__restrict__ q, const double *__restrict__ m,
                              const int32_t *__restrict__ st, const double *__restrict__ tinj, int64_t n,
                              int has_v, int has_t, double *__restrict__ x, double *__restrict__ y,
                              double *__restrict__ z, double *__restrict__ vx, double *__restrict__ vy,
                              double *__restrict__ vz, double *__restrict__ qo, double *__restrict__ mo,
                              int32_t *__restrict__ so, double *__restrict__ to) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < 3 * n; t += stride) {
        const int64_t i = t / 3;
        const int d = (int)(t - 3 * i);
        (d == 0 ? x : (d == 1 ? y : z))[i] = x3[t];
        (d == 0 ? vx : (d == 1 ? vy : vz))[i] = has_v ? v3[t] : 0.0;
        if (t < n) {
            qo[t] = q[t];
            mo[t] = m[t];
            so[t] = st[t];
            to[t] = has_t ? tinj[t] : 0.0;
        }
    }
}

// sv_update_state's unpacking: positions, velocities (optional) and statuses
// (optional), from device staging or in place from mapped host memory, each
// thread taking consecutive doubles of the interleaved arrays
__global__ void unpack_state(const double *__restrict__ x3, const double *__restrict__ v3,
                             const int32_t *__restrict__ st, int64_t n, double *__restrict__ x,
                             double *__restrict__ y, double *__restrict__ z, double *__restrict__ vx,
                             double *__restrict__ vy, double *__restrict__ vz, int32_t *__restrict__ so) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < 3 * n; t += stride) {
        const int64_t i = t / 3;
        const int d = (int)(t - 3 * i);
        (d == 0 ? x : (d == 1 ? y : z))[i] = x3[t];
        if (v3) (d == 0 ? vx : (d == 1 ? vy : vz))[i] = v3[t];
        if (st && t < n) so[t] = st[t];
    }
}

// ParticleSpeciesFunction::getMass (particles.h:65-87): EMI 111, BF4 87 amu
__device__ double species_mass(int s) {
    switch (s) {
    case 0: return 111.0;
    case 1: return 2 * 111.0 + 87.0;
    case 2: return 3 * 111.0 + 2 * 87.0;
    case 4: return 111.0 + 87.0;
    case 5: return 87.0;
    case 6: return 111.0 + 2 * 87.0;
    case 7: return 2 * 111.0 + 3 * 87.0;
    default: return 0.0;  // droplet (3): unsupported in the reference, mass 0
    }
}

__global__ void unpack_ref32(const float4 *__restrict__ pos4, const float4 *__restrict__ vel4,
                             const float4 *__restrict__ acc4, const float *__restrict__ tinj, int64_t n,
                             int has_t, double *__restrict__ x, double *__restrict__ y,
                             double *__restrict__ z, double *__restrict__ vx, double *__restrict__ vy,
                             double *__restrict__ vz, double *__restrict__ qo, double *__restrict__ mo,
                             int32_t *__restrict__ so, double *__restrict__ to) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = pos4[i], v = vel4[i], a = acc4[i];
    x[i] = p.x; y[i] = p.y; z[i] = p.z; qo[i] = p.w;
    vx[i] = v.x; vy[i] = v.y; vz[i] = v.z;
    mo[i] = species_mass((int)v.w);
    so[i] = (int32_t)a.w;
    to[i] = has_t ? (double)tinj[i] : 0.0;
}

__global__ void pack_fp64(const double *__restrict__ x, const double *__restrict__ y,
                          const double *__restrict__ z, const double *__restrict__ vx,
                          const double *__restrict__ vy, const double *__restrict__ vz, int64_t n,
                          double *__restrict__ x3, double *__restrict__ v3) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    x3[3 * i] = x[i]; x3[3 * i + 1] = y[i]; x3[3 * i + 2] = z[i];
    v3[3 * i] = vx[i]; v3[3 * i + 1] = vy[i]; v3[3 * i + 2] = vz[i];
}

// pack_fp64 writing the caller's arrays in place in mapped host memory,
// consecutive doubles per thread (v3 and st optional)
__global__ void pack_mapped(const double *__restrict__ x, const double *__restrict__ y,
                            const double *__restrict__ z, const double *__restrict__ vx,
                            const double *__restrict__ vy, const double *__restrict__ vz,
                            const int32_t *__restrict__ st, int64_t n, double *__restrict__ x3,
                            double *__restrict__ v3, int32_t *__restrict__ st_out) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < 3 * n; t += stride) {
        const int64_t i = t / 3;
        const int d = (int)(t - 3 * i);
        if (x3) x3[t] = (d == 0 ? x : (d == 1 ? y : z))[i];
        if (v3) v3[t] = (d == 0 ? vx : (d == 1 ? vy : vz))[i];
        if (st_out && t < n) st_out[t] = st[t];
    }
}

// pack_accel over all particles, writing mapped host memory in place,
// consecutive doubles per thread
__global__ void pack_accel_mapped(const double *__restrict__ ax, const double *__restrict__ ay,
                                  const double *__restrict__ az, const int32_t *__restrict__ st, int64_t n,
                                  double *__restrict__ a3) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < 3 * n; t += stride) {
        const int64_t i = t / 3;
        const int d = (int)(t - 3 * i);
        a3[t] = st[i] == 1 ? (d == 0 ? ax : (d == 1 ? ay : az))[i] : 0.0;
    }
}

__global__ void pack_accel(const double *__restrict__ ax, const double *__restrict__ ay,
                           const double *__restrict__ az, const int32_t *__restrict__ st,
                           int64_t first, int64_t last, int64_t n, double *__restrict__ a3) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const bool t = st[i] == 1 && i >= first && i < last;
    a3[3 * i] = t ? ax[i] : 0.0;
    a3[3 * i + 1] = t ? ay[i] : 0.0;
    a3[3 * i + 2] = t ? az[i] : 0.0;
}

// the status of an evaluation over [first, last): particles outside the range
// take no part, as sources or as targets
__global__ void range_status(const int32_t *__restrict__ st, int64_t first, int64_t last, int64_t n,
                             int32_t *__restrict__ out) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] = (i >= first && i < last) ? st[i] : 0;
}


// Host <-> device copies split in pieces over the copy streams, so that
// several copy engines share a large transfer: ordered after the work already
// on c->stream and joined back into it.
// Device address of a caller's host array that kernels may read and write in
// place: memory pinned by cudaHostAlloc / cudaHostRegister and mapped into
// the device's address space.  Null for anything else (pageable memory goes
// by copies).
static void *mapped_host(const void *h) {
    if (!h) return nullptr;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, h) != cudaSuccess) {
        (void)cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// grid of a grid-stride pass over the host link: enough loads in flight
static int link_grid(int64_t items) {
    const int64_t g = (items + 255) / 256;
    const int64_t cap = 8 * (int64_t)device_sms();
    return (int)std::max<int64_t>(1, std::min(g, cap));
}

struct HostCopy {
    void *dst;
    const void *src;
    size_t bytes;
};
constexpr int kCopyWays = 4;

static sv_status copy_split(sv_ctx *c, const HostCopy *cp, int ncp, cudaMemcpyKind kind) {
    if (!c->cps[0]) {
        for (int k = 0; k < kCopyWays; k++) SV_CK(c, cudaStreamCreateWithFlags(&c->cps[k], cudaStreamNonBlocking));
        for (int k = 0; k <= kCopyWays; k++) SV_CK(c, cudaEventCreateWithFlags(&c->cpe[k], cudaEventDisableTiming));
    }
    SV_CK(c, cudaEventRecord(c->cpe[kCopyWays], c->stream));
    for (int k = 0; k < kCopyWays; k++) SV_CK(c, cudaStreamWaitEvent(c->cps[k], c->cpe[kCopyWays], 0));
    for (int i = 0; i < ncp; i++) {
        const size_t piece = (cp[i].bytes / kCopyWays + 4095) & ~(size_t)4095;
        for (int k = 0; k < kCopyWays && piece * k < cp[i].bytes; k++) {
            const size_t o = piece * k, b = std::min(piece, cp[i].bytes - o);
            SV_CK(c, cudaMemcpyAsync((char *)cp[i].dst + o, (const char *)cp[i].src + o, b, kind, c->cps[k]));
        }
    }
    for (int k = 0; k < kCopyWays; k++) {
        SV_CK(c, cudaEventRecord(c->cpe[k], c->cps[k]));
        SV_CK(c, cudaStreamWaitEvent(c->stream, c->cpe[k], 0));
    }
    return SV_OK;
}

sv_status stage_bytes(sv_ctx *c, size_t bytes, void **p) {
    if (c->d_stage_bytes < bytes) {
        cudaFree(c->d_stage);
        c->d_stage = nullptr;
        c->d_stage_bytes = 0;
        SV_CK(c, cudaMalloc(&c->d_stage, bytes));
        c->d_stage_bytes = bytes;
    }
    *p = c->d_stage;
    return SV_OK;
}

sv_status check_params(sv_ctx *c, const sv_params *p) {
    if (!p) return set_error(c, SV_ERR_INVALID, "params is null");
    if (p->method < SV_METHOD_DIRECT || p->method > SV_METHOD_FMM)
        return set_error(c, SV_ERR_INVALID, "unknown method %d", p->method);
    if (p->precision < SV_PREC_MIXED || p->precision > SV_PREC_FP64)
        return set_error(c, SV_ERR_INVALID, "unknown precision %d", p->precision);
    if (p->symmetry < SV_SYM_NONE || p->symmetry > SV_SYM_TRANSLATIONAL)
        return set_error(c, SV_ERR_INVALID, "unknown symmetry %d", p->symmetry);
    if (!(p->softening2 >= 0.0) || !std::isfinite(p->softening2))
        return set_error(c, SV_ERR_INVALID, "softening2 must be finite and >= 0");
    if (p->fmm_order < 1 || p->fmm_order > 10)
        return set_error(c, SV_ERR_INVALID, "fmm_order %d outside 1..10", p->fmm_order);
    if (p->fmm_ws < 1 || p->fmm_ws > 2) return set_error(c, SV_ERR_INVALID, "fmm_ws must be 1 or 2");
    if (p->leaf_size < 1 || p->leaf_size > 64) return set_error(c, SV_ERR_INVALID, "leaf_size outside 1..64");
    if (!(p->theta >= 0.0f) || p->theta > 1.0f) return set_error(c, SV_ERR_INVALID, "theta outside [0, 1]");
    if (p->fmm_leaf_target < 1 || p->fmm_leaf_target > 4096)
        return set_error(c, SV_ERR_INVALID, "fmm_leaf_target outside 1..4096");
    if (p->fmm_type < SV_FMM_FMM || p->fmm_type > SV_FMM_TREECODE_OUTLIERS)
        return set_error(c, SV_ERR_INVALID, "unknown fmm_type %d", p->fmm_type);
    if (p->fmm_m2l_tc < -1 || p->fmm_m2l_tc > 1) return set_error(c, SV_ERR_INVALID, "fmm_m2l_tc must be -1, 0 or 1");
    if (p->fmm_near < 0 || p->fmm_near > 2) return set_error(c, SV_ERR_INVALID, "fmm_near must be 0, 1 or 2");
    if (!(p->fmm_tune_err >= 0.0f) || !std::isfinite(p->fmm_tune_err))
        return set_error(c, SV_ERR_INVALID, "fmm_tune_err must be finite and >= 0");
    if (!(p->fmm_root_scale == 0.0f || (p->fmm_root_scale >= 1.0f && p->fmm_root_scale < 2.0f)))
        return set_error(c, SV_ERR_INVALID, "fmm_root_scale must be 0 or in [1, 2)");
    if (p->symmetry == SV_SYM_TRANSLATIONAL) {
        if (p->sym_levels < 0 || p->sym_levels > 4) return set_error(c, SV_ERR_INVALID, "sym_levels outside 0..4");
        for (int d = 0; d < 3; d++)
            if (p->sym_axes[d] && !(p->domain_size[d] > 0.0))
                return set_error(c, SV_ERR_INVALID, "periodic axis %d needs domain_size > 0", d);
    }
    return SV_OK;
}

int grid_of(int64_t n) { return (int)((n + 255) / 256 > 0 ? (n + 255) / 256 : 1); }

// Accuracy metric of Integrator::compareAcceleration (integration_schemes.cpp:
// 411-461) over the window [first, last) of the last evaluation: for every
// inbound particle k, r_k = |a_k - ref_k|^2 / |ref_k|^2 (0 when both are 0);
// the metric is sqrt(mean r_k), the largest sqrt(r_k) and its index (the
// first index among equal largest terms, as the reference's strict > over
// ascending k keeps it; index 0 when no term is positive).  Each term is
// evaluated in FP64 without contraction, so terms, maximum and index equal a
// sequential host loop's; the sum is taken per block, then over blocks in
// block order.
constexpr int kCmpThreads = 256;

// The FP64 direct sum at sampled targets (one block per target, threads over
// the sources, a fixed-order block reduction) beside the context's last
// acceleration at those targets: out[6 k ..] = reference xyz, evaluated xyz.
// Targets are the inbound particles, sources status 1 or 2, j != i
// (direct_force_method.cpp:153-190 in FP64).
constexpr int kSmpThreads = 256;

__global__ void __launch_bounds__(kSmpThreads)
sampled_direct_f64_kernel(const int64_t *__restrict__ tg, const double *__restrict__ x, const double *__restrict__ y,
                          const double *__restrict__ z, const double *__restrict__ q, const double *__restrict__ qom,
                          const int32_t *__restrict__ st, int64_t n, double eps2, double kconst,
                          const double *__restrict__ ax, const double *__restrict__ ay,
                          const double *__restrict__ az, double *__restrict__ out) {
    const int64_t i = tg[blockIdx.x];
    const double xi = x[i], yi = y[i], zi = z[i];
    double sx = 0.0, sy = 0.0, sz = 0.0;
    if (st[i] == 1)
        for (int64_t j = threadIdx.x; j < n; j += kSmpThreads) {
            if (j == i || (st[j] != 1 && st[j] != 2)) continue;
            const double dx = xi - x[j], dy = yi - y[j], dz = zi - z[j];
            const double r2 = dx * dx + dy * dy + dz * dz + eps2;
            const double w = q[j] / (r2 * sqrt(r2));
            sx += w * dx;
            sy += w * dy;
            sz += w * dz;
        }
    __shared__ double red[3][kSmpThreads];
    red[0][threadIdx.x] = sx;
    red[1][threadIdx.x] = sy;
    red[2][threadIdx.x] = sz;
    __syncthreads();
    for (int w = kSmpThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w)
            for (int d = 0; d < 3; d++) red[d][threadIdx.x] += red[d][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double c = st[i] == 1 ? kconst * qom[i] : 0.0;
        double *o = out + 6 * blockIdx.x;
        o[0] = red[0][0] * c;
        o[1] = red[1][0] * c;
        o[2] = red[2][0] * c;
        o[3] = ax[i];
        o[4] = ay[i];
        o[5] = az[i];
    }
}

__global__ void __launch_bounds__(kCmpThreads)
compare_partial(const double *__restrict__ ax, const double *__restrict__ ay, const double *__restrict__ az,
                const double *__restrict__ ref3, const int32_t *__restrict__ status, int64_t first, int64_t last,
                double *__restrict__ psum, double *__restrict__ pmax, long long *__restrict__ parg,
                long long *__restrict__ pcnt) {
    double sum = 0.0, mx = 0.0;
    long long am = -1, cnt = 0;
    for (int64_t k = first + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < last;
         k += (int64_t)gridDim.x * blockDim.x) {
        if (status[k] != 1) continue;
        cnt++;
        const double a[3] = {ax[k], ay[k], az[k]};
        double d = 0.0, nr = 0.0;
#pragma unroll
        for (int e = 0; e < 3; e++) {
            const double r = ref3[3 * k + e];
            const double df = __dadd_rn(a[e], -r);
            d = __dadd_rn(d, __dmul_rn(df, df));
            nr = __dadd_rn(nr, __dmul_rn(r, r));
        }
        const double t = (nr == 0.0 && d == 0.0) ? 0.0 : __ddiv_rn(d, nr);
        sum = __dadd_rn(sum, t);
        if (t > mx) {  // ascending k per thread: the first of equal terms stays
            mx = t;
            am = k;
        }
    }
    __shared__ double s_sum[kCmpThreads], s_max[kCmpThreads];
    __shared__ long long s_arg[kCmpThreads], s_cnt[kCmpThreads];
    s_sum[threadIdx.x] = sum;
    s_max[threadIdx.x] = mx;
    s_arg[threadIdx.x] = am;
    s_cnt[threadIdx.x] = cnt;
    __syncthreads();
    for (int w = kCmpThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            const int o = threadIdx.x + w;
            s_sum[threadIdx.x] = __dadd_rn(s_sum[threadIdx.x], s_sum[o]);
            s_cnt[threadIdx.x] += s_cnt[o];
            const double m0 = s_max[threadIdx.x], m1 = s_max[o];
            const long long a0 = s_arg[threadIdx.x], a1 = s_arg[o];
            if (m1 > m0 || (m1 == m0 && a1 >= 0 && (a0 < 0 || a1 < a0))) {
                s_max[threadIdx.x] = m1;
                s_arg[threadIdx.x] = a1;
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        psum[blockIdx.x] = s_sum[0];
        pmax[blockIdx.x] = s_max[0];
        parg[blockIdx.x] = s_arg[0];
        pcnt[blockIdx.x] = s_cnt[0];
    }
}

// out[0] sum of the terms, out[1] largest term, out[2] its index, out[3] count
// (the last two as 64-bit integers)
__global__ void compare_final(int blocks, const double *__restrict__ psum, const double *__restrict__ pmax,
                              const long long *__restrict__ parg, const long long *__restrict__ pcnt,
                              double *__restrict__ out) {
    if (threadIdx.x != 0) return;
    double sum = 0.0, mx = 0.0;
    long long am = -1, cnt = 0;
    for (int b = 0; b < blocks; b++) {
        sum = __dadd_rn(sum, psum[b]);
        cnt += pcnt[b];
        if (pmax[b] > mx || (pmax[b] == mx && parg[b] >= 0 && (am < 0 || parg[b] < am))) {
            mx = pmax[b];
            am = parg[b];
        }
    }
    if (!(mx > 0.0)) am = 0;
    out[0] = sum;
    out[1] = mx;
    reinterpret_cast<long long *>(out)[2] = am;
    reinterpret_cast<long long *>(out)[3] = cnt;
}

}  // namespace
}  // namespace sv

using namespace sv;

extern "C" {

static sv_status upload_state(sv_ctx *c, int64_t n, const double *x3, const double *v3, const double *q,
                              const double *m_amu, const int32_t *status, const double *t_inj);

sv_status sv_upload_batch(sv_ctx *c, int32_t nplumes, const int64_t *counts, const int32_t *method,
                          const int32_t *symmetry, const double *x3, const double *v3, const double *q,
                          const double *m_amu, const int32_t *status, const double *t_inj) {
    if (!c || !counts || !method || !symmetry) return SV_ERR_INVALID;
    if (nplumes < 1) return set_error(c, SV_ERR_INVALID, "a batch needs at least one plume");
    int64_t n = 0;
    for (int p = 0; p < nplumes; p++) n += counts[p];
    SV_CK(c, cudaSetDevice(c->device));
    // a batch of the same shape keeps its plan, capacities and graphs
    const bool same = batch_same_shape(c, nplumes, counts, method, symmetry);
    if (!same) batch_free(c);
    SV_TRY(upload_state(c, n, x3, v3, q, m_amu, status, t_inj));
    if (same) return SV_OK;
    const sv_status st = batch_plan(c, nplumes, counts, method, symmetry);
    if (st != SV_OK) batch_free(c);
    return st;
}

sv_status sv_batch_tune(sv_ctx *c, const char *cache_path, double *best_ms) {
    if (!c) return SV_ERR_INVALID;
    if (!c->batch) return set_error(c, SV_ERR_STATE, "no batch uploaded");
    SV_CK(c, cudaSetDevice(c->device));
    return batch_tune(c, cache_path, best_ms);
}

sv_status sv_get_outliers(sv_ctx *c, int32_t *flags, int64_t *count) {
    if (!c) return SV_ERR_INVALID;
    SV_CK(c, cudaSetDevice(c->device));
    return outliers_get(c, flags, count);
}

sv_status sv_batch_set_tuning(sv_ctx *c, int32_t leaf_target, int32_t direct_chunk) {
    if (!c) return SV_ERR_INVALID;
    if (!c->batch) return set_error(c, SV_ERR_STATE, "no batch uploaded");
    SV_CK(c, cudaSetDevice(c->device));
    return batch_set_tuning(c, leaf_target, direct_chunk);
}

sv_status sv_batch_get_info(const sv_ctx *c, sv_batch_info *out) {
    if (!c || !out) return SV_ERR_INVALID;
    if (!c->batch) return SV_ERR_STATE;
    return batch_info(c, out);
}

int32_t sv_abi_version(void) { return SV_ABI_VERSION; }

sv_status sv_default_params(sv_params *p) {
    if (!p) return SV_ERR_INVALID;
    memset(p, 0, sizeof(*p));
    p->softening2 = 6.4e-19;
    {
        // constants.h:46, evaluated as the reference does (float e^2, long double denominator)
        const float e = 1.6021766e-19f, amu = 1.66053904e-27f, eps0 = 8.85419e-12f;
        const long double pi = 3.14159265358979323846264338328L;
        const float e2 = e * e;
        p->k_const = (double)((long double)e2 / (4 * pi * eps0 * amu));
        const float eoa = e / amu;
        p->e_over_amu = (double)eoa;
    }
    p->method = SV_METHOD_DIRECT;
    p->precision = SV_PREC_MIXED;
    p->symmetry = SV_SYM_NONE;
    p->theta = 0.5f;
    p->leaf_size = 16;
    p->fmm_order = 8;
    p->fmm_ws = 1;
    p->fmm_leaf_target = 32;
    p->sym_axes[0] = p->sym_axes[1] = 1;
    p->sym_levels = 2;
    p->domain_size[0] = p->domain_size[1] = 2e-6;
    p->device = 0;
    return SV_OK;
}

sv_status sv_create(const sv_params *p, sv_ctx **out) {
    if (!out) return SV_ERR_INVALID;
    *out = nullptr;
    sv_ctx *c = new (std::nothrow) sv_ctx();
    if (!c) return SV_ERR_ALLOC;
    sv_status s = check_params(c, p);
    if (s != SV_OK) {
        delete c;
        return s;
    }
    c->P = *p;
    c->device = p->device;
    cudaError_t e = cudaSetDevice(c->device);
    if (e == cudaSuccess) (void)device_sms();  // query the SM count once, outside any stream capture
    // the context's stream at the highest priority: the FMM's second stream
    // (the near field, which fills every SM) yields to it as its blocks retire
    int prio_lo = 0, prio_hi = 0;
    if (e == cudaSuccess) e = cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&c->stream, cudaStreamNonBlocking, prio_hi);
    if (e == cudaSuccess) e = cudaMalloc(&c->d_scalar, 64 * sizeof(double));
    if (e == cudaSuccess) e = cudaMallocHost(&c->h_scalar, 64 * sizeof(double));
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev_begin);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev_end);
    for (int k = 0; k < 9 && e == cudaSuccess; k++) e = cudaEventCreate(&c->ph_ev[k]);
    if (e != cudaSuccess) {
        sv_destroy(c);
        return e == cudaErrorMemoryAllocation ? SV_ERR_ALLOC : SV_ERR_CUDA;
    }
    *out = c;
    return SV_OK;
}

void sv_destroy(sv_ctx *c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    tree_free(c);
    fmm_free(c);
    bh_free(c);
    adjoint_free(c);
    batch_free(c);
    outliers_free(c);
    events_free(c);
    field_free(c);
    substeps_free(c);
    energy_free(c);
    free_state(c);
    Sorted &S = c->S;
    cudaFree(S.x); cudaFree(S.y); cudaFree(S.z); cudaFree(S.q); cudaFree(S.qm);
    cudaFree(S.idx); cudaFree(S.keys); cudaFree(S.keys_alt); cudaFree(S.idx_alt);
    cudaFree(S.ax); cudaFree(S.ay); cudaFree(S.az); cudaFree(S.cub_tmp);
    cudaFree(S.root); cudaFree(S.red);
    cudaFree(c->d_stage);
    cudaFree(c->d_scalar);
    if (c->h_scalar) cudaFreeHost(c->h_scalar);
    if (c->h_accel) cudaFreeHost(c->h_accel);
    if (c->ev_begin) cudaEventDestroy(c->ev_begin);
    if (c->ev_end) cudaEventDestroy(c->ev_end);
    for (int k = 0; k < 9; k++)
        if (c->ph_ev[k]) cudaEventDestroy(c->ph_ev[k]);
    for (int k = 0; k < 4; k++)
        if (c->cps[k]) cudaStreamDestroy(c->cps[k]);
    for (int k = 0; k < 5; k++)
        if (c->cpe[k]) cudaEventDestroy(c->cpe[k]);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

sv_status sv_set_params(sv_ctx *c, const sv_params *p) {
    if (!c) return SV_ERR_INVALID;
    SV_TRY(check_params(c, p));
    if (p->device != c->device) return set_error(c, SV_ERR_INVALID, "device cannot change on a context");
    c->P = *p;
    batch_invalidate(c);
    return SV_OK;
}

sv_status sv_get_params(const sv_ctx *c, sv_params *p) {
    if (!c || !p) return SV_ERR_INVALID;
    *p = c->P;
    return SV_OK;
}

// state upload shared by sv_upload and sv_upload_batch (keeps any batch plan)
static sv_status upload_state(sv_ctx *c, int64_t n, const double *x3, const double *v3, const double *q,
                              const double *m_amu, const int32_t *status, const double *t_inj) {
    if (n < 0 || n > (int64_t)INT32_MAX) return set_error(c, SV_ERR_INVALID, "n=%lld out of range", (long long)n);
    if (n > 0 && (!x3 || !q || !m_amu || !status)) return set_error(c, SV_ERR_INVALID, "null state array");
    SV_CK(c, cudaSetDevice(c->device));
    SV_TRY(ensure_capacity(c, n));
    c->n = n;
    c->have_state = true;
    c->have_accel = false;
    c->ev_seq = 0;
    if (c->d_ev_count) SV_CK(c, cudaMemsetAsync(c->d_ev_count, 0, sizeof(unsigned long long), c->stream));
    SV_TRY(field_prepare(c));
    SV_TRY(field_reset(c));
    SV_TRY(substeps_reset_levels(c));
    energy_rearm(c);
    if (n == 0) return SV_OK;
    SV_CK(c, cudaMemsetAsync(c->e2, 0, sizeof(float) * 3 * (size_t)n, c->stream));
    SV_CK(c, cudaMemsetAsync(c->e1, 0, sizeof(float) * 3 * (size_t)n, c->stream));
    {
        // pinned, mapped arrays: read in place, no staging copy
        const double *mx = (const double *)mapped_host(x3), *mv = (const double *)mapped_host(v3);
        const double *mq = (const double *)mapped_host(q), *mm = (const double *)mapped_host(m_amu);
        const double *mt = (const double *)mapped_host(t_inj);
        const int32_t *ms = (const int32_t *)mapped_host(status);
        if (mx && mq && mm && ms && (!v3 || mv) && (!t_inj || mt)) {
            unpack_mapped<<<link_grid(3 * n), 256, 0, c->stream>>>(
                mx, mv, mq, mm, ms, mt, n, v3 != nullptr, t_inj != nullptr, c->x, c->y, c->z, c->vx, c->vy, c->vz,
                c->q, c->m, c->status, c->t_inj);
            SV_LAUNCHED(c);
            charge_over_mass<<<grid_of(n), 256, 0, c->stream>>>(c->q, c->m, n, c->qom, c->species);
            SV_LAUNCHED(c);
            return SV_OK;
        }
    }
    const size_t b3 = sizeof(double) * 3 * (size_t)n, b1 = sizeof(double) * (size_t)n;
    void *stg = nullptr;
    SV_TRY(stage_bytes(c, 2 * b3 + 3 * b1 + sizeof(int32_t) * (size_t)n, &stg));
    char *p = (char *)stg;
    double *dx3 = (double *)p; p += b3;
    double *dv3 = (double *)p; p += b3;
    double *dq = (double *)p; p += b1;
    double *dm = (double *)p; p += b1;
    double *dt = (double *)p; p += b1;
    int32_t *ds = (int32_t *)p;
    const HostCopy cp[6] = {{dx3, x3, b3},
                            {dv3, v3, v3 ? b3 : 0},
                            {dq, q, b1},
                            {dm, m_amu, b1},
                            {dt, t_inj, t_inj ? b1 : 0},
                            {ds, status, sizeof(int32_t) * (size_t)n}};
    SV_TRY(copy_split(c, cp, 6, cudaMemcpyHostToDevice));
    unpack_fp64<<<grid_of(n), 256, 0, c->stream>>>(dx3, dv3, dq, dm, ds, dt, n, v3 != nullptr, t_inj != nullptr,
                                                   c->x, c->y, c->z, c->vx, c->vy, c->vz, c->q, c->m,
                                                   c->status, c->t_inj);
    SV_LAUNCHED(c);
    charge_over_mass<<<grid_of(n), 256, 0, c->stream>>>(c->q, c->m, n, c->qom, c->species);
    SV_LAUNCHED(c);
    return SV_OK;
}

sv_status sv_upload(sv_ctx *c, int64_t n, const double *x3, const double *v3, const double *q,
                    const double *m_amu, const int32_t *status, const double *t_inj) {
    if (!c) return SV_ERR_INVALID;
    SV_CK(c, cudaSetDevice(c->device));
    batch_free(c);
    return upload_state(c, n, x3, v3, q, m_amu, status, t_inj);
}

sv_status sv_upload_ref32(sv_ctx *c, int64_t n, const float *pos4, const float *vel4, const float *acc4,
                          const float *t_inj) {
    if (!c) return SV_ERR_INVALID;
    if (n < 0 || n > (int64_t)INT32_MAX) return set_error(c, SV_ERR_INVALID, "n=%lld out of range", (long long)n);
    if (n > 0 && (!pos4 || !vel4 || !acc4)) return set_error(c, SV_ERR_INVALID, "null state array");
    SV_CK(c, cudaSetDevice(c->device));
    batch_free(c);
    SV_TRY(ensure_capacity(c, n));
    c->n = n;
    c->have_state = true;
    c->have_accel = false;
    c->ev_seq = 0;
    if (c->d_ev_count) SV_CK(c, cudaMemsetAsync(c->d_ev_count, 0, sizeof(unsigned long long), c->stream));
    SV_TRY(field_prepare(c));
    SV_TRY(field_reset(c));
    SV_TRY(substeps_reset_levels(c));
    energy_rearm(c);
    if (n == 0) return SV_OK;
    SV_CK(c, cudaMemsetAsync(c->e2, 0, sizeof(float) * 3 * (size_t)n, c->stream));
    SV_CK(c, cudaMemsetAsync(c->e1, 0, sizeof(float) * 3 * (size_t)n, c->stream));
    const size_t b4 = 16 * (size_t)n;
    void *stg = nullptr;
    SV_TRY(stage_bytes(c, 3 * b4 + 4 * (size_t)n, &stg));
    char *p = (char *)stg;
    float4 *dp = (float4 *)p; p += b4;
    float4 *dv = (float4 *)p; p += b4;
    float4 *da = (float4 *)p; p += b4;
    float *dt = (float *)p;
    SV_CK(c, cudaMemcpyAsync(dp, pos4, b4, cudaMemcpyHostToDevice, c->stream));
    SV_CK(c, cudaMemcpyAsync(dv, vel4, b4, cudaMemcpyHostToDevice, c->stream));
    SV_CK(c, cudaMemcpyAsync(da, acc4, b4, cudaMemcpyHostToDevice, c->stream));
    if (t_inj) SV_CK(c, cudaMemcpyAsync(dt, t_inj, 4 * (size_t)n, cudaMemcpyHostToDevice, c->stream));
    unpack_ref32<<<grid_of(n), 256, 0, c->stream>>>(dp, dv, da, dt, n, t_inj != nullptr, c->x, c->y, c->z,
                                                    c->vx, c->vy, c->vz, c->q, c->m, c->status, c->t_inj);
    SV_LAUNCHED(c);
    charge_over_mass<<<grid_of(n), 256, 0, c->stream>>>(c->q, c->m, n, c->qom, c->species);
    SV_LAUNCHED(c);
    return SV_OK;
}

sv_status sv_update_state(sv_ctx *c, int64_t n, const double *x3, const double *v3, const int32_t *status) {
    if (!c || !x3) return SV_ERR_INVALID;
    if (!c->have_state) return set_error(c, SV_ERR_STATE, "no state uploaded");
    if (c->batch) return set_error(c, SV_ERR_UNSUPPORTED, "a batch's state is replaced by sv_upload_batch");
    if (n != c->n) return set_error(c, SV_ERR_INVALID, "n=%lld, the uploaded plume has %lld", (long long)n,
                                    (long long)c->n);
    SV_CK(c, cudaSetDevice(c->device));
    c->have_accel = false;
    if (n == 0) return SV_OK;
    const double *mx = (const double *)mapped_host(x3), *mv = (const double *)mapped_host(v3);
    const int32_t *ms = (const int32_t *)mapped_host(status);
    if (mx && (!v3 || mv) && (!status || ms)) {  // pinned, mapped arrays: read in place
        unpack_state<<<link_grid(3 * n), 256, 0, c->stream>>>(mx, mv, ms, n, c->x, c->y, c->z, c->vx, c->vy, c->vz,
                                                             c->status);
        SV_LAUNCHED(c);
        return SV_OK;
    }
    const size_t b3 = sizeof(double) * 3 * (size_t)n;
    void *stg = nullptr;
    SV_TRY(stage_bytes(c, 2 * b3 + sizeof(int32_t) * (size_t)n, &stg));
    double *dx3 = (double *)stg, *dv3 = dx3 + 3 * n;
    int32_t *ds = (int32_t *)(dv3 + 3 * n);
    const HostCopy cp[3] = {{dx3, x3, b3}, {dv3, v3, v3 ? b3 : 0}, {ds, status, status ? sizeof(int32_t) * (size_t)n : 0}};
    SV_TRY(copy_split(c, cp, 3, cudaMemcpyHostToDevice));
    unpack_state<<<link_grid(3 * n), 256, 0, c->stream>>>(dx3, v3 ? dv3 : nullptr, status ? ds : nullptr, n, c->x,
                                                         c->y, c->z, c->vx, c->vy, c->vz, c->status);
    SV_LAUNCHED(c);
    return SV_OK;
}

sv_status sv_download(sv_ctx *c, double *x3, double *v3, int32_t *status) {
    if (!c) return SV_ERR_INVALID;
    if (!c->have_state) return set_error(c, SV_ERR_STATE, "no state uploaded");
    const int64_t n = c->n;
    if (n == 0) return SV_OK;
    SV_CK(c, cudaSetDevice(c->device));
    {
        // pinned, mapped arrays: written in place, no staging copy
        double *mx = (double *)mapped_host(x3), *mv = (double *)mapped_host(v3);
        int32_t *ms = (int32_t *)mapped_host(status);
        if ((!x3 || mx) && (!v3 || mv) && (!status || ms)) {
            pack_mapped<<<link_grid(3 * n), 256, 0, c->stream>>>(c->x, c->y, c->z, c->vx, c->vy, c->vz, c->status, n,
                                                                 mx, mv, ms);
            SV_LAUNCHED(c);
            SV_CK(c, cudaStreamSynchronize(c->stream));
            return SV_OK;
        }
    }
    const size_t b3 = sizeof(double) * 3 * (size_t)n;
    void *stg = nullptr;
    SV_TRY(stage_bytes(c, 2 * b3, &stg));
    double *dx3 = (double *)stg, *dv3 = dx3 + 3 * n;
    pack_fp64<<<grid_of(n), 256, 0, c->stream>>>(c->x, c->y, c->z, c->vx, c->vy, c->vz, n, dx3, dv3);
    SV_LAUNCHED(c);
    const HostCopy cp[3] = {{x3, dx3, x3 ? b3 : 0},
                            {v3, dv3, v3 ? b3 : 0},
                            {status, c->status, status ? sizeof(int32_t) * (size_t)n : 0}};
    SV_TRY(copy_split(c, cp, 3, cudaMemcpyDeviceToHost));
    SV_CK(c, cudaStreamSynchronize(c->stream));
    return SV_OK;
}

sv_status sv_download_ref32(sv_ctx *c, float *pos4, float *vel4) {
    if (!c) return SV_ERR_INVALID;
    const int64_t n = c->n;
    std::vector<double> x(3 * n), v(3 * n);
    SV_TRY(sv_download(c, x.data(), v.data(), nullptr));
    for (int64_t i = 0; i < n; i++) {
        for (int d = 0; d < 3; d++) {
            if (pos4) pos4[4 * i + d] = (float)x[3 * i + d];
            if (vel4) vel4[4 * i + d] = (float)v[3 * i + d];
        }
    }
    return SV_OK;
}

}  // extern "C"

sv_status sv::compute_accel_device(sv_ctx *c, int64_t first, int64_t last) {
    if (!c->have_state) return set_error(c, SV_ERR_STATE, "no state uploaded");
    if (first < 0) first = 0;
    if (last > c->n || last < 0) last = c->n;
    const int64_t n = c->n;
    memset(&c->stats, 0, sizeof(c->stats));
    c->near_ev[0] = c->near_ev[1] = nullptr;  // set by an FMM evaluation that times its near field
    if (c->batch) {
        SV_CK(c, cudaEventRecord(c->ev_begin, c->stream));
        SV_TRY(batch_accel(c));
        SV_CK(c, cudaEventRecord(c->ev_end, c->stream));
        c->have_accel = true;
        c->acc_first = 0;
        c->acc_last = n;
        return SV_OK;
    }
    SV_CK(c, cudaEventRecord(c->ev_begin, c->stream));
    const bool outliers = c->P.method == SV_METHOD_FMM &&
                          (c->P.fmm_type == SV_FMM_FMM_OUTLIERS || c->P.fmm_type == SV_FMM_TREECODE_OUTLIERS);
    if (outliers && c->P.symmetry != SV_SYM_NONE)
        return set_error(c, SV_ERR_UNSUPPORTED, "the outlier variants run without symmetry images");
    // a partial range: the reference's methods take their sources from
    // [firstParticle, lastParticle) as well as their targets
    const int32_t *saved_fstatus = c->fstatus;
    if (n > 0 && (first > 0 || last < n)) {
        range_status<<<grid_of(n), 256, 0, c->stream>>>(force_status(c), first, last, n, c->rstatus);
        SV_LAUNCHED(c);
        c->fstatus = c->rstatus;
    }
    const sv_status st_run = [&]() -> sv_status {
    if (n > 0) {
        phase_mark(c, 0);
        c->S.far = nullptr;
        const int32_t *st2 = nullptr;
        if (outliers) SV_TRY(outliers_detect(c, &st2));  // outliers leave the tree; summed directly below
        auto sort_all = [&](int levels) -> sv_status {
            c->S.want_levels = levels;
            if (outliers) {
                const ParticleView v{c->x, c->y, c->z, c->q, c->m, st2, c->n, c->n, c->qom};
                return sort_view(c, v, first, last);
            }
            if (c->P.method == SV_METHOD_FMM && c->P.symmetry != SV_SYM_NONE) return fmm_sort_images(c, first, last);
            return sort_state(c, first, last);
        };
        // the FMM orders its keys down to one level below its last leaf level,
        // the Barnes-Hut two levels below its last tree's deepest
        SV_TRY(sort_all(c->P.method == SV_METHOD_FMM          ? fmm_sort_levels(c)
                        : c->P.method == SV_METHOD_BARNES_HUT ? bh_sort_levels(c)
                                                              : kMortonBits));
        phase_mark(c, 1);
        switch (c->P.method) {
        case SV_METHOD_DIRECT: SV_TRY(direct_accel(c)); break;
        case SV_METHOD_BARNES_HUT:
            SV_TRY(bh_accel(c));
            if (c->S.resort) {  // the tree reached the sorted levels: the full order, then again
                SV_TRY(sort_all(kMortonBits));
                SV_TRY(bh_accel(c));
            }
            break;
        case SV_METHOD_FMM:
            SV_TRY(fmm_accel(c));
            if (c->S.resort) {  // the leaf level moved down: the full order, then the FMM again
                SV_TRY(sort_all(kMortonBits));
                SV_TRY(fmm_accel(c));
            }
            break;
        default: return set_error(c, SV_ERR_INVALID, "unknown method");
        }
        phase_mark(c, 7);
        SV_TRY(unsort_accel(c));  // non-targets get zero
        if (outliers) SV_TRY(outliers_add(c, first, last));
        phase_mark(c, 8);
    }
    return SV_OK;
    }();
    c->fstatus = saved_fstatus;
    SV_TRY(st_run);
    SV_CK(c, cudaEventRecord(c->ev_end, c->stream));
    c->have_accel = true;
    c->acc_first = first;
    c->acc_last = last;
    return SV_OK;
}

extern "C" {

sv_status sv_compute_accel(sv_ctx *c, int64_t first, int64_t last, double *a3_out) {
    if (!c) return SV_ERR_INVALID;
    SV_CK(c, cudaSetDevice(c->device));
    SV_TRY(compute_accel_device(c, first, last));
    if (a3_out && c->n > 0) {
        const int64_t n = c->n;
        if (double *ma = (double *)mapped_host(a3_out)) {  // pinned and mapped: written in place
            pack_accel_mapped<<<link_grid(3 * n), 256, 0, c->stream>>>(c->ax, c->ay, c->az, c->status, n, ma);
            SV_LAUNCHED(c);
            SV_CK(c, cudaStreamSynchronize(c->stream));
            return SV_OK;
        }
        void *stg = nullptr;
        SV_TRY(stage_bytes(c, sizeof(double) * 3 * n, &stg));
        pack_accel<<<grid_of(n), 256, 0, c->stream>>>(c->ax, c->ay, c->az, c->status, 0, n, n, (double *)stg);
        SV_LAUNCHED(c);
        SV_CK(c, cudaMemcpyAsync(a3_out, stg, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, c->stream));
        SV_CK(c, cudaStreamSynchronize(c->stream));
    }
    return SV_OK;
}

sv_status sv_add_accel_ref32(sv_ctx *c, float *acc4) {
    if (!c || !acc4) return SV_ERR_INVALID;
    if (!c->have_accel) return set_error(c, SV_ERR_STATE, "no acceleration computed");
    const int64_t n = c->n;
    if (n == 0) return SV_OK;
    // a page-locked copy kept by the context: no allocation or page faults per call
    if (c->h_accel_cap < 3 * n) {
        if (c->h_accel) cudaFreeHost(c->h_accel);
        c->h_accel = nullptr;
        c->h_accel_cap = 0;
        SV_CK(c, cudaMallocHost(&c->h_accel, sizeof(double) * 3 * n));
        c->h_accel_cap = 3 * n;
    }
    const double *a = c->h_accel;
    if (double *ma = (double *)mapped_host(c->h_accel)) {  // mapped: written in place
        pack_accel_mapped<<<link_grid(3 * n), 256, 0, c->stream>>>(c->ax, c->ay, c->az, c->status, n, ma);
        SV_LAUNCHED(c);
    } else {
        void *stg = nullptr;
        SV_TRY(stage_bytes(c, sizeof(double) * 3 * n, &stg));
        pack_accel<<<grid_of(n), 256, 0, c->stream>>>(c->ax, c->ay, c->az, c->status, 0, n, n, (double *)stg);
        SV_LAUNCHED(c);
        SV_CK(c, cudaMemcpyAsync(c->h_accel, stg, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, c->stream));
    }
    SV_CK(c, cudaStreamSynchronize(c->stream));
    for (int64_t i = 0; i < n; i++) {
        if (acc4[4 * i + 3] != 1.0f) continue;
        for (int d = 0; d < 3; d++) acc4[4 * i + d] = (float)((double)acc4[4 * i + d] + a[3 * i + d]);
    }
    return SV_OK;
}

sv_status sv_leapfrog(sv_ctx *c, int32_t nsteps, double dt, double t0) {
    if (!c) return SV_ERR_INVALID;
    if (!c->have_state) return set_error(c, SV_ERR_STATE, "no state uploaded");
    if (nsteps < 0 || !(dt > 0.0)) return set_error(c, SV_ERR_INVALID, "nsteps >= 0 and dt > 0 required");
    SV_CK(c, cudaSetDevice(c->device));
    if (c->en.on && (c->batch || c->sub.on))
        return set_error(c, SV_ERR_UNSUPPORTED, "energy bookkeeping runs with the single-rate leapfrog of one plume");
    if (c->batch) {
        SV_TRY(batch_leapfrog(c, nsteps, dt, t0));
    } else if (c->sub.on) {
        SV_TRY(substeps_run(c, nsteps, dt, t0));
    } else {
        for (int it = 0; it < nsteps; it++) SV_TRY(leapfrog_step(c, t0 + dt * it, dt));
    }
    return field_check(c);
}

sv_status sv_set_boundary(sv_ctx *c, const sv_boundary *b) {
    if (!c || !b) return SV_ERR_INVALID;
    if (b->crash != SV_CRASH_NONE && b->crash != SV_CRASH_EXTRACTOR_GRID)
        return set_error(c, SV_ERR_INVALID, "unknown crash condition %d", b->crash);
    if (b->bc < SV_BC_NONE || b->bc > SV_BC_SPACE_AND_TIME)
        return set_error(c, SV_ERR_INVALID, "unknown boundary condition %d", b->bc);
    for (int k = 0; k < 4; k++)
        if (!(b->bc_space[k] >= 0.0)) return set_error(c, SV_ERR_INVALID, "spatial limits must be >= 0");
    if (b->fold && c->P.symmetry == SV_SYM_TRANSLATIONAL)
        for (int k = 0; k < 3; k++)
            if (c->P.sym_axes[k] && !(c->P.domain_size[k] > 0.0))
                return set_error(c, SV_ERR_INVALID, "folding a periodic axis needs domain_size > 0");
    c->B = *b;
    if (c->batch) batch_invalidate(c);
    return SV_OK;
}

sv_status sv_get_boundary(const sv_ctx *c, sv_boundary *b) {
    if (!c || !b) return SV_ERR_INVALID;
    *b = c->B;
    return SV_OK;
}

sv_status sv_get_events(sv_ctx *c, sv_event *out, int64_t cap, int64_t *count) {
    if (!c || !count || cap < 0) return SV_ERR_INVALID;
    *count = 0;
    if (!c->d_ev_count) return SV_OK;
    SV_CK(c, cudaSetDevice(c->device));
    unsigned long long recorded = 0;
    SV_CK(c, cudaMemcpyAsync(&recorded, c->d_ev_count, sizeof(recorded), cudaMemcpyDeviceToHost, c->stream));
    SV_CK(c, cudaStreamSynchronize(c->stream));
    *count = (int64_t)recorded;
    if (!out) return recorded > (unsigned long long)c->ev_cap
                         ? set_error(c, SV_ERR_CAPACITY, "%llu events recorded, %lld kept", recorded,
                                     (long long)c->ev_cap)
                         : SV_OK;
    const int64_t kept = std::min<int64_t>((int64_t)recorded, c->ev_cap);
    std::vector<sv_event> ev(kept);
    std::vector<unsigned long long> key(kept);
    if (kept > 0) {
        SV_CK(c, cudaMemcpyAsync(ev.data(), c->d_events, sizeof(sv_event) * kept, cudaMemcpyDeviceToHost, c->stream));
        SV_CK(c, cudaMemcpyAsync(key.data(), c->d_ev_key, sizeof(unsigned long long) * kept, cudaMemcpyDeviceToHost,
                                 c->stream));
    }
    SV_CK(c, cudaMemsetAsync(c->d_ev_count, 0, sizeof(unsigned long long), c->stream));
    SV_CK(c, cudaStreamSynchronize(c->stream));
    // the device appends in arrival order; the reference's file order is by
    // drift, kind of event, particle index
    std::vector<int64_t> ord(kept);
    for (int64_t k = 0; k < kept; k++) ord[k] = k;
    std::sort(ord.begin(), ord.end(), [&](int64_t a, int64_t b) { return key[a] < key[b]; });
    const int64_t ncopy = std::min<int64_t>(kept, cap);
    for (int64_t k = 0; k < ncopy; k++) out[k] = ev[ord[k]];
    if (recorded > (unsigned long long)c->ev_cap)
        return set_error(c, SV_ERR_CAPACITY, "%llu events recorded, %lld kept", recorded, (long long)c->ev_cap);
    return SV_OK;
}

sv_status sv_energy(sv_ctx *c, double *ke, double *pe) {
    if (!c || !ke || !pe) return SV_ERR_INVALID;
    if (!c->have_state) return set_error(c, SV_ERR_STATE, "no state uploaded");
    if (c->batch) return set_error(c, SV_ERR_UNSUPPORTED, "energy of a batch: evaluate the plumes one by one");
    SV_CK(c, cudaSetDevice(c->device));
    if (c->n == 0) {
        *ke = *pe = 0.0;
        return SV_OK;
    }
    return energy(c, ke, pe);
}

// Root-scale sweep of the context's current order and separation: the
// fastest scale is left in the parameters, its time in *best.
static sv_status tune_root_scale(sv_ctx *c, double *best) {
    float best_scale = 1.0f;
    *best = 1e300;
    for (int k = 0; k < 8; k++) {
        c->P.fmm_root_scale = 1.0f + 0.125f * (float)k;
        double t = 1e300;
        for (int r = 0; r < 5; r++) {  // the first evaluation warms the scale's buffers; min of the other four
            SV_TRY(compute_accel_device(c, 0, c->n));
            SV_CK(c, cudaEventSynchronize(c->ev_end));
            float ms = 0.f;
            SV_CK(c, cudaEventElapsedTime(&ms, c->ev_begin, c->ev_end));
            if (r > 0) t = std::min(t, (double)ms);
        }
        if (t < *best) {
            *best = t;
            best_scale = c->P.fmm_root_scale;
        }
    }
    c->P.fmm_root_scale = best_scale;
    return SV_OK;
}

}  // extern "C"

// Per-particle relative-L2 error of the last acceleration on up to k evenly
// spaced targets of [first, first + count) against the FP64 direct sum over
// the sources of that range (compareAcceleration's metric; a batch's plume
// is such a range).
sv_status sv::sampled_error_range(sv_ctx *c, int64_t first, int64_t count, int k_max, double *err) {
    const int k = (int)std::min<int64_t>(count, k_max);
    *err = 0.0;
    if (k == 0) return SV_OK;
    std::vector<int64_t> tg(k);
    for (int i = 0; i < k; i++) tg[i] = (int64_t)((double)i * (double)count / (double)k);
    void *stg = nullptr;
    SV_TRY(stage_bytes(c, sizeof(int64_t) * k + sizeof(double) * 6 * k, &stg));
    int64_t *d_tg = (int64_t *)stg;
    double *d_out = (double *)(d_tg + k);
    SV_CK(c, cudaMemcpyAsync(d_tg, tg.data(), sizeof(int64_t) * k, cudaMemcpyHostToDevice, c->stream));
    sampled_direct_f64_kernel<<<k, kSmpThreads, 0, c->stream>>>(
        d_tg, c->x + first, c->y + first, c->z + first, c->q + first, c->qom + first, c->status + first, count,
        c->P.softening2, c->P.k_const, c->ax + first, c->ay + first, c->az + first, d_out);
    SV_LAUNCHED(c);
    std::vector<double> h(6 * (size_t)k);
    SV_CK(c, cudaMemcpyAsync(h.data(), d_out, sizeof(double) * 6 * k, cudaMemcpyDeviceToHost, c->stream));
    SV_CK(c, cudaStreamSynchronize(c->stream));
    double s = 0.0;
    int cnt = 0;
    for (int i = 0; i < k; i++) {
        const double *o = &h[6 * (size_t)i];
        double d = 0.0, nr = 0.0;
        for (int e = 0; e < 3; e++) {
            d += (o[3 + e] - o[e]) * (o[3 + e] - o[e]);
            nr += o[e] * o[e];
        }
        if (nr == 0.0 && d == 0.0) continue;  // not a target (or no source)
        s += nr > 0.0 ? d / nr : 1.0;
        cnt++;
    }
    *err = cnt ? std::sqrt(s / cnt) : 0.0;
    return SV_OK;
}

static sv_status sampled_error(sv_ctx *c, double *err) { return sv::sampled_error_range(c, 0, c->n, 256, err); }

extern "C" {

sv_status sv_fmm_tune(sv_ctx *c, double *best_ms) {
    if (!c) return SV_ERR_INVALID;
    if (!c->have_state) return set_error(c, SV_ERR_STATE, "no state uploaded");
    if (c->batch) return set_error(c, SV_ERR_UNSUPPORTED, "batches tune with sv_batch_tune");
    if (c->P.method != SV_METHOD_FMM) return set_error(c, SV_ERR_UNSUPPORTED, "sv_fmm_tune tunes the FMM");
    SV_CK(c, cudaSetDevice(c->device));
    double best = 1e300;
    if (c->P.fmm_tune_err > 0.0f) {
        // (order, separation, near field) candidates; both near-field shapes at
        // separation 2 unless the caller fixed one
        struct Cand {
            int p, ws, near;
        };
        std::vector<Cand> cand;
        const int fixed_near = c->P.fmm_near;
        for (const int p : {6, 8, 10})
            for (const int ws : {1, 2}) {
                if (p == 6 && ws == 1) continue;  // the least accurate pair: not tried
                if (ws == 1 || fixed_near != 0) cand.push_back({p, ws, ws == 1 ? 1 : fixed_near});
                else {
                    cand.push_back({p, ws, 2});
                    cand.push_back({p, ws, 1});
                }
            }
        const int nc = (int)cand.size();
        int kept = -1, most_acc = 0;
        double kept_t = 1e300, min_err = 1e300;
        std::vector<double> times(nc);
        std::vector<float> scales(nc);
        for (int k = 0; k < nc; k++) {
            c->P.fmm_order = cand[k].p;
            c->P.fmm_ws = cand[k].ws;
            c->P.fmm_near = cand[k].near;
            double t = 0.0, e = 0.0;
            SV_TRY(tune_root_scale(c, &t));
            scales[k] = c->P.fmm_root_scale;
            times[k] = t;
            SV_TRY(compute_accel_device(c, 0, c->n));
            SV_TRY(sampled_error(c, &e));
            if (e < min_err) {
                min_err = e;
                most_acc = k;
            }
            if (e <= (double)c->P.fmm_tune_err && t < kept_t) {
                kept_t = t;
                kept = k;
            }
        }
        const int k = kept >= 0 ? kept : most_acc;
        c->P.fmm_order = cand[k].p;
        c->P.fmm_ws = cand[k].ws;
        c->P.fmm_near = cand[k].ws == 2 ? cand[k].near : fixed_near;
        c->P.fmm_root_scale = scales[k];
        best = times[k];
    } else {
        SV_TRY(tune_root_scale(c, &best));
    }
    SV_TRY(compute_accel_device(c, 0, c->n));  // the last acceleration and statistics at the kept settings
    if (best_ms) *best_ms = best;
    return SV_OK;
}

sv_status sv_compare_accel(sv_ctx *c, const double *ref3, double *l2, double *maxl2, int64_t *argmax) {
    if (!c || !ref3 || !l2) return SV_ERR_INVALID;
    if (!c->have_accel) return set_error(c, SV_ERR_STATE, "no acceleration computed");
    SV_CK(c, cudaSetDevice(c->device));
    const int64_t n = c->n, first = c->acc_first, last = c->acc_last;
    double sum = 0.0, mx = 0.0;
    long long am = 0, cnt = 0;
    if (last > first) {
        const int blocks = std::max(1, std::min(div_up(last - first, kCmpThreads), 2 * device_sms()));
        // staging: the reference (3n doubles), then per block sum, max, argmax and count
        const size_t b3 = sizeof(double) * 3 * (size_t)n;
        void *stg = nullptr;
        SV_TRY(stage_bytes(c, b3 + (size_t)blocks * 32, &stg));
        double *dref = (double *)stg;
        double *psum = dref + 3 * n, *pmax = psum + blocks;
        long long *parg = (long long *)(pmax + blocks), *pcnt = parg + blocks;
        SV_CK(c, cudaMemcpyAsync(dref, ref3, b3, cudaMemcpyHostToDevice, c->stream));
        compare_partial<<<blocks, kCmpThreads, 0, c->stream>>>(c->ax, c->ay, c->az, dref, c->status, first, last,
                                                               psum, pmax, parg, pcnt);
        SV_LAUNCHED(c);
        compare_final<<<1, 32, 0, c->stream>>>(blocks, psum, pmax, parg, pcnt, c->d_scalar);
        SV_LAUNCHED(c);
        SV_CK(c, cudaMemcpyAsync(c->h_scalar, c->d_scalar, 4 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        SV_CK(c, cudaStreamSynchronize(c->stream));
        sum = c->h_scalar[0];
        mx = c->h_scalar[1];
        memcpy(&am, &c->h_scalar[2], sizeof(am));
        memcpy(&cnt, &c->h_scalar[3], sizeof(cnt));
    }
    *l2 = cnt ? std::sqrt(sum / (double)cnt) : 0.0;
    if (maxl2) *maxl2 = std::sqrt(mx);
    if (argmax) *argmax = am;
    return SV_OK;
}

sv_status sv_get_stats(const sv_ctx *cc, sv_stats *out) {
    if (!cc || !out) return SV_ERR_INVALID;
    sv_ctx *c = const_cast<sv_ctx *>(cc);
    if (c->have_accel && c->P.method == SV_METHOD_FMM) {
        double m2l = 0, pairs = 0;
        SV_TRY(fmm_counts(c, &m2l, &pairs));
        const int p = c->P.fmm_order;
        double rot = 0, zt = 0;
        for (int n = 0; n < p; n++) rot += (n + 1) * (2 * n + 1);
        for (int j = 0; j < p; j++)
            for (int k = 0; k <= j; k++) zt += p - k;
        c->stats.pair_interactions = pairs;
        c->stats.cell_interactions = m2l;
        // 20 flop per pair; 8 flop per complex multiply-add of the M2L
        // rotations and z-translation; P2M + L2P (1 + 3 terms per coefficient)
        c->stats.flops_algorithmic = 20.0 * pairs + m2l * 8.0 * (2.0 * rot + zt) +
                                     (double)c->n * 8.0 * (p * (p + 1) / 2) * 4.0;
    }
    if (c->have_accel && c->P.method == SV_METHOD_BARNES_HUT) {
        double cells = 0, pairs = 0;
        SV_TRY(bh_counts(c, &cells, &pairs));
        c->stats.cell_interactions = cells;
        c->stats.pair_interactions = pairs;
        c->stats.flops_algorithmic = 20.0 * (cells + pairs);
    }
    if (c->have_accel && c->P.profile_phases && cudaEventQuery(c->ph_ev[8]) == cudaSuccess) {
        for (int k = 0; k < 8; k++) {
            float t = 0.f;
            c->stats.ms_phase[k] = cudaEventElapsedTime(&t, c->ph_ev[k], c->ph_ev[k + 1]) == cudaSuccess ? t : 0.0;
        }
        float t = 0.f;
        if (c->near_ev[0] && cudaEventElapsedTime(&t, c->near_ev[0], c->near_ev[1]) == cudaSuccess)
            c->stats.ms_phase[6] = t;
    }
    *out = c->stats;
    float ms = 0.f;
    if (c->have_accel && cudaEventQuery(c->ev_end) == cudaSuccess &&
        cudaEventElapsedTime(&ms, c->ev_begin, c->ev_end) == cudaSuccess)
        out->ms_total = ms;
    return SV_OK;
}

sv_status sv_sync(sv_ctx *c) {
    if (!c) return SV_ERR_INVALID;
    SV_CK(c, cudaStreamSynchronize(c->stream));
    return SV_OK;
}

void *sv_stream(sv_ctx *c) { return c ? (void *)c->stream : nullptr; }
uint64_t sv_launch_count(const sv_ctx *c) { return c ? c->launches : 0; }
const char *sv_last_error(const sv_ctx *c) { return c ? c->err : "null context"; }

}  // extern "C"
