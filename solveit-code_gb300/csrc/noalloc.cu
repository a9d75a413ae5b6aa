// noalloc.cu -- direct-sum entry point that allocates no memory.
//
// For callers that cannot allocate device memory themselves or let a library
// do it: code running inside a memory-pool-managed host framework that owns
// every allocation, real-time loops where an allocation (and the implicit
// synchronisation cudaMalloc / cudaFree can cause) is not allowed, or code
// driven by another runtime that only hands out buffers it already owns.
// sv_direct_accel_noalloc() computes the same mixed-precision direct sum as
// sv_compute_accel(SV_METHOD_DIRECT, SV_PREC_MIXED, SV_SYM_NONE) from device
// buffers the caller passes in; the Morton-sorted working copy, the sort keys
// and the sort's temporary storage live in one file-scope __device__ array of
// SV_NOALLOC_SCRATCH_BYTES, which every GPU that loads this library holds
// until the process exits.
//
// The array's name is only a host-side stand-in in host code, so its device
// address is fetched once per device with cudaGetSymbolAddress (with that
// device current) on the first call made on that device.  That first call is
// the set-up call: under lazy module loading (the CUDA default) it is also the
// one that loads this library's device code on the device, which commits the
// array's memory and can synchronise the device, so a caller that must not
// allocate later makes it during its own set-up, before any stream capture.
// The address is kept for the life of the process: after a cudaDeviceReset of
// a device the entry point must not be called on that device again.  All
// calls share the one array and it keeps the previous call's contents:
// everything that has to start at zero is cleared here, and two calls whose
// work overlaps on the GPU race on the array.  A CUDA error already pending on
// the calling thread when a call starts is left pending (not consumed): the
// call returns SV_ERR_CUDA without doing any work.
#include <cub/device/device_radix_sort.cuh>

#include <mutex>

#include "sv_internal.cuh"

namespace sv {
namespace {

static __device__ __align__(256) unsigned char g_noalloc_scratch[SV_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
void *g_scratch_addr[kMaxDevices] = {nullptr};
std::mutex g_scratch_mu;

cudaError_t scratch_address(int dev, unsigned char **out) {
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_addr[dev] = p;
    }
    *out = (unsigned char *)g_scratch_addr[dev];
    return cudaSuccess;
}

__device__ __forceinline__ bool is_src(int32_t s) { return s == 1 || s == 2; }

__global__ void na_bbox_partial(const double *__restrict__ x3, const int32_t *__restrict__ st, int n,
                                double *__restrict__ out) {
    double mn[3] = {1e300, 1e300, 1e300}, mx[3] = {-1e300, -1e300, -1e300};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (!is_src(st[i])) continue;
#pragma unroll
        for (int d = 0; d < 3; d++) {
            mn[d] = fmin(mn[d], x3[3 * i + d]);
            mx[d] = fmax(mx[d], x3[3 * i + d]);
        }
    }
#pragma unroll
    for (int d = 0; d < 3; d++)
        for (int o = 16; o > 0; o >>= 1) {
            mn[d] = fmin(mn[d], __shfl_xor_sync(0xffffffffu, mn[d], o));
            mx[d] = fmax(mx[d], __shfl_xor_sync(0xffffffffu, mx[d], o));
        }
    __shared__ double sh[6][8];
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0)
        for (int d = 0; d < 3; d++) {
            sh[d][w] = mn[d];
            sh[3 + d][w] = mx[d];
        }
    __syncthreads();
    if (threadIdx.x < 6) {
        const int d = threadIdx.x;
        double v = d < 3 ? 1e300 : -1e300;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) v = d < 3 ? fmin(v, sh[d][k]) : fmax(v, sh[d][k]);
        out[blockIdx.x * 6 + d] = v;
    }
}

// origin = bbox min; cube side = smallest power of two above the extent
__global__ void na_bbox_final(const double *__restrict__ part, int nb, double *__restrict__ root) {
    __shared__ double sh[6];
    if (threadIdx.x < 6) {
        const int d = threadIdx.x;
        double v = d < 3 ? 1e300 : -1e300;
        for (int k = 0; k < nb; k++) v = d < 3 ? fmin(v, part[k * 6 + d]) : fmax(v, part[k * 6 + d]);
        sh[d] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double ext = 0.0;
        for (int d = 0; d < 3; d++) ext = fmax(ext, sh[3 + d] - sh[d]);
        double S = 1e-12;
        if (ext > 0.0) {
            int e;
            frexp(ext, &e);
            S = ldexp(1.0, e);
        }
        root[0] = sh[0] > sh[3] ? 0.0 : sh[0];
        root[1] = sh[0] > sh[3] ? 0.0 : sh[1];
        root[2] = sh[0] > sh[3] ? 0.0 : sh[2];
        root[3] = S;
    }
}

__device__ __forceinline__ uint64_t na_spread3(uint32_t v) {
    uint64_t x = v & 0x1fffffull;
    x = (x | (x << 32)) & 0x1f00000000ffffull;
    x = (x | (x << 16)) & 0x1f0000ff0000ffull;
    x = (x | (x << 8)) & 0x100f00f00f00f00full;
    x = (x | (x << 4)) & 0x10c30c30c30c30c3ull;
    x = (x | (x << 2)) & 0x1249249249249249ull;
    return x;
}

__global__ void na_keys(const double *__restrict__ x3, const int32_t *__restrict__ st, int n,
                        const double *__restrict__ root, uint64_t *__restrict__ keys, uint32_t *__restrict__ idx) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    idx[i] = (uint32_t)i;
    if (!is_src(st[i])) {
        keys[i] = ~0ull;
        return;
    }
    const double inv = (double)(1u << kMortonBits) / root[3];
    uint32_t c[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
        double f = floor((x3[3 * i + d] - root[d]) * inv);
        f = fmin(fmax(f, 0.0), (double)((1u << kMortonBits) - 1));
        c[d] = (uint32_t)f;
    }
    keys[i] = na_spread3(c[0]) | (na_spread3(c[1]) << 1) | (na_spread3(c[2]) << 2);
}

__global__ void na_gather(const uint32_t *__restrict__ idx, int n, const double *__restrict__ x3,
                          const double *__restrict__ q, const double *__restrict__ m,
                          const int32_t *__restrict__ st, double kconst, double *__restrict__ xs,
                          double *__restrict__ ys, double *__restrict__ zs, float *__restrict__ qs,
                          double *__restrict__ qm) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const uint32_t i = idx[s];
    xs[s] = x3[3 * i];
    ys[s] = x3[3 * i + 1];
    zs[s] = x3[3 * i + 2];
    const int32_t w = st[i];
    qs[s] = is_src(w) ? (float)q[i] : 0.0f;
    qm[s] = (w == 1 && m[i] > 0.0) ? kconst * q[i] / m[i] : 0.0;
}

// every output entry is written: targets get their acceleration, everything
// else 0 (entries of the sorted arrays that the kernel did not touch may hold
// the previous call's values and are never passed on)
__global__ void na_scatter(const uint32_t *__restrict__ idx, int n, const double *__restrict__ qm,
                           const double *__restrict__ ax, const double *__restrict__ ay,
                           const double *__restrict__ az, double *__restrict__ a3) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const uint32_t i = idx[s];
    const bool t = qm[s] != 0.0;
    a3[3 * i] = t ? ax[s] : 0.0;
    a3[3 * i + 1] = t ? ay[s] : 0.0;
    a3[3 * i + 2] = t ? az[s] : 0.0;
}

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace
}  // namespace sv

using namespace sv;

extern "C" sv_status sv_direct_accel_noalloc(int64_t n, const double *x3, const double *q, const double *m_amu,
                                             const int32_t *status, double softening2, double k_const,
                                             double *a3, void *stream) {
    if (n < 0 || !(softening2 >= 0.0)) return SV_ERR_INVALID;
    if (n > SV_NOALLOC_MAX_N) return SV_ERR_CAPACITY;
    if (n == 0) return SV_OK;
    if (!x3 || !q || !m_amu || !status || !a3) return SV_ERR_INVALID;
    // the launch checks below read (and clear) the thread's last error: an
    // error the caller's own work left pending is not this call's to consume
    if (cudaPeekAtLastError() != cudaSuccess) return SV_ERR_CUDA;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return SV_ERR_CUDA;
    unsigned char *base = nullptr;
    if (scratch_address(dev, &base) != cudaSuccess) return SV_ERR_CUDA;
    cudaStream_t s = (cudaStream_t)stream;
    const int ni = (int)n;
    // carve the scratch array
    size_t off = 0;
    auto carve = [&](size_t bytes) {
        unsigned char *p = base + off;
        off += align256(bytes);
        return (void *)p;
    };
    uint64_t *keys = (uint64_t *)carve(sizeof(uint64_t) * ni);
    uint64_t *keys_alt = (uint64_t *)carve(sizeof(uint64_t) * ni);
    uint32_t *idx = (uint32_t *)carve(sizeof(uint32_t) * ni);
    uint32_t *idx_alt = (uint32_t *)carve(sizeof(uint32_t) * ni);
    double *xs = (double *)carve(sizeof(double) * ni);
    double *ys = (double *)carve(sizeof(double) * ni);
    double *zs = (double *)carve(sizeof(double) * ni);
    float *qs = (float *)carve(sizeof(float) * ni);
    double *qm = (double *)carve(sizeof(double) * ni);
    double *ax = (double *)carve(sizeof(double) * ni);
    double *ay = (double *)carve(sizeof(double) * ni);
    double *az = (double *)carve(sizeof(double) * ni);
    const int red_blocks = 2 * device_sms();
    double *part = (double *)carve(sizeof(double) * 6 * red_blocks);
    double *root = (double *)carve(sizeof(double) * 8);
    cub::DoubleBuffer<uint64_t> kb(keys, keys_alt);
    cub::DoubleBuffer<uint32_t> vb(idx, idx_alt);
    size_t tmp_bytes = 0;
    if (cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, kb, vb, ni, 0, 3 * kMortonBits + 1, s) != cudaSuccess)
        return SV_ERR_CUDA;
    void *tmp = carve(tmp_bytes);
    if (off > (size_t)SV_NOALLOC_SCRATCH_BYTES) return SV_ERR_CAPACITY;

    const int nb = (ni + 255) / 256;
    na_bbox_partial<<<red_blocks, 256, 0, s>>>(x3, status, ni, part);
    na_bbox_final<<<1, 32, 0, s>>>(part, red_blocks, root);
    na_keys<<<nb, 256, 0, s>>>(x3, status, ni, root, keys, idx);
    if (cudaGetLastError() != cudaSuccess) return SV_ERR_CUDA;
    if (cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, kb, vb, ni, 0, 3 * kMortonBits + 1, s) != cudaSuccess)
        return SV_ERR_CUDA;
    const uint32_t *sidx = vb.Current();
    na_gather<<<nb, 256, 0, s>>>(sidx, ni, x3, q, m_amu, status, k_const, xs, ys, zs, qs, qm);
    if (cudaGetLastError() != cudaSuccess) return SV_ERR_CUDA;
    if (launch_direct_mixed_sorted(xs, ys, zs, qs, qm, ni, (float)softening2, ax, ay, az, s) != cudaSuccess)
        return SV_ERR_CUDA;
    na_scatter<<<nb, 256, 0, s>>>(sidx, ni, qm, ax, ay, az, a3);
    if (cudaGetLastError() != cudaSuccess) return SV_ERR_CUDA;
    return SV_OK;
}
