// outliers.cu -- the outlier variants of the FMM (FmmType::fmmOutliers and
// FmmType::treecodeOutliers, structures.h:283-288).
//
// Detection restates DomainBoundsFunction::isOutlier
// (domain_bounds_functions.cpp:16-99) on the sources (status 1 or 2), in FP32
// as the reference computes it: per axis the true median of the positions
// (findTrueMedian, outlier_detection.h:117-133: the middle element, or the
// mean of the two middle ones), the absolute deviations from it, and their
// median scaled by 1.482602218505602 (domain_bounds_functions.h:37); a source
// deviating by >= 3 scaled deviations (:38) on any axis is an outlier.  (The
// reference takes the deviations' median over all particles of its range,
// sources or not; with every particle a source, as in a plume, both agree.)
// Medians come from CUB radix sorts of the FP32 values, non-sources sorted
// last as +inf.
//
// The reference then places outliers in boxes of their own and couples them
// to the tree with P2P and M2P kernels (p2outlier_p, m2outlier_p,
// outlier_p2p).  Here outliers leave the tree (their status is masked for the
// sort), and every interaction that involves one is summed directly in FP64:
// outlier sources onto inlier targets, and every source onto an outlier
// target.  Outliers are few by construction, so this is O(N * outliers).
#include <cub/device/device_radix_sort.cuh>

#include <algorithm>
#include <cmath>

#include "sv_internal.cuh"

namespace sv {

struct Outliers {
    int64_t cap = 0;
    float *keys = nullptr, *keys_alt = nullptr;  // n FP32 values and their sorted copy
    int32_t *flag = nullptr;     // caller order: 1 outlier source, 0 inlier source, -1 no source
    int32_t *status2 = nullptr;  // caller status with outliers masked to 0 (ignored) for the tree
    int32_t *list = nullptr, *list_alt = nullptr;  // outlier indices, sorted
    int *count = nullptr;        // device [2]: sources, outliers
    float *stats = nullptr;      // device [6]: median x y z, scaled MAD x y z
    void *cub_tmp = nullptr;
    size_t cub_bytes = 0;
    int *h_count = nullptr;      // pinned [2]
    int n_out = 0;
    bool valid = false;
};

namespace {

constexpr float kOutlierFactor = 1.482602218505602f;  // -1 / (sqrt(2) erfcinv(3/2))
constexpr float kMaxDeviation = 3.0f;

__device__ __forceinline__ bool is_src(int32_t w) { return w == 1 || w == 2; }

__global__ void count_sources_kernel(const int32_t *__restrict__ st, int64_t n, int *__restrict__ count) {
    int c = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        c += is_src(st[i]);
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(count, c);
}

// FP32 value of each source on one axis (the reference's state is FP32), or
// the deviation from the axis median; non-sources +inf (sorted last)
__global__ void axis_values_kernel(const double *__restrict__ x, const int32_t *__restrict__ st, int64_t n,
                                   const float *__restrict__ med, float *__restrict__ out) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (!is_src(st[i])) {
        out[i] = INFINITY;
        return;
    }
    const float v = (float)x[i];
    out[i] = med ? fabsf(v - *med) : v;
}

// findTrueMedian on the sorted values of the first `count` entries
__global__ void true_median_kernel(const float *__restrict__ sorted, const int *__restrict__ count, float scale,
                                   float *__restrict__ out) {
    const int n = *count;
    float v = 0.0f;
    if (n > 0) {
        if (n & 1) v = sorted[n / 2];
        else v = (sorted[(n - 1) / 2] + sorted[n / 2]) / 2;
    }
    *out = scale * v;
}

__global__ void flag_kernel(const double *__restrict__ x, const double *__restrict__ y, const double *__restrict__ z,
                            const int32_t *__restrict__ st, int64_t n, const float *__restrict__ stats,
                            int32_t *__restrict__ flag, int32_t *__restrict__ status2, int32_t *__restrict__ list,
                            int *__restrict__ count) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int32_t w = st[i];
    if (!is_src(w)) {
        flag[i] = -1;
        status2[i] = w;
        return;
    }
    const float dx = fabsf((float)x[i] - stats[0]) / stats[3];
    const float dy = fabsf((float)y[i] - stats[1]) / stats[4];
    const float dz = fabsf((float)z[i] - stats[2]) / stats[5];
    const bool out = dx >= kMaxDeviation || dy >= kMaxDeviation || dz >= kMaxDeviation;
    flag[i] = out ? 1 : 0;
    status2[i] = out ? 0 : w;
    if (out) list[atomicAdd(&count[1], 1)] = (int32_t)i;
}

__device__ __forceinline__ double inv3(double dx, double dy, double dz, double eps2) {
    const double r2 = dx * dx + dy * dy + dz * dz + eps2;
    const double r = sqrt(r2);
    return 1.0 / (r2 * r);
}

// inlier targets: + the outlier sources, FP64
__global__ void outlier_sources_kernel(const double *__restrict__ x, const double *__restrict__ y,
                                       const double *__restrict__ z, const double *__restrict__ q,
                                       const double *__restrict__ m, const int32_t *__restrict__ st,
                                       const int32_t *__restrict__ flag, const int32_t *__restrict__ list, int n_out,
                                       int64_t n, int64_t first, int64_t last, double eps2, double kconst,
                                       double *__restrict__ ax, double *__restrict__ ay, double *__restrict__ az) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n || st[i] != 1 || flag[i] != 0 || i < first || i >= last || !(m[i] > 0.0)) return;
    const double xi = x[i], yi = y[i], zi = z[i];
    double sx = 0.0, sy = 0.0, sz = 0.0;
    for (int k = 0; k < n_out; k++) {
        const int32_t j = list[k];
        const double dx = xi - x[j], dy = yi - y[j], dz = zi - z[j];
        const double w = q[j] * inv3(dx, dy, dz, eps2);
        sx += dx * w;
        sy += dy * w;
        sz += dz * w;
    }
    const double c = kconst * q[i] / m[i];
    ax[i] += c * sx;
    ay[i] += c * sy;
    az[i] += c * sz;
}

// outlier targets: every source directly, FP64, one block per outlier
__global__ void __launch_bounds__(256)
outlier_targets_kernel(const double *__restrict__ x, const double *__restrict__ y, const double *__restrict__ z,
                       const double *__restrict__ q, const double *__restrict__ m, const int32_t *__restrict__ st,
                       const int32_t *__restrict__ list, int64_t n, int64_t first, int64_t last, double eps2,
                       double kconst, double *__restrict__ ax, double *__restrict__ ay, double *__restrict__ az) {
    __shared__ double red[3][8];
    const int32_t i = list[blockIdx.x];
    const bool tgt = st[i] == 1 && i >= first && i < last && m[i] > 0.0;
    double sx = 0.0, sy = 0.0, sz = 0.0;
    if (tgt) {
        const double xi = x[i], yi = y[i], zi = z[i];
        for (int64_t j = threadIdx.x; j < n; j += blockDim.x) {
            if (j == i || !is_src(st[j])) continue;
            const double dx = xi - x[j], dy = yi - y[j], dz = zi - z[j];
            const double w = q[j] * inv3(dx, dy, dz, eps2);
            sx += dx * w;
            sy += dy * w;
            sz += dz * w;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        sx += __shfl_xor_sync(0xffffffffu, sx, o);
        sy += __shfl_xor_sync(0xffffffffu, sy, o);
        sz += __shfl_xor_sync(0xffffffffu, sz, o);
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        red[0][w] = sx;
        red[1][w] = sy;
        red[2][w] = sz;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0, b = 0, c = 0;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) {
            a += red[0][k];
            b += red[1][k];
            c += red[2][k];
        }
        const double f = tgt ? kconst * q[i] / m[i] : 0.0;
        ax[i] = f * a;
        ay[i] = f * b;
        az[i] = f * c;
    }
}

sv_status reserve(sv_ctx *c, Outliers &O, int64_t n) {
    if (O.cap >= n && O.keys) return SV_OK;
    cudaFree(O.keys); cudaFree(O.keys_alt); cudaFree(O.flag); cudaFree(O.status2); cudaFree(O.list);
    cudaFree(O.list_alt); cudaFree(O.cub_tmp);
    O.keys = O.keys_alt = nullptr;
    O.flag = O.status2 = O.list = O.list_alt = nullptr;
    O.cub_tmp = nullptr;
    const int64_t cap = std::max<int64_t>(n, 1024);
    SV_CK(c, cudaMalloc(&O.keys, sizeof(float) * cap));
    SV_CK(c, cudaMalloc(&O.keys_alt, sizeof(float) * cap));
    SV_CK(c, cudaMalloc(&O.flag, sizeof(int32_t) * cap));
    SV_CK(c, cudaMalloc(&O.status2, sizeof(int32_t) * cap));
    SV_CK(c, cudaMalloc(&O.list, sizeof(int32_t) * cap));
    SV_CK(c, cudaMalloc(&O.list_alt, sizeof(int32_t) * cap));
    size_t b1 = 0, b2 = 0;
    SV_CK(c, cub::DeviceRadixSort::SortKeys(nullptr, b1, O.keys, O.keys_alt, (int)cap, 0, 32, c->stream));
    SV_CK(c, cub::DeviceRadixSort::SortKeys(nullptr, b2, O.list, O.list_alt, (int)cap, 0, 32, c->stream));
    O.cub_bytes = std::max(b1, b2);
    SV_CK(c, cudaMalloc(&O.cub_tmp, O.cub_bytes));
    if (!O.count) {
        SV_CK(c, cudaMalloc(&O.count, sizeof(int) * 2));
        SV_CK(c, cudaMalloc(&O.stats, sizeof(float) * 6));
        SV_CK(c, cudaMallocHost(&O.h_count, sizeof(int) * 2));
    }
    O.cap = cap;
    return SV_OK;
}

}  // namespace

void outliers_free(sv_ctx *c) {
    if (!c->outliers) return;
    Outliers &O = *c->outliers;
    cudaFree(O.keys); cudaFree(O.keys_alt); cudaFree(O.flag); cudaFree(O.status2); cudaFree(O.list);
    cudaFree(O.list_alt); cudaFree(O.cub_tmp); cudaFree(O.count); cudaFree(O.stats);
    cudaFreeHost(O.h_count);
    delete c->outliers;
    c->outliers = nullptr;
}

sv_status outliers_detect(sv_ctx *c, const int32_t **status_for_tree) {
    if (!c->outliers) c->outliers = new Outliers();
    Outliers &O = *c->outliers;
    const int64_t n = c->n;
    SV_TRY(reserve(c, O, n));
    const int g = div_up(n, 256);
    SV_CK(c, cudaMemsetAsync(O.count, 0, sizeof(int) * 2, c->stream));
    count_sources_kernel<<<std::min(g, 16 * device_sms()), 256, 0, c->stream>>>(force_status(c), n, O.count);
    SV_LAUNCHED(c);
    const double *axis[3] = {c->x, c->y, c->z};
    for (int pass = 0; pass < 2; pass++) {
        for (int d = 0; d < 3; d++) {
            axis_values_kernel<<<g, 256, 0, c->stream>>>(axis[d], force_status(c), n, pass ? O.stats + d : nullptr, O.keys);
            SV_LAUNCHED(c);
            size_t bytes = O.cub_bytes;
            SV_CK(c, cub::DeviceRadixSort::SortKeys(O.cub_tmp, bytes, O.keys, O.keys_alt, (int)n, 0, 32, c->stream));
            c->launches += 8;
            true_median_kernel<<<1, 1, 0, c->stream>>>(O.keys_alt, O.count, pass ? kOutlierFactor : 1.0f,
                                                      O.stats + 3 * pass + d);
            SV_LAUNCHED(c);
        }
    }
    flag_kernel<<<g, 256, 0, c->stream>>>(c->x, c->y, c->z, force_status(c), n, O.stats, O.flag, O.status2, O.list,
                                          O.count);
    SV_LAUNCHED(c);
    SV_CK(c, cudaMemcpyAsync(O.h_count, O.count, sizeof(int) * 2, cudaMemcpyDeviceToHost, c->stream));
    SV_CK(c, cudaStreamSynchronize(c->stream));
    O.n_out = O.h_count[1];
    if (O.n_out > 1) {
        size_t bytes = O.cub_bytes;
        SV_CK(c, cub::DeviceRadixSort::SortKeys(O.cub_tmp, bytes, O.list, O.list_alt, O.n_out, 0, 32, c->stream));
        c->launches += 8;
        std::swap(O.list, O.list_alt);
    }
    O.valid = true;
    *status_for_tree = O.status2;
    return SV_OK;
}

sv_status outliers_add(sv_ctx *c, int64_t first, int64_t last) {
    Outliers &O = *c->outliers;
    if (O.n_out == 0) return SV_OK;
    const int64_t n = c->n;
    outlier_sources_kernel<<<div_up(n, 256), 256, 0, c->stream>>>(
        c->x, c->y, c->z, c->q, c->m, force_status(c), O.flag, O.list, O.n_out, n, first, last, c->P.softening2,
        c->P.k_const, c->ax, c->ay, c->az);
    SV_LAUNCHED(c);
    outlier_targets_kernel<<<O.n_out, 256, 0, c->stream>>>(c->x, c->y, c->z, c->q, c->m, force_status(c), O.list, n,
                                                           first, last, c->P.softening2, c->P.k_const, c->ax,
                                                           c->ay, c->az);
    SV_LAUNCHED(c);
    return SV_OK;
}

sv_status outliers_get(sv_ctx *c, int32_t *flags, int64_t *count) {
    if (!c->outliers || !c->outliers->valid)
        return set_error(c, SV_ERR_STATE, "no outlier-variant FMM evaluation has run");
    Outliers &O = *c->outliers;
    if (flags) {
        SV_CK(c, cudaMemcpyAsync(flags, O.flag, sizeof(int32_t) * c->n, cudaMemcpyDeviceToHost, c->stream));
        SV_CK(c, cudaStreamSynchronize(c->stream));
    }
    if (count) *count = O.n_out;
    return SV_OK;
}

}  // namespace sv
