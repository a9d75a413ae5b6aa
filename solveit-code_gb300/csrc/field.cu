// field.cu -- the single-emitter background field map on the device
// (InterpolationScheme, interpolation_scheme.cpp:66-262, with the walk and
// interpolation of pwl_interp_2d_scattered.c; the per-particle evaluation is
// in field.cuh, called from the kick).
#include <vector>

#include "sv_internal.cuh"

namespace sv {
namespace {

__global__ void field_points_kernel(FieldMesh M, const double *__restrict__ x3, int64_t n, double *__restrict__ e3) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int t = -1;
        double ex, ey, ez;
        field_at(M, x3[3 * i], x3[3 * i + 1], x3[3 * i + 2], &t, &ex, &ey, &ez);
        e3[3 * i] = ex;
        e3[3 * i + 1] = ey;
        e3[3 * i + 2] = ez;
    }
}

__global__ void fill_minus_one(int *p, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = -1;
}

int grid_for(int64_t n) {
    const int64_t b = (n + 255) / 256;
    return (int)(b < 1 ? 1 : (b > 16 * device_sms() ? 16 * device_sms() : b));
}

}  // namespace

void field_free(sv_ctx *c) {
    FieldMesh &M = c->field;
    cudaFree(const_cast<double2 *>(M.node));
    cudaFree(const_cast<double *>(M.er));
    cudaFree(const_cast<double *>(M.ez));
    cudaFree(const_cast<int *>(M.tri));
    cudaFree(const_cast<int *>(M.nbr));
    cudaFree(M.cache);
    cudaFree(M.err);
    M = FieldMesh{};
    c->field_cap = 0;
}

sv_status field_prepare(sv_ctx *c) {
    FieldMesh &M = c->field;
    if (M.nt == 0) return SV_OK;
    const int64_t want = c->n > 1 ? c->n : 1;
    if (c->field_cap < want) {
        cudaFree(M.cache);
        M.cache = nullptr;
        c->field_cap = 0;
        SV_CK(c, cudaMalloc(&M.cache, sizeof(int) * want));
        c->field_cap = want;
        fill_minus_one<<<grid_for(want), 256, 0, c->stream>>>(M.cache, want);
        SV_LAUNCHED(c);
    }
    return SV_OK;
}

// reset the walks' start triangles (a new state has no previous triangles)
sv_status field_reset(sv_ctx *c) {
    FieldMesh &M = c->field;
    if (M.nt == 0 || !M.cache) return SV_OK;
    fill_minus_one<<<grid_for(c->field_cap), 256, 0, c->stream>>>(M.cache, c->field_cap);
    SV_LAUNCHED(c);
    return SV_OK;
}

sv_status field_check(sv_ctx *c) {
    FieldMesh &M = c->field;
    if (M.nt == 0) return SV_OK;
    int err = 0;
    SV_CK(c, cudaMemcpyAsync(&err, M.err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    SV_CK(c, cudaStreamSynchronize(c->stream));
    if (!err) return SV_OK;
    SV_CK(c, cudaMemsetAsync(M.err, 0, sizeof(int), c->stream));
    return set_error(c, SV_ERR_INVALID, "emitter field: %s", (err & 1) ? "a triangulation walk did not end (cycle)"
                                                                        : "degenerate triangle in the field map");
}

}  // namespace sv

using namespace sv;

extern "C" {

sv_status sv_set_emitter_field(sv_ctx *c, int32_t n_nodes, const double *node_rz, const double *e_r,
                               const double *e_z, int32_t n_tri, const int32_t *tri, const int32_t *nbr, double r0,
                               double e0, double z_max) {
    if (!c) return SV_ERR_INVALID;
    SV_CK(c, cudaSetDevice(c->device));
    SV_CK(c, cudaStreamSynchronize(c->stream));
    field_free(c);
    if (c->batch) batch_invalidate(c);
    if (n_nodes == 0) return SV_OK;
    if (n_nodes < 3 || n_tri < 1 || !node_rz || !e_r || !e_z || !tri || !nbr)
        return set_error(c, SV_ERR_INVALID, "field map needs >= 3 nodes, >= 1 triangle and all arrays");
    if (!(r0 > 0.0) || !(z_max >= 0.0)) return set_error(c, SV_ERR_INVALID, "r0 > 0 and z_max >= 0 required");
    for (int64_t k = 0; k < 3 * (int64_t)n_tri; k++) {
        if (tri[k] < 0 || tri[k] >= n_nodes)
            return set_error(c, SV_ERR_INVALID, "triangle %lld: node %d out of range", (long long)(k / 3), tri[k]);
        if (nbr[k] < -1 || nbr[k] >= n_tri)
            return set_error(c, SV_ERR_INVALID, "triangle %lld: neighbour %d out of range", (long long)(k / 3),
                             nbr[k]);
    }
    std::vector<double2> nodes(n_nodes);
    for (int k = 0; k < n_nodes; k++) nodes[k] = make_double2(node_rz[2 * k], node_rz[2 * k + 1]);
    // each buffer is owned by c->field as soon as it exists, so field_free
    // releases a partial allocation too
    FieldMesh &M = c->field;
    double2 *dn = nullptr;
    double *der = nullptr, *dez = nullptr;
    int *dt = nullptr, *dnb = nullptr, *derr = nullptr;
    SV_CK(c, cudaMalloc(&dn, sizeof(double2) * n_nodes));
    M.node = dn;
    SV_CK(c, cudaMalloc(&der, sizeof(double) * n_nodes));
    M.er = der;
    SV_CK(c, cudaMalloc(&dez, sizeof(double) * n_nodes));
    M.ez = dez;
    SV_CK(c, cudaMalloc(&dt, sizeof(int) * 3 * (size_t)n_tri));
    M.tri = dt;
    SV_CK(c, cudaMalloc(&dnb, sizeof(int) * 3 * (size_t)n_tri));
    M.nbr = dnb;
    SV_CK(c, cudaMalloc(&derr, sizeof(int)));
    M.err = derr;
    M.r0 = r0;
    M.e0 = e0;
    M.zmax = z_max;
    SV_CK(c, cudaMemcpy(dn, nodes.data(), sizeof(double2) * n_nodes, cudaMemcpyHostToDevice));
    SV_CK(c, cudaMemcpy(der, e_r, sizeof(double) * n_nodes, cudaMemcpyHostToDevice));
    SV_CK(c, cudaMemcpy(dez, e_z, sizeof(double) * n_nodes, cudaMemcpyHostToDevice));
    SV_CK(c, cudaMemcpy(dt, tri, sizeof(int) * 3 * (size_t)n_tri, cudaMemcpyHostToDevice));
    SV_CK(c, cudaMemcpy(dnb, nbr, sizeof(int) * 3 * (size_t)n_tri, cudaMemcpyHostToDevice));
    SV_CK(c, cudaMemset(derr, 0, sizeof(int)));
    M.nt = n_tri;  // the field is on once the map is complete
    return SV_OK;
}

sv_status sv_emitter_field_at(sv_ctx *c, int64_t n, const double *x3, double *e3) {
    if (!c || n < 0 || (n > 0 && (!x3 || !e3))) return SV_ERR_INVALID;
    if (c->field.nt == 0) return set_error(c, SV_ERR_STATE, "no emitter field set");
    if (n == 0) return SV_OK;
    SV_CK(c, cudaSetDevice(c->device));
    double *d = nullptr;
    SV_CK(c, cudaMalloc(&d, sizeof(double) * 6 * (size_t)n));
    cudaError_t e = cudaMemcpyAsync(d, x3, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) {
        field_points_kernel<<<grid_for(n), 256, 0, c->stream>>>(c->field, d, n, d + 3 * n);
        c->launches++;
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(e3, d + 3 * n, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(d);
    SV_CK(c, e);
    return field_check(c);
}

}  // extern "C"
