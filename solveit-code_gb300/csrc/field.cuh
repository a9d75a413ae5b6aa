// field.cuh -- background field of a single emitter, evaluated per particle.
//
// InterpolationScheme::computeEfieldSingleEmitter (interpolation_scheme.cpp:
// 206-262) over the axisymmetric field map (r, z nodes in units of r0, field
// in units of E0, a triangulation with its neighbour table):
//   - (r, z) = (sqrt(x^2 + y^2), z) / r0; z outside [0, z_max] has no field;
//   - the triangle holding (r, z) is found by the walk of
//     triangulation_search_delaunay (pwl_interp_2d_scattered.c:1762-1992):
//     barycentric coordinates (alpha, beta, gamma) of the current triangle
//     (vertex c as the base), step across the edge opposite the first
//     negative coordinate whose neighbour exists, stop when all are >= 0 or
//     the negative ones face the hull (the field is then extrapolated from that
//     triangle);
//   - E_r, E_z = alpha f(a) + beta f(b) + gamma f(c)
//     (pwl_interp_2d_scattered_value, :887-957), E = E0 (E_r cos phi,
//     E_r sin phi, E_z) with the reference's phi (phi = pi/2 on x = 0, y != 0).
// The barycentric arithmetic uses the reference's operation order without
// fused multiply-adds, so a point next to an edge takes the same step.  Each
// particle starts its walk at its triangle of the previous evaluation (the
// mesh's middle triangle the first time), so a walk is a few steps.
#pragma once

#include <cstdint>

namespace sv {

struct FieldMesh {
    const double2 *node = nullptr;  // (r, z) / r0
    const double *er = nullptr, *ez = nullptr;
    const int *tri = nullptr, *nbr = nullptr;
    int nt = 0;                     // triangles (0: no emitter field)
    double r0 = 0, e0 = 0, zmax = 0;
    int *cache = nullptr;           // per particle: last triangle, -1 = none
    int *err = nullptr;             // bit 0: a walk did not end; bit 1: degenerate triangle
};

// Walk to the triangle of (pr, pz) from triangle t; returns it with the
// barycentric coordinates, or -1 (error bits set).
__device__ inline int field_walk(const FieldMesh &M, double pr, double pz, int t, double *alpha, double *beta,
                                 double *gamma) {
    for (int step = 0; step <= M.nt; step++) {
        const int a = M.tri[3 * t], b = M.tri[3 * t + 1], c = M.tri[3 * t + 2];
        const double2 A = M.node[a], B = M.node[b], Cc = M.node[c];
        const double dxa = __dsub_rn(A.x, Cc.x), dya = __dsub_rn(A.y, Cc.y);
        const double dxb = __dsub_rn(B.x, Cc.x), dyb = __dsub_rn(B.y, Cc.y);
        const double dxp = __dsub_rn(pr, Cc.x), dyp = __dsub_rn(pz, Cc.y);
        const double det = __dsub_rn(__dmul_rn(dxa, dyb), __dmul_rn(dya, dxb));
        const double al = __ddiv_rn(__dsub_rn(__dmul_rn(dxp, dyb), __dmul_rn(dyp, dxb)), det);
        const double be = __ddiv_rn(__dsub_rn(__dmul_rn(dxa, dyp), __dmul_rn(dya, dxp)), det);
        const double ga = __dsub_rn(__dsub_rn(1.0, al), be);
        *alpha = al;
        *beta = be;
        *gamma = ga;
        if (0.0 <= al && 0.0 <= be && 0.0 <= ga) return t;
        const int n0 = M.nbr[3 * t], n1 = M.nbr[3 * t + 1], n2 = M.nbr[3 * t + 2];
        if (al < 0.0 && n0 >= 0) {
            t = n0;
            continue;
        }
        if (be < 0.0 && n1 >= 0) {
            t = n1;
            continue;
        }
        if (ga < 0.0 && n2 >= 0) {
            t = n2;
            continue;
        }
        if (al < 0.0 || be < 0.0 || ga < 0.0) return t;  // outside the hull: extrapolate from t
        atomicOr(M.err, 2);                               // NaN coordinates: a degenerate triangle
        return -1;
    }
    atomicOr(M.err, 1);
    return -1;
}

// E (V/m) of the emitter at (x, y, z) m; *t: the walk's start, updated.
__device__ inline void field_at(const FieldMesh &M, double x, double y, double z, int *t, double *ex, double *ey,
                                double *ez) {
    *ex = *ey = *ez = 0.0;
    const double pz = z / M.r0;
    if (pz < 0.0 || pz > M.zmax) return;
    const double pr = sqrt(x * x + y * y) / M.r0;
    int t0 = *t;
    if (t0 < 0 || t0 >= M.nt) t0 = (M.nt + 1) / 2 - 1;
    double al, be, ga;
    const int tr = field_walk(M, pr, pz, t0, &al, &be, &ga);
    if (tr < 0) return;
    *t = tr;
    const int a = M.tri[3 * tr], b = M.tri[3 * tr + 1], c = M.tri[3 * tr + 2];
    const double fr = __dadd_rn(__dadd_rn(__dmul_rn(al, M.er[a]), __dmul_rn(be, M.er[b])), __dmul_rn(ga, M.er[c]));
    const double fz = __dadd_rn(__dadd_rn(__dmul_rn(al, M.ez[a]), __dmul_rn(be, M.ez[b])), __dmul_rn(ga, M.ez[c]));
    // phi as the reference forms it: atan(y/x) (+pi for x < 0), pi/2 on the
    // y axis whatever the sign of y, 0 at the origin
    double cph, sph;
    if (x == 0.0) {
        cph = y != 0.0 ? 0.0 : 1.0;
        sph = y != 0.0 ? 1.0 : 0.0;
    } else {
        const double r = sqrt(x * x + y * y);
        cph = x / r;
        sph = y / r;
    }
    *ex = M.e0 * fr * cph;
    *ey = M.e0 * fr * sph;
    *ez = M.e0 * fz;
}

}  // namespace sv
