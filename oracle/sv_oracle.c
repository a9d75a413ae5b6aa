/*
 * sv_oracle.c -- CPU restatement of the SOLVEiT force-evaluation hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker that the CUDA path is compared with
 * (parity tests, smoke check, bench.py cpu_baseline leg).  The product
 * library never links or calls it.
 *
 * Build with -ffp-contract=off so that no multiply-add is fused: the
 * reference is compiled for plain x86-64 (no FMA), and the *_ref32
 * functions reproduce its rounding step by step.  Each function cites the
 * reference file:line it restates (paths inside the SOLVEiT-Code project).
 */
#include "sv_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---- constants (constants.h:28-47) ----------------------------------- */

static const long double REF_PI = 3.14159265358979323846264338328L;
static const float REF_ELEM_CHARGE = 1.6021766e-19f;
static const float REF_AMU = 1.66053904e-27f;
static const float REF_EPS0 = 8.85419e-12f;

double orc_k_const(void) {
    /* K_CONST = (ELEM_CHARGE * ELEM_CHARGE) / (4 * PI * FREE_SPACE_PERMITTIVITY * AMU):
     * float*float in float, the denominator in long double (constants.h:46). */
    float e2 = REF_ELEM_CHARGE * REF_ELEM_CHARGE;
    long double den = 4 * REF_PI * REF_EPS0 * REF_AMU;
    return (double)((long double)e2 / den);
}

double orc_e_over_amu(void) {
    /* factor = ELEM_CHARGE / AMU, float division (particles.cpp:500). */
    float f = REF_ELEM_CHARGE / REF_AMU;
    return (double)f;
}

double orc_coulomb_ke(void) {
    /* ke = 1 / (4 pi eps0) stored as float (particles.cpp:565). */
    float ke = (float)(1 / (4.0 * REF_PI * REF_EPS0));
    return (double)ke;
}

double orc_elem_charge(void) { return (double)REF_ELEM_CHARGE; }
double orc_amu(void) { return (double)REF_AMU; }

/* ParticleSpeciesFunction::getMass (particles.h:65-87), EMI 111, BF4 87. */
static long double species_mass_ld(int s) {
    switch (s) {
    case 0: return 111.0L;                 /* monomerPositive */
    case 1: return 2 * 111.0 + 87.0;       /* dimerPositive */
    case 2: return 3 * 111.0 + 2 * 87.0;   /* trimerPositive */
    case 3: return 0.0L;                   /* droplet: unsupported -> 0 */
    case 4: return 111.0 + 87.0;           /* neutral */
    case 5: return 87.0;                   /* monomerNegative */
    case 6: return 111.0 + 2 * 87.0;       /* dimerNegative */
    case 7: return 2 * 111.0 + 3 * 87.0;   /* trimerNegative */
    default: return 0.0L;
    }
}

double orc_species_mass(int species) { return (double)species_mass_ld(species); }

static int nthreads_or_default(int nthreads) {
#ifdef _OPENMP
    return nthreads > 0 ? nthreads : omp_get_max_threads();
#else
    (void)nthreads;
    return 1;
#endif
}

/* accel_const = K_const * q / getMass(i): double * float, then divided by a
 * long double mass, rounded to double (direct_force_method.cpp:183). */
static double accel_const_ref(const float *pos4, const float *vel4, int i) {
    long double m = species_mass_ld((int)vel4[4 * i + 3]);
    double kq = orc_k_const() * (double)pos4[4 * i + 3];
    return (double)((long double)kq / m);
}

/* ---- reference direct, no symmetry ------------------------------------ */

void orc_direct_ref32(const float *pos4, const float *vel4, float *acc4,
                      int i0, int i1, int j0, int j1, double eps, int nthreads) {
    /* DirectForceFunction::direct (direct_force_method.cpp:153-190). */
    const int nt = nthreads_or_default(nthreads);
#pragma omp parallel for schedule(dynamic, 16) num_threads(nt)
    for (int i = i0; i < i1; i++) {
        if (acc4[4 * i + 3] != 1.0f) continue;
        double ax = 0, ay = 0, az = 0;
        for (int j = j0; j < j1; j++) {
            float wj = acc4[4 * j + 3];
            if (!(wj == 1.0f || wj == 2.0f) || j == i) continue;
            double dx = (float)(pos4[4 * i + 0] - pos4[4 * j + 0]);
            double dy = (float)(pos4[4 * i + 1] - pos4[4 * j + 1]);
            double dz = (float)(pos4[4 * i + 2] - pos4[4 * j + 2]);
            double inv = 1.0 / sqrt(dx * dx + dy * dy + dz * dz + eps);
            double inv3 = (double)pos4[4 * j + 3] * inv * inv * inv;
            ax += dx * inv3;
            ay += dy * inv3;
            az += dz * inv3;
        }
        double c = accel_const_ref(pos4, vel4, i);
        ax *= c; ay *= c; az *= c;
        acc4[4 * i + 0] = (float)((double)acc4[4 * i + 0] + ax);
        acc4[4 * i + 1] = (float)((double)acc4[4 * i + 1] + ay);
        acc4[4 * i + 2] = (float)((double)acc4[4 * i + 2] + az);
    }
}

/* quadrantRotationFunction (auxiliary_functions.h:55-57): cos/sin of k*pi/2
 * as integers. */
static int quadrant_rot(int n) {
    if ((n & 1) == 0) return 0;
    return (((n - 1) >> 1) & 1) ? -1 : 1;
}

void orc_direct_rot4_ref32(const float *pos4, const float *vel4, float *acc4,
                           int i0, int i1, int j0, int j1, double eps,
                           int nthreads) {
    /* directKernelRotationCalculation + direct_rotational
     * (direct_force_method_rotational.cpp:28-94): for each quadrant the
     * source is rotated by k*pi/2 in FP32, no j != i test, and each
     * quadrant's sum is added to the FP32 acceleration in turn. */
    const int nt = nthreads_or_default(nthreads);
    for (int k = 0; k < 4; k++) {
        const int ck = quadrant_rot(k + 1);
        const int sk = quadrant_rot(k);
#pragma omp parallel for schedule(dynamic, 16) num_threads(nt)
        for (int i = i0; i < i1; i++) {
            if (acc4[4 * i + 3] != 1.0f) continue;
            double ax = 0, ay = 0, az = 0;
            const float xi = pos4[4 * i + 0], yi = pos4[4 * i + 1], zi = pos4[4 * i + 2];
            for (int j = j0; j < j1; j++) {
                float wj = acc4[4 * j + 3];
                if (!(wj == 1.0f || wj == 2.0f)) continue;
                const float xj = pos4[4 * j + 0], yj = pos4[4 * j + 1];
                double dz = (float)(zi - pos4[4 * j + 2]);
                double dz2 = dz * dz;
                float rx = (float)ck * xj - (float)sk * yj;
                float ry = (float)sk * xj + (float)ck * yj;
                double dx = (float)(xi - rx);
                double dy = (float)(yi - ry);
                double inv = 1.0 / sqrt(dx * dx + dy * dy + dz2 + eps);
                double inv3 = (double)pos4[4 * j + 3] * inv * inv * inv;
                ax += dx * inv3;
                ay += dy * inv3;
                az += dz * inv3;
            }
            double c = accel_const_ref(pos4, vel4, i);
            ax *= c; ay *= c; az *= c;
            acc4[4 * i + 0] = (float)((double)acc4[4 * i + 0] + ax);
            acc4[4 * i + 1] = (float)((double)acc4[4 * i + 1] + ay);
            acc4[4 * i + 2] = (float)((double)acc4[4 * i + 2] + az);
        }
    }
}

void orc_direct_trans_ref32(const float *pos4, const float *vel4, float *acc4,
                            int i0, int i1, int j0, int j1, double eps,
                            int nimg, const int *images,
                            const float domain_size[3], int nthreads) {
    /* direct_translational (direct_force_method_translational.cpp:320-367),
     * called once per image in the order of the image list. */
    const int nt = nthreads_or_default(nthreads);
    for (int g = 0; g < nimg; g++) {
        const float ox = (float)images[3 * g + 0] * domain_size[0];
        const float oy = (float)images[3 * g + 1] * domain_size[1];
        const float oz = (float)images[3 * g + 2] * domain_size[2];
#pragma omp parallel for schedule(dynamic, 16) num_threads(nt)
        for (int i = i0; i < i1; i++) {
            if (acc4[4 * i + 3] != 1.0f) continue;
            double ax = 0, ay = 0, az = 0;
            const float xi = pos4[4 * i + 0] - ox;
            const float yi = pos4[4 * i + 1] - oy;
            const float zi = pos4[4 * i + 2] - oz;
            for (int j = j0; j < j1; j++) {
                float wj = acc4[4 * j + 3];
                if (!(wj == 1.0f || wj == 2.0f)) continue;
                double dx = (float)(xi - pos4[4 * j + 0]);
                double dy = (float)(yi - pos4[4 * j + 1]);
                double dz = (float)(zi - pos4[4 * j + 2]);
                double inv = 1.0 / sqrt(dx * dx + dy * dy + dz * dz + eps);
                double inv3 = (double)pos4[4 * j + 3] * inv * inv * inv;
                ax += dx * inv3;
                ay += dy * inv3;
                az += dz * inv3;
            }
            double c = accel_const_ref(pos4, vel4, i);
            ax *= c; ay *= c; az *= c;
            acc4[4 * i + 0] = (float)((double)acc4[4 * i + 0] + ax);
            acc4[4 * i + 1] = (float)((double)acc4[4 * i + 1] + ay);
            acc4[4 * i + 2] = (float)((double)acc4[4 * i + 2] + az);
        }
    }
}

/* ---- periodic image list (lattice_point.h:65-131 and
 *      direct_force_method_translational.cpp:35-306) ------------------- */

static int oe(int i) { return (i & 1) ? -1 : 1; } /* ODDEVEN */

static int emit(int *out, int cnt, int max_out, int x, int y, int z) {
    if (cnt < max_out) {
        out[3 * cnt + 0] = x;
        out[3 * cnt + 1] = y;
        out[3 * cnt + 2] = z;
    }
    return cnt + 1;
}

int orc_trans_images(int box_length, const int axes[3], const int *lattice,
                     int nlat, int *out, int max_out) {
    const int n = box_length / 2;
    const int dsum = (axes[0] != 0) + (axes[1] != 0) + (axes[2] != 0);
    int *pts = NULL;
    if (lattice == NULL) {
        int cap = (2 * n + 1) * (2 * n + 1) * (2 * n + 1) + 1;
        pts = (int *)malloc(sizeof(int) * 3 * (size_t)cap);
        int cnt = 0;
        int t[3] = {axes[0] != 0, axes[1] != 0, axes[2] != 0};
        for (int pass = 0; pass < dsum; pass++) {
            int i = t[0];
            do {
                int j = t[1];
                do {
                    int k = t[2];
                    do {
                        pts[3 * cnt + 0] = i; pts[3 * cnt + 1] = j; pts[3 * cnt + 2] = k;
                        cnt++;
                        k++;
                    } while (t[2] != 0 && k <= n);
                    j++;
                } while (t[1] != 0 && j <= n);
                i++;
            } while (t[0] != 0 && i <= n);
            if (t[0] == 0) {
                if (t[1] == 0) t[2] = 0; else t[1] = 0;
            } else {
                t[0] = 0;
            }
        }
        pts[3 * cnt + 0] = 0; pts[3 * cnt + 1] = 0; pts[3 * cnt + 2] = 0;
        cnt++;
        /* descending norm; insertion sort keeps ties in generation order */
        for (int a = 1; a < cnt; a++) {
            int p0 = pts[3 * a], p1 = pts[3 * a + 1], p2 = pts[3 * a + 2];
            int na = p0 * p0 + p1 * p1 + p2 * p2;
            int b = a - 1;
            while (b >= 0) {
                int nb = pts[3 * b] * pts[3 * b] + pts[3 * b + 1] * pts[3 * b + 1] +
                         pts[3 * b + 2] * pts[3 * b + 2];
                if (nb >= na) break;
                memcpy(&pts[3 * (b + 1)], &pts[3 * b], sizeof(int) * 3);
                b--;
            }
            pts[3 * (b + 1)] = p0; pts[3 * (b + 1) + 1] = p1; pts[3 * (b + 1) + 2] = p2;
        }
        lattice = pts;
        nlat = cnt;
    }
    int cnt = 0;
    for (int ii = 0; ii < nlat; ii++) {
        const int px = lattice[3 * ii], py = lattice[3 * ii + 1], pz = lattice[3 * ii + 2];
        const int nz = (px != 0) + (py != 0) + (pz != 0);
        const int ni = 1 + (px != 0), nj = 1 + (py != 0), nk = 1 + (pz != 0);
        if (dsum == 3) {
            if (nz == 3) {
                for (int i = 0; i < 2; i++)
                    for (int j = 0; j < 2; j++)
                        for (int k = 0; k < 2; k++)
                            cnt = emit(out, cnt, max_out, oe(i) * px, oe(j) * py, oe(k) * pz);
            } else if (nz == 2) {
                for (int jj = 0; jj < 3; jj++)
                    for (int i = 0; i < ni; i++)
                        for (int j = 0; j < nj; j++)
                            for (int k = 0; k < nk; k++) {
                                int tx = (jj != 0) * oe(i) * px +
                                         (px == 0) * ((jj == 1) * oe(j) * py + (jj == 2) * oe(k) * pz);
                                int ty = (jj != 1) * oe(j) * py +
                                         (py == 0) * ((jj == 0) * oe(i) * px + (jj == 2) * oe(k) * pz);
                                int tz = (jj != 2) * oe(k) * pz +
                                         (pz == 0) * ((jj == 0) * oe(i) * px + (jj == 1) * oe(j) * py);
                                cnt = emit(out, cnt, max_out, tx, ty, tz);
                            }
            } else if (nz == 1) {
                for (int jj = 0; jj < 3; jj++)
                    for (int i = 0; i < ni; i++)
                        for (int j = 0; j < nj; j++)
                            for (int k = 0; k < nk; k++) {
                                int tx = (jj == 0) * oe(i) * px + (jj == 1) * oe(j) * py + (jj == 2) * oe(k) * pz;
                                int ty = (jj == 0) * oe(j) * py + (jj == 1) * oe(k) * pz + (jj == 2) * oe(i) * px;
                                int tz = (jj == 0) * oe(k) * pz + (jj == 1) * oe(i) * px + (jj == 2) * oe(j) * py;
                                cnt = emit(out, cnt, max_out, tx, ty, tz);
                            }
            } else {
                cnt = emit(out, cnt, max_out, 0, 0, 0);
            }
        } else if (dsum == 2) {
            if (nz == 2) {
                for (int i = 0; i < ni; i++)
                    for (int j = 0; j < nj; j++)
                        for (int k = 0; k < nk; k++)
                            cnt = emit(out, cnt, max_out, oe(i) * px, oe(j) * py, oe(k) * pz);
            } else if (nz == 1) {
                const int ax = axes[0] != 0, ay = axes[1] != 0, az = axes[2] != 0;
                for (int jj = 0; jj < 2; jj++)
                    for (int i = 0; i < ni; i++)
                        for (int j = 0; j < nj; j++)
                            for (int k = 0; k < nk; k++) {
                                int tx = ax * ((jj == 0) * oe(i) * px + (jj == 1) * (oe(j) * py + oe(k) * pz));
                                int ty = ay * ((jj == 0) * oe(j) * py + (jj == 1) * (oe(i) * px + oe(k) * pz));
                                int tz = az * ((jj == 0) * oe(k) * pz + (jj == 1) * (oe(i) * px + oe(j) * py));
                                cnt = emit(out, cnt, max_out, tx, ty, tz);
                            }
            } else {
                cnt = emit(out, cnt, max_out, 0, 0, 0);
            }
        } else if (dsum == 1) {
            if (nz == 1) {
                for (int i = 0; i < ni; i++)
                    for (int j = 0; j < nj; j++)
                        for (int k = 0; k < nk; k++)
                            cnt = emit(out, cnt, max_out, oe(i) * px, oe(j) * py, oe(k) * pz);
            } else {
                cnt = emit(out, cnt, max_out, 0, 0, 0);
            }
        }
    }
    free(pts);
    return cnt;
}

/* ---- FP64 ground truth ------------------------------------------------- */

void orc_direct_f64(int64_t n, const double *x, const double *q,
                    const double *m, const int32_t *status,
                    const int64_t *targets, int64_t ntargets, double eps2,
                    double kconst, int sym, int nimg, const double *img_off,
                    double *a_out, int nthreads) {
    /* Same pair law as direct_force_method.cpp:163-189 (and the rotational /
     * translational variants), all in FP64. */
    const int nt = nthreads_or_default(nthreads);
    const int64_t nt_count = targets ? ntargets : n;
    static const double rc[4] = {1, 0, -1, 0}, rs[4] = {0, 1, 0, -1};
#pragma omp parallel for schedule(dynamic, 8) num_threads(nt)
    for (int64_t t = 0; t < nt_count; t++) {
        const int64_t i = targets ? targets[t] : t;
        double *ao = a_out + 3 * t;
        ao[0] = ao[1] = ao[2] = 0.0;
        if (status[i] != 1) continue;
        double ax = 0, ay = 0, az = 0;
        const double xi = x[3 * i], yi = x[3 * i + 1], zi = x[3 * i + 2];
        if (sym == 0) {
            for (int64_t j = 0; j < n; j++) {
                if (!(status[j] == 1 || status[j] == 2) || j == i) continue;
                double dx = xi - x[3 * j], dy = yi - x[3 * j + 1], dz = zi - x[3 * j + 2];
                double inv = 1.0 / sqrt(dx * dx + dy * dy + dz * dz + eps2);
                double w = q[j] * inv * inv * inv;
                ax += dx * w; ay += dy * w; az += dz * w;
            }
        } else if (sym == 1) {
            for (int k = 0; k < 4; k++) {
                double bx = 0, by = 0, bz = 0;
                for (int64_t j = 0; j < n; j++) {
                    if (!(status[j] == 1 || status[j] == 2)) continue;
                    double sx = rc[k] * x[3 * j] - rs[k] * x[3 * j + 1];
                    double sy = rs[k] * x[3 * j] + rc[k] * x[3 * j + 1];
                    double dx = xi - sx, dy = yi - sy, dz = zi - x[3 * j + 2];
                    double inv = 1.0 / sqrt(dx * dx + dy * dy + dz * dz + eps2);
                    double w = q[j] * inv * inv * inv;
                    bx += dx * w; by += dy * w; bz += dz * w;
                }
                ax += bx; ay += by; az += bz;
            }
        } else {
            for (int g = 0; g < nimg; g++) {
                const double tx = xi - img_off[3 * g], ty = yi - img_off[3 * g + 1],
                             tz = zi - img_off[3 * g + 2];
                double bx = 0, by = 0, bz = 0;
                for (int64_t j = 0; j < n; j++) {
                    if (!(status[j] == 1 || status[j] == 2)) continue;
                    double dx = tx - x[3 * j], dy = ty - x[3 * j + 1], dz = tz - x[3 * j + 2];
                    double inv = 1.0 / sqrt(dx * dx + dy * dy + dz * dz + eps2);
                    double w = q[j] * inv * inv * inv;
                    bx += dx * w; by += dy * w; bz += dz * w;
                }
                ax += bx; ay += by; az += bz;
            }
        }
        const double c = kconst * q[i] / m[i];
        ao[0] = ax * c; ao[1] = ay * c; ao[2] = az * c;
    }
}

void orc_potential_f64(int64_t n, const double *x, const double *q,
                       const int32_t *status, const int64_t *targets,
                       int64_t ntargets, double eps2, double *phi_out,
                       int nthreads) {
    const int nt = nthreads_or_default(nthreads);
    const int64_t nt_count = targets ? ntargets : n;
#pragma omp parallel for schedule(dynamic, 8) num_threads(nt)
    for (int64_t t = 0; t < nt_count; t++) {
        const int64_t i = targets ? targets[t] : t;
        double phi = 0;
        for (int64_t j = 0; j < n; j++) {
            if (!(status[j] == 1 || status[j] == 2) || j == i) continue;
            double dx = x[3 * i] - x[3 * j], dy = x[3 * i + 1] - x[3 * j + 1],
                   dz = x[3 * i + 2] - x[3 * j + 2];
            phi += q[j] / sqrt(dx * dx + dy * dy + dz * dz + eps2);
        }
        phi_out[t] = phi;
    }
}

/* ---- leapfrog DKD ------------------------------------------------------ */

static float clampf_dt(float v, float dt) {
    /* std::min(std::max(v, 0.0f), dt) */
    float a = v > 0.0f ? v : 0.0f;
    return dt < a ? dt : a;
}

/* std::max / std::min as the reference calls them */
static float ref_maxf(float a, float b) { return a < b ? b : a; }
static float ref_minf(float a, float b) { return b < a ? b : a; }
static double ref_max(double a, double b) { return a < b ? b : a; }
static double ref_min(double a, double b) { return b < a ? b : a; }

/* CrashParameters::checkExtractorGridCrash (structures.h:467-517), FP32:
 * returns 1 on a crash with *fz the crossing's z. */
static int crash_ref32(const orc_boundary *bd, float ix, float iy, float iz, float fx, float fy, float fz0,
                       float *fz) {
    const float zd = (float)bd->crash_z, zw = (float)bd->crash_width, rd = (float)bd->crash_r;
    float initial_r = sqrtf(ix * ix + iy * iy);
    float final_r = sqrtf(fx * fx + fy * fy);
    float m = (fz0 - iz) / (final_r - initial_r);
    float b = iz - m * initial_r;
    float min_r = ref_minf(initial_r, final_r), max_r = ref_maxf(initial_r, final_r);
    float min_z = ref_minf(iz, fz0), max_z = ref_maxf(iz, fz0);
    float temp_r, temp_z;
    if (zd >= min_z && zd <= max_z) {
        temp_r = (zd - b) / m;
        if (temp_r >= ref_maxf(min_r, rd) && temp_r <= max_r) {
            *fz = zd;
            return 1;
        }
    }
    if (zd + zw >= min_z && zd + zw <= max_z) {
        temp_r = (zd + zw - b) / m;
        if (temp_r >= ref_maxf(min_r, rd) && temp_r <= max_r) {
            *fz = zd + zw;
            return 1;
        }
    }
    if (rd >= min_r && rd <= max_r) {
        temp_z = m * rd + b;
        if (temp_z >= ref_maxf(min_z, zd) && temp_z <= ref_minf(max_z, zd + zw)) {
            *fz = temp_z;
            return 1;
        }
    }
    return 0;
}

static int crash_f64(const orc_boundary *bd, double ix, double iy, double iz, double fx, double fy, double fz0,
                     double *fz) {
    const double zd = bd->crash_z, zw = bd->crash_width, rd = bd->crash_r;
    const double ri = sqrt(ix * ix + iy * iy), rf = sqrt(fx * fx + fy * fy);
    const double m = (fz0 - iz) / (rf - ri), b = iz - m * ri;
    const double rmin = ref_min(ri, rf), rmax = ref_max(ri, rf);
    const double zmin = ref_min(iz, fz0), zmax = ref_max(iz, fz0);
    if (zd >= zmin && zd <= zmax) {
        const double tr = (zd - b) / m;
        if (tr >= ref_max(rmin, rd) && tr <= rmax) {
            *fz = zd;
            return 1;
        }
    }
    if (zd + zw >= zmin && zd + zw <= zmax) {
        const double tr = (zd + zw - b) / m;
        if (tr >= ref_max(rmin, rd) && tr <= rmax) {
            *fz = zd + zw;
            return 1;
        }
    }
    if (rd >= rmin && rd <= rmax) {
        const double tz = m * rd + b;
        if (tz >= ref_max(zmin, zd) && tz <= ref_min(zmax, zd + zw)) {
            *fz = tz;
            return 1;
        }
    }
    return 0;
}

static void push_event(orc_event *ev, int ev_cap, int *ev_count, float t, float x, float y, float z, float vx,
                       float vy, float vz, int index, uint32_t species, int32_t status) {
    if (ev && *ev_count < ev_cap) {
        orc_event *e = &ev[*ev_count];
        e->time = t;
        e->x = x; e->y = y; e->z = z;
        e->vx = vx; e->vy = vy; e->vz = vz;
        e->index = index;
        e->species = species;
        e->status = status;
    }
    (*ev_count)++;
}

/* ChargedParticles::findMostRecentInjected (particles.cpp:1328-1359) */
static int most_recent_injected(int n, const float *t_inj, float time) {
    int max_i = n - 1, min_i = 0, t;
    do {
        t = (max_i + min_i) / 2;
        if (t_inj[t] <= time)
            min_i = t + 1;
        else if (t_inj[t] > time)
            max_i = t - 1;
    } while (max_i > min_i);
    t = max_i;
    if (t_inj[t] > time) t--;
    return t;
}

/* ParticleSystem::translateToSymmetryDomain, one axis (particles.cpp:278-333), FP32 */
static float wrap_ref32(float p, float L) {
    float temp = p + L / 2;
    if (temp >= 0) return fmodf(temp, L) - L / 2;
    temp = fmodf(temp, L);
    return temp < 0 ? temp + L / 2 : temp - L / 2;
}

static double wrap_f64(double p, double L) {
    double temp = p + L / 2;
    if (temp >= 0) return fmod(temp, L) - L / 2;
    temp = fmod(temp, L);
    return temp < 0 ? temp + L / 2 : temp - L / 2;
}

/* triangulation_search_delaunay (pwl_interp_2d_scattered.c:1762-1992): walk
 * from *t to the triangle holding p; returns it (or -1 at a dead end) and the
 * barycentric coordinates; *t keeps the start for the next search when the
 * walk ended normally (the reference's triangle_index_save). */
static int field_walk(const orc_field *f, const double p[2], int *t, double *al, double *be, double *ga) {
    int ti = (*t < 0 || f->n_tri <= *t) ? (f->n_tri + 1) / 2 - 1 : *t;
    for (int step = 0;; step++) {
        if (f->n_tri < step) return -1;
        const int a = f->tri[3 * ti], b = f->tri[3 * ti + 1], c = f->tri[3 * ti + 2];
        const double dxa = f->node_rz[2 * a] - f->node_rz[2 * c];
        const double dya = f->node_rz[2 * a + 1] - f->node_rz[2 * c + 1];
        const double dxb = f->node_rz[2 * b] - f->node_rz[2 * c];
        const double dyb = f->node_rz[2 * b + 1] - f->node_rz[2 * c + 1];
        const double dxp = p[0] - f->node_rz[2 * c];
        const double dyp = p[1] - f->node_rz[2 * c + 1];
        const double det = dxa * dyb - dya * dxb;
        *al = (dxp * dyb - dyp * dxb) / det;
        *be = (dxa * dyp - dya * dxp) / det;
        *ga = 1.0 - *al - *be;
        if (0.0 <= *al && 0.0 <= *be && 0.0 <= *ga) break;
        if (*al < 0.0 && 0 <= f->nbr[3 * ti]) {
            ti = f->nbr[3 * ti];
            continue;
        } else if (*be < 0.0 && 0 <= f->nbr[3 * ti + 1]) {
            ti = f->nbr[3 * ti + 1];
            continue;
        } else if (*ga < 0.0 && 0 <= f->nbr[3 * ti + 2]) {
            ti = f->nbr[3 * ti + 2];
            continue;
        }
        if (*al < 0.0 || *be < 0.0 || *ga < 0.0) break; /* outside the hull */
        return -1;
    }
    *t = ti;
    return ti;
}

/* pwl_interp_2d_scattered_value (pwl_interp_2d_scattered.c:887-957), one point */
static double field_value(const orc_field *f, const double *zd, int t, double al, double be, double ga) {
    return al * zd[f->tri[3 * t]] + be * zd[f->tri[3 * t + 1]] + ga * zd[f->tri[3 * t + 2]];
}

/* InterpolationScheme::computeEfieldSingleEmitter (interpolation_scheme.cpp:206-262) */
static void efield_ref32(const orc_field *f, float x, float y, float z, int *save, float out[3]) {
    const long double PI = 3.14159265358979323846264338328L;
    const float r0 = (float)f->r0, e0 = (float)f->e0;
    float phi = atanf(y / x);
    if (x < 0) phi = (float)((long double)phi + PI);
    if (x == 0 && y != 0)
        phi = (float)(PI / 2);
    else if (x == 0 && y == 0)
        phi = 0;
    x /= r0;
    y /= r0;
    z /= r0;
    float e[3] = {0, 0, 0};
    double coords[2];
    coords[0] = (double)sqrt((double)(x * x + y * y));
    coords[1] = (double)z;
    if (!(z < 0 || z > (float)f->zmax)) {
        double al, be, ga;
        int t = field_walk(f, coords, save, &al, &be, &ga);
        const double ri = t < 0 ? -1.0 : field_value(f, f->er, t, al, be, ga);
        t = field_walk(f, coords, save, &al, &be, &ga);
        const double zi = t < 0 ? -1.0 : field_value(f, f->ez, t, al, be, ga);
        e[0] = (float)ri;
        e[0] *= cosf(phi);
        e[1] = (float)ri;
        e[1] *= sinf(phi);
        e[2] = (float)zi;
    }
    for (int d = 0; d < 3; d++) out[d] = (float)((double)e[d] * (double)e0);
}

void orc_emitter_field_ref32(const orc_field *f, int n, const float *pos4, float *e3, int *save) {
    for (int i = 0; i < n; i++) efield_ref32(f, pos4[4 * i], pos4[4 * i + 1], pos4[4 * i + 2], save, &e3[3 * i]);
}

static void efield_f64(const orc_field *f, const double *x, double out[3]) {
    out[0] = out[1] = out[2] = 0.0;
    const double pz = x[2] / f->r0;
    if (pz < 0.0 || pz > f->zmax) return;
    const double rr = sqrt(x[0] * x[0] + x[1] * x[1]);
    const double p[2] = {rr / f->r0, pz};
    int t = -1;
    double al, be, ga;
    if (field_walk(f, p, &t, &al, &be, &ga) < 0) return;
    const double fr = field_value(f, f->er, t, al, be, ga), fz = field_value(f, f->ez, t, al, be, ga);
    double c = 1.0, sn = 0.0;
    if (x[0] == 0.0) {
        c = x[1] != 0.0 ? 0.0 : 1.0;
        sn = x[1] != 0.0 ? 1.0 : 0.0;
    } else {
        c = x[0] / rr;
        sn = x[1] / rr;
    }
    out[0] = f->e0 * fr * c;
    out[1] = f->e0 * fr * sn;
    out[2] = f->e0 * fz;
}

void orc_emitter_field_f64(const orc_field *f, int64_t n, const double *x3, double *e3) {
    for (int64_t i = 0; i < n; i++) efield_f64(f, &x3[3 * i], &e3[3 * i]);
}

/* ParticleSystem::propagatePositionNew (particles.cpp:33-40) for the charged
 * particles of [first, last), FP32: drift with the crash test
 * (particles.cpp:693-739), symmetry folding (particles.cpp:199-333; sym 1
 * rotational, 2 translational), boundary conditions (particles.cpp:73-177). */
static void drift_ref32(int first, int last, float *pos4, float *vel4, float *acc4, const float *t_inj,
                        float tstart, float dt, int sym, const float domain[3], const orc_boundary *bd,
                        orc_event *ev, int ev_cap, int *ev_count) {
    const float tend = tstart + dt;
    for (int i = first; i < last; i++) {
        float w = acc4[4 * i + 3];
        if (!(w == 1.0f || w == 2.0f)) continue;
        float *p = &pos4[4 * i];
        const float *v = &vel4[4 * i];
        const float ix = p[0], iy = p[1], iz = p[2];
        float s = clampf_dt(tend - t_inj[i], dt);
        p[0] += v[0] * s;
        p[1] += v[1] * s;
        p[2] += v[2] * s;
        float fz;
        if (bd && bd->crash && crash_ref32(bd, ix, iy, iz, p[0], p[1], p[2], &fz)) {
            acc4[4 * i + 3] = -1.0f;
            p[2] = fz;
            float temp_dt = (fz - iz) / v[2];
            p[0] = ix + temp_dt * v[0];
            p[1] = iy + temp_dt * v[1];
            push_event(ev, ev_cap, ev_count, tstart + temp_dt, p[0], p[1], p[2], v[0], v[1], v[2], i,
                       (uint32_t)(int)vel4[4 * i + 3], -1);
        }
    }
    if (sym == 1) {
        for (int i = first; i < last; i++) {
            float *p = &pos4[4 * i], *v = &vel4[4 * i];
            float tx, ty;
            if (p[0] < 0 && p[1] < 0) {
                p[0] = -p[0]; p[1] = -p[1]; v[0] = -v[0]; v[1] = -v[1];
            } else if (p[0] < 0) {
                tx = p[1]; ty = -p[0]; p[0] = tx; p[1] = ty;
                tx = v[1]; ty = -v[0]; v[0] = tx; v[1] = ty;
            } else if (p[1] < 0) {
                tx = -p[1]; ty = p[0]; p[0] = tx; p[1] = ty;
                tx = -v[1]; ty = v[0]; v[0] = tx; v[1] = ty;
            }
        }
    } else if (sym == 2 && bd) {
        for (int i = first; i < last; i++)
            for (int d = 0; d < 3; d++)
                if (bd->axes[d]) pos4[4 * i + d] = wrap_ref32(pos4[4 * i + d], domain[d]);
    }
    if (!bd) return;
    const float now = tstart + dt;
    if (bd->bc == 1 || bd->bc == 3) {
        const float X = (float)bd->bc_space[0], Y = (float)bd->bc_space[1], Z = (float)bd->bc_space[2],
                    W = (float)bd->bc_space[3];
        for (int i = first; i < last; i++) {
            if (acc4[4 * i + 3] != 1.0f) continue;
            const float x = pos4[4 * i], y = pos4[4 * i + 1], z = pos4[4 * i + 2];
            int out = (X != 0 && fabsf(x) > X) || (Y != 0 && fabsf(y) > Y) || (Z != 0 && fabsf(z) > Z) ||
                      (W != 0 && sqrtf(x * x + y * y) > W);
            if (out) {
                acc4[4 * i + 3] = 0.0f;
                push_event(ev, ev_cap, ev_count, now, x, y, z, vel4[4 * i], vel4[4 * i + 1], vel4[4 * i + 2], i,
                           (uint32_t)(int)vel4[4 * i + 3], 0);
            }
        }
    }
    if (bd->bc == 2 || bd->bc == 3) {
        const float T = (float)bd->bc_time;
        for (int i = first; i < last; i++) {
            if (acc4[4 * i + 3] != 1.0f) continue;
            if (now - t_inj[i] > T) {
                acc4[4 * i + 3] = 0.0f;
                push_event(ev, ev_cap, ev_count, now, pos4[4 * i], pos4[4 * i + 1], pos4[4 * i + 2], vel4[4 * i],
                           vel4[4 * i + 1], vel4[4 * i + 2], i, (uint32_t)(int)vel4[4 * i + 3], 0);
            }
        }
    }
}

/* ParticleSystem::resetFirstChargedParticle (particles.cpp:179-193) */
static int reset_first(int first, int last, const float *acc4) {
    for (int i = first; i < last; i++) {
        const float w = acc4[4 * i + 3];
        if (w == 2.0f || w == 1.0f) return i;
    }
    return first;
}

/* ---- energy bookkeeping, FP32 as the reference ------------------------ */

/* ParticleSystem::computeChargedKineticEnergy (particles.cpp:535-542):
 * ((0.5 * AMU) * getMass) * |v|^2, the mass a long double */
static float ke_ref32(const float *vel4, int i) {
    const float *v = vel4 + 4 * i;
    const float s = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    return (float)((long double)(0.5 * (double)REF_AMU) * species_mass_ld((int)v[3]) * (long double)s);
}

/* ParticleSystem::computeChargedElectricPotentialEnergy (particles.cpp:
 * 551-571): r^2 in float plus the softening in double, sqrt, q_i q_j / r
 * summed in float over [first, last) in index order */
static float pe_ref32(const float *pos4, int i, int first, int last, double eps) {
    const float ke = (float)(1 / (4.0 * REF_PI * REF_EPS0));
    const float q2 = REF_ELEM_CHARGE * REF_ELEM_CHARGE;
    const float *p = pos4 + 4 * i;
    float epe = 0;
    for (int j = first; j < last; j++) {
        if (j == i) continue;
        const float *o = pos4 + 4 * j;
        const float dx = p[0] - o[0], dy = p[1] - o[1], dz = p[2] - o[2];
        float r = (float)((double)(dx * dx + dy * dy + dz * dz) + eps);
        r = sqrtf(r);
        epe += p[3] * o[3] / r;
    }
    return epe * q2 * ke;
}

/* ParticleSystem::updateChargedFieldEnergy (particles.cpp:594-638): the work
 * of the field from init to the particle, first along z at init's (x, y),
 * then along (x, y) at the particle's z, steps left-point samples each */
static void fe_update_ref32(const orc_field *f, int *save, const float *pos4, int i, int steps, const float init[3],
                            float *fe) {
    if (!f) return;
    const float *p = pos4 + 4 * i;
    const double dx = (double)(p[0] - init[0]), dy = (double)(p[1] - init[1]), dz = (double)(p[2] - init[2]);
    const double px = init[0], py = init[1];
    double pz = init[2];
    double tz = 0, tr = 0;
    float e[3];
    for (int k = 0; k < steps; k++) {
        efield_ref32(f, (float)px, (float)py, (float)(pz + k * dz / steps), save, e);
        tz += e[2] * dz / steps;
    }
    pz += dz;
    for (int k = 0; k < steps; k++) {
        efield_ref32(f, (float)(px + k * dx / steps), (float)(py + k * dy / steps), (float)pz, save, e);
        tr += e[0] * dx / steps + e[1] * dy / steps;
    }
    double t = tz + tr;
    t *= (double)(-REF_ELEM_CHARGE * p[3]);
    fe[i] = (float)((double)fe[i] + t);
}

typedef struct {
    float *fe, *ke_inj, *init;   /* per particle; init: 3 per particle */
    float KE_inj, PE_inj, FE_inj;
    int prev;                    /* the integrator's tempLastParticlePrev */
} energy_state;

/* Integrator::initializeEnergyData (integration_schemes.cpp:757-775) at the
 * state before the first step; the reference position is (0, 0, 140 r0)
 * (InterpolationScheme::setReferencePosition, interpolation_scheme.cpp:38-47) */
static void energy_init_ref32(energy_state *E, int n, const float *pos4, const float *vel4, const orc_field *f,
                              int *save, int steps) {
    const float ref[3] = {0.0f, 0.0f, f ? 140 * (float)f->r0 : 0.0f};
    for (int i = 0; i < n; i++) {
        E->fe[i] = 0;
        fe_update_ref32(f, save, pos4, i, steps, ref, E->fe);
        E->ke_inj[i] = ke_ref32(vel4, i);
        for (int d = 0; d < 3; d++) E->init[3 * i + d] = pos4[4 * i + d];
    }
    E->KE_inj = E->PE_inj = E->FE_inj = 0;
    E->prev = 0;
}

/* Integrator::updateEnergyInjectionData (integration_schemes.cpp:783-793),
 * called by driftNew after it set lastParticle, before the drift */
static void energy_inject_ref32(energy_state *E, const float *pos4, int first, int last, double eps) {
    for (int i = E->prev; i < last; i++) {
        E->KE_inj += E->ke_inj[i];
        E->PE_inj += pe_ref32(pos4, i, first, last, eps);
        E->FE_inj += E->fe[i];
    }
    E->prev = last;
}

/* Integrator::updateEnergyIntervalData (integration_schemes.cpp:799-835) */
static void energy_interval_ref32(energy_state *E, orc_energy *en, const float *pos4, const float *vel4,
                                  const float *t_inj, int first, int last, float tpos, float dt,
                                  const orc_field *f, int *save, double eps) {
    float KE = 0, PE = 0, FE = 0;
    for (int i = first; i < last; i++) {
        const float tt = fminf(dt * en->interval, tpos - t_inj[i]);
        const int fe_steps = (int)fmaxf(tt * en->steps / dt, 2.0f);
        fe_update_ref32(f, save, pos4, i, fe_steps, &E->init[3 * i], E->fe);
        for (int d = 0; d < 3; d++) E->init[3 * i + d] = pos4[4 * i + d];
        KE += ke_ref32(vel4, i);
        PE += pe_ref32(pos4, i, first, last, eps);
        FE += E->fe[i];
    }
    PE /= 2;
    if (en->rec && en->rec_count < en->rec_cap) {
        float *r = en->rec + 6 * en->rec_count;
        r[0] = E->KE_inj; r[1] = E->PE_inj; r[2] = E->FE_inj;
        r[3] = KE; r[4] = PE; r[5] = FE;
    }
    en->rec_count++;
}

static void leapfrog_ref32_impl(int n, float *pos4, float *vel4, float *acc4,
                                const float *t_inj, int nsteps, float dt, double eps,
                                const float efield[3], int sym, int nimg,
                                const int *images, const float domain_size[3],
                                const orc_boundary *bd, const orc_field *field,
                                orc_event *ev, int ev_cap, int *ev_count, orc_energy *en,
                                int nthreads) {
    /* LeapfrogDKD::runSimulation (integration_schemes.cpp:856-891):
     * driftNew(dt/2), kick(dt), driftNew(dt/2) per step; driftNew
     * (integration_schemes.cpp:705-723) sets lastParticle from the injection
     * times, drifts, then moves firstParticle past inactive particles. */
    const float factor = REF_ELEM_CHARGE / REF_AMU;
    int first = 0, last = 0, cnt = 0, save = -1;
    energy_state E = {0};
    if (en) {
        E.fe = (float *)malloc(sizeof(float) * (size_t)n);
        E.ke_inj = (float *)malloc(sizeof(float) * (size_t)n);
        E.init = (float *)malloc(sizeof(float) * 3 * (size_t)n);
        energy_init_ref32(&E, n, pos4, vel4, field, &save, en->init_steps);
        en->rec_count = 0;
    }
    for (int it = 1; it <= nsteps; it++) {
        float tpos = dt * (float)(it - 1);
        float tvel = dt * (float)(it - 1);
        last = most_recent_injected(n, t_inj, tpos + dt / 2) + 1;
        if (en) energy_inject_ref32(&E, pos4, first, last, eps);
        drift_ref32(first, last, pos4, vel4, acc4, t_inj, tpos, dt / 2, sym, domain_size, bd, ev, ev_cap, &cnt);
        first = reset_first(first, last, acc4);
        tpos += dt / 2;
        /* kick: zeroAcceleration (particles.cpp:1031-1044) + force */
        for (int i = first; i < last; i++)
            if (acc4[4 * i + 3] == 1.0f) acc4[4 * i] = acc4[4 * i + 1] = acc4[4 * i + 2] = 0.0f;
        if (sym == 0)
            orc_direct_ref32(pos4, vel4, acc4, first, last, first, last, eps, nthreads);
        else if (sym == 1)
            orc_direct_rot4_ref32(pos4, vel4, acc4, first, last, first, last, eps, nthreads);
        else
            orc_direct_trans_ref32(pos4, vel4, acc4, first, last, first, last, eps, nimg, images,
                                   domain_size, nthreads);
        /* computeBackgroundAcceleration with a uniform field
         * (particles.cpp:496-520): Efactor in float, E*Efactor per axis. */
        for (int i = first; i < last; i++) {
            if (acc4[4 * i + 3] != 1.0f) continue;
            long double m = species_mass_ld((int)vel4[4 * i + 3]);
            float ef = (float)((double)factor * (double)pos4[4 * i + 3] / m);
            float ev3[3] = {efield[0], efield[1], efield[2]};
            if (field) efield_ref32(field, pos4[4 * i], pos4[4 * i + 1], pos4[4 * i + 2], &save, ev3);
            for (int d = 0; d < 3; d++) {
                float e = (float)((double)ev3[d] * (double)ef);
                acc4[4 * i + d] += e;
            }
        }
        /* propagateVelocityNew (particles.cpp:763-786) */
        {
            const float tend = tvel + dt;
            for (int i = first; i < last; i++) {
                if (acc4[4 * i + 3] != 1.0f) continue;
                float s = clampf_dt(tend - t_inj[i], dt);
                vel4[4 * i + 0] += acc4[4 * i + 0] * s;
                vel4[4 * i + 1] += acc4[4 * i + 1] * s;
                vel4[4 * i + 2] += acc4[4 * i + 2] * s;
            }
        }
        last = most_recent_injected(n, t_inj, tpos + dt / 2) + 1;
        if (en) energy_inject_ref32(&E, pos4, first, last, eps);
        drift_ref32(first, last, pos4, vel4, acc4, t_inj, tpos, dt / 2, sym, domain_size, bd, ev, ev_cap, &cnt);
        first = reset_first(first, last, acc4);
        /* Integrator::finishIter (integration_schemes.cpp:584-601) */
        if (en && it % en->interval == 0)
            energy_interval_ref32(&E, en, pos4, vel4, t_inj, first, last, tpos + dt / 2, dt, field, &save, eps);
    }
    if (ev_count) *ev_count = cnt;
    free(E.fe);
    free(E.ke_inj);
    free(E.init);
}

void orc_leapfrog_ref32_bc(int n, float *pos4, float *vel4, float *acc4,
                           const float *t_inj, int nsteps, float dt, double eps,
                           const float efield[3], int sym, int nimg,
                           const int *images, const float domain_size[3],
                           const orc_boundary *bd, const orc_field *field,
                           orc_event *ev, int ev_cap, int *ev_count, int nthreads) {
    leapfrog_ref32_impl(n, pos4, vel4, acc4, t_inj, nsteps, dt, eps, efield, sym, nimg, images, domain_size, bd,
                        field, ev, ev_cap, ev_count, NULL, nthreads);
}

void orc_leapfrog_ref32_energy(int n, float *pos4, float *vel4, float *acc4,
                               const float *t_inj, int nsteps, float dt, double eps,
                               const float efield[3], const orc_boundary *bd,
                               const orc_field *field, orc_energy *en, int nthreads) {
    const float dom[3] = {0, 0, 0};
    if (!en || en->interval < 1) return;
    leapfrog_ref32_impl(n, pos4, vel4, acc4, t_inj, nsteps, dt, eps, efield, 0, 0, NULL, dom, bd, field, NULL, 0,
                        NULL, en, nthreads);
}


void orc_leapfrog_ref32(int n, float *pos4, float *vel4, float *acc4,
                        const float *t_inj, int nsteps, float dt, double eps,
                        const float efield[3], int sym, int nimg,
                        const int *images, const float domain_size[3],
                        int nthreads) {
    orc_leapfrog_ref32_bc(n, pos4, vel4, acc4, t_inj, nsteps, dt, eps, efield, sym, nimg, images, domain_size,
                          NULL, NULL, NULL, 0, NULL, nthreads);
}

/* ---- multi-rate leapfrog (LeapfrogDKDSubsteps) -------------------------- */

typedef struct {
    int type;
    float t, s[4];
} ref_bc;

static void bc_most_stringent(ref_bc *b) {
    /* BoundaryConditionParameters::setMostStringentBoundaryConditionType (structures.h:309-326) */
    if (b->type == 0) {
        b->t = 0.0f;
        for (int k = 0; k < 4; k++) b->s[k] = 0.0f;
    } else if (b->type == 1) {
        b->t = 0.0f;
    } else if (b->type == 2) {
        for (int k = 0; k < 4; k++) b->s[k] = 0.0f;
    }
    b->type = 3;
}

static void bc_choose_min(ref_bc *a, const ref_bc *b) {
    /* chooseMinimumBoundaryConditionParameters (structures.h:328-363) */
    a->t = (a->t == 0 && b->t == 0) ? 0.0f : ref_minf(a->t, b->t);
    for (int k = 0; k < 4; k++) a->s[k] = (a->s[k] == 0 && b->s[k] == 0) ? 0.0f : ref_minf(a->s[k], b->s[k]);
}

static void bc_choose_max(ref_bc *a, const ref_bc *b) {
    /* chooseMaximumBoundaryConditionParameters (structures.h:365-400) */
    a->t = (a->t == 0 || b->t == 0) ? 0.0f : ref_maxf(a->t, b->t);
    for (int k = 0; k < 4; k++) a->s[k] = (a->s[k] == 0 || b->s[k] == 0) ? 0.0f : ref_maxf(a->s[k], b->s[k]);
}

#define ORC_MAX_LEVELS 16

typedef struct {
    int L;
    float dt[ORC_MAX_LEVELS];
    ref_bc bc[ORC_MAX_LEVELS];
} sub_table;

static int cmp_substep(const void *a, const void *b) {
    const float x = ((const orc_substep *)a)->dt, y = ((const orc_substep *)b)->dt;
    return (x > y) - (x < y);
}

/* LeapfrogDKDSubsteps::setSubstepTimes (integration_schemes.cpp:1361-1412) */
static int resolve_substeps(float step, int nsub, const orc_substep *subs_in, sub_table *T) {
    orc_substep *in = (orc_substep *)malloc(sizeof(orc_substep) * (size_t)nsub);
    memcpy(in, subs_in, sizeof(orc_substep) * (size_t)nsub);
    qsort(in, (size_t)nsub, sizeof(orc_substep), cmp_substep);
    float temp_dt = step;
    int L = 0;
    while (temp_dt > in[0].dt) {
        temp_dt /= 3.0;
        L++;
    }
    if (L >= ORC_MAX_LEVELS) {
        free(in);
        return -1;
    }
    memset(T, 0, sizeof(*T));
    T->L = L;
    if (L != 0) {
        T->dt[L] = in[0].dt;
        T->bc[L].type = in[0].bc;
        T->bc[L].t = in[0].t;
        for (int k = 0; k < 4; k++) T->bc[L].s[k] = in[0].s[k];
    }
    for (int i = 0; i <= L; i++) bc_most_stringent(&T->bc[i]);
    for (int i = 1; i < nsub; i++) {
        int ind = 0;
        temp_dt = step;
        while (temp_dt > in[i].dt) {
            temp_dt /= 3.0;
            ind++;
        }
        ref_bc b;
        b.type = in[i].bc;
        b.t = in[i].t;
        for (int k = 0; k < 4; k++) b.s[k] = in[i].s[k];
        if (T->dt[ind] == 0) {
            T->dt[ind] = temp_dt;
            if (ind != 0) T->bc[ind] = b;
        } else {
            bc_choose_min(&T->bc[ind], &b);
        }
    }
    T->dt[0] = step;
    for (int i = 1; i <= L; i++) T->dt[i] = (float)(T->dt[i - 1] / 3.0);
    for (int i = L - 1; i >= 0; i--) bc_choose_max(&T->bc[i], &T->bc[i + 1]);
    free(in);
    return 0;
}

/* the scan of checkSpatialConditions / checkTemporalConditions
 * (integration_schemes.cpp:956-1094) for one coordinate (comp 0..3: |x|, |y|,
 * |z|, r; comp 4: time since injection) */
static int scan_levels_ref32(const sub_table *T, int level, float value, int comp) {
    int possible = -1;
    float boundary = 0.0f;
    for (int i = T->L; i >= level; i--) {
        const float lim = comp < 4 ? T->bc[i].s[comp] : T->bc[i].t;
        if (possible == -1) {
            const int in = comp < 4 ? (fabsf(value) < lim || lim == 0) : (value < lim || lim == 0);
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

typedef struct {
    int n, first, last, nthreads, sym;
    float *pos4, *vel4, *acc4;
    const float *t_inj;
    const float *efield;
    const float *domain;
    const orc_boundary *bd;
    double eps;
    float t_pos, t_vel;
    const sub_table *T;
    int *lev;
    int ev_count;
} sub_run;

static void sub_crossover(sub_run *r, int level) {
    /* crossoverParticles / checkConditions (integration_schemes.cpp:932-1111) */
    const sub_table *T = r->T;
    for (int i = r->first; i < r->last; i++) {
        if (r->lev[i] != level && r->lev[i] != level + 1) continue;
        const int type = T->bc[level + 1].type;
        const float *p = &r->pos4[4 * i];
        const float w = sqrtf(p[0] * p[0] + p[1] * p[1]);
        const float ts = r->t_pos - r->t_inj[i];
        int out = r->lev[i], sp = 0;
        if (type == 1 || type == 3) {
            sp = scan_levels_ref32(T, level, p[0], 0);
            int q = scan_levels_ref32(T, level, p[1], 1);
            sp = sp > q ? sp : q;
            q = scan_levels_ref32(T, level, p[2], 2);
            sp = sp > q ? sp : q;
            q = scan_levels_ref32(T, level, w, 3);
            sp = sp > q ? sp : q;
            out = sp;
        }
        if (type == 2) out = scan_levels_ref32(T, level, ts, 4);
        if (type == 3) {
            const int q = scan_levels_ref32(T, level, ts, 4);
            out = q > sp ? q : sp;
        }
        r->lev[i] = out < 0 ? level : out;
    }
}

static void sub_drift(sub_run *r, int level, int toggle);

static void sub_kick(sub_run *r, int level, int top) {
    const sub_table *T = r->T;
    if (level != T->L) {
        sub_drift(r, level + 1, 0);
        sub_kick(r, level + 1, top);
        sub_drift(r, level + 1, 1);
        return;
    }
    /* setParticleStatus (integration_schemes.cpp:1216-1236) */
    for (int i = r->first; i < r->last; i++) {
        float *w = &r->acc4[4 * i + 3];
        if (*w != 0.0f && *w != -1.0f) {
            if (r->lev[i] <= level && r->lev[i] >= top)
                *w = 1.0f;
            else if (r->lev[i] < top)
                *w = 2.0f;
        }
    }
    /* updateAcceleration / updateAccelerationSubsteps: zeroAcceleration + force */
    for (int i = r->first; i < r->last; i++)
        if (r->acc4[4 * i + 3] == 1.0f) r->acc4[4 * i] = r->acc4[4 * i + 1] = r->acc4[4 * i + 2] = 0.0f;
    orc_direct_ref32(r->pos4, r->vel4, r->acc4, r->first, r->last, r->first, r->last, r->eps, r->nthreads);
    /* computeBackgroundAcceleration with a uniform field */
    const float factor = REF_ELEM_CHARGE / REF_AMU;
    for (int i = r->first; i < r->last; i++) {
        if (r->acc4[4 * i + 3] != 1.0f) continue;
        long double m = species_mass_ld((int)r->vel4[4 * i + 3]);
        float ef = (float)((double)factor * (double)r->pos4[4 * i + 3] / m);
        for (int d = 0; d < 3; d++) r->acc4[4 * i + d] += (float)((double)r->efield[d] * (double)ef);
    }
    /* variableTimestepKick (integration_schemes.cpp:1241-1262) */
    float tend[ORC_MAX_LEVELS];
    for (int l = 0; l <= T->L; l++) tend[l] = r->t_vel + T->dt[l];
    for (int i = r->first; i < r->last; i++) {
        if (r->acc4[4 * i + 3] != 1.0f) continue;
        const int l = r->lev[i];
        const float temp_dt = T->dt[l];
        const float s = clampf_dt(tend[l] - r->t_inj[i], temp_dt);
        for (int d = 0; d < 3; d++) r->vel4[4 * i + d] += r->acc4[4 * i + d] * s;
    }
    r->t_vel += T->dt[T->L];
}

static void sub_drift(sub_run *r, int level, int toggle) {
    const sub_table *T = r->T;
    if (level != T->L) {
        sub_drift(r, level + 1, 0);
        sub_kick(r, level + 1, level + 1);
        sub_drift(r, level + 1, 1);
        if (toggle) sub_crossover(r, level);
        return;
    }
    /* LeapfrogDKDSubsteps::driftNew at the finest level (integration_schemes.cpp:1162-1201) */
    const float h = T->dt[T->L] / 2;
    r->last = most_recent_injected(r->n, r->t_inj, r->t_pos + h) + 1;
    drift_ref32(r->first, r->last, r->pos4, r->vel4, r->acc4, r->t_inj, r->t_pos, h, r->sym, r->domain, r->bd,
                NULL, 0, &r->ev_count);
    r->first = reset_first(r->first, r->last, r->acc4);
    r->t_pos += h;
}

void orc_leapfrog_substeps_ref32(int n, float *pos4, float *vel4, float *acc4,
                                 const float *t_inj, int nsteps, float dt, double eps,
                                 const float efield[3], int sym, int nsub,
                                 const orc_substep *subs, const orc_boundary *bd,
                                 int8_t *levels_out, int nthreads) {
    sub_table T;
    if (resolve_substeps(dt, nsub, subs, &T) != 0) return;
    int *lev = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    for (int i = 0; i < n; i++) lev[i] = T.L;  /* initializeParticleLevels */
    const float dom0[3] = {0, 0, 0};
    sub_run r;
    memset(&r, 0, sizeof(r));
    r.n = n;
    r.nthreads = nthreads;
    r.sym = sym;
    r.pos4 = pos4;
    r.vel4 = vel4;
    r.acc4 = acc4;
    r.t_inj = t_inj;
    r.efield = efield;
    r.domain = bd ? NULL : dom0;
    r.bd = bd;
    r.eps = eps;
    r.T = &T;
    r.lev = lev;
    float dom[3] = {0, 0, 0};
    if (bd)
        for (int d = 0; d < 3; d++) dom[d] = (float)bd->domain[d];
    r.domain = dom;
    for (int it = 1; it <= nsteps; it++) {
        r.t_pos = dt * (float)(it - 1);
        r.t_vel = dt * (float)(it - 1);
        sub_drift(&r, 0, 0);
        sub_kick(&r, 0, 0);
        sub_drift(&r, 0, 1);
    }
    if (levels_out)
        for (int i = 0; i < n; i++) levels_out[i] = (int8_t)lev[i];
    free(lev);
}

static uint32_t species_of_mass(double m) {
    for (int k = 0; k < 8; k++)
        if (k != 3 && m == (double)species_mass_ld(k)) return (uint32_t)k;
    return 0xffffffffu;
}

/* Events of one drift in the reference's file order: crashes (drift loop),
 * then spatial, then temporal boundary hits, each in index order. */
static void drift_f64(int64_t n, double *x, double *v, const double *m, int32_t *status, const double *t_inj,
                      double t_start, double h, const orc_boundary *bd, orc_event *ev, int ev_cap, int *cnt) {
    const double T = t_start + h;
    int fold = bd ? bd->fold : 0;
    for (int64_t i = 0; i < n; i++) {
        if (!(t_inj[i] <= T)) continue;
        if (!(status[i] == 1 || status[i] == 2)) continue;
        double *p = &x[3 * i];
        const double *u = &v[3 * i];
        const double ix = p[0], iy = p[1], iz = p[2];
        double s = T - t_inj[i];
        s = s < 0 ? 0 : (s > h ? h : s);
        for (int d = 0; d < 3; d++) p[d] += u[d] * s;
        double zc;
        if (bd && bd->crash && crash_f64(bd, ix, iy, iz, p[0], p[1], p[2], &zc)) {
            status[i] = -1;
            p[2] = zc;
            const double td = (zc - iz) / u[2];
            p[0] = ix + td * u[0];
            p[1] = iy + td * u[1];
            push_event(ev, ev_cap, cnt, (float)(t_start + td), (float)p[0], (float)p[1], (float)p[2], (float)u[0],
                       (float)u[1], (float)u[2], (int)i, species_of_mass(m[i]), -1);
        }
    }
    for (int64_t i = 0; i < n && fold; i++) {
        if (!(t_inj[i] <= T)) continue;
        double *p = &x[3 * i], *u = &v[3 * i];
        if (fold == 1) {
            double tx, ty;
            if (p[0] < 0 && p[1] < 0) {
                p[0] = -p[0]; p[1] = -p[1]; u[0] = -u[0]; u[1] = -u[1];
            } else if (p[0] < 0) {
                tx = p[1]; ty = -p[0]; p[0] = tx; p[1] = ty;
                tx = u[1]; ty = -u[0]; u[0] = tx; u[1] = ty;
            } else if (p[1] < 0) {
                tx = -p[1]; ty = p[0]; p[0] = tx; p[1] = ty;
                tx = -u[1]; ty = u[0]; u[0] = tx; u[1] = ty;
            }
        } else {
            for (int d = 0; d < 3; d++)
                if (bd->axes[d]) p[d] = wrap_f64(p[d], bd->domain[d]);
        }
    }
    if (!bd) return;
    for (int pass = 0; pass < 2; pass++) {
        if (pass == 0 && !(bd->bc == 1 || bd->bc == 3)) continue;
        if (pass == 1 && !(bd->bc == 2 || bd->bc == 3)) continue;
        for (int64_t i = 0; i < n; i++) {
            if (!(t_inj[i] <= T) || status[i] != 1) continue;
            const double *p = &x[3 * i];
            int out;
            if (pass == 0)
                out = (bd->bc_space[0] != 0 && fabs(p[0]) > bd->bc_space[0]) ||
                      (bd->bc_space[1] != 0 && fabs(p[1]) > bd->bc_space[1]) ||
                      (bd->bc_space[2] != 0 && fabs(p[2]) > bd->bc_space[2]) ||
                      (bd->bc_space[3] != 0 && sqrt(p[0] * p[0] + p[1] * p[1]) > bd->bc_space[3]);
            else
                out = T - t_inj[i] > bd->bc_time;
            if (out) {
                status[i] = 0;
                push_event(ev, ev_cap, cnt, (float)T, (float)p[0], (float)p[1], (float)p[2], (float)v[3 * i],
                           (float)v[3 * i + 1], (float)v[3 * i + 2], (int)i, species_of_mass(m[i]), 0);
            }
        }
    }
}

static void leapfrog_f64(int64_t n, double *x, double *v, const double *q, const double *m, int32_t *status,
                         const double *t_inj, int nsteps, double dt, double t0, double eps2, double kconst,
                         const double efield[3], int sym, int nimg, const double *img_off, const orc_boundary *bd,
                         const orc_field *field, orc_event *ev, int ev_cap, int *ev_count, double *a_out,
                         int nthreads) {
    double *a = (double *)malloc(sizeof(double) * 3 * (size_t)(n > 0 ? n : 1));
    int32_t *win = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    const double eoa = orc_e_over_amu();
    const double h = 0.5 * dt;
    int cnt = 0;
    for (int it = 0; it < nsteps; it++) {
        const double ts = t0 + dt * it;
        drift_f64(n, x, v, m, status, t_inj, ts, h, bd, ev, ev_cap, &cnt);
        /* force and kick over the particles injected by the mid time */
        for (int64_t i = 0; i < n; i++) win[i] = t_inj[i] <= ts + h ? status[i] : 0;
        orc_direct_f64(n, x, q, m, win, NULL, 0, eps2, kconst, sym, nimg, img_off, a, nthreads);
        for (int64_t i = 0; i < n; i++) {
            if (win[i] != 1) continue;
            const double ef = eoa * q[i] / m[i];
            double s = ts + dt - t_inj[i];
            s = s < 0 ? 0 : (s > dt ? dt : s);
            double e3[3] = {0.0, 0.0, 0.0};
            if (field) efield_f64(field, &x[3 * i], e3);
            for (int d = 0; d < 3; d++) {
                a[3 * i + d] += (efield[d] + e3[d]) * ef;
                v[3 * i + d] += a[3 * i + d] * s;
            }
        }
        drift_f64(n, x, v, m, status, t_inj, ts + h, h, bd, ev, ev_cap, &cnt);
    }
    if (a_out) memcpy(a_out, a, sizeof(double) * 3 * (size_t)n);
    free(a);
    free(win);
    if (ev_count) *ev_count = cnt;
}

void orc_leapfrog_f64_bc(int64_t n, double *x, double *v, const double *q,
                         const double *m, int32_t *status, const double *t_inj,
                         int nsteps, double dt, double t0, double eps2,
                         double kconst, const double efield[3], int sym, int nimg,
                         const double *img_off, const orc_boundary *bd,
                         const orc_field *field, orc_event *ev, int ev_cap,
                         int *ev_count, int nthreads) {
    leapfrog_f64(n, x, v, q, m, status, t_inj, nsteps, dt, t0, eps2, kconst, efield, sym, nimg, img_off, bd,
                 field, ev, ev_cap, ev_count, NULL, nthreads);
}

void orc_leapfrog_f64(int64_t n, double *x, double *v, const double *q,
                      const double *m, int32_t *status, const double *t_inj,
                      int nsteps, double dt, double t0, double eps2,
                      double kconst, const double efield[3], int sym, int nimg,
                      const double *img_off, double *a_out, int nthreads) {
    leapfrog_f64(n, x, v, q, m, status, t_inj, nsteps, dt, t0, eps2, kconst, efield, sym, nimg, img_off, NULL,
                 NULL, NULL, 0, NULL, a_out, nthreads);
}

/* ---- energy ------------------------------------------------------------ */

void orc_energy_f64(int64_t n, const double *x, const double *v,
                    const double *q, const double *m, double eps2,
                    double *ke, double *pe, int nthreads) {
    /* computeChargedKineticEnergy / computeChargedElectricPotentialEnergy
     * (particles.cpp:535-578) and the halving in updateEnergyIntervalData
     * (integration_schemes.cpp:815). */
    const int nt = nthreads_or_default(nthreads);
    const double amu = orc_amu(), e = orc_elem_charge(), kc = orc_coulomb_ke();
    double k_sum = 0, p_sum = 0;
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : k_sum, p_sum) num_threads(nt)
    for (int64_t i = 0; i < n; i++) {
        const double v2 = v[3 * i] * v[3 * i] + v[3 * i + 1] * v[3 * i + 1] + v[3 * i + 2] * v[3 * i + 2];
        k_sum += 0.5 * amu * m[i] * v2;
        double s = 0;
        for (int64_t j = 0; j < n; j++) {
            if (j == i) continue;
            double dx = x[3 * i] - x[3 * j], dy = x[3 * i + 1] - x[3 * j + 1],
                   dz = x[3 * i + 2] - x[3 * j + 2];
            s += q[i] * q[j] / sqrt(dx * dx + dy * dy + dz * dz + eps2);
        }
        p_sum += s;
    }
    *ke = k_sum;
    *pe = 0.5 * p_sum * e * e * kc;
}

/* ---- accuracy metric --------------------------------------------------- */

void orc_rel_l2(int64_t n, const double *a, const double *r,
                const int32_t *status, double *l2, double *maxl2,
                int64_t *argmax, double *global_l2) {
    double s = 0, mx = 0, num = 0, den = 0;
    int64_t cnt = 0, arg = 0;
    for (int64_t k = 0; k < n; k++) {
        if (status && status[k] != 1) continue;
        cnt++;
        double d = 0, nr = 0;
        for (int c = 0; c < 3; c++) {
            double e = a[3 * k + c] - r[3 * k + c];
            d += e * e;
            nr += r[3 * k + c] * r[3 * k + c];
        }
        num += d;
        den += nr;
        double ratio = (nr == 0 && d == 0) ? 0.0 : d / nr;
        s += ratio;
        if (ratio > mx) { mx = ratio; arg = k; }
    }
    *l2 = cnt ? sqrt(s / (double)cnt) : 0.0;
    *maxl2 = sqrt(mx);
    *argmax = arg;
    *global_l2 = den > 0 ? sqrt(num / den) : 0.0;
}

/* ------------------------------------------------------------- outliers -- */
static int cmp_float(const void *a, const void *b) {
    const float x = *(const float *)a, y = *(const float *)b;
    return (x > y) - (x < y);
}

/* findTrueMedian (outlier_detection.h:117-133) by sorting a copy */
static float true_median(float *v, int64_t n) {
    if (n <= 0) return 0.0f;
    qsort(v, (size_t)n, sizeof(float), cmp_float);
    if (n & 1) return v[n / 2];
    return (v[(n - 1) / 2] + v[n / 2]) / 2;
}

int64_t orc_outliers(int64_t n, const double *x3, const int32_t *status, int32_t *flags) {
    const float factor = 1.482602218505602f; /* domain_bounds_functions.h:37 */
    const float max_dev = 3.0f;              /* domain_bounds_functions.h:38 */
    float *pos[3], *dev[3], *tmp = (float *)malloc(sizeof(float) * (size_t)(n > 0 ? n : 1));
    float med[3], mad[3];
    int64_t nv = 0, nout = 0;
    for (int d = 0; d < 3; d++) {
        pos[d] = (float *)malloc(sizeof(float) * (size_t)(n > 0 ? n : 1));
        dev[d] = (float *)malloc(sizeof(float) * (size_t)(n > 0 ? n : 1));
    }
    for (int64_t i = 0; i < n; i++)
        if (status[i] == 1 || status[i] == 2) {
            for (int d = 0; d < 3; d++) pos[d][nv] = (float)x3[3 * i + d];
            nv++;
        }
    for (int d = 0; d < 3; d++) {
        memcpy(tmp, pos[d], sizeof(float) * (size_t)nv);
        med[d] = true_median(tmp, nv);
        for (int64_t k = 0; k < nv; k++) dev[d][k] = fabsf(pos[d][k] - med[d]);
        memcpy(tmp, dev[d], sizeof(float) * (size_t)nv);
        mad[d] = factor * true_median(tmp, nv);
    }
    int64_t k = 0;
    for (int64_t i = 0; i < n; i++) {
        if (!(status[i] == 1 || status[i] == 2)) {
            flags[i] = -1;
            continue;
        }
        int out = 0;
        for (int d = 0; d < 3; d++) out |= (dev[d][k] / mad[d]) >= max_dev;
        flags[i] = out;
        nout += out;
        k++;
    }
    for (int d = 0; d < 3; d++) {
        free(pos[d]);
        free(dev[d]);
    }
    free(tmp);
    return nout;
}
