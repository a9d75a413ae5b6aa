// fmm_tables.cpp -- host precompute of the FMM translation tables.
//
// Plays the role of MultipoleMethodConstants::precalc
// (multipole_method_constants.cpp:40-226: factorials, Anm, Ynm at theta = 0,
// Wigner rotation matrices Dnm for the primitive directions).  Conventions:
//   Y_n^m(t, f) = sqrt((n-|m|)!/(n+|m|)!) P_n^|m|(cos t) e^{imf}, P without
//   the Condon-Shortley phase;  multipole M_n^m = sum q r^n Y_n^-m,
//   potential sum M_n^m Y_n^m / r^{n+1};  local potential sum L_j^k Y_j^k r^j.
// An M2L from a source box to a target box at offset d (target - source, in
// box units) is done as: phase e^{imf}, rotation about y by -theta (d -> +z),
// translation along z, rotation about y by +theta, phase e^{-imf}.  The two
// y-rotation matrices of every polar angle are computed by exact quadrature on
// the sphere (Gauss-Legendre x trapezoid), so no sign convention of a Wigner
// formula has to be matched.
#include "fmm_tables.h"

#include <cmath>
#include <complex>
#include <map>
#include <vector>

namespace sv {
namespace {

using cd = std::complex<double>;

double fact(int n) {
    double f = 1.0;
    for (int k = 2; k <= n; k++) f *= k;
    return f;
}

// associated Legendre P_n^m(x), m >= 0, no Condon-Shortley phase, n < p
void legendre(int p, double x, std::vector<double> &P) {
    P.assign(p * p, 0.0);
    const double s = std::sqrt(std::max(0.0, (1 - x) * (1 + x)));
    double pmm = 1.0;
    for (int m = 0; m < p; m++) {
        if (m > 0) pmm *= (2 * m - 1) * s;
        P[m * p + m] = pmm;
        if (m + 1 < p) P[(m + 1) * p + m] = x * (2 * m + 1) * pmm;
        for (int n = m + 2; n < p; n++)
            P[n * p + m] = ((2 * n - 1) * x * P[(n - 1) * p + m] - (n + m - 1) * P[(n - 2) * p + m]) / (n - m);
    }
}

cd ynm(int n, int m, const std::vector<double> &P, int p, double phi) {
    const int am = std::abs(m);
    const double nrm = std::sqrt(fact(n - am) / fact(n + am));
    return nrm * P[n * p + am] * std::polar(1.0, m * phi);
}

void gauss_legendre(int n, std::vector<double> &x, std::vector<double> &w) {
    x.resize(n);
    w.resize(n);
    for (int i = 0; i < n; i++) {
        double z = std::cos(M_PI * (i + 0.75) / (n + 0.5));
        for (int it = 0; it < 100; it++) {
            double p1 = 1, p2 = 0;
            for (int k = 1; k <= n; k++) {
                double p3 = p2;
                p2 = p1;
                p1 = ((2 * k - 1) * z * p2 - (k - 1) * p3) / k;
            }
            double pp = n * (z * p1 - p2) / (z * z - 1);
            double dz = p1 / pp;
            z -= dz;
            if (std::fabs(dz) < 1e-15) break;
        }
        double p1 = 1, p2 = 0;
        for (int k = 1; k <= n; k++) {
            double p3 = p2;
            p2 = p1;
            p1 = ((2 * k - 1) * z * p2 - (k - 1) * p3) / k;
        }
        double pp = n * (z * p1 - p2) / (z * z - 1);
        x[i] = z;
        w[i] = 2 / ((1 - z * z) * pp * pp);
    }
}

// G[n][(mp+n)*(2n+1) + (m+n)] for f(u) -> f(Ry(a) u')
std::vector<std::vector<cd>> yrot(int p, double a, double *max_imag) {
    std::vector<double> gx, gw;
    gauss_legendre(p + 1, gx, gw);
    const int nph = 2 * p + 1;
    std::vector<std::vector<cd>> G(p);
    for (int n = 0; n < p; n++) G[n].assign((2 * n + 1) * (2 * n + 1), cd(0, 0));
    std::vector<double> P0, P1;
    const double ca = std::cos(a), sa = std::sin(a);
    for (size_t it = 0; it < gx.size(); it++) {
        const double ct = gx[it], st = std::sqrt(std::max(0.0, 1 - ct * ct));
        legendre(p, ct, P0);
        for (int ip = 0; ip < nph; ip++) {
            const double ph = 2 * M_PI * ip / nph;
            const double w = gw[it] * 2 * M_PI / nph;
            const double ux = st * std::cos(ph), uy = st * std::sin(ph), uz = ct;
            // v = Ry(a) u
            const double vx = ca * ux + sa * uz, vy = uy, vz = -sa * ux + ca * uz;
            const double vr = std::sqrt(vx * vx + vy * vy + vz * vz);
            const double vct = std::max(-1.0, std::min(1.0, vz / vr));
            const double vph = std::atan2(vy, vx);
            legendre(p, vct, P1);
            for (int n = 0; n < p; n++) {
                const double f = w * (2 * n + 1) / (4 * M_PI);
                for (int m = -n; m <= n; m++) {
                    const cd fv = ynm(n, m, P1, p, vph);
                    for (int mp = -n; mp <= n; mp++) {
                        G[n][(mp + n) * (2 * n + 1) + (m + n)] += f * fv * std::conj(ynm(n, mp, P0, p, ph));
                    }
                }
            }
        }
    }
    double mi = 0;
    for (auto &g : G)
        for (auto &v : g) mi = std::max(mi, std::fabs(v.imag()));
    *max_imag = mi;
    return G;
}

// fold a real (2n+1)^2 rotation block into E ((n+1) rows) and O (n rows) of
// `stride` zero-padded floats; O rows carry a leading zero so that both
// blocks pair with the coefficients m = 0..n.  Storage is group-major: the
// 4-float group g of row r sits at (g * rows + r) * 4, so lanes that read
// the same group of consecutive rows read consecutive 16-byte pieces.
void fold(const std::vector<cd> &G, int n, int stride, float *E, float *O) {
    (void)stride;
    const int w = 2 * n + 1;
    auto g = [&](int mp, int m) { return G[(mp + n) * w + (m + n)].real(); };
    auto at = [](int rows, int r, int m) { return ((m / 4) * rows + r) * 4 + (m % 4); };
    for (int mp = 0; mp <= n; mp++) {
        E[at(n + 1, mp, 0)] = (float)g(mp, 0);
        for (int m = 1; m <= n; m++) E[at(n + 1, mp, m)] = (float)(g(mp, m) + g(mp, -m));
    }
    for (int mp = 1; mp <= n; mp++)
        for (int m = 1; m <= n; m++) O[at(n, mp - 1, m)] = (float)(g(mp, m) - g(mp, -m));
}

}  // namespace

int rot_stride(int p) { return (p + 3) / 4 * 4; }

OctLayout oct_layout(int p) {
    const int rs = rot_stride(p), dsz = 2 * rs * p * p, zsz = p * p * rs;
    OctLayout o;
    o.rot = 0;
    o.zm2m = 2 * dsz;
    o.zl2l = o.zm2m + zsz;
    o.ph_m2m = o.zl2l + zsz;
    o.ph_l2l = o.ph_m2m + 16 * p;
    o.th_m2m = o.ph_l2l + 16 * p;
    o.th_l2l = o.th_m2m + 8;
    o.size = o.th_l2l + 8;
    return o;
}
int dmat_offset_e(int n, int p) { return rot_stride(p) * n * (n + 1) / 2; }
int dmat_offset_o(int n, int p) { return rot_stride(p) * n * (n - 1) / 2; }

bool build_fmm_tables(int p, int ws, FmmTables &T, std::string &err) {
    T = FmmTables();
    T.p = p;
    T.ws = ws;
    T.nc = p * (p + 1) / 2;
    T.range = 2 * ws + 1;
    const int R = T.range;
    T.side = 2 * R + 1;
    T.ncls = T.side * T.side * T.side;
    T.stride = rot_stride(p);
    T.esz = dmat_offset_e(p, p);
    T.osz = dmat_offset_o(p, p);
    T.dsz = 2 * (T.esz + T.osz);
    T.cls_theta.assign(T.ncls, -1);
    T.cls_phase.assign((size_t)T.ncls * p * 2, 0.f);
    T.cls_rho2.assign(T.ncls, 0.f);
    std::map<long long, int> theta_index;
    std::vector<double> thetas;
    for (int dx = -R; dx <= R; dx++)
        for (int dy = -R; dy <= R; dy++)
            for (int dz = -R; dz <= R; dz++) {
                const int id = ((dx + R) * T.side + (dy + R)) * T.side + (dz + R);
                if (!fmm_m2l_class(dx, dy, dz, ws)) continue;
                const double r = std::sqrt((double)(dx * dx + dy * dy + dz * dz));
                const double th = std::acos(dz / r);
                const double ph = std::atan2((double)dy, (double)dx);
                const long long key = std::llround(th * 1e12);
                auto itk = theta_index.find(key);
                int ti;
                if (itk == theta_index.end()) {
                    ti = (int)thetas.size();
                    theta_index[key] = ti;
                    thetas.push_back(th);
                } else {
                    ti = itk->second;
                }
                T.cls_theta[id] = ti;
                T.cls_rho2[id] = (float)(dx * dx + dy * dy + dz * dz);
                for (int m = 0; m < p; m++) {
                    T.cls_phase[((size_t)id * p + m) * 2 + 0] = (float)std::cos(m * ph);
                    T.cls_phase[((size_t)id * p + m) * 2 + 1] = (float)std::sin(m * ph);
                }
            }
    T.ntheta = (int)thetas.size();
    T.dmat.assign((size_t)T.ntheta * T.dsz, 0.f);
    for (int ti = 0; ti < T.ntheta; ti++) {
        double mi1 = 0, mi2 = 0;
        // forward rotation Ry(-theta) acts on coefficients as f(u) -> f(Ry(theta) u'),
        // the backward one Ry(theta) as f(u) -> f(Ry(-theta) u')
        auto Gf = yrot(p, thetas[ti], &mi1);
        auto Gb = yrot(p, -thetas[ti], &mi2);
        if (mi1 > 1e-9 || mi2 > 1e-9) {
            err = "y-rotation matrix is not real";
            return false;
        }
        float *base = &T.dmat[(size_t)ti * T.dsz];
        for (int n = 0; n < p; n++) {
            fold(Gf[n], n, T.stride, base + dmat_offset_e(n, p), base + T.esz + dmat_offset_o(n, p));
            fold(Gb[n], n, T.stride, base + T.esz + T.osz + dmat_offset_e(n, p),
                 base + 2 * T.esz + T.osz + dmat_offset_o(n, p));
        }
    }
    // z translation constants C[k][j][n] = (-1)^{j+k} (j+n)! / (N_n^k N_j^k)
    // rows of n padded to the rotation stride, zero for n < k
    T.zc.assign((size_t)p * p * T.stride, 0.f);
    auto N = [](int n, int m) { return std::sqrt(fact(n - m) * fact(n + m)); };
    for (int k = 0; k < p; k++)
        for (int j = k; j < p; j++)
            for (int n = k; n < p; n++)
                T.zc[((size_t)k * p + j) * T.stride + n] =
                    (float)(((j + k) & 1 ? -1.0 : 1.0) * fact(j + n) / (N(n, k) * N(j, k)));
    T.nrm.assign((size_t)p * p, 0.f);
    for (int n = 0; n < p; n++)
        for (int m = 0; m <= n; m++) T.nrm[n * p + m] = (float)N(n, m);
    // rotation-based M2M / L2L tables (see oct_layout)
    {
        const OctLayout L = oct_layout(p);
        T.otab.assign(L.size, 0.f);
        const double th0 = std::acos(1.0 / std::sqrt(3.0)), rho = std::sqrt(3.0) / 2.0;
        const double ths[2] = {th0, M_PI - th0};
        for (int ti = 0; ti < 2; ti++) {
            double mi1 = 0, mi2 = 0;
            auto Gf = yrot(p, ths[ti], &mi1);
            auto Gb = yrot(p, -ths[ti], &mi2);
            if (mi1 > 1e-9 || mi2 > 1e-9) {
                err = "octant y-rotation matrix is not real";
                return false;
            }
            float *base = &T.otab[(size_t)L.rot + (size_t)ti * T.dsz];
            for (int n = 0; n < p; n++) {
                fold(Gf[n], n, T.stride, base + dmat_offset_e(n, p), base + T.esz + dmat_offset_o(n, p));
                fold(Gb[n], n, T.stride, base + T.esz + T.osz + dmat_offset_e(n, p),
                     base + 2 * T.esz + T.osz + dmat_offset_o(n, p));
            }
        }
        auto Nn = [](int n, int m) { return std::sqrt(fact(n - m) * fact(n + m)); };
        for (int k = 0; k < p; k++)
            for (int j = k; j < p; j++)
                for (int n = k; n < p; n++) {
                    // multipole: new centre = old + rho z (child -> parent centre), child -> parent units
                    if (n <= j)
                        T.otab[L.zm2m + ((size_t)k * p + j) * T.stride + n] =
                            (float)(Nn(j, k) / Nn(n, k) * std::pow(-rho, j - n) / fact(j - n) * std::ldexp(1.0, -j));
                    // local: new centre = old + rho z (parent -> child centre), parent -> child units
                    if (n >= j)
                        T.otab[L.zl2l + ((size_t)k * p + j) * T.stride + n] =
                            (float)(Nn(n, k) / Nn(j, k) * std::pow(rho, n - j) / fact(n - j) * std::ldexp(1.0, -(n + 1)));
                }
        for (int oc = 0; oc < 8; oc++) {
            // child centre - parent centre, child box units
            const double d[3] = {(oc & 1) ? 0.5 : -0.5, (oc & 2) ? 0.5 : -0.5, (oc & 4) ? 0.5 : -0.5};
            for (int kind = 0; kind < 2; kind++) {
                const double sgn = kind == 0 ? -1.0 : 1.0;  // M2M moves parent-ward, L2L child-ward
                const double tx = sgn * d[0], ty = sgn * d[1], tz = sgn * d[2];
                const double ph = std::atan2(ty, tx);
                const int ph0 = kind == 0 ? L.ph_m2m : L.ph_l2l, th = kind == 0 ? L.th_m2m : L.th_l2l;
                T.otab[th + oc] = tz > 0 ? 0.f : 1.f;
                for (int m = 0; m < p; m++) {
                    T.otab[ph0 + ((size_t)oc * p + m) * 2 + 0] = (float)std::cos(m * ph);
                    T.otab[ph0 + ((size_t)oc * p + m) * 2 + 1] = (float)std::sin(m * ph);
                }
            }
        }
    }
    return true;
}

bool build_m2l_dense(int p, int ws, std::vector<double> &K, std::string &err) {
    const int R = p * p, range = 2 * ws + 1, side = 2 * range + 1, ncls = side * side * side;
    K.assign((size_t)ncls * R * R, 0.0);
    auto N = [](int n, int m) { return std::sqrt(fact(n - m) * fact(n + m)); };
    // z-translation constants C[k][j][n], as build_fmm_tables has them
    std::vector<double> zc((size_t)p * p * p, 0.0);
    for (int k = 0; k < p; k++)
        for (int j = k; j < p; j++)
            for (int n = k; n < p; n++)
                zc[((size_t)k * p + j) * p + n] = ((j + k) & 1 ? -1.0 : 1.0) * fact(j + n) / (N(n, k) * N(j, k));
    std::map<long long, std::pair<std::vector<std::vector<cd>>, std::vector<std::vector<cd>>>> rot;
    // real index of (n, m, part): n^2 for Re(c_n^0); n^2 + 2m - 1 / n^2 + 2m for Re / Im(c_n^m)
    auto ri = [](int n, int m, int im) { return m == 0 ? n * n : n * n + 2 * m - 1 + im; };
    std::vector<cd> A(p * p), B(p * p), Cz(p * p), Rr(p * p);  // [n][m], m = 0..n
    for (int dx = -range; dx <= range; dx++)
        for (int dy = -range; dy <= range; dy++)
            for (int dz = -range; dz <= range; dz++) {
                if (!fmm_m2l_class(dx, dy, dz, ws)) continue;
                const int id = ((dx + range) * side + (dy + range)) * side + (dz + range);
                const double r = std::sqrt((double)(dx * dx + dy * dy + dz * dz));
                const double th = std::acos(dz / r), ph = std::atan2((double)dy, (double)dx);
                const long long key = std::llround(th * 1e12);
                if (!rot.count(key)) {
                    double mi1 = 0, mi2 = 0;
                    auto gf = yrot(p, th, &mi1);
                    auto gb = yrot(p, -th, &mi2);
                    if (mi1 > 1e-9 || mi2 > 1e-9) {
                        err = "y-rotation matrix is not real";
                        return false;
                    }
                    rot[key] = {gf, gb};
                }
                const auto &Gf = rot[key].first, &Gb = rot[key].second;
                // a real y-rotation of degree n on coefficients m = 0..n of a
                // real-symmetric expansion (c_n^-m = conj c_n^m)
                auto yrot_apply = [&](const std::vector<std::vector<cd>> &G, const std::vector<cd> &in,
                                      std::vector<cd> &out) {
                    for (int n = 0; n < p; n++) {
                        const int w = 2 * n + 1;
                        auto g = [&](int mp, int m) { return G[n][(mp + n) * w + (m + n)].real(); };
                        for (int mp = 0; mp <= n; mp++) {
                            double re = g(mp, 0) * in[n * p].real(), im = 0.0;
                            for (int m = 1; m <= n; m++) {
                                re += (g(mp, m) + g(mp, -m)) * in[n * p + m].real();
                                if (mp > 0) im += (g(mp, m) - g(mp, -m)) * in[n * p + m].imag();
                            }
                            out[n * p + mp] = cd(re, im);
                        }
                    }
                };
                for (int n0 = 0; n0 < p; n0++)
                    for (int m0 = 0; m0 <= n0; m0++)
                        for (int part = 0; part < (m0 == 0 ? 1 : 2); part++) {
                            std::fill(A.begin(), A.end(), cd(0, 0));
                            // unit input, then the phase e^{i m phi}
                            A[n0 * p + m0] = (part == 0 ? cd(1, 0) : cd(0, 1)) * std::polar(1.0, m0 * ph);
                            yrot_apply(Gf, A, B);
                            // translation along z: C_j^k = sum_n C[k][j][n] r^-(j+n+1) B_n^k
                            std::fill(Cz.begin(), Cz.end(), cd(0, 0));
                            for (int k = 0; k < p; k++)
                                for (int j = k; j < p; j++) {
                                    cd acc(0, 0);
                                    for (int n = k; n < p; n++)
                                        acc += zc[((size_t)k * p + j) * p + n] * std::pow(r, -(j + n + 1)) * B[n * p + k];
                                    Cz[j * p + k] = acc;
                                }
                            yrot_apply(Gb, Cz, Rr);
                            const int kin = ri(n0, m0, part);
                            for (int j = 0; j < p; j++)
                                for (int k = 0; k <= j; k++) {
                                    const cd v = Rr[j * p + k] * std::polar(1.0, -k * ph);
                                    K[((size_t)id * R + ri(j, k, 0)) * R + kin] = v.real();
                                    if (k > 0) K[((size_t)id * R + ri(j, k, 1)) * R + kin] = v.imag();
                                }
                        }
            }
    return true;
}

}  // namespace sv
