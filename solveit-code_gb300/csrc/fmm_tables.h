// fmm_tables.h -- host-built FMM operator tables (uploaded once per order / separation).
#pragma once

#include <string>
#include <vector>

#ifdef __CUDACC__
#define SV_HD __host__ __device__
#else
#define SV_HD
#endif

namespace sv {

struct FmmTables {
    int p = 0, ws = 0, nc = 0;
    int range = 0;   // 2*ws+1: largest |offset| component of an M2L pair
    int side = 0;    // 2*range+1: offsets per axis in the class index
    int ncls = 0;    // side^3 offset classes (target - source, box units)
    int ntheta = 0;  // distinct polar angles among the M2L offsets
    int stride = 0;  // floats per rotation / translation row: p rounded up to 4 (16-byte rows)
    int esz = 0, osz = 0, dsz = 0;
    std::vector<int> cls_theta;    // [ncls] polar-angle index, -1 for offsets never translated (fmm_m2l_class)
    std::vector<float> cls_phase;  // [ncls][p][2] cos(m phi), sin(m phi)
    std::vector<float> cls_rho2;   // [ncls] |offset|^2
    std::vector<float> dmat;       // [ntheta][Ef | Of | Eb | Ob] folded y-rotations, group-major rows of `stride`
    std::vector<float> zc;         // [p][p][stride] z-translation constants C[k][j][n]
    std::vector<float> nrm;        // [p][p] sqrt((n-m)!(n+m)!)
    // rotation-based M2M / L2L along the 8 child directions (layout: oct_layout)
    std::vector<float> otab;
};

// Offsets (floats) inside FmmTables::otab for order p.  The child offsets
// (+-1/2)^3 (child box units) have two polar angles, theta0 = acos(1/sqrt 3)
// and pi - theta0:
//   rot    [2][dsz]        folded y-rotation blocks of both angles (dmat layout)
//   zm2m   [p][p][stride]  z-shift of a multipole by -sqrt(3)/2, child -> parent units
//   zl2l   [p][p][stride]  z-shift of a local expansion by +sqrt(3)/2, parent -> child units
//   ph_m2m, ph_l2l [8][p][2]  e^{i m phi} of each octant's translation direction
//   th_m2m, th_l2l [8]        polar-angle index (0 or 1) of each octant's direction
struct OctLayout {
    int rot, zm2m, zl2l, ph_m2m, ph_l2l, th_m2m, th_l2l, size;
};
OctLayout oct_layout(int p);

// Near-field offsets that the trimmed near field of ws = 2 hands to the M2L:
// the (2,2,1) and (2,2,2) types (32 of the 125 boxes).  Their worst-case
// separation ratio (sum of the two boxes' circumradii over the centre distance)
// is sqrt(3)/3 for (2,2,1) and 1/2 for (2,2,2), no larger than that of the
// closest M2L offsets of the full cube, (3,0,0).
SV_HD inline bool fmm_trimmable(int dx, int dy, int dz, int ws) {
    if (ws != 2) return false;
    const int a = dx < 0 ? -dx : dx, b = dy < 0 ? -dy : dy, c = dz < 0 ? -dz : dz;
    const int n2 = (a == 2) + (b == 2) + (c == 2);
    return n2 == 3 || (n2 == 2 && a + b + c == 5);
}
// An offset class the M2L tables carry: outside the near cube, or trimmable.
SV_HD inline bool fmm_m2l_class(int dx, int dy, int dz, int ws) {
    const int a = dx < 0 ? -dx : dx, b = dy < 0 ? -dy : dy, c = dz < 0 ? -dz : dz;
    const int am = a > b ? (a > c ? a : c) : (b > c ? b : c);
    return am > ws || fmm_trimmable(dx, dy, dz, ws);
}

int rot_stride(int p);              // p rounded up to a multiple of 4
int dmat_offset_e(int n, int p);    // stride * sum_{k<n} (k+1): E block of degree n
int dmat_offset_o(int n, int p);    // stride * sum_{k<n} k: O block of degree n (rows mp = 1..n)
bool build_fmm_tables(int p, int ws, FmmTables &T, std::string &err);

// The M2L of every offset class as a dense real matrix, built in FP64 from
// the same steps as the rotation-based M2L (phase, y-rotation, translation
// along z, back-rotation, phase) without the softening of the distance.
// Coefficients are taken as R = p^2 reals in degree order: for degree n,
// Re(c_n^0), then Re(c_n^m), Im(c_n^m) for m = 1..n (the zero imaginary part
// of c_n^0 is left out).  K[(cls * R + j) * R + k] maps input real k of the
// source multipole to output real j of the target's local expansion (zero
// for the classes fmm_m2l_class leaves out).
bool build_m2l_dense(int p, int ws, std::vector<double> &K, std::string &err);

}  // namespace sv
