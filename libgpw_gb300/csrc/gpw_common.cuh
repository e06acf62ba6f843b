// Shared host/device definitions of libgpw_gb300.
//
// Conventions (fixed by the reference's interface, mtaillefumier/libgpw):
//   * Cartesian index coset(lx,ly,lz) as src/lib/grid_base_ref_c.cc:39-46;
//   * grid arrays double[ngrid[2]][ngrid[1]][ngrid[0]], x fastest (grid_base_ref_c.cc:496);
//   * dh rows are the grid step vectors, dh_inv is applied transposed
//     (grid_base_ref_c.cc:535-547, :637-644).
#pragma once

#include <cmath>
#include <cstdint>

#include "../../include/gpw.h"

#if defined(__CUDACC__)
#define GPW_HD __host__ __device__ __forceinline__
#else
#define GPW_HD inline
#endif

namespace gpw {

constexpr int kMaxL = GPW_MAX_L;    // per primitive
constexpr int kMaxLp = GPW_MAX_LP;  // la_max + lb_max (+2 with tau)
constexpr int kNPow = kMaxLp + 1;
// the backward pass needs moments two degrees beyond the forward coefficients
constexpr int kMaxLpB = kMaxLp + 2;
constexpr int kNPowB = kMaxLpB + 1;

GPW_HD int ncoset(int l) { return l < 0 ? 0 : ((l + 1) * (l + 2) * (l + 3)) / 6; }
GPW_HD int nshell(int l) { return ((l + 1) * (l + 2)) / 2; }
GPW_HD int coset(int lx, int ly, int lz) {
    const int l = lx + ly + lz;
    return l == 0 ? 0 : ncoset(l - 1) + ((l - lx) * (l - lx + 1)) / 2 + lz;
}
GPW_HD int imod(int a, int m) {
    int r = a % m;
    return r < 0 ? r + m : r;
}
// Packed index of (lz, ly, lx), lx + ly + lz <= lp, lz outermost (the order of
// coef_xyz in grid_base_ref_c.cc:250-257).
GPW_HD int pidx(int lp, int lz, int ly, int lx) {
    // entries with z < lz: sum_{z<lz} (lp-z+1)(lp-z+2)/2
    int before_z = 0;
    for (int z = 0; z < lz; z++) before_z += ((lp - z + 1) * (lp - z + 2)) / 2;
    const int q = lp - lz;  // triangle ly + lx <= q
    const int before_y = ly * (q + 1) - (ly * (ly - 1)) / 2;
    return before_z + before_y + lx;
}
GPW_HD int ncoef(int lp) { return ncoset(lp); }

// Round-to-nearest arithmetic that never contracts to FMA, so that host and
// device decide cube membership identically.
GPW_HD double rmul(double a, double b) {
#if defined(__CUDA_ARCH__)
    return __dmul_rn(a, b);
#else
    return a * b;
#endif
}
GPW_HD double radd(double a, double b) {
#if defined(__CUDA_ARCH__)
    return __dadd_rn(a, b);
#else
    return a + b;
#endif
}
GPW_HD double rsub(double a, double b) {
#if defined(__CUDA_ARCH__)
    return __dsub_rn(a, b);
#else
    return a - b;
#endif
}
GPW_HD double rdiv(double a, double b) {
#if defined(__CUDA_ARCH__)
    return __ddiv_rn(a, b);
#else
    return a / b;
#endif
}
GPW_HD double rsqrt_rn(double a) {
#if defined(__CUDA_ARCH__)
    return __dsqrt_rn(a);
#else
    return std::sqrt(a);
#endif
}

// ---------------------------------------------------------------------------
// The library's sphere rule for orthorhombic cubes.  Offsets g of a cube axis
// fold to f = g <= 0 ? g : 1 - g (the cube is symmetric about +1/2 cell, as the
// mirror writes of grid_base_ref_c.cc:496-503 assume).  With r2 = r*r:
//   kmax        = floor(r / hz)
//   remk(kf)    = max(r2 - (kf*hz)^2, 0),   jmax(kf) = floor(sqrt(remk)/hy)
//   imax(kf,jf) = floor(sqrt(max(remk - (jf*hy)^2, 0)) / hx)
// A point is in the cube when kf >= -kmax, jf >= -jmax(kf), if >= -imax(kf,jf).
GPW_HD int rule_kmax(double r, double hz) { return (int)floor(rdiv(r, hz)); }
GPW_HD double rule_remk(double r2, int kf, double hz) {
    const double dz = rmul((double)(-kf), hz);
    const double rem = rsub(r2, rmul(dz, dz));
    return rem < 0.0 ? 0.0 : rem;
}
GPW_HD int rule_jmax(double remk, double hy) { return (int)floor(rdiv(rsqrt_rn(remk), hy)); }
GPW_HD int rule_imax(double remk, int jf, double hy, double hx) {
    const double dy = rmul((double)(-jf), hy);
    double rem = rsub(remk, rmul(dy, dy));
    if (rem < 0.0) rem = 0.0;
    return (int)floor(rdiv(rsqrt_rn(rem), hx));
}
GPW_HD int fold(int g) { return g <= 0 ? g : 1 - g; }

// Grid index of cube offset g on one axis (grid_base_ref_c.cc:318-351): periodic
// axes wrap; non-periodic axes address a local window and return -1 outside it.
GPW_HD int axis_index(int periodic, int cc, int g, int lbc, int lbg, int npts, int ngrid) {
    if (periodic) return imod(cc + g, npts);
    const int idx = g + imod(cc + lbc + lbg, npts) - lbc;
    return (idx < 0 || idx >= ngrid) ? -1 : idx;
}

// General cell: the i-range of the index-box row (dj, dk) from the quadratic
// |i h0 + v|^2 <= r^2, with the reference's operation order (grid_base_ref_c.cc:781-807).
GPW_HD bool general_row(const double dh[3][3], const double gp[3], double dj, double dk,
                        double radius, int &ismin, int &ismax) {
    double a = 0.0, b = 0.0, c = 0.0;
    for (int i = 0; i < 3; i++) {
        const double pointk = rmul(dh[2][i], dk);
        const double pointj = radd(pointk, rmul(dh[1][i], dj));
        const double v = rsub(pointj, rmul(gp[0], dh[0][i]));
        a = radd(a, rmul(dh[0][i], dh[0][i]));
        b = radd(b, rmul(rmul(2.0, v), dh[0][i]));
        c = radd(c, rmul(v, v));
    }
    double d = rsub(rmul(b, b), rmul(rmul(4.0, a), rsub(c, rmul(radius, radius))));
    if (d < 0.0) return false;
    d = rsqrt_rn(d);
    const double a2 = rmul(2.0, a);
    ismin = (int)ceil(rdiv(rsub(-b, d), a2));
    ismax = (int)floor(rdiv(radd(-b, d), a2));
    return true;
}


// ---------------------------------------------------------------------------
// Per-level constants on the device.
struct LevelDev {
    int npts[3];
    int ngrid[3];
    int lb_grid[3];
    int periodic[3];
    int ortho;
    int pad_;
    double dh[3][3];
    double dh_inv[3][3];
    int64_t grid_elems;
    int64_t tmat_off;  // general cells: offset of the lattice transform blocks
};

// Pair geometry, computed once per task set on the host (FP64, no contraction).
struct PairGeom {
    double rp[3];
    double off[3];    // ortho: roffset (rp - cc*h); general: gp = dh_inv^T rp
    double zetp;
    double prefactor; // rscale * exp(-zeta*f*|rab|^2)
    double radius;
    double ra[3];
    double rb[3];
    int cc[3];        // ortho: cube centre; general: lowest index of the box
    int hi[3];        // general: highest index of the box; ortho: ub_cube
    int lb[3];        // ortho: lb_cube
    int kgmin;        // ortho
    int lp;
    int level;
    int task;         // index in the caller's task array
    int la_max, la_min, lb_max, lb_min;  // after the tau shift
    int la0_max, la0_min, lb0_max, lb0_min;  // as given
    int maxco, o1, o2;
    int ortho;
    int64_t pab_offset;
    int64_t coef_off;  // scratch offset of the packed coefficients
    int64_t table_off; // CP2K-format cube list (ortho), -1: sphere rule
    int64_t cost;      // estimated cube points
    int64_t mom_ext_off; // scratch offset of the degree lp+2 moments (backward)
    double zeta, zetb;
    double rscale;
    double rab[3];
    int ext0[3];       // general: the box extents the task set was planned with
    int pad_;
};

// Device status bits (OR-ed by kernels, read by gpw_taskset_check).
enum : int {
    kStatOutOfWindow = 1,
    kStatTimeout = 2,
    kStatBadTable = 4,
    kStatTooManyImages = 8,
    kStatBadTile = 16,
    kStatBadGeom = 32,      // a geometry update that the task set cannot take
};

}  // namespace gpw
