/*
 * gpw_oracle.c -- TEST INFRASTRUCTURE ONLY.  A plain-C, FP64, single-pair CPU
 * restatement of libgpw's collocate path (mtaillefumier/libgpw,
 * src/lib/grid_base_ref_c.cc), plus its adjoint (integrate) which the
 * reference does not have.  Only tests, the smoke check and the CPU-baseline
 * leg of the benchmark call it; the library never links it.
 *
 * Pinned by: the reference's own task fixtures (src/lib/collocate_*.task, via
 * tests/golden) and by the reference code itself compiled from its sources
 * (oracle/_ref/libgpwref.so, built by oracle/ref/Makefile).
 *
 * Structure of one pair (reference call stack grid_base_ref_c.cc:849-1014):
 *   prefactor, rp, rb                          :878-886
 *   density block -> local block (rho / tau)  :158-192 / :65-155
 *   1-D re-centring binomials                  :195-231
 *   product-centre coefficients c[lz][ly][lx]  :234-315
 *   orthorhombic cube  (tables, map, contraction) :318-508, :511-589
 *   general cell (lattice polynomial, rows)       :593-846
 * The arithmetic is written independently (dense coefficient arrays, direct
 * exponentials instead of the exp recurrences, explicit adjoints), so results
 * agree with the reference to rounding, not bit for bit.
 *
 * Build: gcc -O2 -fPIC -ffp-contract=off -shared (oracle/Makefile).
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/gpw.h"

#define LPMAX 12              /* lp <= 10 with tau; a little headroom        */
#define NPOW (LPMAX + 1)

static const int ncoset_tab[] = {1, 4, 10, 20, 35, 56, 84, 120, 165, 220, 286, 364, 455, 560};

static int ncoset(int l) { return l < 0 ? 0 : ncoset_tab[l]; }

/* Cartesian index of (lx,ly,lz): the coset ordering of grid_base_ref_c.cc:39-46.
 * It is the layout of the density block, so it has to be the same. */
static int coset(int lx, int ly, int lz) {
    int l = lx + ly + lz;
    if (l == 0) return 0;
    return ncoset_tab[l - 1] + ((l - lx) * (l - lx + 1)) / 2 + lz;
}

static int imod(int a, int m) { int r = a % m; return r < 0 ? r + m : r; }

/* ------------------------------------------------------------------------- */
/* Pair geometry (grid_base_ref_c.cc:878-886)                                  */
typedef struct {
    double zetp, prefactor;
    double ra[3], rb[3], rp[3];
    int la_max, la_min, lb_max, lb_min;      /* after the tau shift          */
    int lp;
} pair_t;

static void pair_setup(int tau, int la_max, int la_min, int lb_max, int lb_min, double zeta,
                       double zetb, double rscale, const double ra[3], const double rab[3],
                       pair_t *p) {
    p->zetp = zeta + zetb;
    double f = zetb / p->zetp;
    double rab2 = rab[0] * rab[0] + rab[1] * rab[1] + rab[2] * rab[2];
    p->prefactor = rscale * exp(-zeta * f * rab2);
    for (int i = 0; i < 3; i++) {
        p->ra[i] = ra[i];
        p->rp[i] = ra[i] + f * rab[i];
        p->rb[i] = ra[i] + rab[i];
    }
    if (tau) { /* grid_base_ref_c.cc:890-895 */
        p->la_max = la_max + 1; p->la_min = la_min - 1 > 0 ? la_min - 1 : 0;
        p->lb_max = lb_max + 1; p->lb_min = lb_min - 1 > 0 ? lb_min - 1 : 0;
    } else {
        p->la_max = la_max; p->la_min = la_min; p->lb_max = lb_max; p->lb_min = lb_min;
    }
    p->lp = p->la_max + p->lb_max;
}

/* ------------------------------------------------------------------------- */
/* Density block -> local block.  loc[jco][ico] with ld = ncoset(la_max_local).
 * func 0, rho: copy of the [la_min,la_max] x [lb_min,lb_max] shells (grid_base_ref_c.cc:158-192).
 * func 1, tau: 1/2 grad(a).grad(b) by d/dx x^l e^{-z x^2} = l x^{l-1} - 2 z x^{l+1}
 *      (grid_base_ref_c.cc:65-155; compute_polynomial_coefficients_DADB, coefficient.hpp:67-196).
 * func 2, 3, 4: phi_a d_d phi_b - d_d phi_a phi_b along x, y, z by the same rule
 *      (compute_polynomial_coefficients_ADBmDAB, coefficient.hpp:209-354, with every
 *      term accumulated).  `adj` runs the transposed map: block[...] += M^T loc.     */
static void block_map(int tau, int adj, int la_max, int la_min, int lb_max, int lb_min,
                      double zeta, double zetb, const double *blk, double *blk_out, int maxco,
                      int o1, int o2, double *loc, const double *loc_in, int ldl) {
    for (int la = la_min; la <= la_max; la++)
    for (int lxa = la; lxa >= 0; lxa--)
    for (int lza = 0; lza <= la - lxa; lza++) {
        int lya = la - lxa - lza;
        int ico = coset(lxa, lya, lza);
        for (int lb = lb_min; lb <= lb_max; lb++)
        for (int lxb = lb; lxb >= 0; lxb--)
        for (int lzb = 0; lzb <= lb - lxb; lzb++) {
            int lyb = lb - lxb - lzb;
            int jco = coset(lxb, lyb, lzb);
            int64_t bidx = (int64_t)(o2 + jco) * maxco + (o1 + ico);
            if (!tau) {
                if (!adj) loc[jco * ldl + ico] = blk[bidx];
                else blk_out[bidx] += loc_in[jco * ldl + ico];
                continue;
            }
            int a[3] = {lxa, lya, lza}, b[3] = {lxb, lyb, lzb};
            double acc = 0.0;
            double p = adj ? 0.0 : blk[bidx];
            if (tau >= 2) {
                /* (a, b - e): b_d;  (a, b + e): -2 zetb;  (a - e, b): -a_d;  (a + e, b): 2 zeta */
                int d = tau - 2;
                for (int k = 0; k < 4; k++) {
                    int a2[3] = {a[0], a[1], a[2]}, b2[3] = {b[0], b[1], b[2]};
                    double w;
                    if (k == 0) { if (b[d] == 0) continue; b2[d] -= 1; w = (double)b[d]; }
                    else if (k == 1) { b2[d] += 1; w = -2.0 * zetb; }
                    else if (k == 2) { if (a[d] == 0) continue; a2[d] -= 1; w = -(double)a[d]; }
                    else { a2[d] += 1; w = 2.0 * zeta; }
                    int ic2 = coset(a2[0], a2[1], a2[2]), jc2 = coset(b2[0], b2[1], b2[2]);
                    if (!adj) loc[jc2 * ldl + ic2] += w * p;
                    else acc += w * loc_in[jc2 * ldl + ic2];
                }
                if (adj) blk_out[bidx] += acc;
                continue;
            }
            for (int d = 0; d < 3; d++) {
                /* two terms from each side: lower (coefficient l) and raise (-2 zeta) */
                for (int sa = 0; sa < 2; sa++) {
                    double ca = sa == 0 ? (double)a[d] : -2.0 * zeta;
                    int da = sa == 0 ? -1 : 1;
                    if (sa == 0 && a[d] == 0) continue;
                    int a2[3] = {a[0], a[1], a[2]};
                    a2[d] += da;
                    int ic2 = coset(a2[0], a2[1], a2[2]);
                    for (int sb = 0; sb < 2; sb++) {
                        double cb = sb == 0 ? (double)b[d] : -2.0 * zetb;
                        int db = sb == 0 ? -1 : 1;
                        if (sb == 0 && b[d] == 0) continue;
                        int b2[3] = {b[0], b[1], b[2]};
                        b2[d] += db;
                        int jc2 = coset(b2[0], b2[1], b2[2]);
                        double w = 0.5 * ca * cb;
                        if (!adj) loc[jc2 * ldl + ic2] += w * p;
                        else acc += w * loc_in[jc2 * ldl + ic2];
                    }
                }
            }
            if (adj) blk_out[bidx] += acc;
        }
    }
}

/* (x-a)^i (x-b)^j = sum_k al[i][j][k] (x-p)^k, one axis (grid_base_ref_c.cc:195-231). */
static void recentre(double pa, double pb, int imax, int jmax, double al[NPOW][NPOW][2 * NPOW]) {
    double binom[NPOW][NPOW];
    memset(binom, 0, sizeof(binom));
    for (int n = 0; n < NPOW; n++) {
        binom[n][0] = 1.0;
        for (int k = 1; k <= n; k++) binom[n][k] = binom[n - 1][k - 1] + (k <= n - 1 ? binom[n - 1][k] : 0.0);
    }
    double ppa[NPOW], ppb[NPOW];
    ppa[0] = ppb[0] = 1.0;
    for (int n = 1; n < NPOW; n++) { ppa[n] = ppa[n - 1] * pa; ppb[n] = ppb[n - 1] * pb; }
    for (int i = 0; i <= imax; i++)
        for (int j = 0; j <= jmax; j++) {
            for (int k = 0; k < 2 * NPOW; k++) al[i][j][k] = 0.0;
            /* (x-a) = (x-p) + (p-a): choose k1 powers of (x-p) from the first factor */
            for (int k1 = 0; k1 <= i; k1++)
                for (int k2 = 0; k2 <= j; k2++)
                    al[i][j][k1 + k2] += binom[i][k1] * ppa[i - k1] * binom[j][k2] * ppb[j - k2];
        }
}

/* local block <-> product-centre coefficients c[lz][ly][lx] (dense, NPOW^3),
 * grid_base_ref_c.cc:234-315.  adj: loc_out = prefactor * M^T c_in. */
typedef struct { double al[3][NPOW][NPOW][2 * NPOW]; } alpha_t;

static void coef_map(const pair_t *p, int adj, const double *loc, double *loc_out, int ldl,
                     double *c, const double *c_in) {
    alpha_t *A = (alpha_t *)malloc(sizeof(alpha_t));
    for (int d = 0; d < 3; d++)
        recentre(p->rp[d] - p->ra[d], p->rp[d] - p->rb[d], p->la_max, p->lb_max, A->al[d]);
    if (!adj) memset(c, 0, sizeof(double) * NPOW * NPOW * NPOW);
    for (int la = p->la_min; la <= p->la_max; la++)
    for (int lxa = la; lxa >= 0; lxa--)
    for (int lza = 0; lza <= la - lxa; lza++) {
        int lya = la - lxa - lza;
        int ico = coset(lxa, lya, lza);
        for (int lb = p->lb_min; lb <= p->lb_max; lb++)
        for (int lxb = lb; lxb >= 0; lxb--)
        for (int lzb = 0; lzb <= lb - lxb; lzb++) {
            int lyb = lb - lxb - lzb;
            int jco = coset(lxb, lyb, lzb);
            double acc = 0.0;
            double pv = adj ? 0.0 : p->prefactor * loc[jco * ldl + ico];
            for (int lz = 0; lz <= lza + lzb; lz++) {
                double az = A->al[2][lza][lzb][lz];
                for (int ly = 0; ly <= lya + lyb; ly++) {
                    double ayz = az * A->al[1][lya][lyb][ly];
                    for (int lx = 0; lx <= lxa + lxb; lx++) {
                        double w = ayz * A->al[0][lxa][lxb][lx];
                        int ci = (lz * NPOW + ly) * NPOW + lx;
                        if (!adj) c[ci] += w * pv;
                        else acc += w * c_in[ci];
                    }
                }
            }
            if (adj) loc_out[jco * ldl + ico] += p->prefactor * acc;
        }
    }
    free(A);
}

/* ------------------------------------------------------------------------- */
/* Cube shapes.  The list format is the one grid_collocate_core consumes
 * (grid_base_ref_c.cc:413-471): kgmin, then for kg = kgmin..0 one jgmin followed
 * by one igmin per jg = jgmin..0.  Each entry covers the row and its mirror
 * 1-ig etc.                                                                    */
typedef struct {
    int kgmin;
    int *jgmin;      /* [nk]  */
    int *rowstart;   /* [nk]  */
    int *igmin;      /* rows  */
} cube_t;

static int cube_parse(const int *sb, int nsb, cube_t *cb) {
    if (nsb < 1) return -1;
    int pos = 0;
    cb->kgmin = sb[pos++];
    if (cb->kgmin > 0) return -1;
    int nk = 1 - cb->kgmin;
    cb->jgmin = (int *)malloc(sizeof(int) * nk);
    cb->rowstart = (int *)malloc(sizeof(int) * nk);
    cb->igmin = (int *)malloc(sizeof(int) * (nsb > 0 ? nsb : 1));
    int nrow = 0;
    for (int k = 0; k < nk; k++) {
        if (pos >= nsb) return -1;
        int jg = sb[pos++];
        if (jg > 0) return -1;
        cb->jgmin[k] = jg;
        cb->rowstart[k] = nrow;
        for (int j = jg; j <= 0; j++) {
            if (pos >= nsb) return -1;
            int ig = sb[pos++];
            if (ig > 0) return -1;
            cb->igmin[nrow++] = ig;
        }
    }
    return 0;
}

static void cube_free(cube_t *cb) { free(cb->jgmin); free(cb->rowstart); free(cb->igmin); }

/* Length of a well-formed list, or -1. */
static int cube_list_len(const int *sb, int limit) {
    int pos = 0;
    if (limit < 1 || sb[0] > 0) return -1;
    int kgmin = sb[pos++];
    for (int k = kgmin; k <= 0; k++) {
        if (pos >= limit) return -1;
        int jg = sb[pos++];
        if (jg > 0) return -1;
        pos += 1 - jg;
        if (pos > limit) return -1;
    }
    return pos;
}

/* The library's sphere rule (mirrors gpw_sphere_bounds): point offsets folded
 * to d = max(-g, g-1) >= 0 per axis are kept while the nested extents
 *   kmax = floor(r/hz), jmax(k) = floor(sqrt(r^2-(k hz)^2)/hy),
 *   imax(k,j) = floor(sqrt(r^2-(k hz)^2-(j hy)^2)/hx)
 * allow it.  No fused multiply-add anywhere (the device evaluates the same
 * expressions with round-to-nearest intrinsics). */
int gpwo_sphere_bounds(double radius, const double *dh9, int lb_cube[3], int ub_cube[3], int *sb,
                       int cap) {
    double h[3] = {dh9[0], dh9[4], dh9[8]};
    if (!(radius > 0.0) || !(h[0] > 0.0) || !(h[1] > 0.0) || !(h[2] > 0.0)) return 0;
    double r2 = radius * radius;
    int kmax = (int)floor(radius / h[2]);
    int n = 0;
#define PUSH(v) do { if (n < cap) sb[n] = (v); n++; } while (0)
    PUSH(-kmax);
    for (int kg = -kmax; kg <= 0; kg++) {
        double dz = (double)(-kg) * h[2];
        double remk = r2 - dz * dz;
        if (remk < 0.0) remk = 0.0;
        int jmax = (int)floor(sqrt(remk) / h[1]);
        PUSH(-jmax);
        for (int jg = -jmax; jg <= 0; jg++) {
            double dy = (double)(-jg) * h[1];
            double remj = remk - dy * dy;
            if (remj < 0.0) remj = 0.0;
            int imax = (int)floor(sqrt(remj) / h[0]);
            PUSH(-imax);
        }
    }
#undef PUSH
    for (int d = 0; d < 3; d++) {
        int m = (int)floor(radius / h[d]);
        lb_cube[d] = -m;
        ub_cube[d] = 1 + m;
    }
    return n <= cap ? n : -n;
}

/* ------------------------------------------------------------------------- */
/* Orthorhombic cube (grid_base_ref_c.cc:318-508, :511-589).
 * adj == 0: grid += sum c * Z * Y * X;  adj == 1: w[lz][ly][lx] += sum V * Z * Y * X. */
static int grid_index(int periodic, int cc, int g, int lbc, int lbg, int npts, int ngrid) {
    if (periodic) return imod(cc + g, npts);
    int idx = g + imod(cc + lbc + lbg, npts) - lbc;         /* grid_base_ref_c.cc:343 */
    if (idx < 0 || idx >= ngrid) return -1;
    return idx;
}

static int ortho_cube(const pair_t *p, int adj, const double dh[3][3], const double dh_inv[3][3],
                      const int npts[3], const int ngrid[3], const int lb_grid[3],
                      const int periodic[3], const int lb_cube[3], const int ub_cube[3],
                      const cube_t *cb, const double *c, double *w, double *grid,
                      const double *V) {
    int lp = p->lp;
    int cc[3];
    double roff[3];
    for (int i = 0; i < 3; i++) { /* cubecenter = floor(dh_inv^T rp), grid_base_ref_c.cc:535-547 */
        double s = 0.0;
        for (int j = 0; j < 3; j++) s += dh_inv[j][i] * p->rp[j];
        cc[i] = (int)floor(s);
        roff[i] = p->rp[i] - (double)cc[i] * dh[i][i];
    }
    /* 1-D tables over [lb_cube, ub_cube]: t^k exp(-zetp t^2), t = g*h - roffset */
    double *tab[3];
    int lo[3], n[3];
    for (int d = 0; d < 3; d++) {
        lo[d] = lb_cube[d];
        n[d] = ub_cube[d] - lb_cube[d] + 1;
        tab[d] = (double *)malloc(sizeof(double) * n[d] * (lp + 1));
        for (int g = 0; g < n[d]; g++) {
            double t = (double)(g + lo[d]) * dh[d][d] - roff[d];
            double e = exp(-p->zetp * t * t);
            for (int k = 0; k <= lp; k++) { tab[d][g * (lp + 1) + k] = e; e *= t; }
        }
    }
    /* every row of the list must lie inside [lb_cube, ub_cube] */
    for (int kf = cb->kgmin; kf <= 0; kf++) {
        int kidx = kf - cb->kgmin;
        int jgmin = cb->jgmin[kidx];
        int bad = kf < lb_cube[2] || 1 - kf > ub_cube[2] || jgmin < lb_cube[1] || 1 - jgmin > ub_cube[1];
        for (int jf = jgmin; jf <= 0 && !bad; jf++) {
            int igmin = cb->igmin[cb->rowstart[kidx] + (jf - jgmin)];
            bad = igmin < lb_cube[0] || 1 - igmin > ub_cube[0];
        }
        if (bad) {
            for (int d = 0; d < 3; d++) free(tab[d]);
            return GPW_ERR_INVALID_ARG;
        }
    }
    /* grid index of every x of the cube box, once per pair (as the reference's map,
     * grid_base_ref_c.cc:318-351): no modulo per point */
    int *xmap = (int *)malloc(sizeof(int) * n[0]);
    for (int g = 0; g < n[0]; g++)
        xmap[g] = grid_index(periodic[0], cc[0], g + lo[0], lb_cube[0], lb_grid[0], npts[0], ngrid[0]);
    double cxy[NPOW][NPOW], cx[NPOW];
    int status = 0;
    for (int kg = cb->kgmin; kg <= 1 - cb->kgmin && !status; kg++) {
        int kf = kg <= 0 ? kg : 1 - kg;
        int kidx = kf - cb->kgmin;
        int k = grid_index(periodic[2], cc[2], kg, lb_cube[2], lb_grid[2], npts[2], ngrid[2]);
        if (k < 0) { status = GPW_ERR_OUT_OF_WINDOW; break; }
        const double *Z = tab[2] + (kg - lo[2]) * (lp + 1);
        if (!adj) {
            for (int ly = 0; ly <= lp; ly++)
                for (int lx = 0; lx <= lp - ly; lx++) {
                    double s = 0.0;
                    for (int lz = 0; lz <= lp - ly - lx; lz++) s += c[(lz * NPOW + ly) * NPOW + lx] * Z[lz];
                    cxy[ly][lx] = s;
                }
        } else {
            memset(cxy, 0, sizeof(cxy));
        }
        int jgmin = cb->jgmin[kidx];
        for (int jg = jgmin; jg <= 1 - jgmin; jg++) {
            int jf = jg <= 0 ? jg : 1 - jg;
            int igmin = cb->igmin[cb->rowstart[kidx] + (jf - jgmin)];
            int j = grid_index(periodic[1], cc[1], jg, lb_cube[1], lb_grid[1], npts[1], ngrid[1]);
            if (j < 0) { status = GPW_ERR_OUT_OF_WINDOW; break; }
            const double *Y = tab[1] + (jg - lo[1]) * (lp + 1);
            if (!adj) {
                for (int lx = 0; lx <= lp; lx++) {
                    double s = 0.0;
                    for (int ly = 0; ly <= lp - lx; ly++) s += cxy[ly][lx] * Y[ly];
                    cx[lx] = s;
                }
            } else {
                memset(cx, 0, sizeof(cx));
            }
            int ig = igmin;
            if (!adj) {
                /* four points at a time: four independent sums, each in the order of the
                 * one-point loop below (the same result); groups with a point outside the
                 * window are left to that loop */
                for (; ig + 3 <= 1 - igmin; ig += 4) {
                    const int *im = xmap + (ig - lo[0]);
                    if (im[0] < 0 || im[1] < 0 || im[2] < 0 || im[3] < 0) break;
                    const double *X = tab[0] + (ig - lo[0]) * (lp + 1);
                    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
                    for (int lx = 0; lx <= lp; lx++) {
                        s0 += cx[lx] * X[lx];
                        s1 += cx[lx] * X[(lp + 1) + lx];
                        s2 += cx[lx] * X[2 * (lp + 1) + lx];
                        s3 += cx[lx] * X[3 * (lp + 1) + lx];
                    }
                    const int64_t row = ((int64_t)k * ngrid[1] + j) * ngrid[0];
                    grid[row + im[0]] += s0;
                    grid[row + im[1]] += s1;
                    grid[row + im[2]] += s2;
                    grid[row + im[3]] += s3;
                }
            }
            for (; ig <= 1 - igmin; ig++) {
                int i = xmap[ig - lo[0]];
                if (i < 0) { status = GPW_ERR_OUT_OF_WINDOW; break; }
                const double *X = tab[0] + (ig - lo[0]) * (lp + 1);
                int64_t gidx = ((int64_t)k * ngrid[1] + j) * ngrid[0] + i;
                if (!adj) {
                    double s = 0.0;
                    for (int lx = 0; lx <= lp; lx++) s += cx[lx] * X[lx];
                    grid[gidx] += s;
                } else {
                    double v = V[gidx];
                    for (int lx = 0; lx <= lp; lx++) cx[lx] += v * X[lx];
                }
            }
            if (adj)
                for (int ly = 0; ly <= lp; ly++)
                    for (int lx = 0; lx <= lp - ly; lx++) cxy[ly][lx] += cx[lx] * Y[ly];
        }
        if (adj)
            for (int ly = 0; ly <= lp; ly++)
                for (int lx = 0; lx <= lp - ly; lx++)
                    for (int lz = 0; lz <= lp - ly - lx; lz++)
                        w[(lz * NPOW + ly) * NPOW + lx] += cxy[ly][lx] * Z[lz];
    }
    free(xmap);
    for (int d = 0; d < 3; d++) free(tab[d]);
    return status;
}

/* ------------------------------------------------------------------------- */
/* General cell (grid_base_ref_c.cc:593-846).  The Cartesian polynomial around rp
 * is re-expressed in lattice offsets d_a = idx_a - gp_a, since
 * r - rp = sum_a d_a dh[a][:], so (x_c - p_c) = sum_a dh[a][c] d_a.
 * T maps c[lz][ly][lx] to q[k][j][i] (coefficient of d0^i d1^j d2^k).          */
#define NQ (NPOW * NPOW * NPOW)

static void poly_mul(const double *a, int da, const double *b, int db, double *out) {
    /* dense polynomials in (d0,d1,d2) of total degree <= da / db, index [k][j][i] */
    memset(out, 0, sizeof(double) * NQ);
    for (int ka = 0; ka <= da; ka++)
    for (int ja = 0; ja <= da - ka; ja++)
    for (int ia = 0; ia <= da - ka - ja; ia++) {
        double va = a[(ka * NPOW + ja) * NPOW + ia];
        if (va == 0.0) continue;
        for (int kb = 0; kb <= db; kb++)
        for (int jb = 0; jb <= db - kb; jb++)
        for (int ib = 0; ib <= db - kb - jb; ib++)
            out[((ka + kb) * NPOW + (ja + jb)) * NPOW + (ia + ib)] += va * b[(kb * NPOW + jb) * NPOW + ib];
    }
}

/* adj == 0: q = T c.  adj == 1: c_out += T^T q_in. */
static void lattice_map(int lp, const double dh[3][3], int adj, const double *c, double *q,
                        const double *q_in, double *c_out) {
    double *U = (double *)calloc((size_t)3 * NPOW * NQ, sizeof(double)); /* U[comp][power] */
    for (int comp = 0; comp < 3; comp++) {
        double *P0 = U + ((size_t)comp * NPOW + 0) * NQ;
        P0[0] = 1.0;
        double lin[NQ];
        memset(lin, 0, sizeof(lin));
        lin[1] = dh[0][comp];                    /* d0 */
        lin[NPOW] = dh[1][comp];                 /* d1 */
        lin[NPOW * NPOW] = dh[2][comp];          /* d2 */
        for (int n = 1; n <= lp; n++)
            poly_mul(U + ((size_t)comp * NPOW + n - 1) * NQ, n - 1, lin, 1,
                     U + ((size_t)comp * NPOW + n) * NQ);
    }
    if (!adj) memset(q, 0, sizeof(double) * NQ);
    double *tmp = (double *)malloc(sizeof(double) * NQ);
    double *col = (double *)malloc(sizeof(double) * NQ);
    for (int lz = 0; lz <= lp; lz++)
        for (int ly = 0; ly <= lp - lz; ly++) {
            poly_mul(U + ((size_t)2 * NPOW + lz) * NQ, lz, U + ((size_t)1 * NPOW + ly) * NQ, ly, tmp);
            for (int lx = 0; lx <= lp - lz - ly; lx++) {
                poly_mul(tmp, lz + ly, U + ((size_t)0 * NPOW + lx) * NQ, lx, col);
                int ci = (lz * NPOW + ly) * NPOW + lx;
                int deg = lz + ly + lx;
                if (!adj) {
                    double cv = c[ci];
                    for (int k = 0; k <= deg; k++)
                        for (int j = 0; j <= deg - k; j++)
                            for (int i = 0; i <= deg - k - j; i++) {
                                int qi = (k * NPOW + j) * NPOW + i;
                                q[qi] += cv * col[qi];
                            }
                } else {
                    double s = 0.0;
                    for (int k = 0; k <= deg; k++)
                        for (int j = 0; j <= deg - k; j++)
                            for (int i = 0; i <= deg - k - j; i++) {
                                int qi = (k * NPOW + j) * NPOW + i;
                                s += q_in[qi] * col[qi];
                            }
                    c_out[ci] += s;
                }
            }
        }
    free(tmp); free(col); free(U);
}

static int general_cube(const pair_t *p, int adj, const double dh[3][3], const double dh_inv[3][3],
                        const int npts[3], const int ngrid[3], const int lb_grid[3],
                        const int periodic[3], double radius, const double *q, double *wq,
                        double *grid, const double *V) {
    int lp = p->lp;
    double gp[3];
    for (int i = 0; i < 3; i++) {
        gp[i] = 0.0;
        for (int j = 0; j < 3; j++) gp[i] += dh_inv[j][i] * p->rp[j];
    }
    /* index box of the cube [rp - r, rp + r]^3 (grid_base_ref_c.cc:703-721) */
    int imin[3] = {INT32_MAX, INT32_MAX, INT32_MAX}, imax[3] = {INT32_MIN, INT32_MIN, INT32_MIN};
    for (int a = -1; a <= 1; a++)
        for (int b = -1; b <= 1; b++)
            for (int e = -1; e <= 1; e++) {
                double x = p->rp[0] + a * radius, y = p->rp[1] + b * radius, z = p->rp[2] + e * radius;
                for (int d = 0; d < 3; d++) {
                    double s = dh_inv[0][d] * x + dh_inv[1][d] * y + dh_inv[2][d] * z;
                    int fl = (int)floor(s), ce = (int)ceil(s);
                    if (fl < imin[d]) imin[d] = fl;
                    if (ce > imax[d]) imax[d] = ce;
                }
            }
    int off[3];
    for (int d = 0; d < 3; d++) off[d] = imod(imin[d] + lb_grid[d], npts[d]);
    double powi[NPOW], powj[NPOW], powk[NPOW];
    double qj[NPOW], qjk[NPOW][NPOW];
    for (int k = imin[2]; k <= imax[2]; k++) {
        double dk = k - gp[2];
        int kidx = periodic[2] ? imod(k, npts[2]) : k - imin[2] + off[2];
        if (kidx < 0 || kidx >= ngrid[2]) return GPW_ERR_OUT_OF_WINDOW;
        powk[0] = 1.0;
        for (int n = 1; n <= lp; n++) powk[n] = powk[n - 1] * dk;
        if (!adj) {
            for (int j = 0; j <= lp; j++)
                for (int i = 0; i <= lp - j; i++) {
                    double s = 0.0;
                    for (int kk = 0; kk <= lp - j - i; kk++) s += q[(kk * NPOW + j) * NPOW + i] * powk[kk];
                    qjk[j][i] = s;
                }
        } else {
            memset(qjk, 0, sizeof(qjk));
        }
        for (int j = imin[1]; j <= imax[1]; j++) {
            double dj = j - gp[1];
            int jidx = periodic[1] ? imod(j, npts[1]) : j - imin[1] + off[1];
            if (jidx < 0 || jidx >= ngrid[1]) return GPW_ERR_OUT_OF_WINDOW;
            /* row bounds from |i h0 + v|^2 <= r^2 (grid_base_ref_c.cc:790-807); the
             * point set must be the reference's, so the same expressions are used */
            double a = 0.0, b = 0.0, cq = 0.0;
            for (int i = 0; i < 3; i++) {
                double pointk = dh[2][i] * dk;
                double pointj = pointk + dh[1][i] * dj;
                double v = pointj - gp[0] * dh[0][i];
                a += dh[0][i] * dh[0][i];
                b += 2.0 * v * dh[0][i];
                cq += v * v;
            }
            double disc = b * b - 4 * a * (cq - radius * radius);
            if (disc < 0.0) continue;
            disc = sqrt(disc);
            int ismin = (int)ceil((-b - disc) / (2.0 * a));
            int ismax = (int)floor((-b + disc) / (2.0 * a));
            powj[0] = 1.0;
            for (int n = 1; n <= lp; n++) powj[n] = powj[n - 1] * dj;
            if (!adj) {
                for (int i = 0; i <= lp; i++) {
                    double s = 0.0;
                    for (int jj = 0; jj <= lp - i; jj++) s += qjk[jj][i] * powj[jj];
                    qj[i] = s;
                }
            } else {
                memset(qj, 0, sizeof(qj));
            }
            for (int i = ismin; i <= ismax; i++) {
                double di = i - gp[0];
                int iidx = periodic[0] ? imod(i, npts[0]) : i - imin[0] + off[0];
                if (iidx < 0 || iidx >= ngrid[0]) return GPW_ERR_OUT_OF_WINDOW;
                double r2 = 0.0;
                for (int cdim = 0; cdim < 3; cdim++) {
                    double rc = di * dh[0][cdim] + dj * dh[1][cdim] + dk * dh[2][cdim];
                    r2 += rc * rc;
                }
                double e = exp(-p->zetp * r2);
                int64_t gidx = ((int64_t)kidx * ngrid[1] + jidx) * ngrid[0] + iidx;
                powi[0] = 1.0;
                for (int n = 1; n <= lp; n++) powi[n] = powi[n - 1] * di;
                if (!adj) {
                    double s = 0.0;
                    for (int n = 0; n <= lp; n++) s += qj[n] * powi[n];
                    grid[gidx] += s * e;
                } else {
                    double ve = V[gidx] * e;
                    for (int n = 0; n <= lp; n++) qj[n] += ve * powi[n];
                }
            }
            if (adj)
                for (int jj = 0; jj <= lp; jj++)
                    for (int i = 0; i <= lp - jj; i++) qjk[jj][i] += qj[i] * powj[jj];
        }
        if (adj)
            for (int j = 0; j <= lp; j++)
                for (int i = 0; i <= lp - j; i++)
                    for (int kk = 0; kk <= lp - j - i; kk++)
                        wq[(kk * NPOW + j) * NPOW + i] += qjk[j][i] * powk[kk];
    }
    return 0;
}

/* ------------------------------------------------------------------------- */
/* One pair, both directions.  adj == 0: grid += rho.  adj == 1: hab += <V|basis>. */
static int pair_run(int adj, int compute_tau, int use_ortho, int la_max, int la_min, int lb_max,
                    int lb_min, double zeta, double zetb, double rscale, const double dh[3][3],
                    const double dh_inv[3][3], const double ra[3], const double rab[3],
                    const int npts[3], const int ngrid[3], const int lb_grid[3],
                    const int periodic[3], double radius, const int lb_cube[3],
                    const int ub_cube[3], int nspheres, const int *sphere_bounds, int maxco,
                    int o1, int o2, const double *pab, double *hab, double *grid,
                    const double *V) {
    if (la_max < 0 || lb_max < 0 || la_min < 0 || lb_min < 0 || la_min > la_max ||
        lb_min > lb_max || la_max > GPW_MAX_L || lb_max > GPW_MAX_L)
        return GPW_ERR_INVALID_ARG;
    pair_t p;
    pair_setup(compute_tau, la_max, la_min, lb_max, lb_min, zeta, zetb, rscale, ra, rab, &p);
    int ldl = ncoset(p.la_max);
    int nloc = ncoset(p.lb_max) * ldl;
    double *loc = (double *)calloc((size_t)nloc, sizeof(double));
    double *c = (double *)calloc(NQ, sizeof(double));
    double *w = (double *)calloc(NQ, sizeof(double));
    int status = 0;
    if (!adj) {
        block_map(compute_tau, 0, la_max, la_min, lb_max, lb_min, zeta, zetb, pab, NULL, maxco, o1,
                  o2, loc, NULL, ldl);
        coef_map(&p, 0, loc, NULL, ldl, c, NULL);
    }
    if (use_ortho) {
        cube_t cb;
        if (cube_parse(sphere_bounds, nspheres, &cb) != 0) {
            status = GPW_ERR_INVALID_ARG;
        } else {
            status = ortho_cube(&p, adj, dh, dh_inv, npts, ngrid, lb_grid, periodic, lb_cube,
                                ub_cube, &cb, c, w, grid, V);
            cube_free(&cb);
        }
    } else {
        double *q = (double *)calloc(NQ, sizeof(double));
        double *wq = (double *)calloc(NQ, sizeof(double));
        if (!adj) lattice_map(p.lp, dh, 0, c, q, NULL, NULL);
        status = general_cube(&p, adj, dh, dh_inv, npts, ngrid, lb_grid, periodic, radius, q, wq,
                              grid, V);
        if (adj) lattice_map(p.lp, dh, 1, NULL, NULL, wq, w);
        free(q); free(wq);
    }
    if (adj && status == 0) {
        coef_map(&p, 1, NULL, loc, ldl, NULL, w);
        block_map(compute_tau, 1, la_max, la_min, lb_max, lb_min, zeta, zetb, NULL, hab, maxco, o1,
                  o2, NULL, loc, ldl);
    }
    free(loc); free(c); free(w);
    return status;
}

static void unpack_dh(const double *dh9, const double *dhi9, double dh[3][3], double dhi[3][3]) {
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) { dh[i][j] = dh9[3 * i + j]; dhi[i][j] = dhi9[3 * i + j]; }
}

/* Same arguments as grid_collocate_pgf_product_rspace (grid_base_ref_c.h:40-67),
 * arrays flattened row-major; grid += rho. */
int gpwo_collocate(int compute_tau, int use_ortho, int la_max, int la_min, int lb_max, int lb_min,
                   double zeta, double zetb, double rscale, const double *dh9,
                   const double *dh_inv9, const double *ra, const double *rab, const int *npts,
                   const int *ngrid, const int *lb_grid, const int *periodic, int lmax,
                   double radius, const int *lb_cube, const int *ub_cube, int nspheres,
                   const int *sphere_bounds, int maxco, int o1, int o2, const double *pab,
                   double *grid) {
    (void)lmax;
    double dh[3][3], dhi[3][3];
    unpack_dh(dh9, dh_inv9, dh, dhi);
    return pair_run(0, compute_tau, use_ortho, la_max, la_min, lb_max, lb_min, zeta, zetb, rscale,
                    dh, dhi, ra, rab, npts, ngrid, lb_grid, periodic, radius, lb_cube, ub_cube,
                    nspheres, sphere_bounds, maxco, o1, o2, pab, NULL, grid, NULL);
}

/* Adjoint: hab[(o2+jco)*maxco + o1+ico] += sum_grid V * d rho / d pab(o2+jco, o1+ico). */
int gpwo_integrate(int compute_tau, int use_ortho, int la_max, int la_min, int lb_max, int lb_min,
                   double zeta, double zetb, double rscale, const double *dh9,
                   const double *dh_inv9, const double *ra, const double *rab, const int *npts,
                   const int *ngrid, const int *lb_grid, const int *periodic, int lmax,
                   double radius, const int *lb_cube, const int *ub_cube, int nspheres,
                   const int *sphere_bounds, int maxco, int o1, int o2, const double *V,
                   double *hab) {
    (void)lmax;
    double dh[3][3], dhi[3][3];
    unpack_dh(dh9, dh_inv9, dh, dhi);
    return pair_run(1, compute_tau, use_ortho, la_max, la_min, lb_max, lb_min, zeta, zetb, rscale,
                    dh, dhi, ra, rab, npts, ngrid, lb_grid, periodic, radius, lb_cube, ub_cube,
                    nspheres, sphere_bounds, maxco, o1, o2, NULL, hab, NULL, V);
}

/* ------------------------------------------------------------------------- */
/* Batches of gpw_task over gpw_grid_desc levels, spread over threads.  Each
 * thread owns private copies of the outputs, summed at the end.             */
typedef struct {
    int adj, tau;
    const gpw_task *tasks;
    int64_t n, first, step;
    const gpw_grid_desc *levels;
    int nlevels;
    const double *pab;
    const double *const *V;
    const int *sphere_table;
    double **grids;   /* private */
    double *hab;      /* private */
    int status;
} job_t;

static int64_t level_size(const gpw_grid_desc *g) {
    return (int64_t)g->ngrid[0] * g->ngrid[1] * g->ngrid[2];
}

static void *job_run(void *arg) {
    job_t *J = (job_t *)arg;
    int *sb = NULL;
    int cap = 0;
    for (int64_t t = J->first; t < J->n; t += J->step) {
        const gpw_task *T = &J->tasks[t];
        const gpw_grid_desc *g = &J->levels[T->level];
        double dh[3][3], dhi[3][3];
        memcpy(dh, g->dh, sizeof(dh));
        memcpy(dhi, g->dh_inv, sizeof(dhi));
        int lbc[3], ubc[3], nsb = 0;
        const int *sbp = NULL;
        if (g->ortho) {
            if (T->sphere_offset >= 0) {
                sbp = J->sphere_table + T->sphere_offset;
                memcpy(lbc, T->lb_cube, sizeof(lbc));
                memcpy(ubc, T->ub_cube, sizeof(ubc));
                nsb = cube_list_len(sbp, 1 << 24);
                if (nsb < 0) { J->status = GPW_ERR_INVALID_ARG; break; }
            } else {
                int need = gpwo_sphere_bounds(T->radius, &g->dh[0][0], lbc, ubc, sb, cap);
                if (need < 0) {
                    cap = -need;
                    sb = (int *)realloc(sb, sizeof(int) * cap);
                    need = gpwo_sphere_bounds(T->radius, &g->dh[0][0], lbc, ubc, sb, cap);
                }
                if (need <= 0) { J->status = GPW_ERR_INVALID_ARG; break; }
                sbp = sb;
                nsb = need;
            }
        }
        int st = pair_run(J->adj, J->tau, g->ortho, T->la_max, T->la_min, T->lb_max, T->lb_min,
                          T->zeta, T->zetb, T->rscale, dh, dhi, T->ra, T->rab, g->npts, g->ngrid,
                          g->lb_grid, g->periodic, T->radius, lbc, ubc, nsb, sbp, T->maxco, T->o1,
                          T->o2, J->pab ? J->pab + T->pab_offset : NULL,
                          J->hab ? J->hab + T->pab_offset : NULL,
                          J->grids ? J->grids[T->level] : NULL,
                          J->V ? J->V[T->level] : NULL);
        if (st) { J->status = st; break; }
    }
    free(sb);
    return NULL;
}

/* The threads' private grids (or hab arrays) summed into thread 0's, each
 * element over t = 1, 2, ... in order (the result of a serial sum); nparts
 * threads take contiguous parts of the arrays. */
typedef struct {
    job_t *jobs;
    int nthreads, adj, nlevels, part, nparts;
    const gpw_grid_desc *levels;
    double *const *grids;
    double *hab;
    int64_t hab_len;
} reduce_t;

static void *reduce_run(void *arg) {
    const reduce_t *R = (const reduce_t *)arg;
    for (int l = 0; l < (R->adj ? 1 : R->nlevels); l++) {
        const int64_t n = R->adj ? R->hab_len : level_size(&R->levels[l]);
        const int64_t i0 = n * R->part / R->nparts, i1 = n * (R->part + 1) / R->nparts;
        double *out = R->adj ? R->hab : R->grids[l];
        for (int t = 1; t < R->nthreads; t++) {
            const double *src = R->adj ? R->jobs[t].hab : R->jobs[t].grids[l];
            for (int64_t i = i0; i < i1; i++) out[i] += src[i];
        }
    }
    return NULL;
}

/* grids[l] += rho (adj 0) or hab += <V|basis> (adj 1) for a task batch. */
int gpwo_batch(int adj, int compute_tau, const gpw_task *tasks, int64_t ntasks,
               const gpw_grid_desc *levels, int nlevels, const int *sphere_table,
               const double *pab, double *const *grids, const double *const *V, double *hab,
               int64_t hab_len, int nthreads) {
    if (nthreads < 1) nthreads = 1;
    job_t *jobs = (job_t *)calloc((size_t)nthreads, sizeof(job_t));
    pthread_t *th = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
    int status = 0;
    for (int t = 0; t < nthreads; t++) {
        job_t *J = &jobs[t];
        J->adj = adj; J->tau = compute_tau; J->tasks = tasks; J->n = ntasks;
        J->first = t; J->step = nthreads; J->levels = levels; J->nlevels = nlevels;
        J->pab = pab; J->V = V; J->sphere_table = sphere_table;
        if (!adj) {
            J->grids = (double **)calloc((size_t)nlevels, sizeof(double *));
            for (int l = 0; l < nlevels; l++)
                J->grids[l] = t == 0 ? grids[l] : (double *)calloc((size_t)level_size(&levels[l]), sizeof(double));
        } else {
            J->hab = t == 0 ? hab : (double *)calloc((size_t)hab_len, sizeof(double));
        }
    }
    for (int t = 1; t < nthreads; t++) pthread_create(&th[t], NULL, job_run, &jobs[t]);
    job_run(&jobs[0]);
    for (int t = 1; t < nthreads; t++) pthread_join(th[t], NULL);
    if (nthreads > 1) {
        reduce_t *R = (reduce_t *)calloc((size_t)nthreads, sizeof(reduce_t));
        for (int t = 0; t < nthreads; t++) {
            R[t].jobs = jobs; R[t].nthreads = nthreads; R[t].adj = adj; R[t].nlevels = nlevels;
            R[t].part = t; R[t].nparts = nthreads; R[t].levels = levels; R[t].grids = grids;
            R[t].hab = hab; R[t].hab_len = hab_len;
        }
        for (int t = 1; t < nthreads; t++) pthread_create(&th[t], NULL, reduce_run, &R[t]);
        reduce_run(&R[0]);
        for (int t = 1; t < nthreads; t++) pthread_join(th[t], NULL);
        free(R);
    }
    for (int t = 0; t < nthreads; t++) {
        job_t *J = &jobs[t];
        if (J->status && !status) status = J->status;
        if (t > 0) {
            if (!adj)
                for (int l = 0; l < nlevels; l++) free(J->grids[l]);
            else
                free(J->hab);
        }
        free(J->grids);
    }
    free(jobs); free(th);
    return status;
}
