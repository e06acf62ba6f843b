// Plain FP64 collocate / integrate: one CTA per pair, FP64 everywhere, grid
// updates by FP64 atomics.  This is the straightforward GPU form of the
// reference's per-pair loops (grid_collocate_core, grid_base_ref_c.cc:403-508;
// grid_collocate_general, :593-846) and the denominator the tiled path is
// measured against.
#include <cuda_runtime.h>

#include "gpw_coef.cuh"
#include "gpw_ff.cuh"
#include "gpw_internal.h"

namespace gpw {

// ---------------------------------------------------------------------------
// cube lists: sphere rule or explicit (random-access) table
// table layout at g.table_off: kgmin, then (jgmin, rowstart) per kf, then igmin per row
__device__ __forceinline__ int cube_jgmin(const PairGeom &g, const LevelDev &lv, const int *table,
                                          int kf, double r2, double &remk) {
    if (g.table_off < 0) {
        remk = rule_remk(r2, kf, lv.dh[2][2]);
        return -rule_jmax(remk, lv.dh[1][1]);
    }
    const int *T = table + g.table_off;
    remk = 0.0;
    return T[1 + 2 * (kf - T[0])];
}
__device__ __forceinline__ int cube_igmin(const PairGeom &g, const LevelDev &lv, const int *table,
                                          int kf, int jf, int jgmin, double remk) {
    if (g.table_off < 0) return -rule_imax(remk, jf, lv.dh[1][1], lv.dh[0][0]);
    const int *T = table + g.table_off;
    const int nk = 1 - T[0];
    return T[1 + 2 * nk + T[2 + 2 * (kf - T[0])] + (jf - jgmin)];
}

// 1-D tables tab[k][gi] = t^k exp(-zetp t^2), t = (lo+gi)*h - off, k < L  (grid_fill_pol,
// grid_base_ref_c.cc:355-400; evaluated directly instead of by recurrence)
__device__ __forceinline__ void fill_table(double *tab, int n, int L, int lo, double h, double off,
                                           double zetp) {
    for (int gi = threadIdx.x; gi < n; gi += blockDim.x) {
        const double t = (double)(lo + gi) * h - off;
        double e = exp(-zetp * t * t);
        for (int k = 0; k < L; k++) {
            tab[k * n + gi] = e;
            e *= t;
        }
    }
}

// ---------------------------------------------------------------------------
// pair set-up: packed coefficients c (ortho) or q (general, lattice basis)
__global__ void k_prep(const PairGeom *__restrict__ geoms, const LevelDev *__restrict__ levels,
                       const double *__restrict__ tmat, int tau, const double *__restrict__ pab,
                       double *__restrict__ coef) {
    extern __shared__ double sm[];
    const PairGeom &g = geoms[blockIdx.x];  // read in place (L1), not copied per thread
    CoefWs w;
    w.carve(sm, g.la_max, g.lb_max);
    fill_alpha(w, g);
    fill_local_block(w, g, tau, pab);
    __syncthreads();
    const int nc = ncoef(g.lp);
    if (g.ortho) {
        forward_coef(w, g, coef + g.coef_off);
        return;
    }
    double *c = w.end();  // packed c, before the lattice transform
    forward_coef(w, g, c);
    __syncthreads();
    // q[k][j][i] = sum over same-degree (lz,ly,lx) of T * c; T in lp = kMaxLp packing
    const LevelDev &lv = levels[g.level];
    const double *Tm = tmat + lv.tmat_off;
    const int NT = ncoef(kMaxLp);
    for (int t = threadIdx.x; t < nc; t += blockDim.x) {
        // decode t -> (k, j, i) in lp packing
        int k = 0, j = 0, i = 0;
        {
            int r = t;
            for (k = 0; k <= g.lp; k++) {
                const int cnt = ((g.lp - k + 1) * (g.lp - k + 2)) / 2;
                if (r < cnt) break;
                r -= cnt;
            }
            const int q = g.lp - k;
            for (j = 0; j <= q; j++) {
                if (r <= q - j) break;
                r -= q - j + 1;
            }
            i = r;
        }
        const int n = i + j + k;
        const int row = pidx(kMaxLp, k, j, i);
        double s = 0.0;
        for (int lz = 0; lz <= n; lz++)
            for (int ly = 0; ly <= n - lz; ly++) {
                const int lx = n - lz - ly;
                s += Tm[(int64_t)row * NT + pidx(kMaxLp, lz, ly, lx)] * c[pidx(g.lp, lz, ly, lx)];
            }
        coef[g.coef_off + t] = s;
    }
}

int smem_prep(int A, int B) {
    // workspace + a packed coefficient vector for the general-cell transform
    return 8 * (coef_ws_doubles(A, B) + ncoef(A + B));
}

// ---------------------------------------------------------------------------
// integrate back-transform: moments -> hab
__global__ void k_backtransform(const PairGeom *__restrict__ geoms, const LevelDev *__restrict__ levels,
                                const double *__restrict__ tmat, int tau,
                                const double *__restrict__ mom, double *__restrict__ hab) {
    extern __shared__ double sm[];
    const PairGeom &g = geoms[blockIdx.x];  // read in place (L1), not copied per thread
    CoefWs w;
    w.carve(sm, g.la_max, g.lb_max);
    fill_alpha(w, g);
    const int nc = ncoef(g.lp);
    const double *W = mom + g.coef_off;
    double *Wc = w.end();
    if (!g.ortho) {
        // Wc[lz][ly][lx] = sum over same-degree (k,j,i) of T[(k,j,i)][(lz,ly,lx)] * Wq[k][j][i]
        const LevelDev &lv = levels[g.level];
        const double *Tm = tmat + lv.tmat_off;
        const int NT = ncoef(kMaxLp);
        for (int t = threadIdx.x; t < nc; t += blockDim.x) {
            int lz = 0, ly = 0, lx = 0;
            int r = t;
            for (lz = 0; lz <= g.lp; lz++) {
                const int cnt = ((g.lp - lz + 1) * (g.lp - lz + 2)) / 2;
                if (r < cnt) break;
                r -= cnt;
            }
            const int q = g.lp - lz;
            for (ly = 0; ly <= q; ly++) {
                if (r <= q - ly) break;
                r -= q - ly + 1;
            }
            lx = r;
            const int n = lx + ly + lz;
            const int col = pidx(kMaxLp, lz, ly, lx);
            double s = 0.0;
            for (int k = 0; k <= n; k++)
                for (int j = 0; j <= n - k; j++) {
                    const int i = n - k - j;
                    s += Tm[(int64_t)pidx(kMaxLp, k, j, i) * NT + col] * W[pidx(g.lp, k, j, i)];
                }
            Wc[t] = s;
        }
        W = Wc;
    }
    __syncthreads();
    adjoint_coef(w, g, tau, W, hab);
}

// ---------------------------------------------------------------------------
// orthorhombic collocate, one CTA per pair
int smem_ortho_fp64(const PairGeom &g, int extra) {
    const int L = g.lp + 1 + extra;
    const int nx = g.hi[0] - g.lb[0] + 1, ny = g.hi[1] - g.lb[1] + 1, nz = g.hi[2] - g.lb[2] + 1;
    return 8 * (L * L * L + L * (nx + ny + nz) + L * L + ny * L) + 8 * ny;
}

// kAcc: the row accumulators of the adjoint, L <= kAcc (kNPow for integrate,
// kNPowB for the backward pass's moments to degree lp + 2: more accumulators cost
// the plain integrate registers and shuffles)
template <bool kAdj, int kAcc = kNPow>
__global__ void __launch_bounds__(256)
k_ortho_fp64(const PairGeom *__restrict__ geoms, int first, const LevelDev *__restrict__ levels,
             const int *__restrict__ table, const double *__restrict__ coef, double *__restrict__ mom,
             GridPtrs grids, int *status, int extra) {
    extern __shared__ double sm[];
    const PairGeom g = geoms[first + blockIdx.x];
    const LevelDev &lv = levels[g.level];
    double *__restrict__ grid = grids.p[g.level];
    const int lp = g.lp + extra, L = lp + 1;
    const int64_t mom_off = extra ? g.mom_ext_off : g.coef_off;
    const int nx = g.hi[0] - g.lb[0] + 1, ny = g.hi[1] - g.lb[1] + 1, nz = g.hi[2] - g.lb[2] + 1;
    double *C = sm;                // [lz][ly][lx] dense: coefficients, or moments (adjoint)
    double *Xt = C + L * L * L;    // [k][gi]
    double *Yt = Xt + L * nx;
    double *Zt = Yt + L * ny;
    double *Cxy = Zt + L * nz;     // [ly][lx]
    double *Cx = Cxy + L * L;      // [row][lx]
    int *rows = (int *)(Cx + ny * L);  // per row: igmin, j
    const int tid = threadIdx.x, nthr = blockDim.x;
    for (int t = tid; t < L * L * L; t += nthr) {
        const int lx = t % L, ly = (t / L) % L, lz = t / (L * L);
        C[t] = (!kAdj && lx + ly + lz <= lp) ? coef[g.coef_off + pidx(lp, lz, ly, lx)] : 0.0;
    }
    fill_table(Xt, nx, L, g.lb[0], lv.dh[0][0], g.off[0], g.zetp);
    fill_table(Yt, ny, L, g.lb[1], lv.dh[1][1], g.off[1], g.zetp);
    fill_table(Zt, nz, L, g.lb[2], lv.dh[2][2], g.off[2], g.zetp);
    __syncthreads();
    const double r2 = rmul(g.radius, g.radius);
    const int lane = tid & 31, warp = tid >> 5, nwarp = nthr >> 5;
    for (int kg = g.kgmin; kg <= 1 - g.kgmin; kg++) {
        const int kf = fold(kg);
        const int k = axis_index(lv.periodic[2], g.cc[2], kg, g.lb[2], lv.lb_grid[2], lv.npts[2],
                                 lv.ngrid[2]);
        if (k < 0) {
            if (tid == 0) atomicOr(status, kStatOutOfWindow);
            continue;
        }
        double remk;
        const int jgmin = cube_jgmin(g, lv, table, kf, r2, remk);
        const int nrows = 2 - 2 * jgmin;
        const double *Zk = Zt + (kg - g.lb[2]);
        if (!kAdj) {
            // Cxy[ly][lx] = sum_lz C[lz][ly][lx] Z[lz]
            for (int t = tid; t < L * L; t += nthr) {
                const int lx = t % L, ly = t / L;
                double s = 0.0;
                for (int lz = 0; lz <= lp - lx - ly; lz++) s += C[(lz * L + ly) * L + lx] * Zk[lz * nz];
                Cxy[t] = s;
            }
            __syncthreads();
        }
        for (int t = tid; t < nrows * L; t += nthr) {
            const int row = t / L, lx = t % L;
            const int jg = jgmin + row;
            if (!kAdj) {
                double s = 0.0;
                for (int ly = 0; ly <= lp - lx; ly++) s += Cxy[ly * L + lx] * Yt[ly * ny + (jg - g.lb[1])];
                Cx[t] = s;
            }
            if (lx == 0) {
                rows[2 * row] = cube_igmin(g, lv, table, kf, fold(jg), jgmin, remk);
                rows[2 * row + 1] = axis_index(lv.periodic[1], g.cc[1], jg, g.lb[1], lv.lb_grid[1],
                                               lv.npts[1], lv.ngrid[1]);
            }
        }
        __syncthreads();
        for (int row = warp; row < nrows; row += nwarp) {
            const int igmin = rows[2 * row], j = rows[2 * row + 1];
            if (j < 0) {
                if (lane == 0) atomicOr(status, kStatOutOfWindow);
                continue;
            }
            const int64_t rowbase = ((int64_t)k * lv.ngrid[1] + j) * lv.ngrid[0];
            double acc[kAcc];
#pragma unroll
            for (int lx = 0; lx < kAcc; lx++) acc[lx] = 0.0;
            for (int ig = igmin + lane; ig <= 1 - igmin; ig += 32) {
                const int i = axis_index(lv.periodic[0], g.cc[0], ig, g.lb[0], lv.lb_grid[0],
                                         lv.npts[0], lv.ngrid[0]);
                if (i < 0) {
                    atomicOr(status, kStatOutOfWindow);
                    continue;
                }
                const double *Xi = Xt + (ig - g.lb[0]);
                if (!kAdj) {
                    double v = 0.0;
                    for (int lx = 0; lx < L; lx++) v += Cx[row * L + lx] * Xi[lx * nx];
                    atomicAdd(grid + rowbase + i, v);
                } else {
                    const double v = grid[rowbase + i];
#pragma unroll
                    for (int lx = 0; lx < kAcc; lx++)
                        if (lx < L) acc[lx] += v * Xi[lx * nx];
                }
            }
            if (kAdj) {
                // warp-shuffle reduction of the row moments
#pragma unroll
                for (int lx = 0; lx < kAcc; lx++) {
                    double v = acc[lx];
                    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
                    acc[lx] = v;
                }
                if (lane == 0)
                    for (int lx = 0; lx < L; lx++) Cx[row * L + lx] = acc[lx];
            }
        }
        __syncthreads();
        if (kAdj) {
            // Cxy[ly][lx] = sum_rows Cx[row][lx] Y[ly][jg];  C[lz][ly][lx] += Cxy * Z[lz]
            for (int t = tid; t < L * L; t += nthr) {
                const int lx = t % L, ly = t / L;
                if (lx + ly > lp) continue;
                double s = 0.0;
                for (int row = 0; row < nrows; row++)
                    if (rows[2 * row + 1] >= 0) s += Cx[row * L + lx] * Yt[ly * ny + (jgmin + row - g.lb[1])];
                for (int lz = 0; lz <= lp - lx - ly; lz++) C[(lz * L + ly) * L + lx] += s * Zk[lz * nz];
            }
            __syncthreads();
        }
    }
    if (kAdj) {
        for (int t = tid; t < L * L * L; t += nthr) {
            const int lx = t % L, ly = (t / L) % L, lz = t / (L * L);
            if (lx + ly + lz <= lp) mom[mom_off + pidx(lp, lz, ly, lx)] = C[t];
        }
    }
}

// ---------------------------------------------------------------------------
// general cell, one CTA per pair (row bounds: general_row, gpw_common.cuh)
// (one row of margin: a geometry update moves a box's extent by at most one)
int smem_general_fp64(const PairGeom &g, int extra) {
    const int L = g.lp + 1 + extra;
    const int ny = g.hi[1] - g.cc[1] + 2;
    return 8 * (L * L * L + L * L + ny * L) + 12 * ny;
}

template <bool kAdj>
__global__ void __launch_bounds__(256)
k_general_fp64(const PairGeom *__restrict__ geoms, int first, const LevelDev *__restrict__ levels,
               const double *__restrict__ coef, double *__restrict__ mom, GridPtrs grids,
               int *status, int extra) {
    extern __shared__ double sm[];
    const PairGeom g = geoms[first + blockIdx.x];
    const LevelDev &lv = levels[g.level];
    double *__restrict__ grid = grids.p[g.level];
    const int lp = g.lp + extra, L = lp + 1;
    const int64_t mom_off = extra ? g.mom_ext_off : g.coef_off;
    const int ny = g.hi[1] - g.cc[1] + 1;
    double *Q = sm;              // [k][j][i] dense
    double *Qjk = Q + L * L * L; // [j][i]
    double *Qj = Qjk + L * L;    // [row][i]
    int *rows = (int *)(Qj + ny * L);  // ismin, ismax, jidx
    const int tid = threadIdx.x, nthr = blockDim.x;
    const int lane = tid & 31, warp = tid >> 5, nwarp = nthr >> 5;
    for (int t = tid; t < L * L * L; t += nthr) {
        const int i = t % L, j = (t / L) % L, k = t / (L * L);
        Q[t] = (!kAdj && i + j + k <= lp) ? coef[g.coef_off + pidx(lp, k, j, i)] : 0.0;
    }
    __syncthreads();
    int off[3];
    for (int d = 0; d < 3; d++) off[d] = imod(g.cc[d] + lv.lb_grid[d], lv.npts[d]);
    for (int kk = g.cc[2]; kk <= g.hi[2]; kk++) {
        const double dk = rsub((double)kk, g.off[2]);
        const int kidx = lv.periodic[2] ? imod(kk, lv.npts[2]) : kk - g.cc[2] + off[2];
        if (kidx < 0 || kidx >= lv.ngrid[2]) {
            if (tid == 0) atomicOr(status, kStatOutOfWindow);
            continue;
        }
        if (!kAdj) {
            for (int t = tid; t < L * L; t += nthr) {
                const int i = t % L, j = t / L;
                double s = 0.0, p = 1.0;
                for (int k = 0; k <= lp - i - j; k++) {
                    s += Q[(k * L + j) * L + i] * p;
                    p *= dk;
                }
                Qjk[t] = s;
            }
            __syncthreads();
        }
        for (int t = tid; t < ny * L; t += nthr) {
            const int row = t / L, i = t % L;
            const int jj = g.cc[1] + row;
            const double dj = rsub((double)jj, g.off[1]);
            if (!kAdj) {
                double s = 0.0, p = 1.0;
                for (int j = 0; j <= lp - i; j++) {
                    s += Qjk[j * L + i] * p;
                    p *= dj;
                }
                Qj[t] = s;
            }
            if (i == 0) {
                int ismin = 0, ismax = -1;
                if (!general_row(lv.dh, g.off, dj, dk, g.radius, ismin, ismax)) { ismin = 0; ismax = -1; }
                rows[3 * row] = ismin;
                rows[3 * row + 1] = ismax;
                rows[3 * row + 2] = lv.periodic[1] ? imod(jj, lv.npts[1]) : jj - g.cc[1] + off[1];
            }
        }
        __syncthreads();
        for (int row = warp; row < ny; row += nwarp) {
            const int ismin = rows[3 * row], ismax = rows[3 * row + 1], jidx = rows[3 * row + 2];
            if (ismax < ismin) continue;
            if (jidx < 0 || jidx >= lv.ngrid[1]) {
                if (lane == 0) atomicOr(status, kStatOutOfWindow);
                continue;
            }
            const double dj = (double)(g.cc[1] + row) - g.off[1];
            const int64_t rowbase = ((int64_t)kidx * lv.ngrid[1] + jidx) * lv.ngrid[0];
            double acc[kNPow];
#pragma unroll
            for (int n = 0; n < kNPow; n++) acc[n] = 0.0;
            for (int ii = ismin + lane; ii <= ismax; ii += 32) {
                const int iidx = lv.periodic[0] ? imod(ii, lv.npts[0]) : ii - g.cc[0] + off[0];
                if (iidx < 0 || iidx >= lv.ngrid[0]) {
                    atomicOr(status, kStatOutOfWindow);
                    continue;
                }
                const double di = (double)ii - g.off[0];
                double r2 = 0.0;
                for (int c = 0; c < 3; c++) {
                    const double rc = di * lv.dh[0][c] + dj * lv.dh[1][c] + dk * lv.dh[2][c];
                    r2 += rc * rc;
                }
                const double e = exp(-g.zetp * r2);
                if (!kAdj) {
                    double s = 0.0, p = 1.0;
                    for (int n = 0; n < L; n++) {
                        s += Qj[row * L + n] * p;
                        p *= di;
                    }
                    atomicAdd(grid + rowbase + iidx, s * e);
                } else {
                    const double ve = grid[rowbase + iidx] * e;
                    double p = 1.0;
#pragma unroll
                    for (int n = 0; n < kNPow; n++) {
                        if (n < L) acc[n] += ve * p;
                        p *= di;
                    }
                }
            }
            if (kAdj) {
#pragma unroll
                for (int n = 0; n < kNPow; n++) {
                    double v = acc[n];
                    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
                    acc[n] = v;
                }
                if (lane == 0)
                    for (int n = 0; n < L; n++) Qj[row * L + n] = acc[n];
            }
        }
        __syncthreads();
        if (kAdj) {
            // Qjk[j][i] = sum_rows Qj[row][i] dj^j;  Q[k][j][i] += Qjk[j][i] dk^k
            for (int t = tid; t < L * L; t += nthr) {
                const int i = t % L, j = t / L;
                if (i + j > lp) continue;
                double s = 0.0;
                for (int row = 0; row < ny; row++) {
                    if (rows[3 * row + 1] < rows[3 * row]) continue;
                    const double dj = (double)(g.cc[1] + row) - g.off[1];
                    double p = 1.0;
                    for (int e = 0; e < j; e++) p *= dj;
                    s += Qj[row * L + i] * p;
                }
                double p = 1.0;
                for (int k = 0; k <= lp - i - j; k++) {
                    Q[(k * L + j) * L + i] += s * p;
                    p *= dk;
                }
            }
            __syncthreads();
        }
    }
    if (kAdj) {
        for (int t = tid; t < L * L * L; t += nthr) {
            const int i = t % L, j = (t / L) % L, k = t / (L * L);
            if (i + j + k <= lp) mom[mom_off + pidx(lp, k, j, i)] = Q[t];
        }
    }
}


// ---------------------------------------------------------------------------
// General cell in float-float (the mixed path): the structure of k_general_fp64
// -- one CTA per pair, the lattice-basis polynomial contracted over k, then j,
// per row of the index box, the row's i-range from the reference's quadratic
// (FP64, general_row, so the point set is the reference's) -- with every
// per-point operation in float-float instead of FP64 (GB300 runs FP64 at ~1/64
// of its FP32 rate):
//   r^2(di) = G00 di^2 + A1 di + A0 per row (metric G = dh dh^T; A1, A0 per row
//   in FP64, split to float-float), exp(-zetp r^2) by ff_exp, the polynomial in
//   di by Horner; collocate adds hi + lo to the grid with FP64 atomics,
//   integrate reduces V exp(..) di^n over each row with warp shuffles.
__device__ __forceinline__ ff ff_shfl_xor(ff v, int o) {
    return {__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
}

template <bool kAdj>
__global__ void __launch_bounds__(256)
k_general_ff(const PairGeom *__restrict__ geoms, int first, const LevelDev *__restrict__ levels,
             const double *__restrict__ coef, double *__restrict__ mom, GridPtrs grids, int *status) {
    extern __shared__ double smd[];
    const PairGeom g = geoms[first + blockIdx.x];
    const LevelDev &lv = levels[g.level];
    double *__restrict__ grid = grids.p[g.level];
    const int lp = g.lp, L = lp + 1;
    const int ny = g.hi[1] - g.cc[1] + 1;
    ff *Q = reinterpret_cast<ff *>(smd);  // [k][j][i] dense
    ff *Qjk = Q + L * L * L;              // [j][i]
    ff *Qj = Qjk + L * L;                 // [row][i]
    ff *rc = Qj + ny * L;                 // per row: a1, a0, d0 (r^2 along the row, first di)
    ff *powj = rc + 3 * ny;               // integrate: per row dj^j, j <= lp
    int *rows = reinterpret_cast<int *>(powj + ny * L);  // ismin, ismax, jidx
    const int tid = threadIdx.x, nthr = blockDim.x;
    const int lane = tid & 31, warp = tid >> 5, nwarp = nthr >> 5;
    for (int t = tid; t < L * L * L; t += nthr) {
        const int i = t % L, j = (t / L) % L, k = t / (L * L);
        Q[t] = (!kAdj && i + j + k <= lp) ? ff_from_double(coef[g.coef_off + pidx(lp, k, j, i)]) : ff{0.0f, 0.0f};
    }
    // metric of the lattice steps
    double G[3][3];
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) G[a][b] = lv.dh[a][0] * lv.dh[b][0] + lv.dh[a][1] * lv.dh[b][1] + lv.dh[a][2] * lv.dh[b][2];
    const ff g00 = ff_from_double(G[0][0]);
    const ff mz = ff_from_double(-g.zetp);
    __syncthreads();
    int off[3];
    for (int d = 0; d < 3; d++) off[d] = imod(g.cc[d] + lv.lb_grid[d], lv.npts[d]);
    for (int kk = g.cc[2]; kk <= g.hi[2]; kk++) {
        const double dk = rsub((double)kk, g.off[2]);
        const int kidx = lv.periodic[2] ? imod(kk, lv.npts[2]) : kk - g.cc[2] + off[2];
        if (kidx < 0 || kidx >= lv.ngrid[2]) {
            if (tid == 0) atomicOr(status, kStatOutOfWindow);
            continue;
        }
        const ff dkf = ff_from_double(dk);
        if (!kAdj) {
            for (int t = tid; t < L * L; t += nthr) {
                const int i = t % L, j = t / L;
                ff s = {0.0f, 0.0f};
                for (int k = lp - i - j; k >= 0; k--) s = ff_fma(s, dkf, Q[(k * L + j) * L + i]);
                Qjk[t] = s;
            }
            __syncthreads();
        }
        // rows: the reference's i-range (FP64 quadratic), one row per lane
        for (int row = tid; row < ny; row += nthr) {
            const int jj = g.cc[1] + row;
            const double dj = rsub((double)jj, g.off[1]);
            int ismin = 0, ismax = -1;
            if (!general_row(lv.dh, g.off, dj, dk, g.radius, ismin, ismax)) { ismin = 0; ismax = -1; }
            rows[3 * row] = ismin;
            rows[3 * row + 1] = ismax;
            rows[3 * row + 2] = lv.periodic[1] ? imod(jj, lv.npts[1]) : jj - g.cc[1] + off[1];
            // r^2 = G00 di^2 + A1 di + A0 along the row; di = (ismin - off0) + n
            rc[3 * row] = ff_from_double(2.0 * (G[0][1] * dj + G[0][2] * dk));
            rc[3 * row + 1] = ff_from_double(G[1][1] * dj * dj + 2.0 * G[1][2] * dj * dk + G[2][2] * dk * dk);
            rc[3 * row + 2] = ff_from_double((double)ismin - g.off[0]);
            if (kAdj) {
                const ff djf = ff_from_double(dj);
                ff p = {1.0f, 0.0f};
                for (int j = 0; j <= lp; j++) {
                    powj[row * L + j] = p;
                    p = ff_mul(p, djf);
                }
            }
        }
        if (!kAdj) {
            for (int t = tid; t < ny * L; t += nthr) {
                const int row = t / L, i = t % L;
                const ff djf = ff_from_double(rsub((double)(g.cc[1] + row), g.off[1]));
                ff s = {0.0f, 0.0f};
                for (int j = lp - i; j >= 0; j--) s = ff_fma(s, djf, Qjk[j * L + i]);
                Qj[t] = s;
            }
        }
        __syncthreads();
        for (int row = warp; row < ny; row += nwarp) {
            const int ismin = rows[3 * row], ismax = rows[3 * row + 1], jidx = rows[3 * row + 2];
            if (ismax < ismin) continue;
            if (jidx < 0 || jidx >= lv.ngrid[1]) {
                if (lane == 0) atomicOr(status, kStatOutOfWindow);
                continue;
            }
            const ff a1 = rc[3 * row], a0 = rc[3 * row + 1], d0 = rc[3 * row + 2];
            const int64_t rowbase = ((int64_t)kidx * lv.ngrid[1] + jidx) * lv.ngrid[0];
            ff acc[kNPow];
#pragma unroll
            for (int n = 0; n < kNPow; n++) acc[n] = ff{0.0f, 0.0f};
            for (int ii = ismin + lane; ii <= ismax; ii += 32) {
                const int iidx = lv.periodic[0] ? imod(ii, lv.npts[0]) : ii - g.cc[0] + off[0];
                if (iidx < 0 || iidx >= lv.ngrid[0]) {
                    atomicOr(status, kStatOutOfWindow);
                    continue;
                }
                const ff di = ff_add(d0, ff{(float)(ii - ismin), 0.0f});
                const ff r2 = ff_fma(ff_fma(g00, di, a1), di, a0);
                const ff e = ff_exp(ff_mul(r2, mz));
                if (!kAdj) {
                    ff s = Qj[row * L + lp];
                    for (int n = lp - 1; n >= 0; n--) s = ff_fma(s, di, Qj[row * L + n]);
                    const ff v = ff_mul(s, e);
                    atomicAdd(grid + rowbase + iidx, (double)v.hi + (double)v.lo);
                } else {
                    ff p = ff_mul(ff_from_double(grid[rowbase + iidx]), e);
#pragma unroll
                    for (int n = 0; n < kNPow; n++) {  // L is uniform over the CTA
                        if (n >= L) break;
                        acc[n] = ff_add(acc[n], p);
                        p = ff_mul(p, di);
                    }
                }
            }
            if (kAdj) {
#pragma unroll
                for (int n = 0; n < kNPow; n++) {
                    if (n >= L) break;
                    ff v = acc[n];
                    for (int o = 16; o > 0; o >>= 1) v = ff_add(v, ff_shfl_xor(v, o));
                    acc[n] = v;
                }
                if (lane == 0)
                    for (int n = 0; n < L; n++) Qj[row * L + n] = acc[n];
            }
        }
        __syncthreads();
        if (kAdj) {
            // Qjk[j][i] = sum_rows Qj[row][i] dj^j;  Q[k][j][i] += Qjk[j][i] dk^k
            for (int t = tid; t < L * L; t += nthr) {
                const int i = t % L, j = t / L;
                if (i + j > lp) continue;
                ff s = {0.0f, 0.0f};
                for (int row = 0; row < ny; row++) {
                    if (rows[3 * row + 1] < rows[3 * row]) continue;
                    s = ff_fma(Qj[row * L + i], powj[row * L + j], s);
                }
                ff p = {1.0f, 0.0f};
                for (int k = 0; k <= lp - i - j; k++) {
                    Q[(k * L + j) * L + i] = ff_fma(s, p, Q[(k * L + j) * L + i]);
                    p = ff_mul(p, dkf);
                }
            }
            __syncthreads();
        }
    }
    if (kAdj) {
        for (int t = tid; t < L * L * L; t += nthr) {
            const int i = t % L, j = (t / L) % L, k = t / (L * L);
            if (i + j + k <= lp) mom[g.coef_off + pidx(lp, k, j, i)] = (double)Q[t].hi + (double)Q[t].lo;
        }
    }
}

// ---------------------------------------------------------------------------
// bytes: the CTA's whole shared memory; a kernel's static shared arrays come out of it
static cudaError_t set_smem(const void *fn, int bytes) {
    cudaFuncAttributes a;
    cudaError_t e = cudaFuncGetAttributes(&a, fn);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes - (int)a.sharedSizeBytes);
}

// Opt every dynamic-shared-memory kernel of this file into the device maximum once,
// so that launches (and CUDA graph capture) need no attribute calls.
cudaError_t fp64_kernel_attributes(int smem_max) {
    const void *fns[] = {(const void *)k_prep, (const void *)k_backtransform,
                         (const void *)k_ortho_fp64<false>, (const void *)k_ortho_fp64<true>,
                         (const void *)k_ortho_fp64<true, kNPowB>,
                         (const void *)k_general_fp64<false>, (const void *)k_general_fp64<true>,
                         (const void *)k_general_ff<false>, (const void *)k_general_ff<true>};
    for (const void *fn : fns) {
        cudaError_t e = set_smem(fn, smem_max);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t launch_prep(const TaskSet &ts, const double *d_pab, cudaStream_t s) {
    if (ts.ntasks == 0) return cudaSuccess;
    const int smem = smem_prep(ts.max_A, ts.max_B);
    ts.n_kernels++;
    k_prep<<<(unsigned)ts.ntasks, 128, smem, s>>>(ts.d_geom, ts.plan->d_levels, ts.plan->d_tmat,
                                                  ts.tau, d_pab, ts.d_coef);
    return cudaGetLastError();
}

static cudaError_t launch_fp64_impl(const TaskSet &ts, const GridPtrs &g, bool adj, int kind, int extra,
                                    double *mom, cudaStream_t s) {
    for (const Chunk &c0 : ts.chunks) {
        Chunk c = c0;
        if (extra) c.smem_bytes = c0.smem_ext;
        if (c.count == 0 || (kind >= 0 && c.kind != kind)) continue;
        cudaError_t e;
        ProfScope prof(ts, s);
        if (c.kind == 0) {
            if (adj && extra)
                k_ortho_fp64<true, kNPowB><<<c.count, 256, c.smem_bytes, s>>>(ts.d_geom, c.first, ts.plan->d_levels,
                                                                             ts.d_table, ts.d_coef, mom, g,
                                                                             ts.d_status, extra);
            else if (adj)
                k_ortho_fp64<true><<<c.count, 256, c.smem_bytes, s>>>(ts.d_geom, c.first, ts.plan->d_levels,
                                                                     ts.d_table, ts.d_coef, mom, g,
                                                                     ts.d_status, 0);
            else
                k_ortho_fp64<false><<<c.count, 256, c.smem_bytes, s>>>(ts.d_geom, c.first, ts.plan->d_levels,
                                                                      ts.d_table, ts.d_coef, mom, g,
                                                                      ts.d_status, 0);
        } else {
            if (adj)
                k_general_fp64<true><<<c.count, 256, c.smem_bytes, s>>>(ts.d_geom, c.first, ts.plan->d_levels,
                                                                       ts.d_coef, mom, g, ts.d_status, extra);
            else
                k_general_fp64<false><<<c.count, 256, c.smem_bytes, s>>>(ts.d_geom, c.first, ts.plan->d_levels,
                                                                        ts.d_coef, mom, g, ts.d_status, 0);
        }
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// general-cell pairs of a mixed call: the float-float kernel
int smem_general_ff(const PairGeom &g) {
    const int L = g.lp + 1;
    const int ny = g.hi[1] - g.cc[1] + 2;  // one row of margin, as smem_general_fp64
    return 8 * (L * L * L + L * L + 2 * ny * L + 3 * ny) + 12 * ny;
}

// one launch over all general-cell pairs (contiguous in the sorted order)
cudaError_t launch_general_ff(const TaskSet &ts, const GridPtrs &g, bool adj, cudaStream_t s) {
    if (ts.gen_count == 0) return cudaSuccess;
    ProfScope prof(ts, s);
    if (adj)
        k_general_ff<true><<<ts.gen_count, 256, ts.gen_smem, s>>>(ts.d_geom, ts.gen_first, ts.plan->d_levels,
                                                                 ts.d_coef, ts.d_mom, g, ts.d_status);
    else
        k_general_ff<false><<<ts.gen_count, 256, ts.gen_smem, s>>>(ts.d_geom, ts.gen_first, ts.plan->d_levels,
                                                                  ts.d_coef, ts.d_mom, g, ts.d_status);
    return cudaGetLastError();
}

cudaError_t launch_fp64_kind(const TaskSet &ts, const GridPtrs &g, bool adj, int kind, cudaStream_t s) {
    return launch_fp64_impl(ts, g, adj, kind, 0, ts.d_mom, s);
}

cudaError_t launch_moments_fp64(const TaskSet &ts, const GridPtrs &g, int extra, double *out, cudaStream_t s) {
    return launch_fp64_impl(ts, g, true, -1, extra, out, s);
}

cudaError_t launch_pairs_fp64(const PairGeom *d_geoms, const LevelDev *d_levels, const double *d_tmat,
                              double *d_coef, int *d_status, int n, int tau, int max_A, int max_B,
                              int smem_coll, const double *d_pab, double *d_grid, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_prep<<<(unsigned)n, 128, smem_prep(max_A, max_B), s>>>(d_geoms, d_levels, d_tmat, tau, d_pab, d_coef);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    GridPtrs g;
    for (int l = 0; l < GPW_MAX_LEVELS; l++) g.p[l] = d_grid;
    k_ortho_fp64<false><<<(unsigned)n, 256, smem_coll, s>>>(d_geoms, 0, d_levels, nullptr, d_coef, nullptr, g,
                                                          d_status, 0);
    return cudaGetLastError();
}

// One pair from raw device pointers, orthorhombic (with its cube list in d_table
// when the pair has one) or general cell: set-up, then the FP64 collocation.
cudaError_t launch_one_fp64(const PairGeom &g, const PairGeom *d_geom, const LevelDev *d_levels, const double *d_tmat,
                            const int *d_table, double *d_coef, int *d_status, int func, const double *d_pab,
                            double *d_grid, cudaStream_t s) {
    k_prep<<<1, 128, smem_prep(g.la_max, g.lb_max), s>>>(d_geom, d_levels, d_tmat, func, d_pab, d_coef);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    GridPtrs gp;
    for (int l = 0; l < GPW_MAX_LEVELS; l++) gp.p[l] = d_grid;
    if (g.ortho)
        k_ortho_fp64<false><<<1, 256, smem_ortho_fp64(g), s>>>(d_geom, 0, d_levels, d_table, d_coef, nullptr, gp,
                                                             d_status, 0);
    else
        k_general_fp64<false><<<1, 256, smem_general_fp64(g), s>>>(d_geom, 0, d_levels, d_coef, nullptr, gp,
                                                                  d_status, 0);
    return cudaGetLastError();
}

cudaError_t launch_collocate_fp64(const TaskSet &ts, const GridPtrs &g, cudaStream_t s) {
    return launch_fp64_kind(ts, g, false, -1, s);
}

cudaError_t launch_integrate_fp64(const TaskSet &ts, const GridPtrs &g, cudaStream_t s) {
    return launch_fp64_kind(ts, g, true, -1, s);
}

cudaError_t launch_backtransform(const TaskSet &ts, const double *d_mom, double *d_hab,
                                 cudaStream_t s) {
    if (ts.ntasks == 0) return cudaSuccess;
    const int smem = smem_prep(ts.max_A, ts.max_B);
    ts.n_kernels++;
    k_backtransform<<<(unsigned)ts.ntasks, 128, smem, s>>>(ts.d_geom, ts.plan->d_levels,
                                                           ts.plan->d_tmat, ts.tau, d_mom, d_hab);
    return cudaGetLastError();
}

}  // namespace gpw
