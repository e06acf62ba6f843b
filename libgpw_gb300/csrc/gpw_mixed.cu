// Tiled mixed-precision collocate / integrate.
//
// Each CTA owns one tile of one grid level (TX x TY x TZ points, x fastest) and
// walks every pair whose cube touches the tile.  Per pair and tile:
//   1-D tables t^k exp(-zetp t^2) over the tile's three ranges   (float-float)
//   stage 1  Cxy[z][b][a] = sum_g c[g][b][a] Z[g][z]              (float-float)
//   stage 2  Cx[(z,y)][a] = sum_b Cxy[z][b][a] Y[b][y]            (float-float)
//   stage 3  rho[(z,y)][x] = sum_a Cx[(z,y)][a] X[a][x]           (exact fp16 slices)
// (the three contractions of collocate_core, collocate.cc:543-623, with the
// cube culling of grid_collocate_core, grid_base_ref_c.cc:413-471).
//
// Stage 3 operands are split into NSL fixed-point fp16 slices of SLB bits: each
// row of Cx is scaled by a power of two so its largest entry is < 2^SLB, each
// column of X likewise, and the slices are integers in [-2^SLB, 2^SLB].  Every
// product of two slices (<= 2^20) and every sum of 16 of them (<= 2^24) is then
// exact in FP32, so the slice products summed per anti-diagonal s = i+j
// (D_s = sum over i+j=s of A_i B_j) carry the tensor-core result without FP32
// accumulation error; the diagonals are recombined in float-float.  The tile sum
// over pairs is float-float in registers, added to the FP64 grid once per tile.
//
// Integrate is the transpose: S[(z,y)][a] = sum_x V[(z,y)][x] X[a][x] by the same
// slices (V sliced once per tile), then the adjoint stages, and the per-pair
// moments are added to FP64 scratch with atomics.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <numeric>
#include <string>
#include <vector>

#include "gpw_coef.cuh"
#include "gpw_ff.cuh"
#include "gpw_internal.h"

namespace gpw {

constexpr int TX = 32, TY = 8, TZ = 16;
constexpr int MROWS = TY * TZ;  // 128 rows per tile, one per thread
constexpr int NTHR = MROWS;
constexpr int NSL = 3;          // slices per operand
constexpr int SLB = 10;         // bits per slice
constexpr int KP = 16;          // padded contraction length (alpha)
constexpr int NPAIR_MAX = (kNPow * (kNPow + 1)) / 2;  // (b, a) with b + a <= lp
constexpr int NCOEF_MAX = ((kMaxLp + 1) * (kMaxLp + 2) * (kMaxLp + 3)) / 6;

constexpr int kMaxImages = 4;  // periodic images of one cube axis over one tile

struct TileDesc {
    int level;
    int t[3];  // tile indices
};

struct MixedState {
    int ntiles = 0;
    int64_t nitems = 0;
    TileDesc *d_tiles = nullptr;
    int64_t *d_start = nullptr;  // ntiles + 1
    int *d_items = nullptr;      // sorted-task indices per tile
    float2 *d_coef_ff = nullptr;
    int *d_queue = nullptr;      // [0]: collocate, [1]: integrate
    int northo = 0;              // ortho tasks come first in sorted order
    int grid_ctas = 0;
};

// ---------------------------------------------------------------------------
// pair data a tile needs, staged in shared memory
struct TPair {
    double r2;          // radius^2 (FP64, rule decisions)
    double hz, hy, hx;
    float r2f, hzf, hyf, hxf;
    ff zetp;
    ff off[3];          // roffset
    ff h[3];
    int lb[3], hi[3], cc[3];
    int kgmin, lp, L;
    int64_t coef_off, table_off;
    int o[3];           // cube offset of the tile origin (current image)
    int gx0, gx1;       // tile-local x range inside the cube box
};

// ---------------------------------------------------------------------------
// Sphere rule with an FP32 fast path.  The FP32 estimate decides unless it lies
// within its error bound of an integer; then the exact FP64 rule (the one the
// host and the oracle use) decides.
__device__ __forceinline__ int fast_floor_checked(float rem, float r2f, float h, bool &unsure) {
    const float rc = fmaxf(rem, 0.0f);
    const float v = __fdiv_rn(sqrtf(rc), h);
    const float fl = floorf(v);
    // error of rem ~ 4 ulp(r2f); of sqrt ~ err/(2 sqrt); plus relative 2^-21
    const float erem = r2f * 4.8e-7f;
    const float ev = (rc > erem ? erem / (2.0f * sqrtf(rc)) : sqrtf(erem)) / h + v * 1e-6f + 1e-6f;
    unsure = (v - fl) <= ev || (fl + 1.0f - v) <= ev || rem <= erem;
    return (int)fl;
}

__device__ __forceinline__ int row_jmax(const TPair &p, int kf) {
    const float dz = (float)(-kf) * p.hzf;
    bool unsure;
    int j = fast_floor_checked(__fmaf_rn(-dz, dz, p.r2f), p.r2f, p.hyf, unsure);
    if (unsure) j = rule_jmax(rule_remk(p.r2, kf, p.hz), p.hy);
    return j;
}

__device__ __forceinline__ int row_imax(const TPair &p, int kf, int jf) {
    const float dz = (float)(-kf) * p.hzf, dy = (float)(-jf) * p.hyf;
    bool unsure;
    int i = fast_floor_checked(__fmaf_rn(-dy, dy, __fmaf_rn(-dz, dz, p.r2f)), p.r2f, p.hxf, unsure);
    if (unsure) i = rule_imax(rule_remk(p.r2, kf, p.hz), jf, p.hy, p.hx);
    return i;
}

// Row (z, y) of the tile: cube-local x range [x0, x1] (empty if x0 > x1).
__device__ __forceinline__ void row_range(const TPair &p, const int *table, int gz, int gy, int ext_ok,
                                          int &x0, int &x1) {
    x0 = 1;
    x1 = 0;
    if (!ext_ok || gz < p.lb[2] || gz > p.hi[2] || gy < p.lb[1] || gy > p.hi[1]) return;
    const int kf = fold(gz), jf = fold(gy);
    if (kf < p.kgmin) return;
    int jmin, imin;
    if (p.table_off < 0) {
        const int jmax = row_jmax(p, kf);
        if (jf < -jmax) return;
        imin = -row_imax(p, kf, jf);
    } else {
        const int *T = table + p.table_off;
        const int kidx = kf - T[0];
        jmin = T[1 + 2 * kidx];
        if (jf < jmin) return;
        imin = T[1 + 2 * (1 - T[0]) + T[2 + 2 * kidx] + (jf - jmin)];
    }
    // cube offsets [imin, 1 - imin] -> tile-local
    x0 = max(imin - p.o[0], p.gx0);
    x1 = min(1 - imin - p.o[0], p.gx1);
}

// ---------------------------------------------------------------------------
// fixed-point slicing of one vector (n entries, float-float) into NSL slices
__device__ __forceinline__ int slice_exponent(const ff *v, int n) {
    float m = 0.0f;
    for (int a = 0; a < n; a++) m = fmaxf(m, fabsf(v[a].hi));
    int e = 0;
    if (m > 0.0f) frexpf(m, &e);  // m = f * 2^e, f in [0.5, 1)
    return m > 0.0f ? e : -1000;
}

__device__ __forceinline__ void slice_value(ff v, int e, float *s) {
    if (e == -1000) {
        s[0] = s[1] = s[2] = 0.0f;
        return;
    }
    // v * 2^(SLB - e): |.| < 2^SLB
    const float hi = ldexpf(v.hi, SLB - e), lo = ldexpf(v.lo, SLB - e);
    const float s1 = rintf(hi);
    float r = __fadd_rn(__fsub_rn(hi, s1), lo);  // |r| <= 1/2 (+ tiny)
    r = __fmul_rn(r, 1024.0f);
    const float s2 = rintf(r);
    r = __fmul_rn(__fsub_rn(r, s2), 1024.0f);
    s[0] = s1;
    s[1] = s2;
    s[2] = rintf(r);
}

// UMMA canonical K-major layout, no swizzle: core matrices of 8 rows x 16 bytes
// (8 halves of K).  Element (row r, k) of an operand with R rows, K = 16:
//   byte offset = (r / 8) * SBO + (k / 8) * LBO + (r % 8) * 16 + (k % 8) * 2,
// LBO = 128 (next 8 K-elements), SBO = 256 (next 8 rows).
__device__ __forceinline__ int umma_off(int r, int k) {
    return (r >> 3) * 256 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2;
}

// Combine the diagonals of one product into float-float and scale by 2^E.
__device__ __forceinline__ ff combine(float d2, float d3, float d4, int E) {
    ff s = two_sum(d2, __fmul_rn(d3, 0.0009765625f));
    s.lo = __fmaf_rn(d4, 9.5367431640625e-07f, s.lo);
    if (E < -126) return {0.0f, 0.0f};  // below 2^-102 of unit scale: dropped
    const float sc = __int_as_float((127 + E) << 23);
    return {__fmul_rn(s.hi, sc), __fmul_rn(s.lo, sc)};
}

// ---------------------------------------------------------------------------
struct MixedArgs {
    const PairGeom *geoms;
    const LevelDev *levels;
    const TileDesc *tiles;
    const int64_t *start;
    const int *items;
    const float2 *coef;
    const int *table;
    double *mom;  // integrate: per-pair moments
    GridPtrs grids;
    int *queue;
    int *status;
    int ntiles;
};

struct TileSmem {
    TPair p;
    float2 coef[NCOEF_MAX];
    ff X[KP][TX];
    ff Y[KP][TY];
    ff Z[KP][TZ];
    ff Cxy[TZ][NPAIR_MAX];  // collocate stage 1; integrate stage-2 output T[z][pair]
    __half A[NSL][MROWS * KP];
    __half B[NSL][TX * KP];
    int fx[TX];             // column exponents (collocate: per x; integrate: per alpha)
    ff S[MROWS][KP];        // integrate: per-row moments
    int tile;
    int img[3][kMaxImages];  // image offsets per axis
    int nimg[3];
};

// pair index of (b, a), b + a <= lp, rows of constant b
__device__ __forceinline__ int pair_index(int L, int b, int a) { return b * L - (b * (b - 1)) / 2 + a; }

__device__ void load_pair(TileSmem &sm, const MixedArgs &A, const LevelDev &lv, int task) {
    if (threadIdx.x == 0) {
        const PairGeom &g = A.geoms[task];
        TPair &p = sm.p;
        p.r2 = rmul(g.radius, g.radius);
        p.hx = lv.dh[0][0];
        p.hy = lv.dh[1][1];
        p.hz = lv.dh[2][2];
        p.r2f = (float)p.r2;
        p.hxf = (float)p.hx;
        p.hyf = (float)p.hy;
        p.hzf = (float)p.hz;
        p.zetp = ff_from_double(g.zetp);
        for (int d = 0; d < 3; d++) {
            p.off[d] = ff_from_double(g.off[d]);
            p.h[d] = ff_from_double(lv.dh[d][d]);
            p.lb[d] = g.lb[d];
            p.hi[d] = g.hi[d];
            p.cc[d] = g.cc[d];
        }
        p.kgmin = g.kgmin;
        p.lp = g.lp;
        p.L = g.lp + 1;
        p.coef_off = g.coef_off;
        p.table_off = g.table_off;
    }
    __syncthreads();
    const int nc = ncoef(sm.p.lp);
    for (int t = threadIdx.x; t < nc; t += blockDim.x) sm.coef[t] = A.coef[sm.p.coef_off + t];
}

// images of one axis: cube offsets o such that the tile [tT, tT+ext) maps onto [lb, hi]
__device__ void axis_images(const LevelDev &lv, int d, int tt, int T, const TPair &p, int *img, int &n, int *status) {
    n = 0;
    const int N = lv.ngrid[d];
    const int ext = min(T, N - tt * T);
    if (lv.periodic[d]) {
        const int np = lv.npts[d];
        // o = k*np + tt*T - cc, need [o, o+ext-1] to meet [lb, hi]
        const int base = tt * T - p.cc[d];
        const int num = p.lb[d] - base - ext + 1;
        const int kmin = (num >= 0 ? num / np : -((-num + np - 1) / np)) - 1;
        for (int k = kmin;; k++) {
            const int o = k * np + base;
            if (o > p.hi[d]) break;
            if (o + ext - 1 >= p.lb[d]) {
                if (n == kMaxImages) {
                    atomicOr(status, kStatTooManyImages);
                    break;
                }
                img[n++] = o;
            }
        }
    } else {
        const int b = imod(p.cc[d] + p.lb[d] + lv.lb_grid[d], lv.npts[d]) - p.lb[d];
        const int o = tt * T - b;
        if (o <= p.hi[d] && o + ext - 1 >= p.lb[d]) img[n++] = o;
    }
}

// tables over the tile's range on one axis: tab[k][i] = t^k exp(-zetp t^2), t = g h - off,
// g = o + i; zero outside [lb, hi] and outside the valid tile extent.
__device__ __forceinline__ void table_entry(const TPair &p, int d, int g, bool inside, ff *col, int stride,
                                            int L) {
    if (!inside) {
        for (int k = 0; k < KP; k++) col[k * stride] = ff{0.0f, 0.0f};
        return;
    }
    const ff t = ff_add(ff_mul_f(p.h[d], (float)g), ff{-p.off[d].hi, -p.off[d].lo});
    const ff a = ff_mul(ff_mul(t, t), ff{-p.zetp.hi, -p.zetp.lo});
    ff e = ff_exp(a);
    for (int k = 0; k < KP; k++) {
        col[k * stride] = k < L ? e : ff{0.0f, 0.0f};
        if (k + 1 < L) e = ff_mul(e, t);
    }
}

__device__ void build_tables(TileSmem &sm, const LevelDev &lv, const TileDesc &td) {
    const TPair &p = sm.p;
    const int tid = threadIdx.x;
    // 32 x + 8 y + 16 z = 56 entries
    if (tid < TX) {
        const int g = p.o[0] + tid;
        const bool in = tid < min(TX, lv.ngrid[0] - td.t[0] * TX) && g >= p.lb[0] && g <= p.hi[0];
        table_entry(p, 0, g, in, &sm.X[0][tid], TX, p.L);
    } else if (tid < TX + TY) {
        const int i = tid - TX, g = p.o[1] + i;
        const bool in = i < min(TY, lv.ngrid[1] - td.t[1] * TY) && g >= p.lb[1] && g <= p.hi[1];
        table_entry(p, 1, g, in, &sm.Y[0][i], TY, p.L);
    } else if (tid < TX + TY + TZ) {
        const int i = tid - TX - TY, g = p.o[2] + i;
        const bool in = i < min(TZ, lv.ngrid[2] - td.t[2] * TZ) && g >= p.lb[2] && g <= p.hi[2];
        table_entry(p, 2, g, in, &sm.Z[0][i], TZ, p.L);
    }
}

// ---------------------------------------------------------------------------
// SIMT stage 3 on the slices: rows m, columns c, K = 16.
__device__ __forceinline__ void slice_dot(const __half *A0, const __half *A1, const __half *A2, const __half *B0,
                                          const __half *B1, const __half *B2, int m, int c, float &d2, float &d3,
                                          float &d4) {
    d2 = d3 = d4 = 0.0f;
#pragma unroll
    for (int k = 0; k < KP; k++) {
        const int oa = umma_off(m, k) >> 1, ob = umma_off(c, k) >> 1;
        const float a0 = __half2float(A0[oa]), a1 = __half2float(A1[oa]), a2 = __half2float(A2[oa]);
        const float b0 = __half2float(B0[ob]), b1 = __half2float(B1[ob]), b2 = __half2float(B2[ob]);
        d2 = __fmaf_rn(a0, b0, d2);
        d3 = __fmaf_rn(a0, b1, __fmaf_rn(a1, b0, d3));
        d4 = __fmaf_rn(a0, b2, __fmaf_rn(a1, b1, __fmaf_rn(a2, b0, d4)));
    }
}

// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(NTHR, 2) k_collocate_tiled(MixedArgs A) {
    extern __shared__ __align__(128) unsigned char smraw[];
    TileSmem &sm = *reinterpret_cast<TileSmem *>(smraw);
    const int tid = threadIdx.x;
    const int m = tid, z = m / TY, y = m % TY;
    for (;;) {
        if (tid == 0) sm.tile = atomicAdd(A.queue, 1);
        __syncthreads();
        const int tile = sm.tile;
        if (tile >= A.ntiles) break;
        const TileDesc td = A.tiles[tile];
        const LevelDev &lv = A.levels[td.level];
        float acc_hi[TX], acc_lo[TX];
#pragma unroll
        for (int x = 0; x < TX; x++) acc_hi[x] = acc_lo[x] = 0.0f;
        const int ext_z = min(TZ, lv.ngrid[2] - td.t[2] * TZ), ext_y = min(TY, lv.ngrid[1] - td.t[1] * TY);
        const int ext_x = min(TX, lv.ngrid[0] - td.t[0] * TX);
        for (int64_t it = A.start[tile]; it < A.start[tile + 1]; it++) {
            const int task = A.items[it];
            load_pair(sm, A, lv, task);
            if (tid < 3) {
                const int T = tid == 0 ? TX : (tid == 1 ? TY : TZ);
                axis_images(lv, tid, td.t[tid], T, sm.p, sm.img[tid], sm.nimg[tid], A.status);
            }
            __syncthreads();
            const int L = sm.p.L, lp = sm.p.lp;
            for (int iz = 0; iz < sm.nimg[2]; iz++)
            for (int iy = 0; iy < sm.nimg[1]; iy++)
            for (int ix = 0; ix < sm.nimg[0]; ix++) {
                if (tid == 0) {
                    sm.p.o[0] = sm.img[0][ix];
                    sm.p.o[1] = sm.img[1][iy];
                    sm.p.o[2] = sm.img[2][iz];
                    sm.p.gx0 = max(0, sm.p.lb[0] - sm.p.o[0]);
                    sm.p.gx1 = min(ext_x - 1, sm.p.hi[0] - sm.p.o[0]);
                }
                __syncthreads();
                build_tables(sm, lv, td);
                __syncthreads();
                // stage 1: Cxy[z][(b,a)] = sum_g c[g][b][a] Z[g][z]
                const int npair = (L * (L + 1)) / 2;
                for (int t = tid; t < TZ * npair; t += NTHR) {
                    const int zz = t / npair;
                    int q = t % npair, b = 0;
                    while (q >= L - b) { q -= L - b; b++; }
                    const int a = q;
                    ff s = {0.0f, 0.0f};
                    for (int g = 0; g <= lp - a - b; g++) {
                        const float2 c = sm.coef[pidx(lp, g, b, a)];
                        s = ff_fma(ff{c.x, c.y}, sm.Z[g][zz], s);
                    }
                    sm.Cxy[zz][pair_index(L, b, a)] = s;
                }
                // B slices: column x over alpha
                if (tid < TX) {
                    ff col[KP];
#pragma unroll
                    for (int k = 0; k < KP; k++) col[k] = sm.X[k][tid];
                    const int e = slice_exponent(col, KP);
                    sm.fx[tid] = e;
#pragma unroll
                    for (int k = 0; k < KP; k++) {
                        float s[3];
                        slice_value(col[k], e, s);
                        const int o = umma_off(tid, k) >> 1;
                        sm.B[0][o] = __float2half_rn(s[0]);
                        sm.B[1][o] = __float2half_rn(s[1]);
                        sm.B[2][o] = __float2half_rn(s[2]);
                    }
                }
                __syncthreads();
                // stage 2 + row culling + A slices (thread = row)
                int x0, x1;
                row_range(sm.p, A.table, sm.p.o[2] + z, sm.p.o[1] + y, z < ext_z && y < ext_y, x0, x1);
                ff cx[KP];
#pragma unroll
                for (int a = 0; a < KP; a++) cx[a] = ff{0.0f, 0.0f};
                if (x0 <= x1) {
#pragma unroll
                    for (int a = 0; a < KP; a++) {
                        if (a >= L) break;
                        ff s = {0.0f, 0.0f};
                        for (int b = 0; b <= lp - a; b++) s = ff_fma(sm.Cxy[z][pair_index(L, b, a)], sm.Y[b][y], s);
                        cx[a] = s;
                    }
                }
                const int em = slice_exponent(cx, KP);
#pragma unroll
                for (int k = 0; k < KP; k++) {
                    float s[3];
                    slice_value(cx[k], em, s);
                    const int o = umma_off(m, k) >> 1;
                    sm.A[0][o] = __float2half_rn(s[0]);
                    sm.A[1][o] = __float2half_rn(s[1]);
                    sm.A[2][o] = __float2half_rn(s[2]);
                }
                __syncthreads();
                // stage 3 (SIMT on the slices) and accumulation
                if (x0 <= x1) {
#pragma unroll
                    for (int x = 0; x < TX; x++) {
                        if (x < x0 || x > x1) continue;
                        float d2, d3, d4;
                        slice_dot(sm.A[0], sm.A[1], sm.A[2], sm.B[0], sm.B[1], sm.B[2], m, x, d2, d3, d4);
                        const ff v = combine(d2, d3, d4, em + sm.fx[x] - 2 * SLB);
                        const ff s = two_sum(acc_hi[x], v.hi);
                        acc_hi[x] = s.hi;
                        acc_lo[x] = __fadd_rn(acc_lo[x], __fadd_rn(s.lo, v.lo));
                    }
                }
                __syncthreads();
            }
        }
        // flush: grid += tile sum (FP64)
        if (z < ext_z && y < ext_y) {
            double *grid = A.grids.p[td.level];
            const int64_t row = ((int64_t)(td.t[2] * TZ + z) * lv.ngrid[1] + (td.t[1] * TY + y)) * lv.ngrid[0] +
                                td.t[0] * TX;
#pragma unroll
            for (int x = 0; x < TX; x++)
                if (x < ext_x) grid[row + x] += (double)acc_hi[x] + (double)acc_lo[x];
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(NTHR, 2) k_integrate_tiled(MixedArgs A) {
    extern __shared__ __align__(128) unsigned char smraw[];
    TileSmem &sm = *reinterpret_cast<TileSmem *>(smraw);
    const int tid = threadIdx.x;
    const int m = tid, z = m / TY, y = m % TY;
    for (;;) {
        if (tid == 0) sm.tile = atomicAdd(A.queue, 1);
        __syncthreads();
        const int tile = sm.tile;
        if (tile >= A.ntiles) break;
        const TileDesc td = A.tiles[tile];
        const LevelDev &lv = A.levels[td.level];
        const int ext_z = min(TZ, lv.ngrid[2] - td.t[2] * TZ), ext_y = min(TY, lv.ngrid[1] - td.t[1] * TY);
        const int ext_x = min(TX, lv.ngrid[0] - td.t[0] * TX);
        // V row of this thread, float-float
        ff v[TX];
        {
            const double *grid = A.grids.p[td.level];
            const bool ok = z < ext_z && y < ext_y;
            const int64_t row = ((int64_t)(td.t[2] * TZ + z) * lv.ngrid[1] + (td.t[1] * TY + y)) * lv.ngrid[0] +
                                td.t[0] * TX;
#pragma unroll
            for (int x = 0; x < TX; x++) v[x] = (ok && x < ext_x) ? ff_from_double(grid[row + x]) : ff{0.0f, 0.0f};
        }
        for (int64_t it = A.start[tile]; it < A.start[tile + 1]; it++) {
            const int task = A.items[it];
            load_pair(sm, A, lv, task);
            if (tid < 3) {
                const int T = tid == 0 ? TX : (tid == 1 ? TY : TZ);
                axis_images(lv, tid, td.t[tid], T, sm.p, sm.img[tid], sm.nimg[tid], A.status);
            }
            __syncthreads();
            const int L = sm.p.L, lp = sm.p.lp;
            const int npair = (L * (L + 1)) / 2;
            const int64_t moff = sm.p.coef_off;
            for (int iz = 0; iz < sm.nimg[2]; iz++)
            for (int iy = 0; iy < sm.nimg[1]; iy++)
            for (int ix = 0; ix < sm.nimg[0]; ix++) {
                if (tid == 0) {
                    sm.p.o[0] = sm.img[0][ix];
                    sm.p.o[1] = sm.img[1][iy];
                    sm.p.o[2] = sm.img[2][iz];
                    sm.p.gx0 = max(0, sm.p.lb[0] - sm.p.o[0]);
                    sm.p.gx1 = min(ext_x - 1, sm.p.hi[0] - sm.p.o[0]);
                }
                __syncthreads();
                build_tables(sm, lv, td);
                __syncthreads();
                // stage 3 transposed: S[m][a] = sum_{x in row range} V[m][x] X[a][x]  (float-float)
                int x0, x1;
                row_range(sm.p, A.table, sm.p.o[2] + z, sm.p.o[1] + y, z < ext_z && y < ext_y, x0, x1);
                for (int a = 0; a < KP; a++) {
                    ff s = {0.0f, 0.0f};
                    if (a < L && x0 <= x1) {
#pragma unroll
                        for (int x = 0; x < TX; x++)
                            if (x >= x0 && x <= x1) s = ff_fma(v[x], sm.X[a][x], s);
                    }
                    sm.S[m][a] = s;
                }
                __syncthreads();
                // stage 2 transposed: T[z][(b,a)] = sum_y S[(z,y)][a] Y[b][y]
                for (int t = tid; t < TZ * npair; t += NTHR) {
                    const int zz = t / npair;
                    int q = t % npair, b = 0;
                    while (q >= L - b) { q -= L - b; b++; }
                    const int a = q;
                    ff s = {0.0f, 0.0f};
                    for (int yy = 0; yy < TY; yy++) s = ff_fma(sm.S[zz * TY + yy][a], sm.Y[b][yy], s);
                    sm.Cxy[zz][pair_index(L, b, a)] = s;
                }
                __syncthreads();
                // stage 1 transposed: W[g][b][a] += sum_z T[z][(b,a)] Z[g][z]
                const int nc = ncoef(lp);
                for (int t = tid; t < nc; t += NTHR) {
                    int g = 0, b = 0, a = 0;
                    {
                        int r = t;
                        for (g = 0; g <= lp; g++) {
                            const int cnt = ((lp - g + 1) * (lp - g + 2)) / 2;
                            if (r < cnt) break;
                            r -= cnt;
                        }
                        const int q = lp - g;
                        for (b = 0; b <= q; b++) {
                            if (r <= q - b) break;
                            r -= q - b + 1;
                        }
                        a = r;
                    }
                    ff s = {0.0f, 0.0f};
                    const int pi = pair_index(L, b, a);
                    for (int zz = 0; zz < TZ; zz++) s = ff_fma(sm.Cxy[zz][pi], sm.Z[g][zz], s);
                    if (s.hi != 0.0f) atomicAdd(A.mom + moff + t, (double)s.hi + (double)s.lo);
                }
                __syncthreads();
            }
        }
    }
}

__global__ void k_coef_to_ff(const double *__restrict__ c, float2 *__restrict__ out, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double d = c[i];
        const float h = __double2float_rn(d);
        out[i] = make_float2(h, __double2float_rn(d - (double)h));
    }
}

// ---------------------------------------------------------------------------
// host: bin the orthorhombic pairs by tile
namespace {
void axis_tiles(const LevelDev &lv, int d, const PairGeom &g, int T, std::vector<int> &out) {
    out.clear();
    const int N = lv.ngrid[d];
    const int nt = (N + T - 1) / T;
    std::vector<char> seen(nt, 0);
    for (int gg = g.lb[d]; gg <= g.hi[d];) {
        int w;
        if (lv.periodic[d]) w = imod(g.cc[d] + gg, lv.npts[d]);
        else w = gg + imod(g.cc[d] + g.lb[d] + lv.lb_grid[d], lv.npts[d]) - g.lb[d];
        if (w < 0 || w >= N) { gg++; continue; }
        const int t = w / T;
        if (!seen[t]) { seen[t] = 1; out.push_back(t); }
        gg += std::min(T - (w - t * T), N - w);
    }
}
}  // namespace

int mixed_build(TaskSet &ts, std::string &err) {
    MixedState *M = new MixedState();
    ts.mixed = M;
    const Plan &P = *ts.plan;
    int64_t northo = 0;
    while (northo < ts.ntasks && ts.h_geom[northo].ortho) northo++;
    M->northo = (int)northo;
    // tiles of every orthorhombic level
    std::vector<int> lvl_first(P.nlevels, -1);
    std::vector<TileDesc> tiles;
    int ntx[GPW_MAX_LEVELS], nty[GPW_MAX_LEVELS], ntz[GPW_MAX_LEVELS];
    for (int l = 0; l < P.nlevels; l++) {
        if (!P.lv[l].ortho) continue;
        ntx[l] = (P.lv[l].ngrid[0] + TX - 1) / TX;
        nty[l] = (P.lv[l].ngrid[1] + TY - 1) / TY;
        ntz[l] = (P.lv[l].ngrid[2] + TZ - 1) / TZ;
        lvl_first[l] = (int)tiles.size();
        for (int a = 0; a < ntz[l]; a++)
            for (int b = 0; b < nty[l]; b++)
                for (int c = 0; c < ntx[l]; c++) tiles.push_back(TileDesc{l, {c, b, a}});
    }
    const int ntiles = (int)tiles.size();
    std::vector<int64_t> count(ntiles + 1, 0);
    std::vector<int> ax, ay, az;
    auto each = [&](auto &&fn) {
        for (int64_t k = 0; k < northo; k++) {
            const PairGeom &g = ts.h_geom[k];
            const LevelDev &lv = P.lv[g.level];
            axis_tiles(lv, 0, g, TX, ax);
            axis_tiles(lv, 1, g, TY, ay);
            axis_tiles(lv, 2, g, TZ, az);
            const int base = lvl_first[g.level];
            for (int c : az)
                for (int b : ay)
                    for (int a : ax) fn(base + (c * nty[g.level] + b) * ntx[g.level] + a, (int)k);
        }
    };
    each([&](int t, int) { count[t + 1]++; });
    // order tiles by decreasing work for the persistent queue
    std::vector<int> order(ntiles);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return count[a + 1] > count[b + 1]; });
    std::vector<int> rank(ntiles);
    for (int i = 0; i < ntiles; i++) rank[order[i]] = i;
    std::vector<int64_t> start(ntiles + 1, 0);
    for (int i = 0; i < ntiles; i++) start[i + 1] = start[i] + count[order[i] + 1];
    const int64_t nitems = start[ntiles];
    std::vector<int> items((size_t)std::max<int64_t>(nitems, 1));
    std::vector<int64_t> fill(start.begin(), start.end() - 1);
    each([&](int t, int k) { items[fill[rank[t]]++] = k; });
    std::vector<TileDesc> tiles_sorted(ntiles);
    for (int i = 0; i < ntiles; i++) tiles_sorted[i] = tiles[order[i]];
    M->ntiles = ntiles;
    M->nitems = nitems;
    cudaError_t e = cudaSuccess;
    auto alloc = [&](void **p, size_t bytes) {
        if (e == cudaSuccess) e = cudaMalloc(p, std::max<size_t>(bytes, 16));
    };
    alloc((void **)&M->d_tiles, sizeof(TileDesc) * ntiles);
    alloc((void **)&M->d_start, sizeof(int64_t) * (ntiles + 1));
    alloc((void **)&M->d_items, sizeof(int) * items.size());
    alloc((void **)&M->d_coef_ff, sizeof(float2) * std::max<int64_t>(ts.coef_len, 1));
    alloc((void **)&M->d_queue, sizeof(int) * 2);
    if (e == cudaSuccess && ntiles)
        e = cudaMemcpy(M->d_tiles, tiles_sorted.data(), sizeof(TileDesc) * ntiles, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(M->d_start, start.data(), sizeof(int64_t) * (ntiles + 1), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && nitems)
        e = cudaMemcpy(M->d_items, items.data(), sizeof(int) * nitems, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        err = std::string("mixed_build: ") + cudaGetErrorString(e);
        return GPW_ERR_CUDA;
    }
    int sms = 0, per_sm = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, P.device);
    for (const void *fn : {(const void *)k_collocate_tiled, (const void *)k_integrate_tiled}) {
        e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(TileSmem));
        if (e != cudaSuccess) {
            err = std::string("mixed_build: ") + cudaGetErrorString(e);
            return GPW_ERR_CUDA;
        }
    }
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_collocate_tiled, NTHR, sizeof(TileSmem));
    M->grid_ctas = std::max(1, std::min(ntiles, sms * std::max(per_sm, 1)));
    return GPW_SUCCESS;
}

void mixed_free(TaskSet &ts) {
    MixedState *M = ts.mixed;
    if (!M) return;
    cudaFree(M->d_tiles);
    cudaFree(M->d_start);
    cudaFree(M->d_items);
    cudaFree(M->d_coef_ff);
    cudaFree(M->d_queue);
    delete M;
    ts.mixed = nullptr;
}

static MixedArgs make_args(const TaskSet &ts, const GridPtrs &g, int which) {
    const MixedState &M = *ts.mixed;
    MixedArgs a;
    a.geoms = ts.d_geom;
    a.levels = ts.plan->d_levels;
    a.tiles = M.d_tiles;
    a.start = M.d_start;
    a.items = M.d_items;
    a.coef = M.d_coef_ff;
    a.table = ts.d_table;
    a.mom = ts.d_mom;
    a.grids = g;
    a.queue = M.d_queue + which;
    a.status = ts.d_status;
    a.ntiles = M.ntiles;
    return a;
}

// general-cell pairs of a mixed call run on the FP64 kernels
static cudaError_t general_fp64(const TaskSet &ts, const GridPtrs &g, bool adj, cudaStream_t s) {
    return adj ? launch_fp64_kind(ts, g, true, 1, s) : launch_fp64_kind(ts, g, false, 1, s);
}

cudaError_t launch_collocate_mixed(const TaskSet &ts, const GridPtrs &g, cudaStream_t s) {
    const MixedState &M = *ts.mixed;
    cudaError_t e = cudaSuccess;
    if (M.northo > 0 && M.ntiles > 0) {
        const int64_t n = ts.coef_len;
        ts.n_kernels++;
        k_coef_to_ff<<<(unsigned)std::min<int64_t>((n + 255) / 256, 4096), 256, 0, s>>>(ts.d_coef, M.d_coef_ff, n);
        if ((e = cudaMemsetAsync(M.d_queue, 0, sizeof(int), s)) != cudaSuccess) return e;
        ProfScope prof(ts, s);
        k_collocate_tiled<<<M.grid_ctas, NTHR, sizeof(TileSmem), s>>>(make_args(ts, g, 0));
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    return general_fp64(ts, g, false, s);
}

cudaError_t launch_integrate_mixed(const TaskSet &ts, const GridPtrs &g, cudaStream_t s) {
    const MixedState &M = *ts.mixed;
    cudaError_t e = cudaSuccess;
    if (M.northo > 0 && M.ntiles > 0) {
        if ((e = cudaMemsetAsync(ts.d_mom, 0, sizeof(double) * ts.coef_len, s)) != cudaSuccess) return e;
        if ((e = cudaMemsetAsync(M.d_queue + 1, 0, sizeof(int), s)) != cudaSuccess) return e;
        ProfScope prof(ts, s);
        k_integrate_tiled<<<M.grid_ctas, NTHR, sizeof(TileSmem), s>>>(make_args(ts, g, 1));
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    return general_fp64(ts, g, true, s);
}

}  // namespace gpw
