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
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "gpw_coef.cuh"
#include "gpw_ff.cuh"
#include "gpw_internal.h"
#include "gpw_tc.cuh"

namespace gpw {

constexpr int TX = 32, TY = 8, TZ = 16;
constexpr int MROWS = TY * TZ;  // 128 rows per tile, one per thread
constexpr int NTHR = MROWS;
constexpr int NSL = 4;          // slices per operand
constexpr int SLB = 10;         // bits per slice
constexpr int KP = 16;          // padded contraction length (alpha)
constexpr int NPAIR_MAX = (kNPow * (kNPow + 1)) / 2;  // (b, a) with b + a <= lp
constexpr int NCOEF_MAX = ((kMaxLp + 1) * (kMaxLp + 2) * (kMaxLp + 3)) / 6;

constexpr int kMaxImages = 4;  // periodic images of one cube axis over one tile

struct TileDesc {
    int level;
    int t[3];  // tile indices
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
    ff tc;              // collocate: x of the re-expansion column minus xp
    int ic;             // collocate: tile-local re-expansion column
    int sb;             // collocate: x-variable scale 2^sb of the slices (balancing)
};

struct MixedState {
    int ntiles = 0;
    int64_t nitems = 0;
    TileDesc *d_tiles = nullptr;
    TPair *d_pairs = nullptr;    // per sorted task
    int64_t *d_start = nullptr;  // ntiles + 1
    int *d_items = nullptr;      // sorted-task indices per tile
    float2 *d_coef_ff = nullptr;
    int *d_queue = nullptr;      // [0]: collocate, [1]: integrate
    int northo = 0;              // ortho tasks come first in sorted order
    int grid_ctas = 0;    // collocate
    int grid_ctas_i = 0;  // integrate
    int per_sm = 0, per_sm_i = 0;
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

// UMMA canonical K-major layout, no swizzle: core matrices of 8 rows x 16 bytes
// (8 halves of K).  Element (row r, k) of an operand with R rows, K = 16:
//   byte offset = (r / 8) * SBO + (k / 8) * LBO + (r % 8) * 16 + (k % 8) * 2,
// LBO = 128 (next 8 K-elements), SBO = 256 (next 8 rows).
__device__ __forceinline__ int umma_off(int r, int k) {
    return (r >> 3) * 256 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2;
}

constexpr int kZeroExp = -1000;
// 2^k as a float, -126 <= k <= 127
__device__ __forceinline__ float pow2i(int k) { return __int_as_float((127 + k) << 23); }
// e with m = f 2^e, f in [0.5, 1); values below 2^-100 count as zero
__device__ __forceinline__ int exp_of(float m) {
    return m >= 7.888609052210118e-31f ? ((__float_as_int(m) >> 23) & 0xff) - 126 : kZeroExp;
}
// the NSL fixed-point slices of v * scale, scale = 2^(SLB - e)
__device__ __forceinline__ void slice_scaled(ff v, float scale, float *sl) {
    const float hi = __fmul_rn(v.hi, scale), lo = __fmul_rn(v.lo, scale);
    sl[0] = rintf(hi);
    float r = __fadd_rn(__fsub_rn(hi, sl[0]), lo);
#pragma unroll
    for (int i = 1; i < NSL; i++) {
        r = __fmul_rn(r, 1024.0f);
        sl[i] = rintf(r);
        r = __fsub_rn(r, sl[i]);
    }
}
// two consecutive K entries (k even) of one operand row as packed halves
__device__ __forceinline__ void store_pair(__half *base, int r, int k, float a, float b) {
    *reinterpret_cast<__half2 *>(base + (umma_off(r, k) >> 1)) = __floats2half2_rn(a, b);
}

// Combine the diagonals D_2..D_5 of one product (weights 1, 2^-10, 2^-20, 2^-30)
// into float-float and scale by 2^E.
__device__ __forceinline__ ff combine(float d2, float d3, float d4, float d5, int E) {
    ff s = two_sum(d2, __fmul_rn(d3, 0.0009765625f));
    s.lo = __fmaf_rn(d4, 9.5367431640625e-07f, __fmaf_rn(d5, 9.313225746154785e-10f, s.lo));
    if (E < -126) return {0.0f, 0.0f};  // below 2^-102 of unit scale: dropped
    const float sc = __int_as_float((127 + E) << 23);
    return {__fmul_rn(s.hi, sc), __fmul_rn(s.lo, sc)};
}

struct MixedArgs {
    const TPair *pairs;
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

// shared state of both tiled kernels
struct TileCommon {
    TPair p;
    float2 coef[NCOEF_MAX];
    ff X[KP][TX];
    ff Y[KP][TY];
    ff Z[KP][TZ];
    ff Cxy[TZ][NPAIR_MAX];  // collocate stage 1; integrate stage-2 output T[z][pair]
    int tile;
    int img[3][kMaxImages];
    int nimg[3];
    uint64_t mbar;
    uint32_t tmem;
    int abort;
    int kmax;  // collocate: K slots of A/B written by the previous pair (zeroed up to here)
};

struct alignas(128) SmemColl {
    __half A[NSL][MROWS * KP];  // Cx slices, M=128 x K=16
    __half B[NSL][TX * KP];     // X slices, N=32 x K=16
    ff cxs[KP][MROWS];          // stage-2 rows (column m belongs to thread m)
    float cs[TX];               // 2^fx per column (0 for an empty column)
    TileCommon c;
};

struct alignas(128) SmemInt {
    __half A[2][NSL][MROWS * KP];  // masked V slices, K halves x in [0,16) and [16,32)
    __half B[2][NSL][KP * KP];     // X' slices, N=16 (alpha) x K=16 per half
    __half Vs[NSL][MROWS][TX];     // this tile's V slices, unmasked
    ff S[MROWS][KP];
    int gexp[KP];
    TileCommon c;
};

// pair index of (b, a), b + a <= lp, rows of constant b
__device__ __forceinline__ int pair_index(int L, int b, int a) { return b * L - (b * (b - 1)) / 2 + a; }

// The pair record is prepared on the host (float-float splits included) and
// copied word by word; then the packed coefficients.
__device__ __forceinline__ void load_coef(TileCommon &sm, const MixedArgs &A) {
    const int nc = ncoef(sm.p.lp);
    for (int t = threadIdx.x; t < nc; t += blockDim.x) sm.coef[t] = A.coef[sm.p.coef_off + t];
}

__device__ void load_pair(TileCommon &sm, const MixedArgs &A, int task, bool with_coef = true) {
    static_assert(sizeof(TPair) % 4 == 0, "TPair must be word-sized");
    const uint32_t *src = reinterpret_cast<const uint32_t *>(A.pairs + task);
    uint32_t *dst = reinterpret_cast<uint32_t *>(&sm.p);
    for (int t = threadIdx.x; t < (int)(sizeof(TPair) / 4); t += blockDim.x) dst[t] = src[t];
    __syncthreads();
    if (with_coef) load_coef(sm, A);
}

// Re-expands the x dependence of the coefficients around column ic of the tile:
// c'[g][b][a] = sum_{a' >= a} C(a', a) tc^(a' - a) c[g][b][a'], in place (one
// thread per (g, b) row).  Powers of the small offsets u = x - x_ic keep the
// stage-3 operands well conditioned for the fixed-point slices.
__constant__ float c_binom[kNPow][kNPow] = {
    {1},
    {1, 1},
    {1, 2, 1},
    {1, 3, 3, 1},
    {1, 4, 6, 4, 1},
    {1, 5, 10, 10, 5, 1},
    {1, 6, 15, 20, 15, 6, 1},
    {1, 7, 21, 35, 35, 21, 7, 1},
    {1, 8, 28, 56, 70, 56, 28, 8, 1},
    {1, 9, 36, 84, 126, 126, 84, 36, 9, 1},
    {1, 10, 45, 120, 210, 252, 210, 120, 45, 10, 1}};

__device__ void recentre_x(TileCommon &sm) {
    const int lp = sm.p.lp;
    const ff tc = sm.p.tc;
    const int nrow = ((lp + 1) * (lp + 2)) / 2;
    for (int t = threadIdx.x; t < nrow; t += blockDim.x) {
        int g = 0, r = t;
        while (r >= lp + 1 - g) { r -= lp + 1 - g; g++; }
        const int b = r, amax = lp - g - b;
        const int base = pidx(lp, g, b, 0);
        ff c[kNPow];
#pragma unroll
        for (int a = 0; a < kNPow; a++) c[a] = a <= amax ? ff{sm.coef[base + a].x, sm.coef[base + a].y} : ff{0.0f, 0.0f};
        for (int a = 0; a <= amax; a++) {
            // Horner in tc over a' = amax .. a with weights C(a', a)
            ff s = {0.0f, 0.0f};
            for (int ap = amax; ap >= a; ap--) s = ff_fma(s, tc, ff_mul_f(c[ap], c_binom[ap][a]));
            sm.coef[base + a] = make_float2(s.hi, s.lo);
        }
    }
}

// images of one axis: cube offsets o such that the tile [tT, tT+ext) maps onto [lb, hi]
__device__ void axis_images(const LevelDev &lv, int d, int tt, int T, const TPair &p, int *img, int &n, int *status) {
    n = 0;
    const int N = lv.ngrid[d];
    const int ext = min(T, N - tt * T);
    if (lv.periodic[d]) {
        const int np = lv.npts[d];
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

// Per image: tile origin in cube offsets and the x range inside the cube box.
__device__ __forceinline__ void set_image(TPair &p, int ox, int oy, int oz, int ext_x) {
    p.o[0] = ox;
    p.o[1] = oy;
    p.o[2] = oz;
    p.gx0 = max(0, p.lb[0] - ox);
    p.gx1 = min(ext_x - 1, p.hi[0] - ox);
    // Re-expansion column: start from the column nearest to the product centre and
    // move toward the tile centre by at most one Gaussian width 1/sqrt(zetp) --
    // the largest values stay near u = 0, and broad Gaussians get the smallest
    // |u| over the whole tile.
    const float hx = p.h[0].hi;
    int i0 = (int)rintf(p.off[0].hi / hx) - ox;
    i0 = min(max(i0, p.gx0), max(p.gx0, p.gx1));
    const float rg = rsqrtf(p.zetp.hi) / hx;
    const float dc = fminf(fmaxf((float)(TX / 2 - i0), -rg), rg);
    p.ic = i0 + (int)rintf(dc);
    p.tc = ff_add(ff_mul_f(p.h[0], (float)(ox + p.ic)), ff{-p.off[0].hi, -p.off[0].lo});
    // Balance the powers: u -> u / 2^sb with 2^sb ~ the extent that matters on this
    // tile, min(max |u|, 2 / sqrt(zetp)); the row coefficients take 2^(k sb), so the
    // product is unchanged and both operands' slices keep their bits where the
    // values are.
    const float umax = (float)max(p.ic - p.gx0, p.gx1 - p.ic) * hx;
    const float ext = fminf(umax, 2.0f * rsqrtf(p.zetp.hi));
    int e = 0;
    if (ext > 0.0f) frexpf(ext, &e);
    p.sb = ext > 0.0f ? min(max(e, -10), 10) : 0;
}

// tab[k][i] = u^k exp(-zetp t^2), t = g h - off, g = o + i, and u = t or, with
// recentre, u = (i - ic) h / 2^sb (the balanced offset from the re-expansion
// column); zero outside the cube box and outside the valid tile extent.
__device__ __forceinline__ void table_entry(const TPair &p, int d, int g, bool inside, ff *col, int stride,
                                            int L, bool recentre = false, int i = 0) {
    if (!inside) {
        for (int k = 0; k < KP; k++) col[k * stride] = ff{0.0f, 0.0f};
        return;
    }
    const ff t = ff_add(ff_mul_f(p.h[d], (float)g), ff{-p.off[d].hi, -p.off[d].lo});
    const ff a = ff_mul(ff_mul(t, t), ff{-p.zetp.hi, -p.zetp.lo});
    ff e = ff_exp(a);
    const ff u = recentre ? ff_mul_f(p.h[d], ldexpf((float)(i - p.ic), -p.sb)) : t;
    for (int k = 0; k < KP; k++) {
        col[k * stride] = k < L ? e : ff{0.0f, 0.0f};
        if (k + 1 < L) e = ff_mul(e, u);
    }
}

__device__ void build_tables(TileCommon &sm, const LevelDev &lv, const TileDesc &td, bool recentre_x = false) {
    const TPair &p = sm.p;
    const int tid = threadIdx.x;
    if (tid < TX) {
        const int g = p.o[0] + tid;
        const bool in = tid >= p.gx0 && tid <= p.gx1;
        table_entry(p, 0, g, in, &sm.X[0][tid], TX, p.L, recentre_x, tid);
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


// TMEM set-up shared by both kernels: warp 0 allocates, thread 0 inits the mbarrier
__device__ __forceinline__ void tc_setup(TileCommon &c, uint32_t ncols) {
    if (threadIdx.x == 0) {
        tc::mbar_init(&c.mbar, 1);
        tc::fence_mbar_init();
        c.abort = 0;
        c.kmax = KP;  // operand buffers start uninitialised: write every slot once
    }
    if (threadIdx.x < 32) {
        tc::tmem_alloc(&c.tmem, ncols);
        tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
}

__device__ __forceinline__ void tc_teardown(TileCommon &c, uint32_t ncols, uint32_t phase) {
    if (c.abort) tc::mbar_wait_bounded(&c.mbar, phase, 1u << 22);  // let an MMA in flight finish
    tc::fence_before_sync();
    __syncthreads();
    if (threadIdx.x < 32) tc::tmem_dealloc(c.tmem, ncols);
}

// waits for the MMAs of this round; false (and abort flagged) on timeout
__device__ __forceinline__ bool tc_wait(TileCommon &c, uint32_t phase, int *status) {
    if (!tc::mbar_wait_bounded(&c.mbar, phase, 1u << 24)) {
        atomicOr(status, kStatTimeout);
        c.abort = 1;
    }
    __syncthreads();
    tc::fence_after_sync();
    return !c.abort;
}

constexpr uint32_t kWaitLimit = 1u << 24;

// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(NTHR, 4) k_collocate_tiled(MixedArgs A) {
    extern __shared__ __align__(128) unsigned char smraw[];
    SmemColl &sm = *reinterpret_cast<SmemColl *>(smraw);
    TileCommon &cm = sm.c;
    const int tid = threadIdx.x, warp = tid >> 5;
    const int m = tid, z = m / TY, y = m % TY;
    constexpr uint32_t kCols = 128;  // diagonals D2..D5: 32 columns each
    tc_setup(cm, kCols);
    const uint32_t tbase = cm.tmem + ((uint32_t)(warp * 32) << 16);
    const uint32_t idesc = tc::idesc_f16_f32(MROWS, TX);
    uint32_t phase = 0;
    for (;;) {
        if (tid == 0) cm.tile = atomicAdd(A.queue, 1);
        __syncthreads();
        const int tile = cm.tile;
        if (tile >= A.ntiles || cm.abort) break;
        const TileDesc td = A.tiles[tile];
        const LevelDev &lv = A.levels[td.level];
        float acc_hi[TX], acc_lo[TX];
#pragma unroll
        for (int x = 0; x < TX; x++) acc_hi[x] = acc_lo[x] = 0.0f;
        const int ext_z = min(TZ, lv.ngrid[2] - td.t[2] * TZ), ext_y = min(TY, lv.ngrid[1] - td.t[1] * TY);
        const int ext_x = min(TX, lv.ngrid[0] - td.t[0] * TX);
        const int64_t it_end = A.start[tile + 1];
        for (int64_t it = A.start[tile]; it < it_end && !cm.abort; it++) {
            load_pair(cm, A, A.items[it], false);
            if (tid < 3) {
                const int T = tid == 0 ? TX : (tid == 1 ? TY : TZ);
                axis_images(lv, tid, td.t[tid], T, cm.p, cm.img[tid], cm.nimg[tid], A.status);
            }
            __syncthreads();
            const int L = cm.p.L, lp = cm.p.lp;
            const int nimg = cm.nimg[0] * cm.nimg[1] * cm.nimg[2];
            for (int im = 0; im < nimg && !cm.abort; im++) {
                if (tid == 0) {
                    const int ix = im % cm.nimg[0], iy = (im / cm.nimg[0]) % cm.nimg[1], iz = im / (cm.nimg[0] * cm.nimg[1]);
                    set_image(cm.p, cm.img[0][ix], cm.img[1][iy], cm.img[2][iz], ext_x);
                }
                __syncthreads();
                if (cm.p.gx0 > cm.p.gx1) continue;  // uniform: no x overlap
                load_coef(cm, A);
                __syncthreads();
                recentre_x(cm);
                build_tables(cm, lv, td, true);
                __syncthreads();
                // stage 1: Cxy[z][(b,a)] = sum_g c[g][b][a] Z[g][z]
                const int npair = (L * (L + 1)) / 2;
                for (int t = tid; t < TZ * npair; t += NTHR) {
                    const int zz = t / npair;
                    int q = t - zz * npair, b = 0;
                    while (q >= L - b) { q -= L - b; b++; }
                    const int a = q;
                    ff s = {0.0f, 0.0f};
                    for (int g = 0; g <= lp - a - b; g++) {
                        const float2 c = cm.coef[pidx(lp, g, b, a)];
                        s = ff_fma(ff{c.x, c.y}, cm.Z[g][zz], s);
                    }
                    cm.Cxy[zz][pair_index(L, b, a)] = s;
                }
                // B slices: column x over alpha, scaled by 2^(SLB - fx); four threads per column
                {
                    const int x = tid >> 2, k0 = (tid & 3) * 4;
                    const bool live = k0 < max(L, cm.kmax);
                    float mx = 0.0f;
#pragma unroll
                    for (int k = k0; k < k0 + 4; k++)
                        if (k < L) mx = fmaxf(mx, fabsf(cm.X[k][x].hi));
                    mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, 1));
                    mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, 2));
                    const int e = exp_of(mx);
                    if ((tid & 3) == 0) sm.cs[x] = e == kZeroExp ? 0.0f : pow2i(e);
                    const float sc = e == kZeroExp ? 0.0f : pow2i(SLB - e);
#pragma unroll
                    for (int k = k0; k < k0 + 4 && live; k += 2) {
                        float s0[NSL], s1[NSL];
                        slice_scaled(k < L ? cm.X[k][x] : ff{0.0f, 0.0f}, sc, s0);
                        slice_scaled(k + 1 < L ? cm.X[k + 1][x] : ff{0.0f, 0.0f}, sc, s1);
#pragma unroll
                        for (int q = 0; q < NSL; q++) store_pair(sm.B[q], x, k, s0[q], s1[q]);
                    }
                }
                __syncthreads();
                // stage 2 (this thread's row) + culling + A slices
                int x0, x1;
                row_range(cm.p, A.table, cm.p.o[2] + z, cm.p.o[1] + y, z < ext_z && y < ext_y, x0, x1);
                float mx = 0.0f;
                if (x0 <= x1) {
                    for (int a = 0; a < L; a++) {
                        ff s = {0.0f, 0.0f};
                        for (int b = 0; b <= lp - a; b++) s = ff_fma(cm.Cxy[z][pair_index(L, b, a)], cm.Y[b][y], s);
                        const float bal = pow2i(a * cm.p.sb);  // balancing of the x powers
                        s.hi = __fmul_rn(s.hi, bal);
                        s.lo = __fmul_rn(s.lo, bal);
                        sm.cxs[a][m] = s;
                        mx = fmaxf(mx, fabsf(s.hi));
                    }
                }
                const int em = exp_of(mx);
                {
                    const float sc = em == kZeroExp ? 0.0f : pow2i(SLB - em);
                    const int kl = cm.kmax;  // K slots that may hold values of an earlier pair
#pragma unroll
                    for (int k = 0; k < KP; k += 2) {
                        if (k >= L && k >= kl) break;
                        float s0[NSL], s1[NSL];
                        slice_scaled(k < L && em != kZeroExp ? sm.cxs[k][m] : ff{0.0f, 0.0f}, sc, s0);
                        slice_scaled(k + 1 < L && em != kZeroExp ? sm.cxs[k + 1][m] : ff{0.0f, 0.0f}, sc, s1);
#pragma unroll
                        for (int q = 0; q < NSL; q++) store_pair(sm.A[q], m, k, s0[q], s1[q]);
                    }
                }
                // stage 3 on the tensor cores: D_s = sum_{i+j=s} A_i B_j^T
                tc::fence_async_smem();
                tc::fence_before_sync();
                __syncthreads();
                if (tid == 0) {
                    tc::fence_after_sync();
                    uint64_t ad[NSL], bd[NSL];
#pragma unroll
                    for (int q = 0; q < NSL; q++) {
                        ad[q] = tc::desc_kmajor(sm.A[q], 128, 256);
                        bd[q] = tc::desc_kmajor(sm.B[q], 128, 256);
                    }
                    // diagonal s = i + j into TMEM columns [32 s, 32 s + 32)
#pragma unroll
                    for (int sd = 0; sd < NSL; sd++)
#pragma unroll
                        for (int i = 0; i <= sd; i++) tc::mma_f16(cm.tmem + 32 * sd, ad[i], bd[sd - i], idesc, i > 0);
                    tc::mma_commit(&cm.mbar);
                }
                const bool ok = tc_wait(cm, phase, A.status);
                phase ^= 1u;
                if (!ok) break;
                if (tid == 0) cm.kmax = L;  // read again only after the next barrier
                // tcgen05.ld is warp-collective: chunk decisions are made per warp
                if (__any_sync(0xffffffffu, x0 <= x1)) {
                    const float rs = pow2i(max(em - 2 * SLB, -126));
#pragma unroll
                    for (int c = 0; c < TX / 8; c++) {
                        if (!__any_sync(0xffffffffu, x0 <= x1 && 8 * c <= x1 && 8 * c + 7 >= x0)) continue;
                        uint32_t r2[8], r3[8], r4[8], r5[8];
                        tc::tmem_ld8(tbase + 8 * c, r2);
                        tc::tmem_ld8(tbase + 32 + 8 * c, r3);
                        tc::tmem_ld8(tbase + 64 + 8 * c, r4);
                        tc::tmem_ld8(tbase + 96 + 8 * c, r5);
                        tc::tmem_wait_ld32(r2, r3, r4, r5);
#pragma unroll
                        for (int i = 0; i < 8; i++) {
                            const int x = 8 * c + i;
                            if (x < x0 || x > x1) continue;
                            // value = scl * (D2 + D3 2^-10 + D4 2^-20 + D5 2^-30) as hi + lo with
                            // lo the exact remainder (fast two-sum), then an exact two-sum into
                            // acc_hi: acc_lo then only gathers rounding errors and remainders,
                            // so it stays ~2^-24 below acc_hi however many pairs a point sees
                            const float d2 = __uint_as_float(r2[i]);
                            const float corr = __fmaf_rn(__uint_as_float(r5[i]), 9.313225746154785e-10f,
                                               __fmaf_rn(__uint_as_float(r4[i]), 9.5367431640625e-07f,
                                                         __fmul_rn(__uint_as_float(r3[i]), 0.0009765625f)));
                            const float scl = __fmul_rn(rs, sm.cs[x]);
                            const float h0 = __fadd_rn(d2, corr);
                            const float hi = __fmul_rn(h0, scl);
                            const float lo = __fmul_rn(__fsub_rn(corr, __fsub_rn(h0, d2)), scl);
                            const float sv = __fadd_rn(acc_hi[x], hi);
                            const float bb = __fsub_rn(sv, acc_hi[x]);
                            const float err = __fadd_rn(__fsub_rn(acc_hi[x], __fsub_rn(sv, bb)), __fsub_rn(hi, bb));
                            acc_hi[x] = sv;
                            acc_lo[x] = __fadd_rn(acc_lo[x], __fadd_rn(err, lo));
                        }
                    }
                }
                tc::fence_before_sync();
                __syncthreads();
            }
        }
        if (cm.abort) break;
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
    tc_teardown(cm, kCols, phase);
}

// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(NTHR, 2) k_integrate_tiled(MixedArgs A) {
    extern __shared__ __align__(128) unsigned char smraw[];
    SmemInt &sm = *reinterpret_cast<SmemInt *>(smraw);
    TileCommon &cm = sm.c;
    const int tid = threadIdx.x, warp = tid >> 5;
    const int m = tid, z = m / TY, y = m % TY;
    constexpr uint32_t kCols = 128;  // D2 (two K halves), D3, D4, D5: 16 columns each
    tc_setup(cm, kCols);
    const uint32_t tbase = cm.tmem + ((uint32_t)(warp * 32) << 16);
    const uint32_t idesc = tc::idesc_f16_f32(MROWS, KP);
    uint32_t phase = 0;
    for (;;) {
        if (tid == 0) cm.tile = atomicAdd(A.queue, 1);
        __syncthreads();
        const int tile = cm.tile;
        if (tile >= A.ntiles || cm.abort) break;
        const TileDesc td = A.tiles[tile];
        const LevelDev &lv = A.levels[td.level];
        const int ext_z = min(TZ, lv.ngrid[2] - td.t[2] * TZ), ext_y = min(TY, lv.ngrid[1] - td.t[1] * TY);
        const int ext_x = min(TX, lv.ngrid[0] - td.t[0] * TX);
        // this thread's V row, sliced once per tile (row exponent vm)
        int vm;
        {
            const double *grid = A.grids.p[td.level];
            const bool ok = z < ext_z && y < ext_y;
            const int64_t row = ((int64_t)(td.t[2] * TZ + z) * lv.ngrid[1] + (td.t[1] * TY + y)) * lv.ngrid[0] +
                                td.t[0] * TX;
            ff v[TX];
#pragma unroll
            for (int x = 0; x < TX; x++) v[x] = (ok && x < ext_x) ? ff_from_double(grid[row + x]) : ff{0.0f, 0.0f};
            float mx = 0.0f;
#pragma unroll
            for (int x = 0; x < TX; x++) mx = fmaxf(mx, fabsf(v[x].hi));
            vm = exp_of(mx);
            const float sc = vm == kZeroExp ? 0.0f : pow2i(SLB - vm);
#pragma unroll
            for (int x = 0; x < TX; x += 2) {
                float s0[NSL], s1[NSL];
                slice_scaled(v[x], sc, s0);
                slice_scaled(v[x + 1], sc, s1);
#pragma unroll
                for (int q = 0; q < NSL; q++)
                    *reinterpret_cast<__half2 *>(&sm.Vs[q][m][x]) = __floats2half2_rn(s0[q], s1[q]);
            }
        }
        for (int64_t it = A.start[tile]; it < A.start[tile + 1] && !cm.abort; it++) {
            load_pair(cm, A, A.items[it]);
            if (tid < 3) {
                const int T = tid == 0 ? TX : (tid == 1 ? TY : TZ);
                axis_images(lv, tid, td.t[tid], T, cm.p, cm.img[tid], cm.nimg[tid], A.status);
            }
            __syncthreads();
            const int L = cm.p.L, lp = cm.p.lp;
            const int npair = (L * (L + 1)) / 2;
            const int64_t moff = cm.p.coef_off;
            const int nimg = cm.nimg[0] * cm.nimg[1] * cm.nimg[2];
            for (int im = 0; im < nimg && !cm.abort; im++) {
                if (tid == 0) {
                    const int ix = im % cm.nimg[0], iy = (im / cm.nimg[0]) % cm.nimg[1], iz = im / (cm.nimg[0] * cm.nimg[1]);
                    set_image(cm.p, cm.img[0][ix], cm.img[1][iy], cm.img[2][iz], ext_x);
                }
                __syncthreads();
                if (cm.p.gx0 > cm.p.gx1) continue;
                build_tables(cm, lv, td);
                // A operand: this row's V slices masked to the row's cube range
                int x0, x1;
                row_range(cm.p, A.table, cm.p.o[2] + z, cm.p.o[1] + y, z < ext_z && y < ext_y, x0, x1);
#pragma unroll
                for (int x = 0; x < TX; x += 2) {
                    const bool in0 = x >= x0 && x <= x1, in1 = x + 1 >= x0 && x + 1 <= x1;
                    const int o = umma_off(m, x & 15) >> 1, h = x >> 4;
#pragma unroll
                    for (int q = 0; q < NSL; q++) {
                        __half2 v2 = *reinterpret_cast<const __half2 *>(&sm.Vs[q][m][x]);
                        if (!in0) v2.x = __float2half_rn(0.0f);
                        if (!in1) v2.y = __float2half_rn(0.0f);
                        *reinterpret_cast<__half2 *>(&sm.A[h][q][o]) = v2;
                    }
                }
                __syncthreads();
                // B operand: X slices per alpha over x (exponent gexp[alpha]); eight threads per alpha
                {
                    const int a = tid >> 3, x0b = (tid & 7) * 4;
                    float mxb = 0.0f;
#pragma unroll
                    for (int x = x0b; x < x0b + 4; x++) mxb = fmaxf(mxb, fabsf(cm.X[a][x].hi));
                    mxb = fmaxf(mxb, __shfl_xor_sync(0xffffffffu, mxb, 1));
                    mxb = fmaxf(mxb, __shfl_xor_sync(0xffffffffu, mxb, 2));
                    mxb = fmaxf(mxb, __shfl_xor_sync(0xffffffffu, mxb, 4));
                    const int e = exp_of(mxb);
                    if ((tid & 7) == 0) sm.gexp[a] = e;
                    const float sc = e == kZeroExp ? 0.0f : pow2i(SLB - e);
#pragma unroll
                    for (int x = x0b; x < x0b + 4; x += 2) {
                        float s0[NSL], s1[NSL];
                        slice_scaled(cm.X[a][x], sc, s0);
                        slice_scaled(cm.X[a][x + 1], sc, s1);
                        const int o = umma_off(a, x & 15) >> 1, h = x >> 4;
#pragma unroll
                        for (int q = 0; q < NSL; q++)
                            *reinterpret_cast<__half2 *>(&sm.B[h][q][o]) = __floats2half2_rn(s0[q], s1[q]);
                    }
                }
                tc::fence_async_smem();
                tc::fence_before_sync();
                __syncthreads();
                if (tid == 0) {
                    tc::fence_after_sync();
                    uint64_t a_[2][NSL], b_[2][NSL];
                    for (int h = 0; h < 2; h++)
                        for (int q = 0; q < NSL; q++) {
                            a_[h][q] = tc::desc_kmajor(sm.A[h][q], 128, 256);
                            b_[h][q] = tc::desc_kmajor(sm.B[h][q], 128, 256);
                        }
                    // D2 per K half (exact: 16 products each); diagonals 3.. over both halves
                    tc::mma_f16(cm.tmem + 0, a_[0][0], b_[0][0], idesc, 0);
                    tc::mma_f16(cm.tmem + 16, a_[1][0], b_[1][0], idesc, 0);
#pragma unroll
                    for (int sd = 1; sd < NSL; sd++) {
                        int first = 1;
#pragma unroll
                        for (int i = 0; i <= sd; i++)
#pragma unroll
                            for (int h = 0; h < 2; h++) {
                                tc::mma_f16(cm.tmem + 16 + 16 * sd, a_[h][i], b_[h][sd - i], idesc, first ? 0u : 1u);
                                first = 0;
                            }
                    }
                    tc::mma_commit(&cm.mbar);
                }
                const bool ok = tc_wait(cm, phase, A.status);
                phase ^= 1u;
                if (!ok) break;
#pragma unroll
                for (int c = 0; c < KP / 8; c++) {
                    uint32_t ra[8], rb[8], r3[8], r4[8], r5[8];
                    tc::tmem_ld8(tbase + 8 * c, ra);
                    tc::tmem_ld8(tbase + 16 + 8 * c, rb);
                    tc::tmem_ld8(tbase + 32 + 8 * c, r3);
                    tc::tmem_ld8(tbase + 48 + 8 * c, r4);
                    tc::tmem_wait_ld32(ra, rb, r3, r4);
                    tc::tmem_ld8(tbase + 64 + 8 * c, r5);
                    tc::tmem_wait_ld8(r5);
#pragma unroll
                    for (int i = 0; i < 8; i++) {
                        const int a = 8 * c + i;
                        ff s = {0.0f, 0.0f};
                        if (a < L && x0 <= x1) {
                            const ff d2 = two_sum(__uint_as_float(ra[i]), __uint_as_float(rb[i]));
                            ff t = two_sum(d2.hi, __fmul_rn(__uint_as_float(r3[i]), 0.0009765625f));
                            t.lo = __fadd_rn(t.lo, __fmaf_rn(__uint_as_float(r4[i]), 9.5367431640625e-07f,
                                                             __fmaf_rn(__uint_as_float(r5[i]), 9.313225746154785e-10f, d2.lo)));
                            t = fast_two_sum(t.hi, t.lo);
                            const int E = vm + sm.gexp[a] - 2 * SLB;
                            if (E >= -126 && vm != kZeroExp && sm.gexp[a] != kZeroExp) {
                                const float scl = pow2i(min(E, 127));
                                s = {__fmul_rn(t.hi, scl), __fmul_rn(t.lo, scl)};
                            }
                        }
                        sm.S[m][a] = s;
                    }
                }
                tc::fence_before_sync();
                __syncthreads();
                // stage 2 transposed: T[z][(b,a)] = sum_y S[(z,y)][a] Y[b][y]
                for (int t = tid; t < TZ * npair; t += NTHR) {
                    const int zz = t / npair;
                    int q = t % npair, b = 0;
                    while (q >= L - b) { q -= L - b; b++; }
                    const int a = q;
                    ff s = {0.0f, 0.0f};
                    for (int yy = 0; yy < TY; yy++) s = ff_fma(sm.S[zz * TY + yy][a], cm.Y[b][yy], s);
                    cm.Cxy[zz][pair_index(L, b, a)] = s;
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
                    for (int zz = 0; zz < TZ; zz++) s = ff_fma(cm.Cxy[zz][pi], cm.Z[g][zz], s);
                    if (s.hi != 0.0f) atomicAdd(A.mom + moff + t, (double)s.hi + (double)s.lo);
                }
                __syncthreads();
            }
        }
        if (cm.abort) break;
    }
    tc_teardown(cm, kCols, phase);
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
// Tiles one cube axis touches, with the smallest folded offset |f| (f = g <= 0 ?
// -g : g - 1) of the cube offsets g that land in each tile.
struct AxisTile {
    int tile;
    int fmin;
};
void axis_tiles(const LevelDev &lv, int d, const PairGeom &g, int T, std::vector<AxisTile> &out) {
    out.clear();
    const int N = lv.ngrid[d];
    const int nt = (N + T - 1) / T;
    std::vector<int> best(nt, INT32_MAX);
    for (int gg = g.lb[d]; gg <= g.hi[d];) {
        int w;
        if (lv.periodic[d]) w = imod(g.cc[d] + gg, lv.npts[d]);
        else w = gg + imod(g.cc[d] + g.lb[d] + lv.lb_grid[d], lv.npts[d]) - g.lb[d];
        if (w < 0 || w >= N) { gg++; continue; }
        const int t = w / T;
        const int len = std::min(T - (w - t * T), N - w);
        const int g1 = std::min(gg + len - 1, g.hi[d]);
        // smallest folded offset over [gg, g1]
        const int f = (gg <= 1 && g1 >= 0) ? 0 : (g1 < 0 ? -g1 : gg - 1);
        best[t] = std::min(best[t], f);
        gg += len;
    }
    for (int t = 0; t < nt; t++)
        if (best[t] != INT32_MAX) out.push_back(AxisTile{t, best[t]});
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
    std::vector<AxisTile> ax, ay, az;
    // a pair visits a tile only if some cube point of the tile can be inside its
    // sphere: folded distance of the tile's nearest offsets <= radius (with margin)
    auto each = [&](auto &&fn) {
        for (int64_t k = 0; k < northo; k++) {
            const PairGeom &g = ts.h_geom[k];
            const LevelDev &lv = P.lv[g.level];
            axis_tiles(lv, 0, g, TX, ax);
            axis_tiles(lv, 1, g, TY, ay);
            axis_tiles(lv, 2, g, TZ, az);
            const int base = lvl_first[g.level];
            const double r2 = g.radius * g.radius * (1.0 + 1e-9) + 1e-12;
            const double hx = lv.dh[0][0], hy = lv.dh[1][1], hz = lv.dh[2][2];
            const bool table = g.table_off >= 0;  // explicit cube lists: no culling
            for (const AxisTile &c : az) {
                const double dz = c.fmin * hz;
                if (!table && dz * dz > r2) continue;
                for (const AxisTile &b : ay) {
                    const double dy = b.fmin * hy;
                    if (!table && dz * dz + dy * dy > r2) continue;
                    for (const AxisTile &a : ax) {
                        const double dx = a.fmin * hx;
                        if (!table && dz * dz + dy * dy + dx * dx > r2) continue;
                        fn(base + (c.tile * nty[g.level] + b.tile) * ntx[g.level] + a.tile, (int)k);
                    }
                }
            }
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
    std::vector<TPair> pairs((size_t)std::max<int64_t>(northo, 1));
    auto split = [](double d) {
        const float h = (float)d;
        return ff{h, (float)(d - (double)h)};
    };
    for (int64_t k = 0; k < northo; k++) {
        const PairGeom &g = ts.h_geom[k];
        const LevelDev &lv = P.lv[g.level];
        TPair &p = pairs[k];
        memset(&p, 0, sizeof p);
        p.r2 = rmul(g.radius, g.radius);
        p.hx = lv.dh[0][0];
        p.hy = lv.dh[1][1];
        p.hz = lv.dh[2][2];
        p.r2f = (float)p.r2;
        p.hxf = (float)p.hx;
        p.hyf = (float)p.hy;
        p.hzf = (float)p.hz;
        p.zetp = split(g.zetp);
        for (int d = 0; d < 3; d++) {
            p.off[d] = split(g.off[d]);
            p.h[d] = split(lv.dh[d][d]);
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
    alloc((void **)&M->d_pairs, sizeof(TPair) * pairs.size());
    if (e == cudaSuccess)
        e = cudaMemcpy(M->d_pairs, pairs.data(), sizeof(TPair) * pairs.size(), cudaMemcpyHostToDevice);
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
    e = cudaFuncSetAttribute((const void *)k_collocate_tiled, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)sizeof(SmemColl));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute((const void *)k_integrate_tiled, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)sizeof(SmemInt));
    if (e != cudaSuccess) {
        err = std::string("mixed_build: ") + cudaGetErrorString(e);
        return GPW_ERR_CUDA;
    }
    // resident CTAs per SM from the kernels' own resources; TMEM (128 of 512
    // columns per CTA) caps it at 4
    auto resident = [&](const void *fn, size_t dyn) {
        cudaFuncAttributes fa;
        if (cudaFuncGetAttributes(&fa, fn) != cudaSuccess) return 1;
        int smem_sm = 0, regs_sm = 0;
        cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, P.device);
        cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, P.device);
        const int by_regs = regs_sm / std::max(1, ((fa.numRegs * 32 + 255) / 256) * 256 * (NTHR / 32));
        const int by_smem = (int)(smem_sm / (dyn + fa.sharedSizeBytes + 1024));
        return std::max(1, std::min({by_regs, by_smem, 4}));
    };
    per_sm = resident((const void *)k_collocate_tiled, sizeof(SmemColl));
    const int per_sm_i = resident((const void *)k_integrate_tiled, sizeof(SmemInt));
    M->per_sm = per_sm;
    M->per_sm_i = per_sm_i;
    M->grid_ctas_i = std::max(1, std::min(ntiles, sms * per_sm_i));
    M->grid_ctas = std::max(1, std::min(ntiles, sms * per_sm));
    return GPW_SUCCESS;
}

void mixed_free(TaskSet &ts) {
    MixedState *M = ts.mixed;
    if (!M) return;
    cudaFree(M->d_tiles);
    cudaFree(M->d_pairs);
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
    a.pairs = M.d_pairs;
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
        k_collocate_tiled<<<M.grid_ctas, NTHR, sizeof(SmemColl), s>>>(make_args(ts, g, 0));
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
        k_integrate_tiled<<<M.grid_ctas_i, NTHR, sizeof(SmemInt), s>>>(make_args(ts, g, 1));
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    return general_fp64(ts, g, true, s);
}

}  // namespace gpw
