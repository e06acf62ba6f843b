// Tiled mixed-precision collocate / integrate.
//
// Persistent CTAs take work units from an atomic queue.  A unit is one tile of
// one grid level (TX x TY x TZ points, x fastest; TX = 32, TY x TZ = 128 rows with
// TZ = 4 or 8 per level, chosen by the tile autotuner) with the pairs whose cube
// touches it, or a part of that list for the busiest tiles (those units flush
// with atomics).  The pair records, coefficients and per-tile images are copied
// one item ahead with cp.async.  Per pair and tile:
//   1-D tables t^k exp(-zetp t^2) over the tile's three ranges   (float-float)
//   stage 1  Cxy[z][b][a] = sum_g c[g][b][a] Z[g][z]              (float-float)
//   stage 2  Cx[(z,y)][a] = sum_b Cxy[z][b][a] Y[b][y]            (float-float)
//   stage 3  rho[(z,y)][x] = sum_a Cx[(z,y)][a] X[a][x]           (exact fp16 slices)
// (the three contractions of collocate_core, collocate.cc:543-623, with the
// cube culling of grid_collocate_core, grid_base_ref_c.cc:413-471).
//
// Stage 3 operands are split into NSL fixed-point fp16 slices of SLB bits: each
// row of Cx is scaled by a power of two so its largest entry is < 2^SLB, each
// column of X likewise, and the slices are integers (the first in [-2^SLB,
// 2^SLB], the others in [-2^(SLB-1), 2^(SLB-1)]).  They carry the float-float
// operand to ~2^-35 of its row's scale (its low part enters through one float32
// remainder).  Every slice product is an integer of at most 2^20, so the
// anti-diagonal sums D_s = sum over i+j=s of A_i B_j are exact in FP32 for the
// leading two (16 and 32 products, at most 2^24); the next two (3 and 4 MMAs
// into one accumulator) can pass 2^24 only in the worst case, where their
// rounding stays below 2^-40 of the scales.  (Integrate contracts 32 x: D2 is
// kept as two K halves of 16 products; its D3 sums 64 and can round in the worst
// case, by less than 2^-35 of the scales.)  The diagonals are recombined in
// float-float.  The tile sum
// over pairs is float-float (high parts in registers, low parts in shared
// memory), added to the FP64 grid once per tile.
//
// Integrate is the transpose: S[(z,y)][a] = sum_x V[(z,y)][x] X[a][x] by the same
// slices (V sliced once per tile into a per-CTA global slot that stays in L1/L2,
// copied per pair into the operand with the pair's row masks), then the adjoint
// stages, and the per-pair moments are added to FP64 scratch with atomics.
//
// General (non-orthorhombic) cells use the same kernels instantiated with
// kGeneral (t_d along the lattice steps, the quadratic row rule, the Gaussian's
// cross factor per point) when their level has a tile shape; by default they
// run on the float-float general kernel (gpw_fp64.cu).
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "gpw_coef.cuh"
#include "gpw_ff.cuh"
#include "gpw_internal.h"
#include "gpw_tc.cuh"

namespace gpw {

constexpr int TX = 32;
constexpr int MROWS = 128;       // TY * TZ rows per tile, one per thread
constexpr int kMaxTY = 32, kMaxTZ = 8;  // tiles of 32 x 16 x 8 or 32 x 32 x 4
constexpr int kMaxTZColl = 8;  // collocate keeps its stage-1 output for at most 8 z (tiles with TZ <= 8)
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
    int lz;    // log2 TZ (TY = MROWS >> lz)
    int split; // the tile's pairs are divided among several work units: flush with atomics
};

// tile extents of a tile descriptor
struct TileShape {
    int TY, TZ, ly, lz;
    __host__ __device__ explicit TileShape(int lz_) : TY(MROWS >> lz_), TZ(1 << lz_), ly(7 - lz_), lz(lz_) {}
};

// ---------------------------------------------------------------------------
// pair data a tile needs, staged in shared memory
struct TPair {
    double r2;          // radius^2 (FP64, rule decisions)
    double hz, hy, hx;  // spacings (orthorhombic rule); general cell: 1 / |v_2|, 1 / |v_1|, 1 / |v_0|
    float r2f, hzf, hyf, hxf;
    float hyinvf, hxinvf;  // 1/hy, 1/hx rounded to float
    ff zetp;
    ff off[3];          // roffset
    ff h[3];
    int lb[3], hi[3], cc[3];
    int kgmin, lp, L;
    int general, pad_;  // general cell: box-relative cube (lb = 0), lattice-step lengths in h
    int64_t coef_off, table_off;
    double gp[3];       // general: the product centre in lattice coordinates (dh_inv^T rp)
    double radius;      // general: the cube radius (the row rule squares it itself)
};
// General-cell level constants of the tiled path: FP32 lattice steps for the row
// rule, and the cosines between the steps (cross terms of the Gaussian).
struct GenLevel {
    float dh[3][3];
    float a, inv2a;     // |v0|^2 and 1 / (2 |v0|^2)
    ff c01, c02, c12;   // cos(v0, v1), cos(v0, v2), cos(v1, v2)
};
// A pair's blob: the record padded to kHdr16 16-byte chunks, then its
// coefficients as float-float (written by every collocate call), padded to 16 bytes.
constexpr int kHdr16 = (int)((sizeof(TPair) + 15) / 16);
constexpr int kCoef16Max = (NCOEF_MAX * (int)sizeof(float2) + 15) / 16;

// the current periodic image of a pair over the tile
struct ImgState {
    ff tc;              // collocate: x of the re-expansion column minus xp
    int o[3];           // cube offset of the tile origin
    int gx0, gx1;       // tile-local x range inside the cube box
    int ic;             // collocate: tile-local re-expansion column
    int sb;             // collocate: x-variable scale 2^sb of the slices (balancing)
};

// Per (tile, pair) item, computed once per task set: the images of the pair's
// cube over the tile (counts per axis packed as n0 | n1 << 8 | n2 << 16) and the
// state of the first image.  Items with more than one image (small periodic
// cells) derive the others in the kernel.
struct alignas(16) ItemImg {
    ImgState im;
    int nimg;
};
static_assert(sizeof(ItemImg) == 48, "ItemImg is three 16-byte chunks");

struct MixedState {
    int ntiles = 0;
    int64_t nitems = 0;
    TileDesc *d_tiles = nullptr;
    uint4 *d_blob = nullptr;       // pair blobs of the orthorhombic tasks (sorted order)
    int64_t *d_blob_off = nullptr; // per task: blob offset in 16-byte chunks
    int64_t *d_start = nullptr;    // per work unit: first item, end
    uint64_t *d_items = nullptr;   // per (tile, pair): blob offset << 16 | chunks
    ItemImg *d_iimg = nullptr;     // per (tile, pair): images
    int *d_queue = nullptr;      // [0]: collocate, [1]: integrate (orthorhombic tiles), [2], [3]: general tiles
    GenLevel *d_glv = nullptr;   // per level (general levels only meaningful)
    int northo = 0;              // ortho tasks come first in sorted order
    int64_t nbin = 0;            // tasks [0, nbin) are binned (the ortho ones, then general ones if tiled)
    bool gen_tiled = false;      // general-cell pairs run on the tiled kernels
    int ntiles_ortho = 0;        // tiles [0, ntiles_ortho) are orthorhombic, the rest general
    int grid_ctas = 0;    // collocate
    int grid_ctas_i = 0;  // integrate
    int sms = 0;
    int per_sm = 0, per_sm_i = 0, per_sm_ig = 0;  // resident CTAs: collocate, integrate (ortho, general)
    uint4 *d_vslot = nullptr;  // orthorhombic integrate: per-CTA V slots
    // binning state kept for re-binning on the device (gpw_taskset_update_geometry)
    std::vector<TileDesc> h_tiles;  // every tile of the binned levels, in tile-index order
    struct BinLevel *d_bl = nullptr;  // per level: first tile index, tiles per axis, tile shape
    int *d_blob_len = nullptr;      // per binned pair: chunks of its blob
    int *d_count = nullptr;         // per tile: items
    unsigned long long *d_cursor = nullptr;  // per tile: next item slot (fill pass)
    int64_t cap_items = 0, cap_units = 0;    // capacities of d_items / d_iimg and d_tiles / d_start
};


// ---------------------------------------------------------------------------
// Sphere rule with an FP32 fast path.  The FP32 estimate decides unless it lies
// within its error bound of an integer; then the exact FP64 rule (the one the
// host and the oracle use) decides.
__device__ __forceinline__ int fast_floor_checked(float rem, float r2f, float hinv, bool &unsure) {
    const float rc = fmaxf(rem, 0.0f);
    const float rs = rsqrtf(fmaxf(rc, 1e-30f));
    const float v = __fmul_rn(__fmul_rn(rc, rs), hinv);  // sqrt(rc) / h, relative error < 2^-21
    const float fl = floorf(v);
    // error of rem ~ 4 ulp(r2f); of sqrt ~ err/(2 sqrt); plus relative 2^-19
    const float erem = r2f * 4.8e-7f;
    const float ev = __fmul_rn(erem * 0.5f, rs) * hinv + v * 2e-6f + 1e-6f;
    unsure = (v - fl) <= ev || (fl + 1.0f - v) <= ev || rem <= erem;
    return (int)fl;
}

// the exact FP64 rule, out of line: taken only where the FP32 estimate is unsure
__device__ __noinline__ int rule_jmax_exact(const TPair &p, int kf) { return rule_jmax(rule_remk(p.r2, kf, p.hz), p.hy); }
__device__ __noinline__ int rule_imax_exact(const TPair &p, int kf, int jf) {
    return rule_imax(rule_remk(p.r2, kf, p.hz), jf, p.hy, p.hx);
}

__device__ __forceinline__ int row_jmax(const TPair &p, int kf) {
    const float dz = (float)(-kf) * p.hzf;
    bool unsure;
    int j = fast_floor_checked(__fmaf_rn(-dz, dz, p.r2f), p.r2f, p.hyinvf, unsure);
    if (unsure) j = rule_jmax_exact(p, kf);
    return j;
}

__device__ __forceinline__ int row_imax(const TPair &p, int kf, int jf) {
    const float dz = (float)(-kf) * p.hzf, dy = (float)(-jf) * p.hyf;
    bool unsure;
    int i = fast_floor_checked(__fmaf_rn(-dy, dy, __fmaf_rn(-dz, dz, p.r2f)), p.r2f, p.hxinvf, unsure);
    if (unsure) i = rule_imax_exact(p, kf, jf);
    return i;
}

// Row (z, y) of the tile: cube-local x range [x0, x1] (empty if x0 > x1).
__device__ __forceinline__ void row_range(const TPair &p, const ImgState &q, const int *table, int gz, int gy,
                                          int ext_ok, int &x0, int &x1) {
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
    x0 = max(imin - q.o[0], q.gx0);
    x1 = min(1 - imin - q.o[0], q.gx1);
}

// General cell: the row (jj, kk) of the index box holds the points i with
// |i v0 + w|^2 <= r^2 (the reference's quadratic, grid_base_ref_c.cc:781-807).
// FP32 estimate in box-relative units i' = i - cc0 with a running error bound;
// the exact FP64 rule (general_row, gpw_common.cuh) decides where a root lies
// within its bound of an integer or the discriminant within its bound of zero.
__device__ __noinline__ bool general_row_exact(const LevelDev &lv, const TPair &p, int jj, int kk, int &ismin,
                                               int &ismax) {
    const double dj = rsub((double)jj, p.gp[1]), dk = rsub((double)kk, p.gp[2]);
    return general_row(lv.dh, p.gp, dj, dk, p.radius, ismin, ismax);
}

__device__ __forceinline__ bool general_row_fast(const LevelDev &lv, const GenLevel &G, const TPair &p, int jj,
                                                 int kk, int &ismin, int &ismax) {
    const float eps = 1.2e-7f;  // 2^-23, with room
    const float gj = (float)(p.gp[1] - (double)p.cc[1]), gk = (float)(p.gp[2] - (double)p.cc[2]);
    const float gi = (float)(p.gp[0] - (double)p.cc[0]);
    const float dj = (float)(jj - p.cc[1]) - gj, dk = (float)(kk - p.cc[2]) - gk;
    float b = 0.0f, c = 0.0f, eb = 0.0f, ec = 0.0f;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        // v_i = dk dh2_i + dj dh1_i - gi dh0_i (box-relative), with its error bound
        const float v = __fsub_rn(__fadd_rn(__fmul_rn(G.dh[2][i], dk), __fmul_rn(G.dh[1][i], dj)),
                                  __fmul_rn(gi, G.dh[0][i]));
        const float ev = eps * (fabsf(G.dh[2][i]) * (2.0f * fabsf(dk) + fabsf(gk)) +
                                fabsf(G.dh[1][i]) * (2.0f * fabsf(dj) + fabsf(gj)) +
                                2.0f * fabsf(gi * G.dh[0][i]) + 2.0f * fabsf(v));
        b = __fadd_rn(b, __fmul_rn(2.0f * v, G.dh[0][i]));
        c = __fadd_rn(c, __fmul_rn(v, v));
        eb += 2.0f * ev * fabsf(G.dh[0][i]) + 2.0f * eps * fabsf(b);
        ec += (2.0f * fabsf(v) + ev) * ev + 2.0f * eps * c;
    }
    // d = b^2 - 4a(c - r^2): propagated input errors, the representation errors of
    // a and r^2, and the rounding of each operation
    const float a = G.a, r2 = p.r2f;
    const float cr = __fsub_rn(c, r2);
    const float d = __fsub_rn(__fmul_rn(b, b), __fmul_rn(4.0f * a, cr));
    const float ed = 2.0f * fabsf(b) * eb + eb * eb + eps * b * b +
                     4.0f * a * (ec + eps * r2 + 2.5f * eps * fabsf(cr)) + eps * fabsf(d);
    bool unsure = fabsf(d) <= 1.5f * ed;
    if (!unsure && d < 0.0f) return false;  // surely empty
    if (!unsure) {
        const float sd = sqrtf(d);
        const float esd = 1.8f * ed / sd + eps * sd;  // d > 1.5 ed: sqrt(d - ed) >= sd / sqrt(3)
        const float lo = __fmul_rn(__fsub_rn(-b, sd), G.inv2a), hi = __fmul_rn(__fadd_rn(-b, sd), G.inv2a);
        const float er = 1.25f * ((eb + esd + eps * (fabsf(b) + sd)) * G.inv2a + 1.5f * eps * (fabsf(lo) + fabsf(hi))) +
                         1e-6f;
        unsure = fabsf(lo - rintf(lo)) <= er || fabsf(hi - rintf(hi)) <= er;
        ismin = p.cc[0] + (int)ceilf(lo);
        ismax = p.cc[0] + (int)floorf(hi);
    }
    if (unsure) return general_row_exact(lv, p, jj, kk, ismin, ismax);
    return true;
}

// Row (z, y) of the tile for a general-cell pair: tile-local x range [x0, x1].
__device__ __forceinline__ void general_row_range(const LevelDev &lv, const GenLevel &G, const TPair &p,
                                                  const ImgState &q, int gz, int gy, int ext_ok, int &x0,
                                                  int &x1) {
    x0 = 1;
    x1 = 0;
    if (!ext_ok || gz < 0 || gz > p.hi[2] || gy < 0 || gy > p.hi[1]) return;
    int ismin, ismax;
    if (!general_row_fast(lv, G, p, p.cc[1] + gy, p.cc[2] + gz, ismin, ismax)) return;
    x0 = max(ismin - p.cc[0] - q.o[0], q.gx0);
    x1 = min(ismax - p.cc[0] - q.o[0], q.gx1);
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

struct MixedArgs {
    const uint4 *blob;        // per pair: record (kHdr16 chunks) then float-float coefficients
    const PairGeom *geoms;
    const LevelDev *levels;
    const TileDesc *tiles;
    const int64_t *start;
    const uint64_t *items;    // per (tile, pair): blob offset in 16-byte chunks << 16 | chunks to copy
    const ItemImg *iimg;      // per (tile, pair): images
    const int *table;
    const GenLevel *glv;  // general levels: FP32 steps, cosines
    double *mom;  // integrate: per-pair moments
    uint4 *vslot;  // orthorhombic integrate: one slot of kVSlot16 chunks per CTA (the tile's V slices)
    GridPtrs grids;
    int *queue;
    int *status;
    int ntiles;
};

// one pair as staged in shared memory: the record, then its coefficients
// (collocate only), in the blob's own layout so that it is copied chunk by chunk
struct alignas(16) PairBuf {
    union {
        TPair p;
        uint4 hdr_[kHdr16];
    };
    float2 coef[2 * kCoef16Max];
};
// the record alone (integrate)
struct alignas(16) PairHdr {
    union {
        TPair p;
        uint4 hdr_[kHdr16];
    };
};

// shared state of both tiled kernels
struct TileCommon {
    ItemImg ii[2];  // images over this tile of the current pair and of the one being fetched
    ImgState im;    // images after the first of a multi-image item
    ff Y[kNPow][kMaxTY + 1];  // rows padded: lanes reading different rows hit different banks
    ff Z[kNPow][kMaxTZ + 1];
    int tile;
    int img[3][kMaxImages];
    int nimg[3];
    uint64_t mbar;
    uint32_t tmem;
    int abort;
    int kmax;  // collocate: K slots of A written by the previous pair (zeroed up to here)
};

struct alignas(128) SmemColl {
    __half A[NSL][MROWS * KP];  // Cx slices, M=128 x K=16
    __half B[NSL][TX * KP];     // X slices, N=32 x K=16
    ff rc[NCOEF_MAX];           // coefficients re-expanded around the tile's column ic
    ff Cxy[kMaxTZColl][NPAIR_MAX];  // stage 1 output
    ff cxy_pad_[4];             // stage-2 reads up to 3 entries past a row
    PairBuf pb[2];              // the current pair and the one being fetched
    float acc_lo[MROWS][TX + 1];  // low parts of the tile sums (row m belongs to thread m; padded rows)
    float bin[kNPow][kNPow];    // binomials C(a', a) of the re-expansion
    alignas(16) float cs[TX];   // 2^fx per column (0 for an empty column)
    unsigned char qb[kNPow][NPAIR_MAX + 2];  // qb[L-1][pair_index(L, b, a)] = b
    int zs[kNPow + 1];          // zs[g]: packed index of (g, 0, 0) for the current pair's lp
    TileCommon c;
};

static_assert(4 * (sizeof(SmemColl) + 1024) <= 228 * 1024, "4 collocate CTAs per SM");

// The V slices of the tile an orthorhombic integrate CTA works on (the A
// operand's layout, both K halves, all slices): 32 KB in a per-CTA global slot
// that stays in L1/L2 while the tile's items are processed.  Kept out of shared
// memory, they leave room for 4 CTAs per SM.  General cells keep V as
// float-float in shared memory (the rows are rescaled per image).
constexpr int kVSlot16 = 2 * NSL * MROWS * KP / 8;
template <bool kGeneral>
struct IntVTile {};
template <>
struct IntVTile<true> {
    ff Vff[TX][MROWS];  // general cell: this tile's V (x-major: lanes read consecutive rows)
};

// Integrate's S[(z,y)][alpha] rows hold KP + 1 values (row stores by thread
// (z,y) spread over the banks), and the block of rows of z starts 8 ceil(z/2)
// values later still: the rows of z = 2w and 2w + 1, which the lanes of stage 2T
// read side by side at the same alpha (16 x 34 words apart, one bank otherwise),
// then lie 16 banks apart, and no block runs into the next.  T rows hold NPAIR_T
// values (2 NPAIR_T = 16 mod 32 words) for the same reason.
constexpr int kSRow = KP + 1;
constexpr int NPAIR_T = NPAIR_MAX + (24 - NPAIR_MAX % 16) % 16;
static_assert((2 * NPAIR_T) % 32 == 16, "T rows of adjacent z 16 banks apart");
__device__ __forceinline__ int s_index(int row, int ly) { return row * kSRow + 8 * (((row >> ly) + 1) >> 1); }

// Integrate's B operand (N = 16 alpha x K = 16 x per half, per slice): core
// matrices 160 bytes apart along K and 288 along N, the second K half 64 bytes
// further on.  Warp 0 stores one alpha row at a time, lane (h, k) the 2-byte
// element (alpha, k) of half h: the four groups of 8 lanes (h, k / 8) then fill
// four disjoint sets of 4 banks (the dense layout, 128 and 2048 bytes apart, put
// all four into the same banks).
constexpr int kBLbo = 160, kBSbo = 288, kBPlane = 576;       // bytes
constexpr int kBHalf = NSL * kBPlane + 64;                   // bytes from half 0 to half 1
__host__ __device__ constexpr int b_off(int row, int k) {    // bytes within a plane
    return (row >> 3) * kBSbo + (k >> 3) * kBLbo + (row & 7) * 16 + (k & 7) * 2;
}
static_assert(b_off(15, 15) + 2 <= kBPlane && kBPlane % 16 == 0 && kBHalf % 16 == 0, "B planes");

template <bool kGeneral>
struct alignas(128) SmemInt : IntVTile<kGeneral> {
    union {
        __half A[2][NSL][MROWS * KP];  // masked V slices, K halves x in [0,16) and [16,32)
        struct {                       // after the MMAs have read A:
            ff S[MROWS * kSRow + 8 * (kMaxTZ / 2)];  //   S[(z,y)][alpha] at s_index((z,y)) + alpha
            ff T[kMaxTZ][NPAIR_T];     //   stage-2 output T[z][(b,a)]
        } st;
    };
    alignas(16) unsigned char B[2 * kBHalf];  // X' slices: plane (h, q) at h kBHalf + q kBPlane
    int vmr[MROWS];  // general cell: each row's exponent of V E in the current image
    int gexp[KP];
    signed char rx0[MROWS], rx1[MROWS];  // each row's cube x range in the current image
    unsigned char qb[kNPow][NPAIR_MAX + 2];  // qb[L-1][pair_index(L, b, a)] = b
    int zs[kNPow + 1];                       // zs[g]: packed index of (g, 0, 0) for the current pair's lp
    PairHdr pb[2];                       // the current pair's record and the one being fetched
    TileCommon c;
};
static_assert(sizeof(((SmemInt<false> *)0)->st) <= sizeof(((SmemInt<false> *)0)->A), "S and T fit in A");
// dynamic shared memory of the orthorhombic integrate CTAs: at least 46 KB, so
// that no fifth CTA (for which TMEM has no columns left) is placed on an SM
constexpr size_t kSmemIntOrtho = sizeof(SmemInt<false>) > 46 * 1024 ? sizeof(SmemInt<false>) : 46 * 1024;
static_assert(kSmemIntOrtho + 1024 <= 228 * 1024 / 4, "4 orthorhombic integrate CTAs per SM");
static_assert(5 * (kSmemIntOrtho + 1024) > 228 * 1024, "at most 4 orthorhombic integrate CTAs per SM");

// pair index of (b, a), b + a <= lp, rows of constant b
__device__ __forceinline__ int pair_index(int L, int b, int a) { return b * L - (b * (b - 1)) / 2 + a; }

// packed index of (g, b, 0) in closed form: sum_{z<g} (lp-z+1)(lp-z+2)/2 + sum_{y<b} (lp-g-y+1)
__device__ __forceinline__ int row_start(int lp, int g, int b) {
    const int n1 = lp + 1, n2 = lp + 1 - g;
    const int q = lp - g;
    return (n1 * (n1 + 1) * (n1 + 2) - n2 * (n2 + 1) * (n2 + 2)) / 6 + b * (q + 1) - (b * (b - 1)) / 2;
}

// ---- asynchronous record copies (cp.async, 16-byte chunks, L2 only)
__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(tc::smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Starts copying item it into buf / ii: the pair's record, its coefficients when
// with_coef, and the item's images.  Each thread waits for its own copies
// (cp_async_wait_all) before the barrier after which the buffers are read.
__device__ __forceinline__ void fetch_pair(uint4 *dst, ItemImg &ii, const MixedArgs &A, int64_t it, uint64_t item,
                                           bool with_coef) {
    const uint4 *src = A.blob + (item >> 16);
    const int n = with_coef ? min((int)(item & 0xFFFFu), kHdr16 + kCoef16Max) : kHdr16;
    const uint4 *isrc = reinterpret_cast<const uint4 *>(A.iimg + it);
    // dst: the record's chunks, the coefficients following without a gap
    uint4 *idst = reinterpret_cast<uint4 *>(&ii);
    for (int t = threadIdx.x; t < n + 3; t += blockDim.x) {
        if (t < n) cp_async16(dst + t, src + t);
        else cp_async16(idst + (t - n), isrc + (t - n));
    }
    cp_async_commit();
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

__device__ __forceinline__ void set_image_x(const TPair &p, ImgState &q, int ox, int ext_x) {
    q.o[0] = ox;
    q.gx0 = max(0, p.lb[0] - ox);
    q.gx1 = min(ext_x - 1, p.hi[0] - ox);
    // Re-expansion column: start from the column nearest to the product centre and
    // move toward the tile centre by at most one Gaussian width 1/sqrt(zetp) --
    // the largest values stay near u = 0, and broad Gaussians get the smallest
    // |u| over the whole tile.
    const float hx = p.h[0].hi;
    int i0 = (int)rintf(__fdividef(p.off[0].hi, hx)) - ox;  // any column is valid: approximate
    i0 = min(max(i0, q.gx0), max(q.gx0, q.gx1));
    const float rg = rsqrtf(p.zetp.hi) / hx;
    const float dc = fminf(fmaxf((float)(TX / 2 - i0), -rg), rg);
    q.ic = i0 + (int)rintf(dc);
    q.tc = ff_add(ff_mul_f(p.h[0], (float)(ox + q.ic)), ff{-p.off[0].hi, -p.off[0].lo});
    // Balance the powers: u -> u / 2^sb with 2^sb ~ the extent that matters on this
    // tile, min(max |u|, 2 / sqrt(zetp)); the row coefficients take 2^(k sb), so the
    // product is unchanged and both operands' slices keep their bits where the
    // values are.
    const float umax = (float)max(q.ic - q.gx0, q.gx1 - q.ic) * hx;
    const float ext = fminf(umax, 2.0f * rsqrtf(p.zetp.hi));
    const int e = ((__float_as_int(ext) >> 23) & 0xff) - 126;  // ext = f 2^e, f in [0.5, 1)
    q.sb = ext >= 1.1754944e-38f ? min(max(e, -10), 10) : 0;
}
__device__ __forceinline__ void set_image(const TPair &p, ImgState &q, int ox, int oy, int oz, int ext_x) {
    q.o[1] = oy;
    q.o[2] = oz;
    set_image_x(p, q, ox, ext_x);
}

// Threads 0-2 derive the periodic images of one axis each and set the first
// image; the caller's next barrier publishes them.
__device__ __forceinline__ void pair_images(TileCommon &sm, const TPair &p, const LevelDev &lv, const TileDesc &td,
                                            int ext_x, int *status) {
    const int tid = threadIdx.x;
    if (tid < 3) {
        const TileShape sh(td.lz);
        const int T = tid == 0 ? TX : (tid == 1 ? sh.TY : sh.TZ);
        axis_images(lv, tid, td.t[tid], T, p, sm.img[tid], sm.nimg[tid], status);
        if (sm.nimg[tid] > 0) {
            if (tid == 0) set_image_x(p, sm.im, sm.img[0][0], ext_x);
            else sm.im.o[tid] = sm.img[tid][0];
        }
    }
}

// tab[k][i] = u^k exp(-zetp t^2), t = g h - off, g = o + i, and u = t or, for x
// with recentre, u = (i - ic) h / 2^sb (the balanced offset from the
// re-expansion column); zero outside the cube box, outside the valid tile extent
// and for k >= L.
//
// One entry per lane: warp 0 entry x of the x column (kept in registers), warp 1
// entry ent of the y table (ent < TY) or of the z table.  In collocate both warps
// run one loop over entries, so that the kernel holds a single copy of the
// float-float exponential, its largest inlined function: collocate is limited by
// instruction fetch, and this alone took it from 995 to 926 ms per launch on the
// 1M-pair workload.
struct TabEntry {
    ff t, e;    // t = g h - off and exp(-zetp t^2) (zero outside)
    int d, i;   // axis and tile-local index
    bool in;    // inside the cube box and the tile's valid extent
};
__device__ __forceinline__ TabEntry tab_entry(const TPair &p, const ImgState &q, const LevelDev &lv,
                                              const TileDesc &td, const TileShape &sh, int warp, int ent) {
    TabEntry r;
    int T;
    if (warp == 0) {
        r.d = 0;
        r.i = ent;
        T = TX;
    } else {
        const bool isy = ent < sh.TY;
        r.d = isy ? 1 : 2;
        r.i = isy ? ent : ent - sh.TY;
        T = isy ? sh.TY : sh.TZ;
    }
    const int g = q.o[r.d] + r.i;
    r.in = r.i < min(T, lv.ngrid[r.d] - td.t[r.d] * T) && g >= p.lb[r.d] && g <= p.hi[r.d];
    r.t = ff_add(ff_mul_f(p.h[r.d], (float)g), ff{-p.off[r.d].hi, -p.off[r.d].lo});
    r.e = r.in ? ff_exp(ff_mul(ff_mul(r.t, r.t), ff{-p.zetp.hi, -p.zetp.lo})) : ff{0.0f, 0.0f};
    return r;
}
// warp 1: one y or z entry into shared memory
__device__ __forceinline__ void yz_fill(TileCommon &sm, const TPair &p, const TabEntry &te) {
    ff *col = te.d == 1 ? &sm.Y[0][te.i] : &sm.Z[0][te.i];
    const int stride = te.d == 1 ? kMaxTY + 1 : kMaxTZ + 1;
    const int L = te.in ? p.L : 0;
    ff e = te.e;
#pragma unroll 1
    for (int k = 0; k < L; k++) {
        col[k * stride] = e;
        e = ff_mul(e, te.t);
    }
#pragma unroll 1
    for (int k = L; k < kNPow; k++) col[k * stride] = ff{0.0f, 0.0f};
}
// warp 0: the x column of entry x in registers, xv[k] for k < kNPow
__device__ __forceinline__ void x_powers(const TPair &p, const ImgState &q, const TabEntry &te, int x, bool recentre,
                                         ff *xv) {
#pragma unroll
    for (int k = 0; k < kNPow; k++) xv[k] = ff{0.0f, 0.0f};
    if (!te.in) return;
    if (recentre) {  // collocate: one chain (its code size matters more than this latency)
        ff e = te.e;
        const ff u = ff_mul_f(p.h[0], ldexpf((float)(x - q.ic), -q.sb));
#pragma unroll
        for (int k = 0; k < kNPow; k++) {
            if (k >= p.L) break;
            xv[k] = e;
            e = ff_mul(e, u);
        }
        return;
    }
    // integrate: even and odd powers of t as two independent chains in t^2
    const ff u2 = ff_mul(te.t, te.t);
    ff e0 = te.e, e1 = ff_mul(te.e, te.t);
#pragma unroll
    for (int k = 0; k < kNPow; k += 2) {
        if (k >= p.L) break;
        xv[k] = e0;
        if (k + 1 < kNPow && k + 1 < p.L) xv[k + 1] = e1;
        e0 = ff_mul(e0, u2);
        e1 = ff_mul(e1, u2);
    }
}

// Binomials C(a', a) of the re-expansion c'[g][b][a] = sum_{a' >= a} C(a', a)
// tc^(a' - a) c[g][b][a'] around column ic of the tile: powers of the small
// offsets u = x - x_ic keep the stage-3 operands well conditioned for the
// fixed-point slices.
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

// One item (g, b, a) per thread of [t0, t0 + nt): Horner in tc over a' = amax .. a
// with the binomials from shared memory (bin[a'][a] = C(a', a)).  zs[g] is the
// packed index of (g, 0, 0) and qb[q][r] the b of row-in-slab r of a slab with
// q = lp - g, so that decoding t needs no arithmetic series.
__device__ void recentre_x(const PairBuf &pb, ff tc, ff *out, const float (*bin)[kNPow], const int *zs,
                           const unsigned char (*qb)[NPAIR_MAX + 2], int t0, int nt) {
    const int lp = pb.p.lp;
    const int nc = ncoef(lp);
    for (int t = (int)threadIdx.x - t0; t < nc; t += nt) {
        int g = 0;
        while (g < lp && zs[g + 1] <= t) g++;
        const int qn = lp - g, r = t - zs[g];
        const int b = qb[qn][r];
        const int a = r - (b * (qn + 1) - (b * (b - 1)) / 2), amax = lp - g - b;
        const int base = t - a;  // packed index of (g, b, 0)
        ff s = {0.0f, 0.0f};
#pragma unroll 1
        for (int ap = amax; ap >= a; ap--) {
            const float2 c = pb.coef[base + ap];
            s = ff_fma(s, tc, ff_mul_f(ff{c.x, c.y}, bin[ap][a]));
        }
        out[t] = s;
    }
}

// masks of the 8 packed halves of one 16-byte chunk from bits 0..7 of b (bit k:
// half k, all ones or zero).  One multiply per 4 bits moves bit k to the top of
// byte k (the copies lie 7 bits apart, so no carries), and prmt, whose selector
// nibbles with the top bit set replicate the sign of the selected byte, spreads
// each byte's top bit over the two bytes of its half.
__device__ __forceinline__ uint4 chunk_mask(uint32_t b) {
    const uint32_t lo = ((b & 0xFu) * 0x10204080u) & 0x80808080u;
    const uint32_t hi = (((b >> 4) & 0xFu) * 0x10204080u) & 0x80808080u;
    uint4 m;
    asm("prmt.b32 %0, %1, 0, 0x9988;" : "=r"(m.x) : "r"(lo));
    asm("prmt.b32 %0, %1, 0, 0xBBAA;" : "=r"(m.y) : "r"(lo));
    asm("prmt.b32 %0, %1, 0, 0x9988;" : "=r"(m.z) : "r"(hi));
    asm("prmt.b32 %0, %1, 0, 0xBBAA;" : "=r"(m.w) : "r"(hi));
    return m;
}

// The NSL slices of one K = 16 operand row (v[k] for k < kNPow, zero beyond),
// scaled by sc, as 16-byte chunks of 8 K values in the UMMA layout (planes of
// plane_halves halves); K groups at or beyond kw are left as they are, and those
// at or beyond nval (v[k] == 0 for k >= nval) are written as zeros directly.
__device__ __forceinline__ void slice_row16(const ff *vin, float sc, int kw, int nval, __half *plane0,
                                            int plane_halves, int row) {
    // one compact loop body for both K groups: the second group's values are moved down
    ff v[8];
#pragma unroll
    for (int k = 0; k < 8; k++) v[k] = vin[k];
#pragma unroll 1
    for (int kg = 0; kg < KP / 8; kg++) {
        if (8 * kg >= kw) break;
        if (8 * kg >= nval) {  // only zeros left: rewrite the stale slots without slicing
            const int o16 = (row >> 3) * 16 + kg * 8 + (row & 7);
#pragma unroll
            for (int q = 0; q < NSL; q++) reinterpret_cast<uint4 *>(plane0 + q * plane_halves)[o16] = make_uint4(0, 0, 0, 0);
            continue;
        }
        uint32_t w[NSL][4];
#pragma unroll
        for (int i = 0; i < 4; i++) {
            float s0[NSL], s1[NSL];
            slice_scaled(v[2 * i], sc, s0);
            slice_scaled(v[2 * i + 1], sc, s1);
#pragma unroll
            for (int q = 0; q < NSL; q++) {
                const __half2 h2 = __floats2half2_rn(s0[q], s1[q]);
                w[q][i] = *reinterpret_cast<const uint32_t *>(&h2);
            }
        }
        const int o16 = (row >> 3) * 16 + kg * 8 + (row & 7);  // umma_off(row, 8 kg) / 16
#pragma unroll
        for (int q = 0; q < NSL; q++)
            reinterpret_cast<uint4 *>(plane0 + q * plane_halves)[o16] = make_uint4(w[q][0], w[q][1], w[q][2], w[q][3]);
#pragma unroll
        for (int k = 0; k < 8; k++) v[k] = 8 + k < kNPow ? vin[8 + k < kNPow ? 8 + k : 0] : ff{0.0f, 0.0f};
    }
}

// named barrier 1 between producer warps (arrive) and consumer warps (sync)
__device__ __forceinline__ void bar_arrive1(int n) { asm volatile("bar.arrive 1, %0;" ::"r"(n) : "memory"); }
__device__ __forceinline__ void bar_sync1(int n) { asm volatile("bar.sync 1, %0;" ::"r"(n) : "memory"); }

// General cell: the cross factor along row (z, y) of the current image, E(x) =
// exp(alpha + beta t0(x)) with beta = -2 zetp (c01 t1 + c02 t2), alpha = -2 zetp
// c12 t1 t2: returns E(x0) and q = E(x + 1) / E(x).
__device__ __forceinline__ void cross_factor_row(const GenLevel &G, const TPair &P, const ImgState &Q, int z, int y,
                                                 int x0, ff &e0, ff &q) {
    const ff t1 = ff_add(ff_mul_f(P.h[1], (float)(Q.o[1] + y)), ff{-P.off[1].hi, -P.off[1].lo});
    const ff t2 = ff_add(ff_mul_f(P.h[2], (float)(Q.o[2] + z)), ff{-P.off[2].hi, -P.off[2].lo});
    const ff t0 = ff_add(ff_mul_f(P.h[0], (float)(Q.o[0] + x0)), ff{-P.off[0].hi, -P.off[0].lo});
    const ff m2z = {-2.0f * P.zetp.hi, -2.0f * P.zetp.lo};
    const ff beta = ff_mul(m2z, ff_add(ff_mul(G.c01, t1), ff_mul(G.c02, t2)));
    const ff alpha = ff_mul(m2z, ff_mul(G.c12, ff_mul(t1, t2)));
    e0 = ff_exp(ff_add(alpha, ff_mul(beta, t0)));
    q = ff_exp(ff_mul(beta, P.h[0]));
}

// General cell, integrate: the A operand row r = the slices of V(x) E(x) over the
// row's cube points (zero elsewhere), with the row's own exponent (vmr[r]).
template <class Smem>
__device__ __forceinline__ void general_a_row(Smem &sm, const GenLevel &G, const TPair &P, const ImgState &Q,
                                              const TileShape &sh, int r, bool &zero_row) {
    const int x0 = sm.rx0[r], x1 = sm.rx1[r];
    if (x0 > x1) {
        sm.vmr[r] = kZeroExp;
        if (zero_row) return;
        zero_row = true;
#pragma unroll
        for (int v = 0; v < TX / 8; v++)
#pragma unroll
            for (int q = 0; q < NSL; q++)
                reinterpret_cast<uint4 *>(sm.A[v >> 1][q])[(r >> 3) * 16 + (v & 1) * 8 + (r & 7)] = make_uint4(0, 0, 0, 0);
        return;
    }
    zero_row = false;
    ff e0, q;
    cross_factor_row(G, P, Q, r >> sh.ly, r & (sh.TY - 1), x0, e0, q);
    // pass 1: the row maximum of |V E|
    float mx = 0.0f;
    {
        ff e = e0;
        for (int x = x0; x <= x1; x++) {
            mx = fmaxf(mx, fabsf(ff_mul(sm.Vff[x][r], e).hi));
            e = ff_mul(e, q);
        }
    }
    const int vmx = exp_of(mx);
    sm.vmr[r] = vmx;
    const float sc = vmx == kZeroExp ? 0.0f : pow2i(SLB - vmx);
    // pass 2: slices, 16-byte chunks of 8 x
    ff e = e0;
#pragma unroll 1
    for (int c = 0; c < TX / 8; c++) {
        uint32_t w[NSL][4];
#pragma unroll
        for (int i = 0; i < 4; i++) {
            ff v2[2];
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int x = 8 * c + 2 * i + h;
                const bool in = x >= x0 && x <= x1;
                v2[h] = in ? ff_mul(sm.Vff[x][r], e) : ff{0.0f, 0.0f};
                if (in) e = ff_mul(e, q);
            }
            float s0[NSL], s1[NSL];
            slice_scaled(v2[0], sc, s0);
            slice_scaled(v2[1], sc, s1);
#pragma unroll
            for (int qq = 0; qq < NSL; qq++) {
                const __half2 h2 = __floats2half2_rn(s0[qq], s1[qq]);
                w[qq][i] = *reinterpret_cast<const uint32_t *>(&h2);
            }
        }
        const int o16 = (r >> 3) * 16 + (c & 1) * 8 + (r & 7);
#pragma unroll
        for (int qq = 0; qq < NSL; qq++)
            reinterpret_cast<uint4 *>(sm.A[c >> 1][qq])[o16] = make_uint4(w[qq][0], w[qq][1], w[qq][2], w[qq][3]);
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
    cp_async_wait_all();
    tc::fence_before_sync();
    __syncthreads();
    if (threadIdx.x < 32) tc::tmem_dealloc(c.tmem, ncols);
}

// waits for the MMAs of the current item; false (and abort flagged) on timeout
__device__ __forceinline__ bool tc_wait(TileCommon &c, uint32_t phase, int *status) {
    if (!tc::mbar_wait_bounded(&c.mbar, phase, 1u << 24)) {
        atomicOr(status, kStatTimeout);
        c.abort = 1;
    }
    __syncthreads();
    tc::fence_after_sync();
    return !c.abort;
}

// The pair loop of a tile: item it + 1 is copied while item it is processed.
// Returns the buffer slot of item it once it is visible to all threads.
template <class Buf>
__device__ __forceinline__ int next_pair(TileCommon &cm, Buf *pb, const MixedArgs &A, int64_t it, int64_t it0,
                                         int64_t it1, uint64_t &nxt, bool with_coef) {
    const int cur = (int)((it - it0) & 1);
    cp_async_wait_all();
    __syncthreads();  // item it visible; every thread is done with the other slot
    if (it + 1 < it1) {
        fetch_pair(pb[cur ^ 1].hdr_, cm.ii[cur ^ 1], A, it + 1, nxt, with_coef);
        if (it + 2 < it1) nxt = A.items[it + 2];
    }
    return cur;
}

template <class Buf>
__device__ __forceinline__ void first_pair(TileCommon &cm, Buf *pb, const MixedArgs &A, int64_t it0, int64_t it1,
                                           uint64_t &nxt, bool with_coef) {
    if (it0 < it1) fetch_pair(pb[0].hdr_, cm.ii[0], A, it0, A.items[it0], with_coef);
    if (it0 + 1 < it1) nxt = A.items[it0 + 1];
}

// images of the current item: 1 for the common case (state precomputed in ii);
// for more, threads 0-2 derive them here (one extra barrier, out of line)
__device__ __noinline__ void item_images_multi(TileCommon &cm, const TPair &P, const LevelDev &lv,
                                               const TileDesc &td, int ext_x, int *status) {
    pair_images(cm, P, lv, td, ext_x, status);
    __syncthreads();
}
__device__ __forceinline__ int item_images(TileCommon &cm, const ItemImg &ii, const TPair &P, const LevelDev &lv,
                                           const TileDesc &td, int ext_x, int *status) {
    const int np = ii.nimg;
    const int nimg = (np & 0xff) * ((np >> 8) & 0xff) * ((np >> 16) & 0xff);
    if (nimg > 1) item_images_multi(cm, P, lv, td, ext_x, status);
    return nimg;
}


// Stage 1 of collocate: Cxy[z][(b,a)] = sum_g c'[g][b][a] Z[g][z]; one output per
// thread (16 consecutive threads share (b, a)), two partial sums over even and
// odd g; the packed index of (g, b, a) is zs[g] - b g + k0.
__device__ __forceinline__ void stage1_cxy(SmemColl &sm, int L, int lp, const TileShape &sh) {
    const TileCommon &cm = sm.c;
    const int npair = (L * (L + 1)) / 2;
    const unsigned char *qbL = sm.qb[L - 1];
    for (int t = threadIdx.x; t < sh.TZ * npair; t += NTHR) {
        const int zz = t & (sh.TZ - 1), q = t >> sh.lz;
        const int b = qbL[q];
        const int a = q - (b * L - (b * (b - 1)) / 2), n = lp - a - b;
        const int k0 = b * (lp + 1) - (b * (b - 1)) / 2 + a;
        ff s0 = {0.0f, 0.0f}, s1 = {0.0f, 0.0f};
        int g = 0, bg = 0;
#pragma unroll 1
        for (; g + 1 <= n; g += 2, bg += 2 * b) {
            s0 = ff_fma(sm.rc[sm.zs[g] - bg + k0], cm.Z[g][zz], s0);
            s1 = ff_fma(sm.rc[sm.zs[g + 1] - bg - b + k0], cm.Z[g + 1][zz], s1);
        }
        if (g <= n) s0 = ff_fma(sm.rc[sm.zs[g] - bg + k0], cm.Z[g][zz], s0);
        sm.Cxy[zz][q] = ff_add(s0, s1);
    }
}

// Stage 2 of collocate for this thread's row (z, y), all a at once, then the
// row's A slices (K slots below kw rewritten); returns the row exponent.  a in
// pairs (a0, a0 + 1; unrolled, uniform exit at lp), b inner (runtime bound
// lp - a0): only the products that exist, two independent float-float sums, each
// renormalised once at the end.
__device__ __forceinline__ int stage2_row(SmemColl &sm, const TileCommon &cm, int L, int lp, int sb, int z, int y,
                                          bool live, int kw, int m) {
    ff cx[kNPow];
#pragma unroll
    for (int a = 0; a < kNPow; a++) cx[a] = ff{0.0f, 0.0f};
    float mx = 0.0f;
    if (live) {
        const ff *crow = sm.Cxy[z];
#pragma unroll
        for (int a0 = 0; a0 < kNPow; a0 += 2) {
            if (a0 > lp) break;
            ff s0 = {0.0f, 0.0f}, s1 = {0.0f, 0.0f};
            const int nb = lp - a0;
            int q = a0;  // pair_index(L, b, a0); (b, a0 + 1) is q + 1
#pragma unroll 1
            for (int b = 0; b <= nb; b++) {
                const ff yb = cm.Y[b][y];
                ff_acc_lazy(s0, crow[q], yb);
                if (b < nb) ff_acc_lazy(s1, crow[q + 1], yb);  // a0 + 1 + b <= lp
                q += L - b;
            }
            cx[a0] = fast_two_sum(s0.hi, s0.lo);
            if (a0 + 1 < kNPow) cx[a0 + 1] = fast_two_sum(s1.hi, s1.lo);
        }
#pragma unroll
        for (int a = 0; a < kNPow; a++) {
            const float bal = pow2i(a * sb);  // balancing of the x powers (exact)
            cx[a].hi = __fmul_rn(cx[a].hi, bal);
            cx[a].lo = __fmul_rn(cx[a].lo, bal);
            mx = fmaxf(mx, fabsf(cx[a].hi));  // entries a > lp are zero
        }
    }
    const int em = exp_of(mx);
    const float sc = em == kZeroExp ? 0.0f : pow2i(SLB - em);
    // entries a > lp of cx are zero; K slots that may hold an earlier pair's values are rewritten
    slice_row16(cx, sc, kw, L, sm.A[0], MROWS * KP, m);
    return em;
}

// ---------------------------------------------------------------------------
// kGeneral: tiles of general-cell levels.  The tables, stages and slices are the
// same in t_d = (index_d - gp_d) |v_d|; the row ranges come from the quadratic
// rule, and every point's value is multiplied by the cross factor
// E = exp(-2 zetp (c01 t0 t1 + c02 t0 t2 + c12 t1 t2)) of the Gaussian
// (exp(-zetp |r|^2) = exp(-zetp (t0^2 + t1^2 + t2^2)) E).  Along a row E(x) is
// exp(alpha + beta t0(x)): one exp at the row's first cube point, then E(x+1) =
// E(x) q, q = exp(beta |v0|), over the row's cube points only (so no intermediate
// leaves the range of the factor inside the cube).
template <bool kGeneral>
__global__ void __launch_bounds__(NTHR, 4) k_collocate_tiled(MixedArgs A) {
    extern __shared__ __align__(128) unsigned char smraw[];
    SmemColl &sm = *reinterpret_cast<SmemColl *>(smraw);
    TileCommon &cm = sm.c;
    const int tid = threadIdx.x, warp = tid >> 5;
    const int m = tid;
    constexpr uint32_t kCols = 128;  // diagonals D2..D5: 32 columns each
    tc_setup(cm, kCols);
    const uint32_t tbase = cm.tmem + ((uint32_t)(warp * 32) << 16);
    const uint32_t idesc = tc::idesc_f16_f32(MROWS, TX);
    uint32_t phase = 0;
    for (int t = tid; t < kNPow * kNPow; t += NTHR) sm.bin[t / kNPow][t % kNPow] = c_binom[t / kNPow][t % kNPow];
    // qb[L-1][pair_index(L, b, a)] = b: the (b, a) of a pair index without a search per use
    for (int t = tid; t < kNPow * (NPAIR_MAX + 2); t += NTHR) {
        const int Lq = t / (NPAIR_MAX + 2) + 1, q = t % (NPAIR_MAX + 2);
        int b = 0, r = q;
        while (b < Lq && r >= Lq - b) r -= Lq - b++;
        sm.qb[Lq - 1][q] = (unsigned char)min(b, kNPow - 1);
    }
    for (;;) {
        if (tid == 0) cm.tile = atomicAdd(A.queue, 1);
        __syncthreads();
        const int tile = cm.tile;
        if (tile >= A.ntiles || cm.abort) break;
        const TileDesc td = A.tiles[tile];
        const LevelDev &lv = A.levels[td.level];
        const TileShape sh(td.lz);
        const int TY = sh.TY, TZ = sh.TZ, z = m >> sh.ly, y = m & (TY - 1);
        if (TZ > kMaxTZColl) {  // shapes are validated on the host; never taken
            if (tid == 0) atomicOr(A.status, kStatBadTile);
            continue;
        }
        float acc_hi[TX];  // the low parts live in shared memory (registers for 4 CTAs per SM)
        float *acc_lo = sm.acc_lo[m];
#pragma unroll
        for (int x = 0; x < TX; x++) acc_hi[x] = acc_lo[x] = 0.0f;
        const int ext_z = min(TZ, lv.ngrid[2] - td.t[2] * TZ), ext_y = min(TY, lv.ngrid[1] - td.t[1] * TY);
        const int ext_x = min(TX, lv.ngrid[0] - td.t[0] * TX);
        const int64_t it0 = A.start[2 * tile], it1 = A.start[2 * tile + 1];
        uint64_t nxt = 0;
        first_pair(cm, sm.pb, A, it0, it1, nxt, true);
        for (int64_t it = it0; it < it1 && !cm.abort; it++) {
            const int cur = next_pair(cm, sm.pb, A, it, it0, it1, nxt, true);
            const PairBuf &pb = sm.pb[cur];
            const TPair &P = pb.p;
            const int L = P.L, lp = P.lp;
            const int nimg = item_images(cm, cm.ii[cur], P, lv, td, ext_x, A.status);
            const ImgState &Q = nimg == 1 ? cm.ii[cur].im : cm.im;
            for (int im = 0; im < nimg && !cm.abort; im++) {
                if (im > 0) {
                    if (tid == 0) {
                        const int ix = im % cm.nimg[0], iy = (im / cm.nimg[0]) % cm.nimg[1],
                                  iz = im / (cm.nimg[0] * cm.nimg[1]);
                        set_image(P, cm.im, cm.img[0][ix], cm.img[1][iy], cm.img[2][iz], ext_x);
                    }
                    __syncthreads();
                }
                if (Q.gx0 > Q.gx1) continue;  // uniform: no x overlap
                // warp 0: X column (lane x) and its B slices, scaled by 2^(SLB - fx); warp 1:
                // Y and Z tables; warps 2-3: re-expansion of the coefficients
                if (warp < 2) {
#pragma unroll 1
                    for (int ent = tid & 31; ent < (warp == 0 ? TX : TY + TZ); ent += 32) {
                        const TabEntry te = tab_entry(P, Q, lv, td, sh, warp, ent);
                        if (warp == 0) {
                            ff xv[kNPow];
                            x_powers(P, Q, te, ent, true, xv);
                            float mx = 0.0f;
#pragma unroll
                            for (int k = 0; k < kNPow; k++) mx = fmaxf(mx, fabsf(xv[k].hi));
                            const int e = exp_of(mx);
                            sm.cs[tid] = e == kZeroExp ? 0.0f : pow2i(e);
                            const float sc = e == kZeroExp ? 0.0f : pow2i(SLB - e);
                            // K slots beyond L may hold an earlier pair's slices: rewritten as zeros
                            slice_row16(xv, sc, max(L, cm.kmax), L, sm.B[0], TX * KP, tid);
                        } else {
                            yz_fill(cm, P, te);
                        }
                    }
                } else {
                    // slab starts zs[g] = packed index of (g, 0, 0), then the re-expansion
                    if (tid - 64 <= kNPow) sm.zs[tid - 64] = tid - 64 <= lp + 1 ? row_start(lp, tid - 64, 0) : 0;
                    asm volatile("bar.sync 2, 64;" ::: "memory");
                    recentre_x(pb, Q.tc, sm.rc, sm.bin, sm.zs, sm.qb, 64, NTHR - 64);
                }
                __syncthreads();
                stage1_cxy(sm, L, lp, sh);
                __syncthreads();
                // stage 2 (this thread's row, all a at once) + culling + A slices
                int x0, x1;
                if constexpr (kGeneral)
                    general_row_range(lv, A.glv[td.level], P, Q, Q.o[2] + z, Q.o[1] + y, z < ext_z && y < ext_y, x0,
                                      x1);
                else
                    row_range(P, Q, A.table, Q.o[2] + z, Q.o[1] + y, z < ext_z && y < ext_y, x0, x1);
                const int em = stage2_row(sm, cm, L, lp, Q.sb, z, y, x0 <= x1, max(L, cm.kmax), m);
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
                // cross factor of the general cell along this row: E0 at x0, ratio q
                ff ecur = {1.0f, 0.0f}, eq = {1.0f, 0.0f};
                if constexpr (kGeneral) {
                    if (x0 <= x1) cross_factor_row(A.glv[td.level], P, Q, z, y, x0, ecur, eq);
                }
                // tcgen05.ld is warp-collective: chunk decisions are made per warp
                if (__any_sync(0xffffffffu, x0 <= x1)) {
                    const float rs = pow2i(max(em - 2 * SLB, -126));
                    // bits x0..x1 of the row: the points of this pair's sphere on the row
                    const uint32_t rmask =
                        x0 > x1 ? 0u : (uint32_t)(((2ull << x1) - 1ull) & ~((1ull << x0) - 1ull));
                    // kCh chunks of 8 x per iteration (a compact loop body: instruction fetch
                    // is a stall of this kernel); acc_hi[0 .. 8 kCh) always holds the current
                    // chunks' sums, rotated by 8 kCh after each iteration (TX / (8 kCh)
                    // rotations restore the order).  Two chunks halve the register moves of
                    // the rotation; the general-cell body, longer by the cross factor, keeps one.
                    constexpr int kCh = kGeneral ? 1 : 2;
#pragma unroll 1
                    for (int c2 = 0; c2 < TX / (8 * kCh); c2++) {
#pragma unroll
                        for (int hh = 0; hh < kCh; hh++) {
                            const int c = kCh * c2 + hh;
                            const uint32_t mc = rmask >> (8 * c);
                            if (__any_sync(0xffffffffu, (mc & 0xFFu) != 0u)) {
                                uint32_t r2[8], r3[8], r4[8], r5[8];
                                const float4 csa = reinterpret_cast<const float4 *>(sm.cs)[2 * c];
                                const float4 csb = reinterpret_cast<const float4 *>(sm.cs)[2 * c + 1];
                                const float csv[8] = {csa.x, csa.y, csa.z, csa.w, csb.x, csb.y, csb.z, csb.w};
                                tc::tmem_ld8(tbase + 8 * c, r2);
                                tc::tmem_ld8(tbase + 32 + 8 * c, r3);
                                tc::tmem_ld8(tbase + 64 + 8 * c, r4);
                                tc::tmem_ld8(tbase + 96 + 8 * c, r5);
                                tc::tmem_wait_ld32(r2, r3, r4, r5);
#pragma unroll
                                for (int i = 0; i < 8; i++) {
                                    const int x = 8 * c + i;
                                    const bool in = (mc >> i) & 1u;  // straight-line code: selects, no branches
                                    // value = scl * (D2 + D3 2^-10 + D4 2^-20 + D5 2^-30) as hi + lo with
                                    // lo the exact remainder (fast two-sum), then an exact two-sum into
                                    // acc_hi: acc_lo then only gathers rounding errors and remainders,
                                    // so it stays ~2^-24 below acc_hi however many pairs a point sees
                                    const float d2 = __uint_as_float(r2[i]);
                                    const float corr = __fmaf_rn(__uint_as_float(r5[i]), 9.313225746154785e-10f,
                                                       __fmaf_rn(__uint_as_float(r4[i]), 9.5367431640625e-07f,
                                                                 __fmul_rn(__uint_as_float(r3[i]), 0.0009765625f)));
                                    float scl = __fmul_rn(rs, csv[i]);
                                    const float h0 = __fadd_rn(d2, corr);
                                    float hi = __fmul_rn(h0, scl);
                                    float rem = __fsub_rn(corr, __fsub_rn(h0, d2));  // lo = rem scl exactly
                                    if constexpr (kGeneral) {
                                        if (x > x0) ecur = ff_mul(ecur, eq);  // E(x) on the row's cube points
                                        const ff v = ff_mul(ff{hi, __fmul_rn(rem, scl)}, ecur);
                                        hi = v.hi;
                                        rem = v.lo;
                                        scl = 1.0f;
                                    }
                                    float &ah = acc_hi[8 * hh + i];
                                    const float sv = __fadd_rn(ah, hi);
                                    const float bb = __fsub_rn(sv, ah);
                                    const float err = __fadd_rn(__fsub_rn(ah, __fsub_rn(sv, bb)), __fsub_rn(hi, bb));
                                    if (in) acc_lo[x] = __fadd_rn(acc_lo[x], __fmaf_rn(rem, scl, err));
                                    ah = in ? sv : ah;
                                }
                            }
                        }
                        float tr[8 * kCh];
#pragma unroll
                        for (int i = 0; i < 8 * kCh; i++) tr[i] = acc_hi[i];
#pragma unroll
                        for (int i = 0; i < TX - 8 * kCh; i++) acc_hi[i] = acc_hi[i + 8 * kCh];
#pragma unroll
                        for (int i = 0; i < 8 * kCh; i++) acc_hi[TX - 8 * kCh + i] = tr[i];
                    }
                }
                tc::fence_before_sync();
                __syncthreads();
            }
        }
        cp_async_wait_all();
        if (cm.abort) break;
        // flush: grid += tile sum (FP64)
        if (z < ext_z && y < ext_y) {
            double *grid = A.grids.p[td.level];
            const int64_t row = ((int64_t)(td.t[2] * TZ + z) * lv.ngrid[1] + (td.t[1] * TY + y)) * lv.ngrid[0] +
                                td.t[0] * TX;
            // 8 points per iteration, acc_hi rotated by 8 after each (compact code)
#pragma unroll 1
            for (int c = 0; c < TX / 8; c++) {
#pragma unroll
                for (int i = 0; i < 8; i++) {
                    const int x = 8 * c + i;
                    if (x >= ext_x) continue;
                    const double v = (double)acc_hi[i] + (double)acc_lo[x];
                    if (td.split) atomicAdd(grid + row + x, v);  // other work units add to the same tile
                    else grid[row + x] += v;
                }
#pragma unroll
                for (int i = 0; i < TX - 8; i++) acc_hi[i] = acc_hi[i + 8];
            }
        }
        __syncthreads();
    }
    tc_teardown(cm, kCols, phase);
}

// kGeneral: tiles of general-cell levels; the A operand holds the slices of
// V(x) E(x) (E the cross factor of the Gaussian along the row), one row per
// thread, with its own exponent per row and image.
template <bool kGeneral>
__global__ void __launch_bounds__(NTHR, kGeneral ? 3 : 4) k_integrate_tiled(MixedArgs A) {
    extern __shared__ __align__(128) unsigned char smraw[];
    SmemInt<kGeneral> &sm = *reinterpret_cast<SmemInt<kGeneral> *>(smraw);
    uint4 *const vslot = kGeneral ? nullptr : A.vslot + (size_t)blockIdx.x * kVSlot16;
    TileCommon &cm = sm.c;
    const int tid = threadIdx.x, warp = tid >> 5;
    const int m = tid;
    constexpr uint32_t kCols = 128;  // D2 (two K halves), D3, D4, D5: 16 columns each
    tc_setup(cm, kCols);
    const uint32_t tbase = cm.tmem + ((uint32_t)(warp * 32) << 16);
    const uint32_t idesc = tc::idesc_f16_f32(MROWS, KP);
    uint32_t phase = 0;
    for (int t = tid; t < kNPow * (NPAIR_MAX + 2); t += NTHR) {
        const int Lq = t / (NPAIR_MAX + 2) + 1, q = t % (NPAIR_MAX + 2);
        int b = 0, r = q;
        while (b < Lq && r >= Lq - b) r -= Lq - b++;
        sm.qb[Lq - 1][q] = (unsigned char)min(b, kNPow - 1);
    }
    // B rows alpha >= L are never written: start them finite (zero)
    for (int t = tid; t < (int)(sizeof(sm.B) / sizeof(uint4)); t += NTHR)
        reinterpret_cast<uint4 *>(sm.B)[t] = make_uint4(0u, 0u, 0u, 0u);
    for (;;) {
        if (tid == 0) cm.tile = atomicAdd(A.queue, 1);
        __syncthreads();
        const int tile = cm.tile;
        if (tile >= A.ntiles || cm.abort) break;
        const TileDesc td = A.tiles[tile];
        const LevelDev &lv = A.levels[td.level];
        const TileShape sh(td.lz);
        const int TY = sh.TY, TZ = sh.TZ, z = m >> sh.ly, y = m & (TY - 1);
        const int ext_z = min(TZ, lv.ngrid[2] - td.t[2] * TZ), ext_y = min(TY, lv.ngrid[1] - td.t[1] * TY);
        const int ext_x = min(TX, lv.ngrid[0] - td.t[0] * TX);
        // this thread's V row, sliced once per tile (row exponent vm)
        int vm;
        {
            const double *grid = A.grids.p[td.level];
            const bool ok = z < ext_z && y < ext_y;
            const int64_t row = ((int64_t)(td.t[2] * TZ + z) * lv.ngrid[1] + (td.t[1] * TY + y)) * lv.ngrid[0] +
                                td.t[0] * TX;
            // compact loops (once per tile): the row maximum, then 16-byte chunks of 8 x
            float mx = 0.0f;
#pragma unroll 1
            for (int x = 0; x < TX; x++) {
                const ff v = (ok && x < ext_x) ? ff_from_double(grid[row + x]) : ff{0.0f, 0.0f};
                if constexpr (kGeneral) sm.Vff[x][m] = v;
                mx = fmaxf(mx, fabsf(v.hi));
            }
            vm = exp_of(mx);
            const float sc = vm == kZeroExp ? 0.0f : pow2i(SLB - vm);
#pragma unroll 1
            for (int c = 0; c < TX / 8 && !kGeneral; c++) {  // 8 x per 16-byte chunk of the UMMA layout
                uint32_t w[NSL][4];
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    const int x = 8 * c + 2 * i;
                    const ff v0 = (ok && x < ext_x) ? ff_from_double(grid[row + x]) : ff{0.0f, 0.0f};
                    const ff v1 = (ok && x + 1 < ext_x) ? ff_from_double(grid[row + x + 1]) : ff{0.0f, 0.0f};
                    float s0[NSL], s1[NSL];
                    slice_scaled(v0, sc, s0);
                    slice_scaled(v1, sc, s1);
#pragma unroll
                    for (int q = 0; q < NSL; q++) {
                        const __half2 h2 = __floats2half2_rn(s0[q], s1[q]);
                        w[q][i] = *reinterpret_cast<const uint32_t *>(&h2);
                    }
                }
                const int o16 = (m >> 3) * 16 + (c & 1) * 8 + (m & 7);  // umma_off / 16
#pragma unroll
                for (int q = 0; q < NSL; q++)
                    vslot[((c >> 1) * NSL + q) * (MROWS * KP / 8) + o16] = make_uint4(w[q][0], w[q][1], w[q][2], w[q][3]);
            }
        }
        bool zero_row[2] = {false, false};  // A rows u, u + 64 hold zeros (warps 2-3)
        const int64_t it0 = A.start[2 * tile], it1 = A.start[2 * tile + 1];
        uint64_t nxt = 0;
        first_pair(cm, sm.pb, A, it0, it1, nxt, false);
        for (int64_t it = it0; it < it1 && !cm.abort; it++) {
            const int cur = next_pair(cm, sm.pb, A, it, it0, it1, nxt, false);
            const TPair &P = sm.pb[cur].p;
            const int L = P.L, lp = P.lp;
            const int npair = (L * (L + 1)) / 2;
            const int64_t moff = P.coef_off;
            const int nimg = item_images(cm, cm.ii[cur], P, lv, td, ext_x, A.status);
            const ImgState &Q = nimg == 1 ? cm.ii[cur].im : cm.im;
            for (int im = 0; im < nimg && !cm.abort; im++) {
                if (im > 0) {
                    if (tid == 0) {
                        const int ix = im % cm.nimg[0], iy = (im / cm.nimg[0]) % cm.nimg[1],
                                  iz = im / (cm.nimg[0] * cm.nimg[1]);
                        set_image(P, cm.im, cm.img[0][ix], cm.img[1][iy], cm.img[2][iz], ext_x);
                    }
                    __syncthreads();
                }
                if (Q.gx0 > Q.gx1) continue;
                {
                    // every thread: its row's cube x range, for the A operand of warps 2-3
                    int x0, x1;
                    if constexpr (kGeneral)
                        general_row_range(lv, A.glv[td.level], P, Q, Q.o[2] + z, Q.o[1] + y, z < ext_z && y < ext_y,
                                          x0, x1);
                    else
                        row_range(P, Q, A.table, Q.o[2] + z, Q.o[1] + y, z < ext_z && y < ext_y, x0, x1);
                    const bool empty = x0 > x1;  // otherwise both lie in [0, TX)
                    sm.rx0[m] = (signed char)(empty ? 1 : x0);
                    sm.rx1[m] = (signed char)(empty ? 0 : x1);
                }
                if (warp == 0) {
                    if constexpr (!kGeneral) bar_arrive1(NTHR);
                    // X column (lane x) in registers, then B: row alpha = X[alpha][x] over x,
                    // scaled by 2^(SLB - gexp[alpha]) (maximum over the warp); rows alpha >= L
                    // are left as they are (their output columns are not read).  Unlike
                    // collocate, integrate is not limited by instruction fetch: warps 0 and 1
                    // keep separate table code.
                    ff xv[kNPow];
                    x_powers(P, Q, tab_entry(P, Q, lv, td, sh, 0, tid), tid, false, xv);
#pragma unroll
                    for (int a = 0; a < kNPow; a++) {
                        if (a >= L) break;
                        // per-alpha maximum over x: one warp reduction (the bit patterns of
                        // non-negative floats order as their values)
                        const float mxb =
                            __uint_as_float(__reduce_max_sync(0xffffffffu, __float_as_uint(fabsf(xv[a].hi))));
                        const int e = exp_of(mxb);
                        if (tid == a) sm.gexp[a] = e;
                        const float sc = e == kZeroExp ? 0.0f : pow2i(SLB - e);
                        float sl[NSL];
                        slice_scaled(xv[a], sc, sl);
                        unsigned char *const bp = sm.B + (tid >> 4) * kBHalf + b_off(a, tid & 15);
#pragma unroll
                        for (int q = 0; q < NSL; q++)
                            *reinterpret_cast<__half *>(bp + q * kBPlane) = __float2half_rn(sl[q]);
                    }
                } else if (warp == 1) {
                    if constexpr (!kGeneral) bar_arrive1(NTHR);
                    if (tid - 32 <= kNPow) sm.zs[tid - 32] = tid - 32 <= lp + 1 ? row_start(lp, tid - 32, 0) : 0;
#pragma unroll 1
                    for (int ent = tid - 32; ent < TY + TZ; ent += 32) yz_fill(cm, P, tab_entry(P, Q, lv, td, sh, 1, ent));
                } else if constexpr (!kGeneral) {
                    bar_sync1(NTHR);
                    // A operand: V slices of rows u and u + 64 (the CTA's slot) masked to the rows' cube ranges,
                    // 16-byte chunks (8 x of one K half); rows already zero stay untouched
                    const int u = tid - 64;
#pragma unroll 1
                    for (int rr = 0; rr < 2; rr++) {
                        const int r = u + 64 * rr;
                        const int x0 = sm.rx0[r], x1 = sm.rx1[r];
                        const uint32_t M =
                            x0 > x1 ? 0u : (uint32_t)(((2ull << x1) - 1ull) & ~((1ull << x0) - 1ull));  // bits x0..x1
                        if (M == 0u && zero_row[rr]) continue;
                        zero_row[rr] = M == 0u;
                        // all loads of the row first (from the slot): latencies overlap; chunks of 8
                        // x outside the row's range are not loaded (they are stored as zeros)
                        uint4 val[TX / 8][NSL];
#pragma unroll
                        for (int v = 0; v < TX / 8; v++)
#pragma unroll
                            for (int q = 0; q < NSL; q++)
                                val[v][q] = ((M >> (8 * v)) & 0xFFu)
                                                ? vslot[((v >> 1) * NSL + q) * (MROWS * KP / 8) + (r >> 3) * 16 +
                                                        (v & 1) * 8 + (r & 7)]
                                                : make_uint4(0u, 0u, 0u, 0u);
#pragma unroll
                        for (int v = 0; v < TX / 8; v++) {
                            const uint4 mk = chunk_mask(M >> (8 * v));
                            const int o16 = (r >> 3) * 16 + (v & 1) * 8 + (r & 7);  // umma_off / 16
#pragma unroll
                            for (int q = 0; q < NSL; q++)
                                reinterpret_cast<uint4 *>(sm.A[v >> 1][q])[o16] =
                                    make_uint4(val[v][q].x & mk.x, val[v][q].y & mk.y, val[v][q].z & mk.z,
                                               val[v][q].w & mk.w);
                        }
                    }
                }
                if constexpr (kGeneral) general_a_row(sm, A.glv[td.level], P, Q, sh, m, zero_row[0]);
                tc::fence_async_smem();
                tc::fence_before_sync();
                __syncthreads();
                if (tid == 0) {
                    tc::fence_after_sync();
                    uint64_t a_[2][NSL], b_[2][NSL];
                    for (int h = 0; h < 2; h++)
                        for (int q = 0; q < NSL; q++) {
                            a_[h][q] = tc::desc_kmajor(sm.A[h][q], 128, 256);
                            b_[h][q] = tc::desc_kmajor(sm.B + h * kBHalf + q * kBPlane, kBLbo, kBSbo);
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
                const bool live = sm.rx0[m] <= sm.rx1[m];
                ff *const srow = sm.st.S + s_index(m, sh.ly);
#pragma unroll 1
                for (int c = 0; c < KP / 8; c++) {
                    if (8 * c >= L) break;  // uniform: S columns alpha >= L are not read
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
                        if (a < L && live) {
                            const ff d2 = two_sum(__uint_as_float(ra[i]), __uint_as_float(rb[i]));
                            ff t = two_sum(d2.hi, __fmul_rn(__uint_as_float(r3[i]), 0.0009765625f));
                            t.lo = __fadd_rn(t.lo, __fmaf_rn(__uint_as_float(r4[i]), 9.5367431640625e-07f,
                                                             __fmaf_rn(__uint_as_float(r5[i]), 9.313225746154785e-10f, d2.lo)));
                            t = fast_two_sum(t.hi, t.lo);
                            const int vrow = kGeneral ? sm.vmr[m] : vm;
                            const int E = vrow + sm.gexp[a] - 2 * SLB;
                            if (E >= -126 && vrow != kZeroExp && sm.gexp[a] != kZeroExp) {
                                const float scl = pow2i(min(E, 127));
                                s = {__fmul_rn(t.hi, scl), __fmul_rn(t.lo, scl)};
                            }
                        }
                        srow[a] = s;
                    }
                }
                tc::fence_before_sync();
                __syncwarp();
                // stage 2 transposed: T[z][(b,a)] = sum_y S[(z,y)][a] Y[b][y], by the warp whose
                // rows have this z (a warp barrier after the readout suffices)
                const int lzw = 5 - sh.ly;  // log2 of the z values per warp
                const int zbase = (warp * 32) >> sh.ly;
                const unsigned char *qbL = sm.qb[L - 1];
                for (int t = tid & 31; t < (npair << lzw); t += 32) {
                    const int zz = zbase + (t & ((1 << lzw) - 1));
                    const int q = t >> lzw, b = qbL[q];  // q = pair_index(L, b, a)
                    const int a = q - (b * L - (b * (b - 1)) / 2);
                    ff s0 = {0.0f, 0.0f}, s1 = {0.0f, 0.0f};
                    const ff *sz = sm.st.S + s_index(zz * TY, sh.ly) + a;  // rows (zz, y) at sz[y * kSRow]
#pragma unroll 2
                    for (int yy = 0; yy < TY; yy += 2) {
                        ff_acc_lazy(s0, sz[yy * kSRow], cm.Y[b][yy]);
                        ff_acc_lazy(s1, sz[(yy + 1) * kSRow], cm.Y[b][yy + 1]);
                    }
                    sm.st.T[zz][q] = ff_add(s0, s1);
                }
                __syncthreads();
                // stage 1 transposed: W[g][b][a] += sum_z T[z][(b,a)] Z[g][z]
                const int nc = ncoef(lp);
                for (int t = tid; t < nc; t += NTHR) {
                    // (g, b, a) of packed index t: slab g by the slab starts, b by the pair table
                    int g = 0;
                    while (g < lp && sm.zs[g + 1] <= t) g++;
                    const int qn = lp - g, r = t - sm.zs[g];
                    const int b = sm.qb[qn][r];
                    const int a = r - (b * (qn + 1) - (b * (b - 1)) / 2);
                    ff s0 = {0.0f, 0.0f}, s1 = {0.0f, 0.0f};
                    const int pi = pair_index(L, b, a);
#pragma unroll 2
                    for (int zz = 0; zz < TZ; zz += 2) {
                        ff_acc_lazy(s0, sm.st.T[zz][pi], cm.Z[g][zz]);
                        ff_acc_lazy(s1, sm.st.T[zz + 1][pi], cm.Z[g][zz + 1]);
                    }
                    const ff s = ff_add(s0, s1);
                    if (s.hi != 0.0f) {
                        double val = (double)s.hi + (double)s.lo;
                        if constexpr (kGeneral) {
                            // moments in powers of t_d = d_d |v_d| -> lattice-index powers d_d
                            for (int e = 0; e < a; e++) val *= P.hx;
                            for (int e = 0; e < b; e++) val *= P.hy;
                            for (int e = 0; e < g; e++) val *= P.hz;
                        }
                        atomicAdd(A.mom + moff + t, val);
                    }
                }
                __syncthreads();
            }
        }
        cp_async_wait_all();
        if (cm.abort) break;
    }
    tc_teardown(cm, kCols, phase);
}

// the float-float coefficients of every orthorhombic pair into its blob; one warp per pair
__global__ void k_coef_to_blob(const double *__restrict__ c, uint4 *blob, const int64_t *__restrict__ off16,
                               int64_t ntask) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t k = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); k < ntask; k += nw) {
        const TPair *p = reinterpret_cast<const TPair *>(blob + off16[k]);
        const int64_t src = p->coef_off;
        const int lp = p->lp;
        const int nc = ncoef(lp);
        float2 *dst = reinterpret_cast<float2 *>(blob + off16[k] + kHdr16);
        // general cell: lattice-index powers di^a dj^b dk^g -> powers of t_d = d_d |v_d|
        double hinv[3] = {1.0, 1.0, 1.0};
        if (p->general)
            for (int d = 0; d < 3; d++) hinv[d] = 1.0 / ((double)p->h[d].hi + (double)p->h[d].lo);
        for (int t = lane; t < nc; t += 32) {
            double d = c[src + t];
            if (p->general) {
                int g = 0, b = 0, r = t;
                for (g = 0; g <= lp; g++) {
                    const int cnt = ((lp - g + 1) * (lp - g + 2)) / 2;
                    if (r < cnt) break;
                    r -= cnt;
                }
                for (b = 0; b <= lp - g; b++) {
                    if (r <= lp - g - b) break;
                    r -= lp - g - b + 1;
                }
                for (int e = 0; e < g; e++) d *= hinv[2];
                for (int e = 0; e < b; e++) d *= hinv[1];
                for (int e = 0; e < r; e++) d *= hinv[0];
            }
            const float h = __double2float_rn(d);
            dst[t] = make_float2(h, __double2float_rn(d - (double)h));
        }
    }
}

// the images of every (tile, pair) item, once per task set; one block per tile
__global__ void k_item_images(const TileDesc *__restrict__ tiles, const int64_t *__restrict__ start,
                              const uint64_t *__restrict__ items, const uint4 *__restrict__ blob,
                              const LevelDev *__restrict__ levels, ItemImg *out, int ntiles, int *status) {
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const TileDesc td = tiles[tile];
        const LevelDev &lv = levels[td.level];
        const int ext_x = min(TX, lv.ngrid[0] - td.t[0] * TX);
        for (int64_t it = start[2 * tile] + threadIdx.x; it < start[2 * tile + 1]; it += blockDim.x) {
            const TPair &p = *reinterpret_cast<const TPair *>(blob + (items[it] >> 16));
            int img[3][kMaxImages], n[3];
            axis_images(lv, 0, td.t[0], TX, p, img[0], n[0], status);
            const TileShape sh(td.lz);
            axis_images(lv, 1, td.t[1], sh.TY, p, img[1], n[1], status);
            axis_images(lv, 2, td.t[2], sh.TZ, p, img[2], n[2], status);
            ItemImg r;
            memset(&r, 0, sizeof r);
            r.nimg = n[0] | (n[1] << 8) | (n[2] << 16);
            if (n[0] > 0 && n[1] > 0 && n[2] > 0) set_image(p, r.im, img[0][0], img[1][0], img[2][0], ext_x);
            out[it] = r;
        }
    }
}

// ---------------------------------------------------------------------------
// Binning on the device: the (tile, pair) items of every binned pair.
struct BinLevel {
    double G[3][3];     // metric of the lattice steps, G_ab = v_a . v_b (general cells)
    int first;          // index of the level's first tile
    int nt[3];          // tiles per axis
    int lz;             // log2 of the tile z extent
};

// Minimum of d^T G d over the box lo <= d <= hi (G symmetric positive definite;
// infinite bounds allowed).  The minimiser has every coordinate either free or
// at one of its bounds; for each such pattern the stationary point of the free
// coordinates is solved and, if it lies in the box, its value kept.  Rounding
// can only accept a point just outside the box, which lowers the result: a test
// "minimum > r^2" built on it never drops a point inside the sphere.
__device__ double box_min_q(const double (&G)[3][3], const double (&lo)[3], const double (&hi)[3]) {
    if (lo[0] <= 0.0 && hi[0] >= 0.0 && lo[1] <= 0.0 && hi[1] >= 0.0 && lo[2] <= 0.0 && hi[2] >= 0.0) return 0.0;
    double best = HUGE_VAL;
    for (int pat = 1; pat < 27; pat++) {  // pattern 0 (all free) is the origin, handled above
        const int s[3] = {pat % 3, (pat / 3) % 3, pat / 9};  // 0 free, 1 at lo, 2 at hi
        double d[3] = {0.0, 0.0, 0.0};
        int fr[2], nf = 0;
        bool ok = true;
        for (int a = 0; a < 3; a++) {
            if (s[a] == 0) {
                fr[nf++] = a;
            } else {
                d[a] = s[a] == 1 ? lo[a] : hi[a];
                ok = ok && isfinite(d[a]);
            }
        }
        if (!ok) continue;
        auto rhs = [&](int a) {  // -(G_aX d_X) over the fixed coordinates
            double r = 0.0;
            for (int b = 0; b < 3; b++)
                if (s[b] != 0) r -= G[a][b] * d[b];
            return r;
        };
        if (nf == 1) {
            d[fr[0]] = rhs(fr[0]) / G[fr[0]][fr[0]];
        } else if (nf == 2) {
            const int a = fr[0], b = fr[1];
            const double ra = rhs(a), rb = rhs(b);
            const double det = G[a][a] * G[b][b] - G[a][b] * G[a][b];
            d[a] = (ra * G[b][b] - rb * G[a][b]) / det;
            d[b] = (G[a][a] * rb - G[a][b] * ra) / det;
        }
        for (int k = 0; k < nf; k++) {
            const int a = fr[k];
            const double tol = 1e-9 * (1.0 + fabs(d[a]));
            ok = ok && d[a] >= lo[a] - tol && d[a] <= hi[a] + tol;
        }
        if (!ok) continue;
        double q = 0.0;
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) q += d[a] * G[a][b] * d[b];
        best = fmin(best, q);
    }
    return best;
}

// One axis of a pair's cube (cube offsets lb..hi around cc, as grid_base_ref_c.cc:318-351
// maps them) cut into runs of consecutive grid indices inside one tile.
struct AxisRuns {
    int lb, hi, cc, T, N, npts, periodic, lbg;
    bool dedupe;  // the cube spans so much of a periodic axis that two runs may hit one tile
    __device__ void init(const LevelDev &lv, int d, int cc_, int lb_, int hi_, int T_) {
        lb = lb_; hi = hi_; cc = cc_; T = T_;
        N = lv.ngrid[d]; npts = lv.npts[d]; periodic = lv.periodic[d]; lbg = lv.lb_grid[d];
        dedupe = periodic && (hi - lb + 1) + T > N;
    }
    // the run starting at offset gg: its tile and its offsets g0..g1; gg moves
    // past the run; false: outside the window
    __device__ bool next(int &gg, int &t, int &g0, int &g1) const {
        const int w = periodic ? imod(cc + gg, npts) : gg + imod(cc + lb + lbg, npts) - lb;
        if (w < 0 || w >= N) {
            gg++;
            return false;
        }
        t = w / T;
        const int len = min(T - (w - t * T), N - w);
        g0 = gg;
        g1 = min(gg + len - 1, hi);
        gg += len;
        return true;
    }
    // calls fn(tile, g0, g1) once per tile the axis touches; where several runs
    // reach one tile, only the first reports it, with the hull of their offsets
    template <class Fn>
    __device__ void each_range(Fn &&fn) const {
        for (int gg = lb; gg <= hi;) {
            const int gs = gg;
            int t, g0, g1;
            if (!next(gg, t, g0, g1)) continue;
            if (dedupe) {
                bool seen = false;
                for (int g2 = lb; g2 < gs && !seen;) {
                    int t2, a2, b2;
                    if (next(g2, t2, a2, b2) && t2 == t) seen = true;
                }
                if (seen) continue;
                for (int g2 = gg; g2 <= hi;) {
                    int t2, a2, b2;
                    if (next(g2, t2, a2, b2) && t2 == t) {
                        g0 = min(g0, a2);
                        g1 = max(g1, b2);
                    }
                }
            }
            fn(t, g0, g1);
        }
    }
    // calls fn(tile, fmin) once per tile the axis touches, fmin the smallest folded
    // offset |f| (f = g <= 0 ? -g : g - 1) over the runs into the tile
    template <class Fn>
    __device__ void each(Fn &&fn) const {
        for (int gg = lb; gg <= hi;) {
            const int gs = gg;
            int t, g0, g1;
            if (!next(gg, t, g0, g1)) continue;
            auto fold = [](int a, int b) { return (a <= 1 && b >= 0) ? 0 : (b < 0 ? -b : a - 1); };
            int f = fold(g0, g1);
            if (dedupe) {  // only the first run into a tile reports it, with the minimum over all runs
                bool seen = false;
                for (int g2 = lb; g2 < gs && !seen;) {
                    int t2, a2, b2;
                    if (next(g2, t2, a2, b2) && t2 == t) seen = true;
                }
                if (seen) continue;
                for (int g2 = gg; g2 <= hi;) {
                    int t2, a2, b2;
                    if (next(g2, t2, a2, b2) && t2 == t) f = min(f, fold(a2, b2));
                }
            }
            fn(t, f);
        }
    }
};

// Pass 0: items per tile (count).  Pass 1: item words into the tile's slots
// (cursor).  A pair visits a tile only if some cube point of the tile can be
// inside its sphere (with a margin): orthorhombic, the folded distance of the
// tile's nearest offsets <= radius; general cell, the least |r - rp|^2 over the
// lattice-index box of the tile's offsets (box_min_q) <= radius^2, tested per z
// run, then per (z, y) runs, then per tile.  Explicit cube lists are not culled.
// kGen: the general-cell pairs [k0, k1) (the culling's box minimum needs registers
// and stack that would slow the orthorhombic launch, kGen = false).
template <bool kGen>
__global__ void k_bin_pairs(const PairGeom *__restrict__ geoms, int64_t k0, int64_t k1,
                            const LevelDev *__restrict__ levels, const BinLevel *__restrict__ bl,
                            const int64_t *__restrict__ off16, const int *__restrict__ len16, int pass, int *count,
                            unsigned long long *cursor, uint64_t *items) {
    for (int64_t k = k0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < k1; k += (int64_t)gridDim.x * blockDim.x) {
        const PairGeom &g = geoms[k];
        const LevelDev &lv = levels[g.level];
        const BinLevel B = bl[g.level];
        const TileShape sh(B.lz);
        int lb[3], hi[3];
        for (int d = 0; d < 3; d++) {  // general cell: the index box as a box-relative cube [0, hi - cc]
            lb[d] = g.ortho ? g.lb[d] : 0;
            hi[d] = g.ortho ? g.hi[d] : g.hi[d] - g.cc[d];
        }
        AxisRuns ax, ay, az;
        ax.init(lv, 0, g.cc[0], lb[0], hi[0], TX);
        ay.init(lv, 1, g.cc[1], lb[1], hi[1], sh.TY);
        az.init(lv, 2, g.cc[2], lb[2], hi[2], sh.TZ);
        const double r2 = g.radius * g.radius * (1.0 + 1e-9) + 1e-12;
        const double hx = lv.dh[0][0], hy = lv.dh[1][1], hz = lv.dh[2][2];
        const bool table = g.table_off >= 0;
        const uint64_t word = ((uint64_t)off16[k] << 16) | (uint64_t)len16[k];
        auto emit = [&](int tz, int ty, int tx) {
            const int tile = B.first + (tz * B.nt[1] + ty) * B.nt[0] + tx;
            if (pass == 0) atomicAdd(count + tile, 1);
            else items[atomicAdd(cursor + tile, 1ull)] = word;
        };
        if constexpr (kGen) {
            // lattice-index offsets from the product centre: d_a = cc_a + gg - gp_a
            const double c[3] = {g.off[0] - g.cc[0], g.off[1] - g.cc[1], g.off[2] - g.cc[2]};
            const double rg = g.radius * g.radius * (1.0 + 1e-6) + 1e-12;
            double lo[3] = {-HUGE_VAL, -HUGE_VAL, 0.0}, up[3] = {HUGE_VAL, HUGE_VAL, 0.0};
            az.each_range([&](int tz, int z0, int z1) {
                lo[2] = z0 - c[2];
                up[2] = z1 - c[2];
                lo[1] = lo[0] = -HUGE_VAL;
                up[1] = up[0] = HUGE_VAL;
                if (box_min_q(B.G, lo, up) > rg) return;
                ay.each_range([&](int ty, int y0, int y1) {
                    lo[1] = y0 - c[1];
                    up[1] = y1 - c[1];
                    lo[0] = -HUGE_VAL;
                    up[0] = HUGE_VAL;
                    if (box_min_q(B.G, lo, up) > rg) return;
                    ax.each_range([&](int tx, int x0, int x1) {
                        lo[0] = x0 - c[0];
                        up[0] = x1 - c[0];
                        if (box_min_q(B.G, lo, up) > rg) return;
                        emit(tz, ty, tx);
                    });
                });
            });
        } else {
        az.each([&](int tz, int fz) {
            const double dz = fz * hz;
            if (!table && dz * dz > r2) return;
            ay.each([&](int ty, int fy) {
                const double dy = fy * hy;
                if (!table && dz * dz + dy * dy > r2) return;
                ax.each([&](int tx, int fx) {
                    const double dx = fx * hx;
                    if (!table && dz * dz + dy * dy + dx * dx > r2) return;
                    emit(tz, ty, tx);
                });
            });
        });
        }
    }
}

// both kinds of pairs of a task set (orthorhombic first in the sorted order)
static cudaError_t bin_pairs(const TaskSet &ts, const MixedState &M, int pass, int *count,
                             unsigned long long *cursor, uint64_t *items) {
    const Plan &P = *ts.plan;
    auto blocks = [](int64_t n) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 127) / 128, 8192)); };
    if (M.northo > 0)
        k_bin_pairs<false><<<blocks(M.northo), 128>>>(ts.d_geom, 0, M.northo, P.d_levels, M.d_bl, M.d_blob_off,
                                                      M.d_blob_len, pass, count, cursor, items);
    if (M.nbin > M.northo)
        k_bin_pairs<true><<<blocks(M.nbin - M.northo), 128>>>(ts.d_geom, M.northo, M.nbin, P.d_levels, M.d_bl,
                                                              M.d_blob_off, M.d_blob_len, pass, count, cursor, items);
    return cudaGetLastError();
}

// The record (TPair) of every binned pair from its geometry, into its blob.
__global__ void k_make_records(const PairGeom *__restrict__ geoms, int64_t nbin, const LevelDev *__restrict__ levels,
                               const int64_t *__restrict__ off16, uint4 *blob) {
    auto split = [](double d) {
        const float h = __double2float_rn(d);
        return ff{h, __double2float_rn(d - (double)h)};
    };
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nbin; k += (int64_t)gridDim.x * blockDim.x) {
        const PairGeom &g = geoms[k];
        const LevelDev &lv = levels[g.level];
        TPair p;
        memset(&p, 0, sizeof p);
        p.r2 = rmul(g.radius, g.radius);
        p.r2f = __double2float_rn(p.r2);
        p.zetp = split(g.zetp);
        p.lp = g.lp;
        p.L = g.lp + 1;
        p.coef_off = g.coef_off;
        if (!g.ortho) {
            // general cell: t_d = (index_d - gp_d) |v_d|, the box as a cube [0, hi - cc] at cc
            p.general = 1;
            double len[3];
            for (int d = 0; d < 3; d++)
                len[d] = rsqrt_rn(radd(radd(rmul(lv.dh[d][0], lv.dh[d][0]), rmul(lv.dh[d][1], lv.dh[d][1])),
                                       rmul(lv.dh[d][2], lv.dh[d][2])));
            p.hx = rdiv(1.0, len[0]);
            p.hy = rdiv(1.0, len[1]);
            p.hz = rdiv(1.0, len[2]);
            p.radius = g.radius;
            for (int d = 0; d < 3; d++) {
                p.h[d] = split(len[d]);
                p.off[d] = split(rmul(rsub(g.off[d], (double)g.cc[d]), len[d]));
                p.lb[d] = 0;
                p.hi[d] = g.hi[d] - g.cc[d];
                p.cc[d] = g.cc[d];
                p.gp[d] = g.off[d];
            }
            p.table_off = -1;
        } else {
            p.hx = lv.dh[0][0];
            p.hy = lv.dh[1][1];
            p.hz = lv.dh[2][2];
            p.hxf = __double2float_rn(p.hx);
            p.hyf = __double2float_rn(p.hy);
            p.hzf = __double2float_rn(p.hz);
            p.hyinvf = __double2float_rn(rdiv(1.0, p.hy));
            p.hxinvf = __double2float_rn(rdiv(1.0, p.hx));
            for (int d = 0; d < 3; d++) {
                p.off[d] = split(g.off[d]);
                p.h[d] = split(lv.dh[d][d]);
                p.lb[d] = g.lb[d];
                p.hi[d] = g.hi[d];
                p.cc[d] = g.cc[d];
            }
            p.kgmin = g.kgmin;
            p.table_off = g.table_off;
        }
        const uint4 *src = reinterpret_cast<const uint4 *>(&p);
        uint4 *dst = blob + off16[k];
        for (int c = 0; c < (int)(sizeof(TPair) / 16); c++) dst[c] = src[c];
        if (sizeof(TPair) % 16) {  // the record's last partial chunk
            uint4 last = make_uint4(0, 0, 0, 0);
            memcpy(&last, reinterpret_cast<const char *>(&p) + (sizeof(TPair) / 16) * 16, sizeof(TPair) % 16);
            dst[sizeof(TPair) / 16] = last;
        }
    }
}

int mixed_build(TaskSet &ts, std::string &err) {
    MixedState *M = new MixedState();
    ts.mixed = M;
    const Plan &P = *ts.plan;
    int64_t northo = 0;
    while (northo < ts.ntasks && ts.h_geom[northo].ortho) northo++;
    M->northo = (int)northo;
    // General-cell levels go on the tiled kernels when the cosine matrix C of the
    // lattice steps satisfies C >= 0.4 I: then sum t_d^2 <= 2.5 r^2, so inside the
    // cube the cross factor exp(-2 zetp sum c_de t_d t_e) of the Gaussian stays
    // within exp(+-58) (float range).  Otherwise they stay on the float-float
    // general kernel.
    std::vector<GenLevel> glv(P.nlevels);
    bool gen_ok = true;
    for (int l = 0; l < P.nlevels; l++) {
        const LevelDev &lv = P.lv[l];
        if (lv.ortho) continue;
        double G[3][3], h[3];
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++)
                G[a][b] = lv.dh[a][0] * lv.dh[b][0] + lv.dh[a][1] * lv.dh[b][1] + lv.dh[a][2] * lv.dh[b][2];
        for (int a = 0; a < 3; a++) h[a] = std::sqrt(G[a][a]);
        double C[3][3];
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) C[a][b] = G[a][b] / (h[a] * h[b]) - (a == b ? 0.4 : 0.0);
        const double m1 = C[0][0], m2 = C[0][0] * C[1][1] - C[0][1] * C[1][0];
        const double m3 = C[0][0] * (C[1][1] * C[2][2] - C[1][2] * C[2][1]) -
                          C[0][1] * (C[1][0] * C[2][2] - C[1][2] * C[2][0]) +
                          C[0][2] * (C[1][0] * C[2][1] - C[1][1] * C[2][0]);
        if (!(m1 > 0.0 && m2 > 0.0 && m3 > 0.0)) gen_ok = false;
        GenLevel &q = glv[l];
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) q.dh[a][b] = (float)lv.dh[a][b];
        q.a = (float)G[0][0];
        q.inv2a = (float)(0.5 / G[0][0]);
        auto sp = [](double d) {
            const float hi = (float)d;
            return ff{hi, (float)(d - (double)hi)};
        };
        q.c01 = sp(G[0][1] / (h[0] * h[1]));
        q.c02 = sp(G[0][2] / (h[0] * h[2]));
        q.c12 = sp(G[1][2] / (h[1] * h[2]));
    }
    const int64_t ngen = ts.ntasks - northo;
    // ... when every general level has a tile shape (not kUntiled) ...
    for (int l = 0; l < P.nlevels; l++)
        if (!P.lv[l].ortho && ts.tile_lz[l] == kUntiled) gen_ok = false;
    // ... and when no general box spans more periodic images of one tile axis
    // than the kernels hold (kMaxImages): count <= (extent + T - 1) / N + 1
    for (int64_t k = northo; k < ts.ntasks && gen_ok; k++) {
        const PairGeom &g = ts.h_geom[k];
        const LevelDev &lv = P.lv[g.level];
        const TileShape sh(ts.tile_lz[g.level]);
        const int T[3] = {TX, sh.TY, sh.TZ};
        for (int d = 0; d < 3; d++)
            if (lv.periodic[d] && (g.hi[d] - g.cc[d] + 1) + T[d] - 1 > (kMaxImages - 1) * lv.npts[d]) gen_ok = false;
    }
    M->gen_tiled = gen_ok && ngen > 0;
    const int64_t nbin = northo + (M->gen_tiled ? ngen : 0);
    M->nbin = nbin;
    std::vector<char> binned_level(P.nlevels, 0);
    for (int64_t k = 0; k < nbin; k++) binned_level[ts.h_geom[k].level] = 1;
    // tiles of every level with binned pairs: orthorhombic levels first
    std::vector<int> lvl_first(P.nlevels, -1);
    std::vector<TileDesc> tiles;
    int ntx[GPW_MAX_LEVELS], nty[GPW_MAX_LEVELS], ntz[GPW_MAX_LEVELS];
    for (int pass = 0; pass < 2; pass++)
    for (int l = 0; l < P.nlevels; l++) {
        if ((pass == 0) != (P.lv[l].ortho != 0)) continue;
        if (!P.lv[l].ortho && !binned_level[l]) continue;
        ntx[l] = (P.lv[l].ngrid[0] + TX - 1) / TX;
        const TileShape sh(ts.tile_lz[l]);
        nty[l] = (P.lv[l].ngrid[1] + sh.TY - 1) / sh.TY;
        ntz[l] = (P.lv[l].ngrid[2] + sh.TZ - 1) / sh.TZ;
        lvl_first[l] = (int)tiles.size();
        for (int a = 0; a < ntz[l]; a++)
            for (int b = 0; b < nty[l]; b++)
                for (int c = 0; c < ntx[l]; c++) tiles.push_back(TileDesc{l, {c, b, a}, ts.tile_lz[l], 0});
    }
    M->h_tiles = tiles;
    std::vector<BinLevel> blv(P.nlevels);
    for (int l = 0; l < P.nlevels; l++) {
        blv[l].first = lvl_first[l];
        blv[l].nt[0] = lvl_first[l] >= 0 ? ntx[l] : 0;
        blv[l].nt[1] = lvl_first[l] >= 0 ? nty[l] : 0;
        blv[l].nt[2] = lvl_first[l] >= 0 ? ntz[l] : 0;
        blv[l].lz = ts.tile_lz[l] >= 0 ? ts.tile_lz[l] : kDefaultTileLz;
        const LevelDev &lv = P.lv[l];
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++)
                blv[l].G[a][b] = lv.dh[a][0] * lv.dh[b][0] + lv.dh[a][1] * lv.dh[b][1] + lv.dh[a][2] * lv.dh[b][2];
    }
    const int ntiles = (int)tiles.size();
    // blob layout: per task the record, then its coefficients
    std::vector<int64_t> off16((size_t)std::max<int64_t>(nbin, 1), 0);
    std::vector<int> len16((size_t)std::max<int64_t>(nbin, 1), 0);
    int64_t nchunks = 0;
    for (int64_t k = 0; k < nbin; k++) {
        off16[k] = nchunks;
        len16[k] = kHdr16 + (ncoef(ts.h_geom[k].lp) * (int)sizeof(float2) + 15) / 16;
        nchunks += len16[k];
    }
    cudaError_t e = cudaSuccess;
    auto alloc = [&](void **p, size_t bytes) {
        if (e == cudaSuccess) e = cudaMalloc(p, std::max<size_t>(bytes, 16));
    };
    alloc((void **)&M->d_blob, sizeof(uint4) * (size_t)std::max<int64_t>(nchunks, 1));
    alloc((void **)&M->d_blob_off, sizeof(int64_t) * off16.size());
    alloc((void **)&M->d_blob_len, sizeof(int) * len16.size());
    alloc((void **)&M->d_bl, sizeof(BinLevel) * blv.size());
    alloc((void **)&M->d_count, sizeof(int) * (size_t)std::max(ntiles, 1));
    alloc((void **)&M->d_cursor, sizeof(unsigned long long) * (size_t)std::max(ntiles, 1));
    alloc((void **)&M->d_queue, sizeof(int) * 5);  // [4]: status sink of the set-up kernels
    alloc((void **)&M->d_glv, sizeof(GenLevel) * glv.size());
    if (e == cudaSuccess) e = cudaMemset(M->d_blob, 0, sizeof(uint4) * (size_t)std::max<int64_t>(nchunks, 1));
    if (e == cudaSuccess)
        e = cudaMemcpy(M->d_blob_off, off16.data(), sizeof(int64_t) * off16.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(M->d_blob_len, len16.data(), sizeof(int) * len16.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(M->d_bl, blv.data(), sizeof(BinLevel) * blv.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(M->d_glv, glv.data(), sizeof(GenLevel) * glv.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(M->d_queue, 0, sizeof(int) * 5);
    if (e != cudaSuccess) {
        err = std::string("mixed_build: ") + cudaGetErrorString(e);
        return GPW_ERR_CUDA;
    }
    int sms = 0, per_sm = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, P.device);
    const void *kc[2] = {(const void *)k_collocate_tiled<false>, (const void *)k_collocate_tiled<true>};
    const void *ki[2] = {(const void *)k_integrate_tiled<false>, (const void *)k_integrate_tiled<true>};
    for (int v = 0; v < 2 && e == cudaSuccess; v++) {
        e = cudaFuncSetAttribute(kc[v], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SmemColl));
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(ki[v], cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)(v ? sizeof(SmemInt<true>) : kSmemIntOrtho));
    }
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
    per_sm = std::min(resident(kc[0], sizeof(SmemColl)), resident(kc[1], sizeof(SmemColl)));
    const int per_sm_i = resident(ki[0], kSmemIntOrtho);
    M->per_sm = per_sm;
    M->per_sm_i = per_sm_i;
    M->per_sm_ig = resident(ki[1], sizeof(SmemInt<true>));
    M->sms = sms;
    // one V slot per resident orthorhombic integrate CTA
    if (northo > 0) {
        e = cudaMalloc(&M->d_vslot, sizeof(uint4) * kVSlot16 * (size_t)sms * per_sm_i);
        if (e != cudaSuccess) {
            err = std::string("mixed_build: ") + cudaGetErrorString(e);
            return GPW_ERR_CUDA;
        }
    }
    return mixed_rebin(ts, err);
}

// Records, items, work units and item images from the task set's current device
// geometry (ts.d_geom): at creation and after a geometry update.  The tile
// grid, the blob layout and the choice of kernels stay as mixed_build made them.
int mixed_rebin(TaskSet &ts, std::string &err) {
    MixedState *M = ts.mixed;
    const Plan &P = *ts.plan;
    const int64_t nbin = M->nbin;
    const int ntiles = (int)M->h_tiles.size();
    cudaError_t e = cudaSuccess;
    auto fail = [&](cudaError_t ce) {
        err = std::string("mixed_rebin: ") + cudaGetErrorString(ce);
        return GPW_ERR_CUDA;
    };
    const unsigned nblk = (unsigned)std::max<int64_t>(1, std::min<int64_t>((nbin + 127) / 128, 8192));
    if (nbin > 0) {
        k_make_records<<<nblk, 128>>>(ts.d_geom, nbin, P.d_levels, M->d_blob_off, M->d_blob);
        if ((e = cudaGetLastError()) != cudaSuccess) return fail(e);
    }
    if ((e = cudaMemset(M->d_count, 0, sizeof(int) * (size_t)std::max(ntiles, 1))) != cudaSuccess) return fail(e);
    if (nbin > 0 && (e = bin_pairs(ts, *M, 0, M->d_count, nullptr, nullptr)) != cudaSuccess) return fail(e);
    std::vector<int> count((size_t)std::max(ntiles, 1), 0);
    if ((e = cudaMemcpy(count.data(), M->d_count, sizeof(int) * count.size(), cudaMemcpyDeviceToHost)) != cudaSuccess)
        return fail(e);
    // items grouped by tile
    std::vector<int64_t> start(ntiles + 1, 0);
    for (int i = 0; i < ntiles; i++) start[i + 1] = start[i] + count[i];
    const int64_t nitems = start[ntiles];
    int nto = 0;
    while (nto < ntiles && P.lv[M->h_tiles[nto].level].ortho) nto++;
    // Work units for the persistent queue: a tile with more items than ~1/64 of
    // an even share per SM is divided into units of consecutive items (their
    // flushes add with FP64 atomics).  Within each group (orthorhombic, general)
    // units run by decreasing work class (item counts within a factor 2^(1/4)
    // share a class), and within a class in the tiles' raster order: the tiles in
    // flight at one time then form a compact slab of the grid, so a pair's record,
    // coefficients and moments stay in L2 between the neighbouring tiles that use
    // them, while the short units still come last.
    const int64_t target = std::max<int64_t>(64, (nitems + 64LL * M->sms - 1) / std::max(1, 64 * M->sms));
    struct Unit {
        int tile;
        int64_t it0, it1;
        bool split;
    };
    std::vector<Unit> units;
    for (int t = 0; t < ntiles; t++) {
        const int64_t n = count[t];
        if (n == 0) continue;
        const int64_t nu = (n + target - 1) / target;
        for (int64_t u = 0; u < nu; u++)
            units.push_back(Unit{t, start[t] + n * u / nu, start[t] + n * (u + 1) / nu, nu > 1});
    }
    auto work_class = [](const Unit &u) { return (int)std::floor(4.0 * std::log2((double)(u.it1 - u.it0))); };
    std::stable_sort(units.begin(), units.end(), [&](const Unit &a, const Unit &b) {
        const bool ga = a.tile >= nto, gb = b.tile >= nto;
        if (ga != gb) return !ga;
        return work_class(a) > work_class(b);
    });
    const int nunits = (int)units.size();
    int nuo = 0;
    while (nuo < nunits && units[nuo].tile < nto) nuo++;
    std::vector<TileDesc> tiles_sorted(std::max(nunits, 1));
    std::vector<int64_t> ubounds(2 * (size_t)std::max(nunits, 1), 0);  // per unit: first item, end
    for (int u = 0; u < nunits; u++) {
        tiles_sorted[u] = M->h_tiles[units[u].tile];
        tiles_sorted[u].split = units[u].split ? 1 : 0;
        ubounds[2 * u] = units[u].it0;
        ubounds[2 * u + 1] = units[u].it1;
    }
    // storage for the items and units (kept when large enough)
    if (nitems > M->cap_items || !M->d_items) {
        cudaFree(M->d_items);
        cudaFree(M->d_iimg);
        M->d_items = nullptr;
        M->d_iimg = nullptr;
        M->cap_items = 0;  // a failed allocation below leaves nothing to reuse
        const int64_t cap = std::max<int64_t>(nitems + nitems / 16, 1);
        if ((e = cudaMalloc(&M->d_items, sizeof(uint64_t) * cap)) != cudaSuccess) return fail(e);
        if ((e = cudaMalloc(&M->d_iimg, sizeof(ItemImg) * cap)) != cudaSuccess) return fail(e);
        M->cap_items = cap;
    }
    if (nunits > M->cap_units || !M->d_tiles) {
        cudaFree(M->d_tiles);
        cudaFree(M->d_start);
        M->d_tiles = nullptr;
        M->d_start = nullptr;
        M->cap_units = 0;
        const int64_t cap = std::max<int64_t>(nunits + nunits / 16, 1);
        if ((e = cudaMalloc(&M->d_tiles, sizeof(TileDesc) * cap)) != cudaSuccess) return fail(e);
        if ((e = cudaMalloc(&M->d_start, sizeof(int64_t) * 2 * cap)) != cudaSuccess) return fail(e);
        M->cap_units = cap;
    }
    if (nunits && (e = cudaMemcpy(M->d_tiles, tiles_sorted.data(), sizeof(TileDesc) * nunits,
                                  cudaMemcpyHostToDevice)) != cudaSuccess)
        return fail(e);
    if ((e = cudaMemcpy(M->d_start, ubounds.data(), sizeof(int64_t) * ubounds.size(), cudaMemcpyHostToDevice)) !=
        cudaSuccess)
        return fail(e);
    std::vector<unsigned long long> cur((size_t)std::max(ntiles, 1), 0ull);
    for (int t = 0; t < ntiles; t++) cur[t] = (unsigned long long)start[t];
    if ((e = cudaMemcpy(M->d_cursor, cur.data(), sizeof(unsigned long long) * cur.size(), cudaMemcpyHostToDevice)) !=
        cudaSuccess)
        return fail(e);
    if (nbin > 0 && (e = bin_pairs(ts, *M, 1, nullptr, M->d_cursor, M->d_items)) != cudaSuccess) return fail(e);
    if (nitems) {
        // image overflows are reported by the tiled kernels when they run (a plain
        // FP64 call on this task set must not see them)
        k_item_images<<<std::max(1, std::min(nunits, 8192)), 128>>>(M->d_tiles, M->d_start, M->d_items, M->d_blob,
                                                                    P.d_levels, M->d_iimg, nunits, M->d_queue + 4);
        if ((e = cudaGetLastError()) != cudaSuccess) return fail(e);
    }
    if ((e = cudaDeviceSynchronize()) != cudaSuccess) return fail(e);
    M->ntiles_ortho = nuo;
    M->ntiles = nunits;
    M->nitems = nitems;
    M->grid_ctas_i = std::max(1, std::min(nunits, M->sms * M->per_sm_i));
    M->grid_ctas = std::max(1, std::min(nunits, M->sms * M->per_sm));
    return GPW_SUCCESS;
}

int64_t mixed_items(const TaskSet &ts) { return ts.mixed ? ts.mixed->nitems : 0; }
int64_t mixed_units(const TaskSet &ts) { return ts.mixed ? ts.mixed->ntiles : 0; }

void mixed_free(TaskSet &ts) {
    MixedState *M = ts.mixed;
    if (!M) return;
    cudaFree(M->d_tiles);
    cudaFree(M->d_blob);
    cudaFree(M->d_blob_off);
    cudaFree(M->d_start);
    cudaFree(M->d_items);
    cudaFree(M->d_iimg);
    cudaFree(M->d_queue);
    cudaFree(M->d_glv);
    cudaFree(M->d_vslot);
    cudaFree(M->d_bl);
    cudaFree(M->d_blob_len);
    cudaFree(M->d_count);
    cudaFree(M->d_cursor);
    delete M;
    ts.mixed = nullptr;
}

static MixedArgs make_args(const TaskSet &ts, const GridPtrs &g, int which, bool general) {
    const MixedState &M = *ts.mixed;
    const int t0 = general ? M.ntiles_ortho : 0;
    MixedArgs a;
    a.blob = M.d_blob;
    a.geoms = ts.d_geom;
    a.levels = ts.plan->d_levels;
    a.tiles = M.d_tiles + t0;
    a.start = M.d_start + 2 * t0;
    a.items = M.d_items;
    a.iimg = M.d_iimg;
    a.table = ts.d_table;
    a.glv = M.d_glv;
    a.mom = ts.d_mom;
    a.vslot = M.d_vslot;
    a.grids = g;
    a.queue = M.d_queue + which + (general ? 2 : 0);
    a.status = ts.d_status;
    a.ntiles = general ? M.ntiles - M.ntiles_ortho : M.ntiles_ortho;
    return a;
}

// general-cell pairs of a mixed call run on the float-float general kernel
static cudaError_t general_ff(const TaskSet &ts, const GridPtrs &g, bool adj, cudaStream_t s) {
    return launch_general_ff(ts, g, adj, s);
}

cudaError_t launch_collocate_mixed(const TaskSet &ts, const GridPtrs &g, cudaStream_t s) {
    if (!ts.mixed) return cudaErrorNotSupported;
    const MixedState &M = *ts.mixed;
    cudaError_t e = cudaSuccess;
    if (M.nbin > 0 && M.ntiles > 0) {
        ts.n_kernels++;
        k_coef_to_blob<<<(unsigned)std::min<int64_t>((M.nbin + 7) / 8, 8192), 256, 0, s>>>(ts.d_coef, M.d_blob,
                                                                                             M.d_blob_off, M.nbin);
        const int nto = M.ntiles_ortho, ntg = M.ntiles - M.ntiles_ortho;
        if (nto > 0) {
            if ((e = cudaMemsetAsync(M.d_queue, 0, sizeof(int), s)) != cudaSuccess) return e;
            ProfScope prof(ts, s);
            k_collocate_tiled<false><<<std::min(nto, M.sms * M.per_sm), NTHR, sizeof(SmemColl), s>>>(
                make_args(ts, g, 0, false));
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
        }
        if (ntg > 0) {
            if ((e = cudaMemsetAsync(M.d_queue + 2, 0, sizeof(int), s)) != cudaSuccess) return e;
            ProfScope prof(ts, s);
            k_collocate_tiled<true><<<std::min(ntg, M.sms * M.per_sm), NTHR, sizeof(SmemColl), s>>>(
                make_args(ts, g, 0, true));
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
        }
    }
    return M.gen_tiled ? cudaSuccess : general_ff(ts, g, false, s);
}

cudaError_t launch_integrate_mixed(const TaskSet &ts, const GridPtrs &g, cudaStream_t s) {
    if (!ts.mixed) return cudaErrorNotSupported;
    const MixedState &M = *ts.mixed;
    cudaError_t e = cudaSuccess;
    if (M.nbin > 0 && M.ntiles > 0) {
        if ((e = cudaMemsetAsync(ts.d_mom, 0, sizeof(double) * ts.coef_len, s)) != cudaSuccess) return e;
        const int nto = M.ntiles_ortho, ntg = M.ntiles - M.ntiles_ortho;
        if (nto > 0) {
            if ((e = cudaMemsetAsync(M.d_queue + 1, 0, sizeof(int), s)) != cudaSuccess) return e;
            ProfScope prof(ts, s);
            k_integrate_tiled<false><<<std::min(nto, M.sms * M.per_sm_i), NTHR, kSmemIntOrtho, s>>>(
                make_args(ts, g, 1, false));
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
        }
        if (ntg > 0) {
            if ((e = cudaMemsetAsync(M.d_queue + 3, 0, sizeof(int), s)) != cudaSuccess) return e;
            ProfScope prof(ts, s);
            k_integrate_tiled<true><<<std::min(ntg, M.sms * M.per_sm_ig), NTHR, sizeof(SmemInt<true>), s>>>(
                make_args(ts, g, 1, true));
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
        }
    }
    return M.gen_tiled ? cudaSuccess : general_ff(ts, g, true, s);
}

}  // namespace gpw
