// C ABI of libgpw_gb300 (include/gpw.h): plans, task sets, dispatch, the
// drop-in single-pair entry, and the host-side geometry every kernel reads.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

#include "gpw_internal.h"

using namespace gpw;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string &msg) {
    g_err = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char *where) {
    return fail(GPW_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define GPW_CUDA(call)                                      \
    do {                                                    \
        cudaError_t e_ = (call);                            \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
    } while (0)

bool finite3(const double *v) { return std::isfinite(v[0]) && std::isfinite(v[1]) && std::isfinite(v[2]); }

// Dense polynomials in (d0, d1, d2) up to total degree kMaxLp, index [k][j][i].
constexpr int NP = kNPow;
constexpr int NQ = NP * NP * NP;
void poly_mul(const std::vector<double> &a, int da, const std::vector<double> &b, int db,
              std::vector<double> &out) {
    std::fill(out.begin(), out.end(), 0.0);
    for (int ka = 0; ka <= da; ka++)
        for (int ja = 0; ja <= da - ka; ja++)
            for (int ia = 0; ia <= da - ka - ja; ia++) {
                const double va = a[(ka * NP + ja) * NP + ia];
                if (va == 0.0) continue;
                for (int kb = 0; kb <= db; kb++)
                    for (int jb = 0; jb <= db - kb; jb++)
                        for (int ib = 0; ib <= db - kb - jb; ib++)
                            out[((ka + kb) * NP + ja + jb) * NP + ia + ib] += va * b[(kb * NP + jb) * NP + ib];
            }
}

// Lattice transform of a general cell: T[q][c], q = (k,j,i) and c = (lz,ly,lx),
// both packed with pidx(kMaxLp, ...).  Column c holds the coefficients of
// (x-xp)^lx (y-yp)^ly (z-zp)^lz in the lattice offsets d_a, since
// r - rp = sum_a d_a dh[a][:]  (the multinomial transform of grid_base_ref_c.cc:646-698).
std::vector<double> lattice_transform(const double dh[3][3]) {
    const int NT = ncoef(kMaxLp);
    std::vector<double> T((size_t)NT * NT, 0.0);
    std::vector<std::vector<double>> U(3 * NP, std::vector<double>(NQ, 0.0));
    for (int c = 0; c < 3; c++) {
        U[c * NP][0] = 1.0;
        std::vector<double> lin(NQ, 0.0);
        lin[1] = dh[0][c];
        lin[NP] = dh[1][c];
        lin[NP * NP] = dh[2][c];
        for (int n = 1; n <= kMaxLp; n++) poly_mul(U[c * NP + n - 1], n - 1, lin, 1, U[c * NP + n]);
    }
    std::vector<double> tmp(NQ), col(NQ);
    for (int lz = 0; lz <= kMaxLp; lz++)
        for (int ly = 0; ly <= kMaxLp - lz; ly++) {
            poly_mul(U[2 * NP + lz], lz, U[1 * NP + ly], ly, tmp);
            for (int lx = 0; lx <= kMaxLp - lz - ly; lx++) {
                poly_mul(tmp, lz + ly, U[0 * NP + lx], lx, col);
                const int ci = pidx(kMaxLp, lz, ly, lx);
                const int deg = lx + ly + lz;
                for (int k = 0; k <= deg; k++)
                    for (int j = 0; j <= deg - k; j++) {
                        const int i = deg - k - j;
                        T[(size_t)pidx(kMaxLp, k, j, i) * NT + ci] = col[(k * NP + j) * NP + i];
                    }
            }
        }
    return T;
}

// CP2K-format cube list -> random-access table (kgmin, (jgmin,rowstart)*, igmin*).
// Returns the number of list entries consumed, or -1 if malformed / outside [lb, ub].
int convert_list(const int *sb, int64_t avail, const int lb[3], const int ub[3], std::vector<int> &out) {
    int64_t pos = 0;
    if (avail < 1) return -1;
    const int kgmin = sb[pos++];
    if (kgmin > 0 || kgmin < lb[2] || 1 - kgmin > ub[2]) return -1;
    const int nk = 1 - kgmin;
    std::vector<int> head(1 + 2 * nk), rows;
    head[0] = kgmin;
    for (int k = 0; k < nk; k++) {
        if (pos >= avail) return -1;
        const int jg = sb[pos++];
        if (jg > 0 || jg < lb[1] || 1 - jg > ub[1]) return -1;
        head[1 + 2 * k] = jg;
        head[2 + 2 * k] = (int)rows.size();
        for (int j = jg; j <= 0; j++) {
            if (pos >= avail) return -1;
            const int ig = sb[pos++];
            if (ig > 0 || ig < lb[0] || 1 - ig > ub[0]) return -1;
            rows.push_back(ig);
        }
    }
    out.insert(out.end(), head.begin(), head.end());
    out.insert(out.end(), rows.begin(), rows.end());
    return (int)pos;
}

// Host geometry of one pair (grid_base_ref_c.cc:878-900, :534-553, :636-726).
int make_geom(const gpw_task &t, int idx, const Plan &P, int func, const int *table, int64_t table_len,
              PairGeom &g, std::vector<int> &dev_table) {
    char buf[256];
    if (t.level < 0 || t.level >= P.nlevels) {
        snprintf(buf, sizeof buf, "task %d: level %d out of range", idx, t.level);
        return fail(GPW_ERR_INVALID_ARG, buf);
    }
    if (t.la_min < 0 || t.lb_min < 0 || t.la_min > t.la_max || t.lb_min > t.lb_max ||
        t.la_max > GPW_MAX_L || t.lb_max > GPW_MAX_L) {
        snprintf(buf, sizeof buf, "task %d: angular momenta out of range (0 <= l_min <= l_max <= %d)", idx,
                 GPW_MAX_L);
        return fail(GPW_ERR_INVALID_ARG, buf);
    }
    if (!(t.zeta > 0.0) || !(t.zetb > 0.0) || !std::isfinite(t.zeta) || !std::isfinite(t.zetb) ||
        !(t.radius > 0.0) || !std::isfinite(t.radius) || !std::isfinite(t.rscale) || !finite3(t.ra) ||
        !finite3(t.rab) || t.maxco < 1) {
        snprintf(buf, sizeof buf, "task %d: exponents, radius, positions must be finite (and positive)", idx);
        return fail(GPW_ERR_INVALID_ARG, buf);
    }
    const LevelDev &lv = P.lv[t.level];
    memset(&g, 0, sizeof g);
    g.task = idx;
    g.level = t.level;
    g.ortho = lv.ortho;
    g.zeta = t.zeta;
    g.zetb = t.zetb;
    g.rscale = t.rscale;
    for (int i = 0; i < 3; i++) g.rab[i] = t.rab[i];
    g.zetp = t.zeta + t.zetb;
    const double f = t.zetb / g.zetp;
    const double rab2 = t.rab[0] * t.rab[0] + t.rab[1] * t.rab[1] + t.rab[2] * t.rab[2];
    g.prefactor = t.rscale * std::exp(-t.zeta * f * rab2);
    for (int i = 0; i < 3; i++) {
        g.ra[i] = t.ra[i];
        g.rp[i] = t.ra[i] + f * t.rab[i];
        g.rb[i] = t.ra[i] + t.rab[i];
    }
    g.la0_max = t.la_max; g.la0_min = t.la_min; g.lb0_max = t.lb_max; g.lb0_min = t.lb_min;
    if (func != GPW_FUNC_AB) {  // the derivative functions need shells l - 1 .. l + 1
        g.la_max = t.la_max + 1; g.la_min = std::max(t.la_min - 1, 0);
        g.lb_max = t.lb_max + 1; g.lb_min = std::max(t.lb_min - 1, 0);
    } else {
        g.la_max = t.la_max; g.la_min = t.la_min; g.lb_max = t.lb_max; g.lb_min = t.lb_min;
    }
    g.lp = g.la_max + g.lb_max;
    g.radius = t.radius;
    g.maxco = t.maxco; g.o1 = t.o1; g.o2 = t.o2;
    g.pab_offset = t.pab_offset;
    g.table_off = -1;
    if (lv.ortho) {
        for (int i = 0; i < 3; i++) {
            double s = 0.0;
            for (int j = 0; j < 3; j++) s += lv.dh_inv[j][i] * g.rp[j];
            g.cc[i] = (int)std::floor(s);
            g.off[i] = g.rp[i] - (double)g.cc[i] * lv.dh[i][i];
        }
        if (t.sphere_offset >= 0) {
            if (!table || t.sphere_offset >= table_len) {
                snprintf(buf, sizeof buf, "task %d: sphere_offset outside the sphere table", idx);
                return fail(GPW_ERR_INVALID_ARG, buf);
            }
            for (int d = 0; d < 3; d++) { g.lb[d] = t.lb_cube[d]; g.hi[d] = t.ub_cube[d]; }
            g.table_off = (int64_t)dev_table.size();
            if (convert_list(table + t.sphere_offset, table_len - t.sphere_offset, g.lb, g.hi, dev_table) < 0) {
                snprintf(buf, sizeof buf, "task %d: malformed cube list or cube outside lb_cube/ub_cube", idx);
                return fail(GPW_ERR_INVALID_ARG, buf);
            }
            g.kgmin = table[t.sphere_offset];
        } else {
            for (int d = 0; d < 3; d++) {
                g.lb[d] = -rule_kmax(t.radius, lv.dh[d][d]);
                g.hi[d] = 1 - g.lb[d];
            }
            g.kgmin = g.lb[2];
        }
        // the reference's window assertion (grid_base_ref_c.cc:343-346)
        for (int d = 0; d < 3; d++) {
            if (lv.periodic[d]) continue;
            const int a = axis_index(0, g.cc[d], g.lb[d], g.lb[d], lv.lb_grid[d], lv.npts[d], lv.ngrid[d]);
            const int b = axis_index(0, g.cc[d], g.hi[d], g.lb[d], lv.lb_grid[d], lv.npts[d], lv.ngrid[d]);
            if (a < 0 || b < 0) {
                snprintf(buf, sizeof buf, "task %d: cube leaves the local grid on non-periodic axis %d", idx, d);
                return fail(GPW_ERR_OUT_OF_WINDOW, buf);
            }
        }
        g.cost = (int64_t)(g.hi[0] - g.lb[0] + 1) * (g.hi[1] - g.lb[1] + 1) * (g.hi[2] - g.lb[2] + 1);
    } else {
        for (int i = 0; i < 3; i++) {
            g.off[i] = 0.0;
            for (int j = 0; j < 3; j++) g.off[i] += lv.dh_inv[j][i] * g.rp[j];
        }
        int imin[3] = {INT32_MAX, INT32_MAX, INT32_MAX}, imax[3] = {INT32_MIN, INT32_MIN, INT32_MIN};
        for (int a = -1; a <= 1; a++)
            for (int b = -1; b <= 1; b++)
                for (int c = -1; c <= 1; c++) {
                    const double x = g.rp[0] + a * t.radius, y = g.rp[1] + b * t.radius, z = g.rp[2] + c * t.radius;
                    for (int d = 0; d < 3; d++) {
                        const double s = lv.dh_inv[0][d] * x + lv.dh_inv[1][d] * y + lv.dh_inv[2][d] * z;
                        imin[d] = std::min(imin[d], (int)std::floor(s));
                        imax[d] = std::max(imax[d], (int)std::ceil(s));
                    }
                }
        for (int d = 0; d < 3; d++) {
            g.cc[d] = imin[d];
            g.hi[d] = imax[d];
            g.ext0[d] = imax[d] - imin[d] + 1;
            if (!lv.periodic[d] && imax[d] - imin[d] + imod(imin[d] + lv.lb_grid[d], lv.npts[d]) >= lv.ngrid[d]) {
                snprintf(buf, sizeof buf, "task %d: box leaves the local grid on non-periodic axis %d", idx, d);
                return fail(GPW_ERR_OUT_OF_WINDOW, buf);
            }
        }
        g.cost = (int64_t)(imax[0] - imin[0] + 1) * (imax[1] - imin[1] + 1) * (imax[2] - imin[2] + 1);
    }
    return GPW_SUCCESS;
}

// New centres and exponents for the pairs of a task set, on the device: the pair
// set-up of make_geom (grid_base_ref_c.cc:878-886 and the cube / box placement)
// with round-to-nearest arithmetic in the host's operation order, so that cube
// centres and boxes land exactly where the host (and the oracle) put them.
// Writes the updated geometry to `out`; flags kStatBadGeom for non-finite or
// non-positive inputs and boxes the task set was not planned for, and
// kStatOutOfWindow for cubes that leave a non-periodic window.
__global__ void k_update_geom(const PairGeom *__restrict__ in, PairGeom *__restrict__ out, int64_t n,
                              const LevelDev *__restrict__ levels, const double *__restrict__ ra,
                              const double *__restrict__ rab, const double *__restrict__ zeta,
                              const double *__restrict__ zetb, int *status) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        PairGeom g = in[k];
        const int64_t t = g.task;
        const LevelDev &lv = levels[g.level];
        if (ra)
            for (int i = 0; i < 3; i++) g.ra[i] = ra[3 * t + i];
        if (rab)
            for (int i = 0; i < 3; i++) g.rab[i] = rab[3 * t + i];
        if (zeta) g.zeta = zeta[t];
        if (zetb) g.zetb = zetb[t];
        bool ok = g.zeta > 0.0 && g.zetb > 0.0 && isfinite(g.zeta) && isfinite(g.zetb);
        for (int i = 0; i < 3; i++) ok = ok && isfinite(g.ra[i]) && isfinite(g.rab[i]);
        if (!ok) {
            atomicOr(status, kStatBadGeom);
            out[k] = in[k];
            continue;
        }
        g.zetp = radd(g.zeta, g.zetb);
        const double f = rdiv(g.zetb, g.zetp);
        const double rab2 = radd(radd(rmul(g.rab[0], g.rab[0]), rmul(g.rab[1], g.rab[1])), rmul(g.rab[2], g.rab[2]));
        g.prefactor = rmul(g.rscale, exp(rmul(rmul(-g.zeta, f), rab2)));
        for (int i = 0; i < 3; i++) {
            g.rp[i] = radd(g.ra[i], rmul(f, g.rab[i]));
            g.rb[i] = radd(g.ra[i], g.rab[i]);
        }
        if (g.ortho) {
            for (int i = 0; i < 3; i++) {
                double sdi = 0.0;
                for (int j = 0; j < 3; j++) sdi = radd(sdi, rmul(lv.dh_inv[j][i], g.rp[j]));
                g.cc[i] = (int)floor(sdi);
                g.off[i] = rsub(g.rp[i], rmul((double)g.cc[i], lv.dh[i][i]));
            }
            for (int d = 0; d < 3; d++) {
                if (lv.periodic[d]) continue;
                const int a = axis_index(0, g.cc[d], g.lb[d], g.lb[d], lv.lb_grid[d], lv.npts[d], lv.ngrid[d]);
                const int b = axis_index(0, g.cc[d], g.hi[d], g.lb[d], lv.lb_grid[d], lv.npts[d], lv.ngrid[d]);
                if (a < 0 || b < 0) atomicOr(status, kStatOutOfWindow);
            }
        } else {
            for (int i = 0; i < 3; i++) {
                double sdi = 0.0;
                for (int j = 0; j < 3; j++) sdi = radd(sdi, rmul(lv.dh_inv[j][i], g.rp[j]));
                g.off[i] = sdi;
            }
            int imin[3] = {INT32_MAX, INT32_MAX, INT32_MAX}, imax[3] = {INT32_MIN, INT32_MIN, INT32_MIN};
            for (int a = -1; a <= 1; a++)
                for (int b = -1; b <= 1; b++)
                    for (int c = -1; c <= 1; c++) {
                        const double x = radd(g.rp[0], rmul((double)a, g.radius));
                        const double y = radd(g.rp[1], rmul((double)b, g.radius));
                        const double z = radd(g.rp[2], rmul((double)c, g.radius));
                        for (int d = 0; d < 3; d++) {
                            const double sd = radd(radd(rmul(lv.dh_inv[0][d], x), rmul(lv.dh_inv[1][d], y)),
                                                   rmul(lv.dh_inv[2][d], z));
                            imin[d] = min(imin[d], (int)floor(sd));
                            imax[d] = max(imax[d], (int)ceil(sd));
                        }
                    }
            for (int d = 0; d < 3; d++) {
                g.cc[d] = imin[d];
                g.hi[d] = imax[d];
                if (imax[d] - imin[d] + 1 > g.ext0[d] + 1) atomicOr(status, kStatBadGeom);
                if (!lv.periodic[d] && imax[d] - imin[d] + imod(imin[d] + lv.lb_grid[d], lv.npts[d]) >= lv.ngrid[d])
                    atomicOr(status, kStatOutOfWindow);
            }
        }
        out[k] = g;
    }
}

GridPtrs grid_ptrs(const Plan &P, double *const *p) {
    GridPtrs g;
    memset(&g, 0, sizeof g);
    for (int l = 0; l < P.nlevels; l++) g.p[l] = p[l];
    return g;
}

struct HostStage {
    double *d_pab = nullptr;
    double *d_grids[GPW_MAX_LEVELS] = {nullptr};
    int64_t pab_len = 0;
};
std::mutex g_stage_mu;
std::map<const gpw_taskset *, HostStage> g_stage;

}  // namespace

namespace gpw {
// One orthorhombic or general level as the kernels see it (host copy).
int level_from_desc(const gpw_grid_desc &d, LevelDev &v) {
    memset(&v, 0, sizeof v);
    for (int i = 0; i < 3; i++) {
        v.npts[i] = d.npts[i];
        v.ngrid[i] = d.ngrid[i];
        v.lb_grid[i] = d.lb_grid[i];
        v.periodic[i] = d.periodic[i] ? 1 : 0;
        if (d.npts[i] < 1 || d.ngrid[i] < 1 || (v.periodic[i] && d.ngrid[i] != d.npts[i]))
            return fail(GPW_ERR_INVALID_ARG, "grid: npts, ngrid >= 1 and ngrid == npts on periodic axes");
        for (int j = 0; j < 3; j++) {
            v.dh[i][j] = d.dh[i][j];
            v.dh_inv[i][j] = d.dh_inv[i][j];
        }
    }
    v.ortho = d.ortho ? 1 : 0;
    v.grid_elems = (int64_t)d.ngrid[0] * d.ngrid[1] * d.ngrid[2];
    v.tmat_off = -1;
    return GPW_SUCCESS;
}

// Host geometry of one pair on a single level (the task's level must be 0).
int host_pair_geom(const gpw_task &t, int idx, const LevelDev &lv, int func, PairGeom &g) {
    Plan P;
    P.nlevels = 1;
    P.lv[0] = lv;
    std::vector<int> no_table;
    return make_geom(t, idx, P, func, nullptr, 0, g, no_table);
}

void set_last_error(const std::string &msg) { fail(0, msg); }
}  // namespace gpw

struct gpw_plan : Plan {};
struct gpw_taskset : TaskSet {};

extern "C" {

const char *gpw_last_error_string(void) { return g_err.c_str(); }

const char *gpw_version(void) { return "libgpw_gb300 0.1 (sm_103a)"; }

int gpw_sphere_bounds(double radius, const double dh[3][3], int lb_cube[3], int ub_cube[3],
                      int *sphere_bounds, int cap) {
    if (!dh || !lb_cube || !ub_cube || !(radius > 0.0) || !std::isfinite(radius) ||
        !(dh[0][0] > 0.0) || !(dh[1][1] > 0.0) || !(dh[2][2] > 0.0)) {
        fail(GPW_ERR_INVALID_ARG, "gpw_sphere_bounds: radius and diagonal steps must be positive");
        return 0;
    }
    const double r2 = rmul(radius, radius);
    const int kmax = rule_kmax(radius, dh[2][2]);
    int n = 0;
    auto push = [&](int v) {
        if (n < cap && sphere_bounds) sphere_bounds[n] = v;
        n++;
    };
    push(-kmax);
    for (int kg = -kmax; kg <= 0; kg++) {
        const double remk = rule_remk(r2, kg, dh[2][2]);
        const int jmax = rule_jmax(remk, dh[1][1]);
        push(-jmax);
        for (int jg = -jmax; jg <= 0; jg++) push(-rule_imax(remk, jg, dh[1][1], dh[0][0]));
    }
    for (int d = 0; d < 3; d++) {
        lb_cube[d] = -rule_kmax(radius, dh[d][d]);
        ub_cube[d] = 1 - lb_cube[d];
    }
    return n <= cap ? n : -n;
}

int gpw_plan_create(gpw_plan **plan, int nlevels, const gpw_grid_desc *levels, int device) {
    if (!plan || !levels || nlevels < 1 || nlevels > GPW_MAX_LEVELS)
        return fail(GPW_ERR_INVALID_ARG, "gpw_plan_create: 1..GPW_MAX_LEVELS levels required");
    *plan = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return fail(GPW_ERR_NO_DEVICE, "gpw_plan_create: no CUDA device");
    if (device < 0 || device >= ndev) return fail(GPW_ERR_INVALID_ARG, "gpw_plan_create: bad device");
    gpw_plan *P = new gpw_plan();
    P->device = device;
    P->nlevels = nlevels;
    std::vector<double> tm;
    for (int l = 0; l < nlevels; l++) {
        const gpw_grid_desc &d = levels[l];
        LevelDev &v = P->lv[l];
        memset(&v, 0, sizeof v);
        for (int i = 0; i < 3; i++) {
            v.npts[i] = d.npts[i];
            v.ngrid[i] = d.ngrid[i];
            v.lb_grid[i] = d.lb_grid[i];
            v.periodic[i] = d.periodic[i] ? 1 : 0;
            if (d.npts[i] < 1 || d.ngrid[i] < 1 || (v.periodic[i] && d.ngrid[i] != d.npts[i])) {
                delete P;
                return fail(GPW_ERR_INVALID_ARG,
                            "gpw_plan_create: npts, ngrid >= 1 and ngrid == npts on periodic axes");
            }
            for (int j = 0; j < 3; j++) {
                v.dh[i][j] = d.dh[i][j];
                v.dh_inv[i][j] = d.dh_inv[i][j];
            }
        }
        v.ortho = d.ortho ? 1 : 0;
        if (v.ortho && (d.dh[0][1] != 0.0 || d.dh[0][2] != 0.0 || d.dh[1][0] != 0.0 || d.dh[1][2] != 0.0 ||
                        d.dh[2][0] != 0.0 || d.dh[2][1] != 0.0 || !(d.dh[0][0] > 0) || !(d.dh[1][1] > 0) ||
                        !(d.dh[2][2] > 0))) {
            delete P;
            return fail(GPW_ERR_INVALID_ARG, "gpw_plan_create: orthorhombic level needs a positive diagonal dh");
        }
        v.grid_elems = (int64_t)d.ngrid[0] * d.ngrid[1] * d.ngrid[2];
        v.tmat_off = -1;
        if (!v.ortho) {
            v.tmat_off = (int64_t)tm.size();
            std::vector<double> T = lattice_transform(v.dh);
            tm.insert(tm.end(), T.begin(), T.end());
        }
    }
    int prev = 0;
    cudaGetDevice(&prev);
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaMalloc(&P->d_levels, sizeof(LevelDev) * nlevels);
    if (e == cudaSuccess) e = cudaMemcpy(P->d_levels, P->lv, sizeof(LevelDev) * nlevels, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !tm.empty()) {
        e = cudaMalloc(&P->d_tmat, sizeof(double) * tm.size());
        if (e == cudaSuccess) e = cudaMemcpy(P->d_tmat, tm.data(), sizeof(double) * tm.size(), cudaMemcpyHostToDevice);
    }
    if (e != cudaSuccess) {
        cudaFree(P->d_levels);
        cudaFree(P->d_tmat);
        delete P;
        return cuda_fail(e, "gpw_plan_create");
    }
    P->h_tmat.swap(tm);
    int smem_max = 0;
    cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    e = fp64_kernel_attributes(smem_max);
    if (e != cudaSuccess) {
        gpw_plan_destroy(P);
        return cuda_fail(e, "gpw_plan_create (kernel attributes)");
    }
    *plan = P;
    return GPW_SUCCESS;
}

int gpw_plan_destroy(gpw_plan *plan) {
    if (!plan) return GPW_SUCCESS;
    cudaFree(plan->d_levels);
    cudaFree(plan->d_tmat);
    delete plan;
    return GPW_SUCCESS;
}

int gpw_taskset_create(gpw_plan *plan, const gpw_task *tasks, int64_t ntasks, int func,
                       const int *sphere_table, int64_t sphere_table_len, gpw_taskset **out) {
    if (!plan || !out || (ntasks > 0 && !tasks) || ntasks < 0 || ntasks > INT32_MAX)
        return fail(GPW_ERR_INVALID_ARG, "gpw_taskset_create: bad arguments");
    if (func < GPW_FUNC_AB || func > GPW_FUNC_ADBMDAB_Z)
        return fail(GPW_ERR_INVALID_ARG, "gpw_taskset_create: func must be a gpw_function (0..4)");
    *out = nullptr;
    std::vector<PairGeom> geo((size_t)ntasks);
    std::vector<int> table;
    int64_t extent = 0;
    for (int64_t i = 0; i < ntasks; i++) {
        int st = make_geom(tasks[i], (int)i, *plan, func, sphere_table, sphere_table_len,
                           geo[i], table);
        if (st) return st;
        const gpw_task &t = tasks[i];
        const int64_t lo = t.pab_offset + (int64_t)(t.o2 + ncoset(t.lb_min - 1)) * t.maxco + t.o1 + ncoset(t.la_min - 1);
        const int64_t hi = t.pab_offset + (int64_t)(t.o2 + ncoset(t.lb_max) - 1) * t.maxco + t.o1 + ncoset(t.la_max) - 1;
        if (lo < 0 || (t.o1 + ncoset(t.la_min - 1)) < 0 || (t.o2 + ncoset(t.lb_min - 1)) < 0) {
            char buf[128];
            snprintf(buf, sizeof buf, "task %lld: density block starts before the buffer", (long long)i);
            return fail(GPW_ERR_INVALID_ARG, buf);
        }
        extent = std::max(extent, hi + 1);
    }
    // sort: kind (ortho first), then the largest cubes first
    std::vector<int> order((size_t)ntasks);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        if (geo[a].ortho != geo[b].ortho) return geo[a].ortho > geo[b].ortho;
        return geo[a].cost > geo[b].cost;
    });
    gpw_taskset *T = new gpw_taskset();
    T->plan = plan;
    for (int l = 0; l < GPW_MAX_LEVELS; l++)  // general-cell levels start on the float-float kernel
        T->tile_lz[l] = (l < plan->nlevels && !plan->lv[l].ortho) ? kUntiled : kDefaultTileLz;
    T->tau = func;
    T->ntasks = ntasks;
    T->pab_extent = extent;
    T->h_geom.resize((size_t)ntasks);
    int64_t coef = 0;
    int64_t mom_ext = 0;
    for (int64_t k = 0; k < ntasks; k++) {
        PairGeom g = geo[order[k]];
        g.coef_off = coef;
        coef += ncoef(g.lp);
        g.mom_ext_off = mom_ext;
        mom_ext += ncoef(g.lp + 2);
        T->max_lp = std::max(T->max_lp, g.lp);
        T->max_A = std::max(T->max_A, g.la_max);
        T->max_B = std::max(T->max_B, g.lb_max);
        T->h_geom[k] = g;
    }
    T->coef_len = coef;
    T->mom_ext_len = mom_ext;
    // FP64 launch chunks: similar shared-memory needs launch together
    int64_t k = 0;
    int smem_limit = 0;
    cudaDeviceGetAttribute(&smem_limit, cudaDevAttrMaxSharedMemoryPerBlockOptin, plan->device);
    while (k < ntasks) {
        Chunk c;
        c.first = (int)k;
        c.kind = T->h_geom[k].ortho ? 0 : 1;
        c.smem_bytes = 0;
        c.smem_ext = 0;
        int64_t m = k;
        while (m < ntasks && (T->h_geom[m].ortho ? 0 : 1) == c.kind) {
            const int need = c.kind == 0 ? smem_ortho_fp64(T->h_geom[m]) : smem_general_fp64(T->h_geom[m]);
            const int need_ext = c.kind == 0 ? smem_ortho_fp64(T->h_geom[m], 2) : smem_general_fp64(T->h_geom[m], 2);
            c.smem_ext = std::max(c.smem_ext, std::min(need_ext, smem_limit));
            if (need > smem_limit) {
                delete T;
                return fail(GPW_ERR_UNSUPPORTED, "gpw_taskset_create: a cube is too large for one CTA");
            }
            if (m > k && need * 2 < c.smem_bytes && m - k >= 64) break;
            c.smem_bytes = std::max(c.smem_bytes, need);
            m++;
        }
        c.count = (int)(m - k);
        T->chunks.push_back(c);
        k = m;
    }
    // general-cell pairs (sorted after the orthorhombic ones) for the float-float kernel
    for (int64_t m = 0; m < ntasks; m++) {
        if (T->h_geom[m].ortho) continue;
        if (T->gen_count == 0) T->gen_first = (int)m;
        T->gen_count++;
        T->gen_smem = std::max(T->gen_smem, smem_general_ff(T->h_geom[m]));
    }
    if (T->gen_smem > smem_limit) {
        delete T;
        return fail(GPW_ERR_UNSUPPORTED, "gpw_taskset_create: a general-cell cube is too large for one CTA");
    }
    if (smem_prep(T->max_A, T->max_B) > smem_limit) {
        delete T;
        return fail(GPW_ERR_UNSUPPORTED, "gpw_taskset_create: angular momenta too high for the set-up kernel");
    }
    cudaError_t e = cudaSetDevice(plan->device);
    auto alloc = [&](void **p, size_t bytes) {
        if (e == cudaSuccess) e = cudaMalloc(p, bytes > 0 ? bytes : 8);
    };
    alloc((void **)&T->d_geom, sizeof(PairGeom) * (size_t)ntasks);
    alloc((void **)&T->d_table, sizeof(int) * table.size());
    alloc((void **)&T->d_coef, sizeof(double) * (size_t)coef);
    alloc((void **)&T->d_mom, sizeof(double) * (size_t)coef);
    alloc((void **)&T->d_status, sizeof(int));
    if (e == cudaSuccess && ntasks > 0)
        e = cudaMemcpy(T->d_geom, T->h_geom.data(), sizeof(PairGeom) * (size_t)ntasks, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !table.empty())
        e = cudaMemcpy(T->d_table, table.data(), sizeof(int) * table.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(T->d_status, 0, sizeof(int));
    if (e != cudaSuccess) {
        gpw_taskset_destroy(T);
        return cuda_fail(e, "gpw_taskset_create");
    }
    std::string err;
    int st = mixed_build(*T, err);
    if (st) {
        gpw_taskset_destroy(T);
        return fail(st, err);
    }
    *out = T;
    return GPW_SUCCESS;
}

int gpw_taskset_destroy(gpw_taskset *ts) {
    if (!ts) return GPW_SUCCESS;
    {
        std::lock_guard<std::mutex> lk(g_stage_mu);
        auto it = g_stage.find(ts);
        if (it != g_stage.end()) {
            cudaFree(it->second.d_pab);
            for (int l = 0; l < GPW_MAX_LEVELS; l++) cudaFree(it->second.d_grids[l]);
            g_stage.erase(it);
        }
    }
    mixed_free(*ts);
    for (cudaEvent_t e : ts->ev_pool) cudaEventDestroy(e);
    cudaFree(ts->d_geom);
    cudaFree(ts->d_geom_next);
    cudaFree(ts->d_table);
    cudaFree(ts->d_coef);
    cudaFree(ts->d_mom);
    cudaFree(ts->d_mom_ext);
    cudaFree(ts->d_status);
    delete ts;
    return GPW_SUCCESS;
}

int64_t gpw_taskset_pab_extent(const gpw_taskset *ts) { return ts ? ts->pab_extent : -1; }

int gpw_collocate(gpw_taskset *ts, int precision, const double *d_pab, double *const *d_grids, void *stream) {
    if (!ts || !d_grids || (ts->ntasks > 0 && !d_pab)) return fail(GPW_ERR_INVALID_ARG, "gpw_collocate: null argument");
    for (int l = 0; l < ts->plan->nlevels; l++)
        if (!d_grids[l]) return fail(GPW_ERR_INVALID_ARG, "gpw_collocate: null grid");
    cudaStream_t s = (cudaStream_t)stream;
    GridPtrs g = grid_ptrs(*ts->plan, d_grids);
    GPW_CUDA(launch_prep(*ts, d_pab, s));
    if (precision == GPW_PREC_FP64) {
        GPW_CUDA(launch_collocate_fp64(*ts, g, s));
    } else if (precision == GPW_PREC_MIXED) {
        cudaError_t e = launch_collocate_mixed(*ts, g, s);
        if (e == cudaErrorNotSupported) return fail(GPW_ERR_UNSUPPORTED, "gpw_collocate: mixed path not built");
        if (e != cudaSuccess) return cuda_fail(e, "gpw_collocate (mixed)");
    } else {
        return fail(GPW_ERR_INVALID_ARG, "gpw_collocate: unknown precision");
    }
    return GPW_SUCCESS;
}

int gpw_integrate(gpw_taskset *ts, int precision, double *const *d_grids, double *d_hab, void *stream) {
    if (!ts || !d_grids || (ts->ntasks > 0 && !d_hab)) return fail(GPW_ERR_INVALID_ARG, "gpw_integrate: null argument");
    for (int l = 0; l < ts->plan->nlevels; l++)
        if (!d_grids[l]) return fail(GPW_ERR_INVALID_ARG, "gpw_integrate: null grid");
    cudaStream_t s = (cudaStream_t)stream;
    GridPtrs g = grid_ptrs(*ts->plan, d_grids);
    if (precision == GPW_PREC_FP64) {
        GPW_CUDA(launch_integrate_fp64(*ts, g, s));
    } else if (precision == GPW_PREC_MIXED) {
        cudaError_t e = launch_integrate_mixed(*ts, g, s);
        if (e == cudaErrorNotSupported) return fail(GPW_ERR_UNSUPPORTED, "gpw_integrate: mixed path not built");
        if (e != cudaSuccess) return cuda_fail(e, "gpw_integrate (mixed)");
    } else {
        return fail(GPW_ERR_INVALID_ARG, "gpw_integrate: unknown precision");
    }
    GPW_CUDA(launch_backtransform(*ts, ts->d_mom, d_hab, s));
    return GPW_SUCCESS;
}

int gpw_backward(gpw_taskset *ts, const double *d_pab, double *const *d_grids, double *d_hab, double *d_dra,
                 double *d_drb, double *d_dzeta, double *d_dzetb, void *stream) {
    if (!ts || !d_grids || (ts->ntasks > 0 && !d_pab)) return fail(GPW_ERR_INVALID_ARG, "gpw_backward: null argument");
    cudaStream_t s = (cudaStream_t)stream;
    GridPtrs g = grid_ptrs(*ts->plan, d_grids);
    if (d_hab) {
        int st = gpw_integrate(ts, GPW_PREC_FP64, d_grids, d_hab, stream);
        if (st) return st;
    }
    if (d_dra || d_drb || d_dzeta || d_dzetb) {
        cudaError_t e = launch_backward(*ts, d_pab, g, d_hab, d_dra, d_drb, d_dzeta, d_dzetb, s);
        if (e == cudaErrorNotSupported) return fail(GPW_ERR_UNSUPPORTED, "gpw_backward: not available");
        if (e != cudaSuccess) return cuda_fail(e, "gpw_backward");
    }
    return GPW_SUCCESS;
}

int gpw_taskset_check(gpw_taskset *ts, void *stream) {
    if (!ts) return fail(GPW_ERR_INVALID_ARG, "gpw_taskset_check: null");
    int h = 0;
    GPW_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
    GPW_CUDA(cudaMemcpy(&h, ts->d_status, sizeof(int), cudaMemcpyDeviceToHost));
    GPW_CUDA(cudaMemset(ts->d_status, 0, sizeof(int)));
    if (h & kStatOutOfWindow) return fail(GPW_ERR_OUT_OF_WINDOW, "a cube left the local grid window");
    if (h & kStatTimeout) return fail(GPW_ERR_TIMEOUT, "a bounded device wait gave up");
    if (h & kStatBadTable) return fail(GPW_ERR_INVALID_ARG, "a cube list was inconsistent on the device");
    if (h & kStatBadTile) return fail(GPW_ERR_INVALID_ARG, "a tile shape the collocate kernel does not hold");
    if (h & kStatTooManyImages)
        return fail(GPW_ERR_UNSUPPORTED, "a cube spans more periodic images than the tiled path handles");
    return GPW_SUCCESS;
}

int gpw_taskset_update_geometry(gpw_taskset *ts, const double *d_ra, const double *d_rab, const double *d_zeta,
                                const double *d_zetb, void *stream) {
    if (!ts) return fail(GPW_ERR_INVALID_ARG, "gpw_taskset_update_geometry: null task set");
    if (ts->ntasks == 0) return GPW_SUCCESS;
    GPW_CUDA(cudaSetDevice(ts->plan->device));
    GPW_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
    GPW_CUDA(cudaDeviceSynchronize());  // no launch of this task set may still read its geometry
    if (!ts->d_geom_next) GPW_CUDA(cudaMalloc(&ts->d_geom_next, sizeof(PairGeom) * (size_t)ts->ntasks));
    GPW_CUDA(cudaMemset(ts->d_status, 0, sizeof(int)));
    const unsigned nblk = (unsigned)std::max<int64_t>(1, std::min<int64_t>((ts->ntasks + 127) / 128, 8192));
    k_update_geom<<<nblk, 128>>>(ts->d_geom, ts->d_geom_next, ts->ntasks, ts->plan->d_levels, d_ra, d_rab, d_zeta,
                                 d_zetb, ts->d_status);
    GPW_CUDA(cudaGetLastError());
    int h = 0;
    GPW_CUDA(cudaMemcpy(&h, ts->d_status, sizeof(int), cudaMemcpyDeviceToHost));
    GPW_CUDA(cudaMemset(ts->d_status, 0, sizeof(int)));
    if (h & kStatBadGeom)
        return fail(GPW_ERR_INVALID_ARG,
                    "gpw_taskset_update_geometry: exponents must be positive and finite, positions finite; "
                    "the task set is unchanged");
    if (h & kStatOutOfWindow)
        return fail(GPW_ERR_OUT_OF_WINDOW,
                    "gpw_taskset_update_geometry: a cube would leave the local grid; the task set is unchanged");
    std::swap(ts->d_geom, ts->d_geom_next);
    ts->h_geom_stale = true;
    if (ts->mixed) {
        std::string err;
        const int st = mixed_rebin(*ts, err);
        if (st) {
            mixed_free(*ts);  // mixed calls then report GPW_ERR_UNSUPPORTED
            return fail(st, err);
        }
    }
    return GPW_SUCCESS;
}

// tz 4 / 8: tiles of that z extent; 0 (general-cell levels only): no tiles, the float-float kernel
static int tile_lz_of(int tz, bool ortho) { return tz == 4 ? 2 : tz == 8 ? 3 : (tz == 0 && !ortho) ? kUntiled : -2; }
static int tile_z_of(int lz) { return lz == kUntiled ? 0 : 1 << lz; }

static int retile(gpw_taskset *ts, const int *lz) {
    bool same = true;
    for (int l = 0; l < ts->plan->nlevels; l++) same = same && ts->tile_lz[l] == lz[l];
    if (same && ts->mixed) return GPW_SUCCESS;
    GPW_CUDA(cudaSetDevice(ts->plan->device));
    GPW_CUDA(cudaDeviceSynchronize());  // the binned state may be in use by earlier launches
    if (ts->h_geom_stale && ts->ntasks > 0) {  // the host copy after a device geometry update
        GPW_CUDA(cudaMemcpy(ts->h_geom.data(), ts->d_geom, sizeof(PairGeom) * (size_t)ts->ntasks,
                            cudaMemcpyDeviceToHost));
        ts->h_geom_stale = false;
    }
    mixed_free(*ts);
    for (int l = 0; l < ts->plan->nlevels; l++) ts->tile_lz[l] = lz[l];
    std::string err;
    const int st = mixed_build(*ts, err);
    if (st) mixed_free(*ts);  // mixed calls then report GPW_ERR_UNSUPPORTED
    return st ? fail(st, err) : GPW_SUCCESS;
}

int gpw_taskset_set_tiles(gpw_taskset *ts, const int *tile_z) {
    if (!ts || !tile_z) return fail(GPW_ERR_INVALID_ARG, "gpw_taskset_set_tiles: null");
    int lz[GPW_MAX_LEVELS];
    for (int l = 0; l < ts->plan->nlevels; l++) {
        lz[l] = tile_lz_of(tile_z[l], ts->plan->lv[l].ortho != 0);
        if (lz[l] == -2)
            return fail(GPW_ERR_INVALID_ARG,
                        "gpw_taskset_set_tiles: tile z extent must be 4 or 8 (or 0 on a general-cell level)");
    }
    return retile(ts, lz);
}

int gpw_taskset_get_tiles(const gpw_taskset *ts, int *tile_z) {
    if (!ts || !tile_z) return fail(GPW_ERR_INVALID_ARG, "gpw_taskset_get_tiles: null");
    for (int l = 0; l < ts->plan->nlevels; l++) tile_z[l] = tile_z_of(ts->tile_lz[l]);
    return GPW_SUCCESS;
}

int gpw_taskset_autotune(gpw_taskset *ts, const double *d_pab, int *tile_z, double *ms, void *stream) {
    if (!ts || (ts->ntasks > 0 && !d_pab)) return fail(GPW_ERR_INVALID_ARG, "gpw_taskset_autotune: null");
    const Plan &P = *ts->plan;
    GPW_CUDA(cudaSetDevice(P.device));
    cudaStream_t s = (cudaStream_t)stream;
    // scratch grids (collocate output, then the integrate input) and matrix elements
    double *grids[GPW_MAX_LEVELS] = {nullptr};
    double *hab = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t ce = cudaMalloc(&hab, sizeof(double) * (size_t)std::max<int64_t>(ts->pab_extent, 1));
    for (int l = 0; l < P.nlevels && ce == cudaSuccess; l++) {
        ce = cudaMalloc(&grids[l], sizeof(double) * P.lv[l].grid_elems);
        if (ce == cudaSuccess) ce = cudaMemsetAsync(grids[l], 0, sizeof(double) * P.lv[l].grid_elems, s);
    }
    if (ce == cudaSuccess) ce = cudaEventCreate(&e0);
    if (ce == cudaSuccess) ce = cudaEventCreate(&e1);
    int st = ce == cudaSuccess ? GPW_SUCCESS : cuda_fail(ce, "gpw_taskset_autotune");
    static const int cand[3] = {3, 2, kUntiled};  // TZ = 8, 4; general-cell levels also untiled
    int best[GPW_MAX_LEVELS];
    for (int l = 0; l < P.nlevels; l++) best[l] = ts->tile_lz[l];
    auto time_once = [&](float &out) -> int {
        // one warm-up and one timed collocate + integrate
        for (int rep = 0; rep < 2; rep++) {
            if (rep == 1 && (ce = cudaEventRecord(e0, s)) != cudaSuccess) return cuda_fail(ce, "autotune");
            int r = gpw_collocate(ts, GPW_PREC_MIXED, d_pab, grids, stream);
            if (!r) r = gpw_integrate(ts, GPW_PREC_MIXED, grids, hab, stream);
            if (r) return r;
        }
        if ((ce = cudaEventRecord(e1, s)) != cudaSuccess || (ce = cudaEventSynchronize(e1)) != cudaSuccess ||
            (ce = cudaEventElapsedTime(&out, e0, e1)) != cudaSuccess)
            return cuda_fail(ce, "autotune");
        return GPW_SUCCESS;
    };
    for (int l = 0; l < P.nlevels && !st; l++) {
        bool used = false;  // levels without tasks keep their shape
        for (int64_t k = 0; k < ts->ntasks && !used; k++) used = ts->h_geom[k].level == l;
        const int ncand = P.lv[l].ortho ? 2 : 3;
        float best_ms = -1.0f;
        for (int c = 0; c < 3 && !st; c++) {
            float t = 0.0f;
            if (used && c < ncand) {
                int lz[GPW_MAX_LEVELS];
                for (int j = 0; j < P.nlevels; j++) lz[j] = best[j];
                lz[l] = cand[c];
                st = retile(ts, lz);
                if (!st) st = time_once(t);
                if (!st && (best_ms < 0.0f || t < best_ms)) best_ms = t, best[l] = cand[c];
            }
            if (ms) ms[3 * l + c] = (used && c < ncand) ? (double)t : -1.0;
        }
    }
    if (!st) st = retile(ts, best);
    if (!st) st = gpw_taskset_check(ts, stream);
    if (tile_z)
        for (int l = 0; l < P.nlevels; l++) tile_z[l] = tile_z_of(ts->tile_lz[l]);
    for (int l = 0; l < P.nlevels; l++) cudaFree(grids[l]);
    cudaFree(hab);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    return st;
}

int gpw_taskset_profile(gpw_taskset *ts, int enable) {
    if (!ts) return fail(GPW_ERR_INVALID_ARG, "gpw_taskset_profile: null");
    ts->profile = enable != 0;
    return GPW_SUCCESS;
}

int gpw_taskset_bins(const gpw_taskset *ts, int64_t *items, int64_t *units) {
    if (!ts) return fail(GPW_ERR_INVALID_ARG, "gpw_taskset_bins: null");
    if (items) *items = mixed_items(*ts);
    if (units) *units = mixed_units(*ts);
    return GPW_SUCCESS;
}

int gpw_taskset_stats(gpw_taskset *ts, double *contraction_ms, int64_t *contraction_launches,
                      int64_t *kernel_launches) {
    if (!ts) return fail(GPW_ERR_INVALID_ARG, "gpw_taskset_stats: null");
    double ms = 0.0;
    if (ts->ev_used > 0) {
        GPW_CUDA(cudaEventSynchronize(ts->ev_pool[ts->ev_used - 1]));
        for (size_t i = 0; i + 1 < ts->ev_used; i += 2) {
            float m = 0.f;
            GPW_CUDA(cudaEventElapsedTime(&m, ts->ev_pool[i], ts->ev_pool[i + 1]));
            ms += m;
        }
    }
    if (contraction_ms) *contraction_ms = ms;
    if (contraction_launches) *contraction_launches = ts->n_contract;
    if (kernel_launches) *kernel_launches = ts->n_kernels;
    ts->ev_used = 0;
    ts->n_contract = 0;
    ts->n_kernels = 0;
    return GPW_SUCCESS;
}

static int stage(gpw_taskset *ts, HostStage **out) {
    std::lock_guard<std::mutex> lk(g_stage_mu);
    HostStage &h = g_stage[ts];
    cudaError_t e = cudaSuccess;
    if (!h.d_pab) {
        e = cudaMalloc(&h.d_pab, sizeof(double) * std::max<int64_t>(ts->pab_extent, 1));
        for (int l = 0; l < ts->plan->nlevels && e == cudaSuccess; l++)
            e = cudaMalloc(&h.d_grids[l], sizeof(double) * ts->plan->lv[l].grid_elems);
        if (e != cudaSuccess) {  // all or nothing: the next call allocates again
            cudaFree(h.d_pab);
            for (int l = 0; l < GPW_MAX_LEVELS; l++) cudaFree(h.d_grids[l]);
            h = HostStage();
            return cuda_fail(e, "host staging");
        }
    }
    *out = &h;
    return GPW_SUCCESS;
}

int gpw_collocate_host(gpw_taskset *ts, int precision, const double *h_pab, double *const *h_grids) {
    if (!ts || !h_grids || (ts->ntasks > 0 && !h_pab)) return fail(GPW_ERR_INVALID_ARG, "gpw_collocate_host: null");
    GPW_CUDA(cudaSetDevice(ts->plan->device));
    HostStage *h;
    int st = stage(ts, &h);
    if (st) return st;
    GPW_CUDA(cudaMemcpy(h->d_pab, h_pab, sizeof(double) * ts->pab_extent, cudaMemcpyHostToDevice));
    for (int l = 0; l < ts->plan->nlevels; l++)
        GPW_CUDA(cudaMemcpy(h->d_grids[l], h_grids[l], sizeof(double) * ts->plan->lv[l].grid_elems,
                            cudaMemcpyHostToDevice));
    st = gpw_collocate(ts, precision, h->d_pab, h->d_grids, nullptr);
    if (st) return st;
    for (int l = 0; l < ts->plan->nlevels; l++)
        GPW_CUDA(cudaMemcpy(h_grids[l], h->d_grids[l], sizeof(double) * ts->plan->lv[l].grid_elems,
                            cudaMemcpyDeviceToHost));
    return gpw_taskset_check(ts, nullptr);
}

int gpw_integrate_host(gpw_taskset *ts, int precision, double *const *h_grids, double *h_hab) {
    if (!ts || !h_grids || (ts->ntasks > 0 && !h_hab)) return fail(GPW_ERR_INVALID_ARG, "gpw_integrate_host: null");
    GPW_CUDA(cudaSetDevice(ts->plan->device));
    HostStage *h;
    int st = stage(ts, &h);
    if (st) return st;
    for (int l = 0; l < ts->plan->nlevels; l++)
        GPW_CUDA(cudaMemcpy(h->d_grids[l], h_grids[l], sizeof(double) * ts->plan->lv[l].grid_elems,
                            cudaMemcpyHostToDevice));
    GPW_CUDA(cudaMemcpy(h->d_pab, h_hab, sizeof(double) * ts->pab_extent, cudaMemcpyHostToDevice));
    st = gpw_integrate(ts, precision, h->d_grids, h->d_pab, nullptr);
    if (st) return st;
    GPW_CUDA(cudaMemcpy(h_hab, h->d_pab, sizeof(double) * ts->pab_extent, cudaMemcpyDeviceToHost));
    return gpw_taskset_check(ts, nullptr);
}

int gpw_collocate_pgf_product_rspace(int compute_tau, int use_ortho, int la_max, int la_min, int lb_max,
                                     int lb_min, double zeta, double zetb, double rscale, const double dh[3][3],
                                     const double dh_inv[3][3], const double ra[3], const double rab[3],
                                     const int npts[3], const int ngrid[3], const int lb_grid[3],
                                     const int periodic[3], int lmax, double radius, const int lb_cube[3],
                                     const int ub_cube[3], int nspheres, const int *sphere_bounds, int maxco,
                                     int o1, int o2, const double *pab, double *grid) {
    (void)lmax;
    if (!dh || !dh_inv || !ra || !rab || !npts || !ngrid || !lb_grid || !periodic || !pab || !grid)
        return fail(GPW_ERR_INVALID_ARG, "gpw_collocate_pgf_product_rspace: null argument");
    if (use_ortho && (!lb_cube || !ub_cube || !sphere_bounds || nspheres < 1))
        return fail(GPW_ERR_INVALID_ARG, "gpw_collocate_pgf_product_rspace: ortho needs the cube and its list");
    int dev = 0;
    cudaGetDevice(&dev);
    gpw_grid_desc gd;
    memset(&gd, 0, sizeof gd);
    for (int i = 0; i < 3; i++) {
        gd.npts[i] = npts[i];
        gd.ngrid[i] = ngrid[i];
        gd.lb_grid[i] = lb_grid[i];
        gd.periodic[i] = periodic[i];
        for (int j = 0; j < 3; j++) {
            gd.dh[i][j] = dh[i][j];
            gd.dh_inv[i][j] = dh_inv[i][j];
        }
    }
    gd.ortho = use_ortho ? 1 : 0;
    // The reference's callers make this call once per pair, many times over the
    // same grid: the plan (one per grid geometry), a device buffer and a pinned
    // host mirror of it stay in a per-thread cache, so a call is the host set-up,
    // one copy in (geometry, cube list, block, grid), two launches and one copy
    // out (status word and grid).
    struct Cache {
        int device = -1;
        gpw_grid_desc desc;
        gpw_plan *plan = nullptr;
        double *d_coef = nullptr;
        unsigned char *d_buf = nullptr, *h_buf = nullptr;
        size_t cap = 0;
        std::vector<int> table;
        ~Cache() { release(); }
        void release() {
            if (plan) gpw_plan_destroy(plan);
            cudaFree(d_coef);
            cudaFree(d_buf);
            if (h_buf) cudaFreeHost(h_buf);
            plan = nullptr;
            d_coef = nullptr;
            d_buf = h_buf = nullptr;
            cap = 0;
        }
    };
    thread_local Cache C;
    if (!C.plan || C.device != dev || memcmp(&C.desc, &gd, sizeof gd) != 0) {
        C.release();
        int st = gpw_plan_create(&C.plan, 1, &gd, dev);
        if (st) return st;
        const cudaError_t e = cudaMalloc(&C.d_coef, sizeof(double) * ncoef(kMaxLp));
        if (e != cudaSuccess) {
            C.release();  // no half-built cache for the next call to reuse
            return cuda_fail(e, "gpw_collocate_pgf_product_rspace: coefficient buffer");
        }
        C.device = dev;
        C.desc = gd;
    }
    gpw_task t;
    memset(&t, 0, sizeof t);
    t.zeta = zeta; t.zetb = zetb; t.rscale = rscale;
    for (int i = 0; i < 3; i++) { t.ra[i] = ra[i]; t.rab[i] = rab[i]; }
    t.radius = radius;
    t.pab_offset = 0;
    t.la_max = la_max; t.la_min = la_min; t.lb_max = lb_max; t.lb_min = lb_min;
    t.level = 0; t.maxco = maxco; t.o1 = o1; t.o2 = o2;
    t.sphere_offset = use_ortho ? 0 : -1;
    if (use_ortho)
        for (int i = 0; i < 3; i++) { t.lb_cube[i] = lb_cube[i]; t.ub_cube[i] = ub_cube[i]; }
    const int func = compute_tau ? GPW_FUNC_DADB : GPW_FUNC_AB;
    PairGeom g;
    C.table.clear();
    int st = make_geom(t, 0, *C.plan, func, use_ortho ? sphere_bounds : nullptr, use_ortho ? nspheres : 0, g,
                       C.table);
    if (st) return st;
    g.coef_off = 0;
    g.mom_ext_off = 0;
    // the block is read at (o2+jco)*maxco + o1+ico < maxco*maxco
    const size_t npab = (size_t)maxco * maxco;
    const size_t ngr = (size_t)C.plan->lv[0].grid_elems;
    int smem_limit = 0;
    cudaDeviceGetAttribute(&smem_limit, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if ((g.ortho ? smem_ortho_fp64(g) : smem_general_fp64(g)) > smem_limit || smem_prep(g.la_max, g.lb_max) > smem_limit)
        return fail(GPW_ERR_UNSUPPORTED, "gpw_collocate_pgf_product_rspace: a cube is too large for one CTA");
    // buffer layout: geometry | cube list | block | status word | grid (256-byte aligned parts)
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t o_table = al(sizeof(PairGeom));
    const size_t o_pab = al(o_table + sizeof(int) * std::max<size_t>(C.table.size(), 1));
    const size_t o_stat = al(o_pab + sizeof(double) * npab);
    const size_t o_grid = o_stat + 256;
    const size_t total = o_grid + sizeof(double) * ngr;
    if (total > C.cap) {
        cudaFree(C.d_buf);
        if (C.h_buf) cudaFreeHost(C.h_buf);
        C.d_buf = C.h_buf = nullptr;
        C.cap = 0;
        GPW_CUDA(cudaMalloc(&C.d_buf, total));
        GPW_CUDA(cudaHostAlloc(&C.h_buf, total, cudaHostAllocDefault));
        C.cap = total;
    }
    memcpy(C.h_buf, &g, sizeof g);
    if (!C.table.empty()) memcpy(C.h_buf + o_table, C.table.data(), sizeof(int) * C.table.size());
    memcpy(C.h_buf + o_pab, pab, sizeof(double) * npab);
    memset(C.h_buf + o_stat, 0, sizeof(int));
    memcpy(C.h_buf + o_grid, grid, sizeof(double) * ngr);
    cudaStream_t s = nullptr;
    GPW_CUDA(cudaMemcpyAsync(C.d_buf, C.h_buf, total, cudaMemcpyHostToDevice, s));
    int *d_status = reinterpret_cast<int *>(C.d_buf + o_stat);
    double *d_grid = reinterpret_cast<double *>(C.d_buf + o_grid);
    GPW_CUDA(launch_one_fp64(g, reinterpret_cast<PairGeom *>(C.d_buf), C.plan->d_levels, C.plan->d_tmat,
                             reinterpret_cast<int *>(C.d_buf + o_table), C.d_coef, d_status, func,
                             reinterpret_cast<double *>(C.d_buf + o_pab), d_grid, s));
    GPW_CUDA(cudaMemcpyAsync(C.h_buf + o_stat, C.d_buf + o_stat, total - o_stat, cudaMemcpyDeviceToHost, s));
    GPW_CUDA(cudaStreamSynchronize(s));
    int h = 0;
    memcpy(&h, C.h_buf + o_stat, sizeof(int));
    memcpy(grid, C.h_buf + o_grid, sizeof(double) * ngr);
    if (h & kStatOutOfWindow) return fail(GPW_ERR_OUT_OF_WINDOW, "a cube left the local grid window");
    if (h) return fail(GPW_ERR_INVALID_ARG, "gpw_collocate_pgf_product_rspace: device status " + std::to_string(h));
    return GPW_SUCCESS;
}

int gpw_selftest_tensorcore(int64_t *mismatches) {
    if (!mismatches) return fail(GPW_ERR_INVALID_ARG, "gpw_selftest_tensorcore: null");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(GPW_ERR_NO_DEVICE, "no CUDA device");
    std::string err;
    const int st = tc_selftest(mismatches, err);
    return st ? fail(st, err) : GPW_SUCCESS;
}

int gpw_selftest_ff_exp(int64_t npoints, double *max_rel_err, double *max_rel_err_low) {
    if (!max_rel_err || !max_rel_err_low || npoints < 16) return fail(GPW_ERR_INVALID_ARG, "gpw_selftest_ff_exp: bad arguments");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(GPW_ERR_NO_DEVICE, "no CUDA device");
    std::string err;
    const int st = ffexp_selftest(npoints, max_rel_err, max_rel_err_low, err);
    return st ? fail(st, err) : GPW_SUCCESS;
}

int gpw_collocate_core(const int length[3], int L, const double *d_co, const double *d_pol, int ld_pol,
                       double *d_out, void *stream) {
    if (!length || L < 1 || L > 16 || !d_co || !d_pol || !d_out || ld_pol < std::max({length[0], length[1], length[2]}))
        return fail(GPW_ERR_INVALID_ARG, "gpw_collocate_core: bad arguments");
    GPW_CUDA(launch_collocate_core(length, L, d_co, d_pol, ld_pol, d_out, (cudaStream_t)stream));
    return GPW_SUCCESS;
}

int gpw_integrate_core(const int length[3], int L, const double *d_pol, int ld_pol, const double *d_V,
                       double *d_co, void *stream) {
    if (!length || L < 1 || L > 16 || !d_co || !d_pol || !d_V || ld_pol < std::max({length[0], length[1], length[2]}))
        return fail(GPW_ERR_INVALID_ARG, "gpw_integrate_core: bad arguments");
    GPW_CUDA(launch_integrate_core(length, L, d_pol, ld_pol, d_V, d_co, (cudaStream_t)stream));
    return GPW_SUCCESS;
}

}  // extern "C"
