// Pair coefficient transforms on the device, FP64, one CTA per pair.
//
// Forward (collocate set-up), following grid_base_ref_c.cc:849-979:
//   density block  -> local block P(b,a)     rho: grid_base_ref_c.cc:158-192
//                                             tau: grid_base_ref_c.cc:65-155
//                                             phi_a d phi_b - d phi_a phi_b:
//                                               coefficient.hpp:209-354 (restated)
//   1-D re-centring (x-a)^i (x-b)^j = sum_k al[i][j][k] (x-p)^k   :195-231
//   P -> c[lz][ly][lx] by three one-axis contractions              :234-315
// Adjoint (integrate back-transform): the same three contractions transposed,
// then the transposed block map, accumulated into the caller's hab.
#pragma once

#include "gpw_common.cuh"

namespace gpw {

GPW_HD void coset_decode(int ico, int &lx, int &ly, int &lz) {
    int l = 0;
    while (ncoset(l) <= ico) l++;
    int s = ico - ncoset(l - 1);
    // s = ((l-lx)(l-lx+1))/2 + lz, 0 <= lz <= l-lx
    lx = l;
    while (((l - lx) * (l - lx + 1)) / 2 + (l - lx) < s) lx--;
    lz = s - ((l - lx) * (l - lx + 1)) / 2;
    ly = l - lx - lz;
}

// (ly, lz) with ly + lz <= A, packed
GPW_HD int tri(int ly, int lz) { return ((ly + lz) * (ly + lz + 1)) / 2 + lz; }
GPW_HD void tri_decode(int t, int &ly, int &lz) {
    int s = 0;
    while (((s + 1) * (s + 2)) / 2 <= t) s++;
    lz = t - (s * (s + 1)) / 2;
    ly = s - lz;
}

struct CoefDims {
    int A, B, L;      // local la_max, lb_max, lp + 1
    int nla, nlb;     // ncoset(A), ncoset(B)
    int na2, nb2;     // (A+1)(A+2)/2, (B+1)(B+2)/2
    GPW_HD void set(int A_, int B_) {
        A = A_; B = B_; L = A + B + 1;
        nla = ncoset(A); nlb = ncoset(B);
        na2 = nshell(A); nb2 = nshell(B);
    }
    GPW_HD int n_P() const { return nla * nlb; }
    GPW_HD int n_al() const { return 3 * (A + 1) * (B + 1) * L; }
    GPW_HD int n_T1() const { return na2 * nb2 * L; }
    GPW_HD int n_T2() const { return (A + 1) * (B + 1) * L * L; }
    // P is dead once T1 is formed (forward) and T2 once T1 is formed (adjoint): they share
    GPW_HD int n_PT2() const { return n_P() > n_T2() ? n_P() : n_T2(); }
    GPW_HD int n_total() const { return n_al() + n_T1() + n_PT2(); }
};

// Shared-memory doubles a CTA needs for pairs up to la, lb (local, after tau).
GPW_HD int coef_ws_doubles(int A, int B) {
    CoefDims d;
    d.set(A, B);
    return d.n_total();
}

struct CoefWs {
    CoefDims d;
    double *P, *al, *T1, *T2;
    __device__ void carve(double *base, int A, int B) {
        d.set(A, B);
        al = base;
        T1 = al + d.n_al();
        T2 = T1 + d.n_T1();
        P = T2;  // shared with T2 (see n_PT2)
    }
    __device__ double *end() const { return T2 + d.n_PT2(); }
    __device__ double &AL(int ax, int i, int j, int k) {
        return al[((ax * (d.A + 1) + i) * (d.B + 1) + j) * d.L + k];
    }
};

// al[ax][i][j][k]: the coefficients of (x-a)^i (x-b)^j in powers of (x-p), as the
// product (u + pa)^i (u + pb)^j with u = x - p, pa = p - a, pb = p - b, expanded by
// one multiplication by (u + pa) or (u + pb) at a time (no divisions, no power
// loops): at most (i + j)(i + j + 3)/2 FP64 multiply-adds per (ax, i, j).
__device__ inline void fill_alpha(CoefWs &w, const PairGeom &g) {
    const int n = 3 * (w.d.A + 1) * (w.d.B + 1);
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
        const int j = t % (w.d.B + 1);
        const int i = (t / (w.d.B + 1)) % (w.d.A + 1);
        const int ax = t / ((w.d.B + 1) * (w.d.A + 1));
        const double pa = g.rp[ax] - g.ra[ax];
        const double pb = g.rp[ax] - g.rb[ax];
        double *out = &w.AL(ax, i, j, 0);
        out[0] = 1.0;
        for (int k = 1; k < w.d.L; k++) out[k] = 0.0;
        for (int m = 0; m < i + j; m++) {  // degree m so far
            const double c = m < i ? pa : pb;
            out[m + 1] = out[m];
            for (int k = m; k >= 1; k--) out[k] = fma(c, out[k], out[k - 1]);
            out[0] *= c;
        }
    }
}

__device__ inline int64_t block_index(const PairGeom &g, int jco, int ico) {
    return g.pab_offset + (int64_t)(g.o2 + jco) * g.maxco + (g.o1 + ico);
}

// The density block element P(bs, as) if (as, bs) lies in the pair's shells, else 0.
__device__ inline double block_entry(const PairGeom &g, const double *pab, const int as[3], const int bs[3]) {
    const int las = as[0] + as[1] + as[2], lbs = bs[0] + bs[1] + bs[2];
    if (las < g.la0_min || las > g.la0_max || lbs < g.lb0_min || lbs > g.lb0_max) return 0.0;
    return pab[block_index(g, coset(bs[0], bs[1], bs[2]), coset(as[0], as[1], as[2]))];
}

// One element P'(b', a') of the local block of function `func` (gpw_function)
// and, when dza / dzb are given, its derivatives with respect to the exponents.
// With d/dx phi_a = l phi_{a - e} - 2 za phi_{a + e} (per axis):
//   rho      P' = P
//   tau      P'(a', b') = 1/2 sum_d sum over the two terms of each side
//   ADBmDAB  phi_a d_d phi_b - d_d phi_a phi_b: P(a', b' + e_d)(b'_d + 1)
//            - 2 zb P(a', b' - e_d) - (a'_d + 1) P(a' + e_d, b') + 2 za P(a' - e_d, b')
__device__ inline double local_entry(const PairGeom &g, int func, const double *pab, const int a[3],
                                     const int b[3], double *dza = nullptr, double *dzb = nullptr) {
    double v = 0.0, va = 0.0, vb = 0.0;
    if (func == GPW_FUNC_AB) {
        v = block_entry(g, pab, a, b);
    } else if (func == GPW_FUNC_DADB) {
        for (int d = 0; d < 3; d++)
            for (int sa = 0; sa < 2; sa++) {
                int as[3] = {a[0], a[1], a[2]};
                double ca, dca;
                if (sa == 0) { as[d] += 1; ca = (double)as[d]; dca = 0.0; }  // source lowered to a'
                else { if (a[d] == 0) continue; as[d] -= 1; ca = -2.0 * g.zeta; dca = -2.0; }  // source raised
                for (int sb = 0; sb < 2; sb++) {
                    int bs[3] = {b[0], b[1], b[2]};
                    double cb, dcb;
                    if (sb == 0) { bs[d] += 1; cb = (double)bs[d]; dcb = 0.0; }
                    else { if (b[d] == 0) continue; bs[d] -= 1; cb = -2.0 * g.zetb; dcb = -2.0; }
                    const double p = 0.5 * block_entry(g, pab, as, bs);
                    v += ca * cb * p;
                    va += dca * cb * p;
                    vb += ca * dcb * p;
                }
            }
    } else {
        const int d = func - GPW_FUNC_ADBMDAB_X;
        int as[3] = {a[0], a[1], a[2]}, bs[3] = {b[0], b[1], b[2]};
        bs[d] = b[d] + 1;
        v += (double)(b[d] + 1) * block_entry(g, pab, a, bs);
        if (b[d] > 0) {
            bs[d] = b[d] - 1;
            const double p = block_entry(g, pab, a, bs);
            v -= 2.0 * g.zetb * p;
            vb -= 2.0 * p;
        }
        as[d] = a[d] + 1;
        v -= (double)(a[d] + 1) * block_entry(g, pab, as, b);
        if (a[d] > 0) {
            as[d] = a[d] - 1;
            const double p = block_entry(g, pab, as, b);
            v += 2.0 * g.zeta * p;
            va += 2.0 * p;
        }
    }
    if (dza) *dza = va;
    if (dzb) *dzb = vb;
    return v;
}

// P(b', a') of the local block of function `func` (gpw_function).
__device__ inline void fill_local_block(CoefWs &w, const PairGeom &g, int func, const double *pab) {
    const int n = w.d.n_P();
    if (func == GPW_FUNC_AB) {
        // rho: the local block is the density block, in the same coset order, and
        // zero below the pair's lowest shells; kU independent loads per thread are
        // in flight together
        constexpr int kU = 8;
        const int nla = w.d.nla, a_lo = ncoset(g.la0_min - 1), b_lo = ncoset(g.lb0_min - 1);
        for (int t0 = threadIdx.x; t0 < n; t0 += kU * blockDim.x) {
            double v[kU];
#pragma unroll
            for (int u = 0; u < kU; u++) {
                const int t = t0 + u * blockDim.x;
                const int jco = t / nla, ico = t - jco * nla;
                v[u] = (t < n && ico >= a_lo && jco >= b_lo) ? __ldg(&pab[block_index(g, jco, ico)]) : 0.0;
            }
#pragma unroll
            for (int u = 0; u < kU; u++) {
                const int t = t0 + u * blockDim.x;
                if (t < n) w.P[t] = v[u];
            }
        }
        return;
    }
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
        const int jco = t / w.d.nla, ico = t % w.d.nla;
        int a[3], b[3];
        coset_decode(ico, a[0], a[1], a[2]);
        coset_decode(jco, b[0], b[1], b[2]);
        w.P[t] = local_entry(g, func, pab, a, b);
    }
}

// c (packed, prefactor included) from P.  Writes packed coefficients to `out`.
// Products with a structurally zero factor are not formed: a lattice power lx of
// T1[(lya,lza)][(lyb,lzb)] is zero beyond (A-lya-lza) + (B-lyb-lzb), the largest
// lxa + lxb of the block, so T2[lza][lzb][ly][lx] is zero for lx + ly beyond
// (A-lza) + (B-lzb); the loop bounds below skip those terms.
__device__ inline void forward_coef(CoefWs &w, const PairGeom &g, double *out) {
    const CoefDims &d = w.d;
    const int L = d.L;
    // X: T1[ta][tb][lx] = sum_{lxa,lxb} P[b][a] al_x[lxa][lxb][lx]
    for (int t = threadIdx.x; t < d.n_T1(); t += blockDim.x) {
        const int lx = t % L;
        const int tb = (t / L) % d.nb2;
        const int ta = t / (L * d.nb2);
        int lya, lza, lyb, lzb;
        tri_decode(ta, lya, lza);
        tri_decode(tb, lyb, lzb);
        double s = 0.0;
        const int xa0 = max(g.la_min - lya - lza, 0), xa1 = g.la_max - lya - lza;
        const int xb0 = max(g.lb_min - lyb - lzb, 0), xb1 = g.lb_max - lyb - lzb;
        for (int lxa = xa0; lxa <= xa1; lxa++)
            for (int lxb = xb0; lxb <= xb1; lxb++) {
                if (lx > lxa + lxb) continue;
                s += w.P[coset(lxb, lyb, lzb) * d.nla + coset(lxa, lya, lza)] * w.AL(0, lxa, lxb, lx);
            }
        w.T1[t] = s;
    }
    __syncthreads();
    // Y: T2[lza][lzb][ly][lx] = sum_{lya,lyb} T1[(lya,lza)][(lyb,lzb)][lx] al_y[lya][lyb][ly]
    for (int t = threadIdx.x; t < d.n_T2(); t += blockDim.x) {
        const int lx = t % L;
        const int ly = (t / L) % L;
        const int lzb = (t / (L * L)) % (d.B + 1);
        const int lza = t / (L * L * (d.B + 1));
        const int cap = d.A + d.B - lza - lzb - lx;  // ly <= lya + lyb <= cap
        double s = 0.0;
        for (int lya = 0; lya <= d.A - lza; lya++) {
            const int b0 = max(ly - lya, 0), b1 = min(d.B - lzb, cap - lya);
            for (int lyb = b0; lyb <= b1; lyb++)
                s += w.T1[(tri(lya, lza) * d.nb2 + tri(lyb, lzb)) * L + lx] * w.AL(1, lya, lyb, ly);
        }
        w.T2[t] = s;
    }
    __syncthreads();
    // Z: c[lz][ly][lx] = pref * sum_{lza,lzb} T2[lza][lzb][ly][lx] al_z[lza][lzb][lz]
    const int lp = g.lp;
    for (int t = threadIdx.x; t < L * L * L; t += blockDim.x) {
        const int lx = t % L, ly = (t / L) % L, lz = t / (L * L);
        if (lx + ly + lz > lp) continue;
        const int cap = d.A + d.B - lx - ly;  // lz <= lza + lzb <= cap
        double s = 0.0;
        for (int lza = 0; lza <= d.A; lza++) {
            const int b0 = max(lz - lza, 0), b1 = min(d.B, cap - lza);
            for (int lzb = b0; lzb <= b1; lzb++)
                s += w.T2[((lza * (d.B + 1) + lzb) * L + ly) * L + lx] * w.AL(2, lza, lzb, lz);
        }
        out[pidx(lp, lz, ly, lx)] = g.prefactor * s;
    }
}

// Cartesian indices of the local shells (la, lb <= kMaxL + 1 after the shift of
// the derivative functions)
constexpr int kNcoLocal = ((kMaxL + 2) * (kMaxL + 3) * (kMaxL + 4)) / 6;

// Adjoint: given moments W (packed like c), accumulate into hab.  Only the
// entries the next stage reads are formed: X^T reads T1[(lya,lza)][(lyb,lzb)][lx]
// for lx <= lxa + lxb <= (A-lya-lza) + (B-lyb-lzb), so Y^T reads T2[lza][lzb][ly][lx]
// only for lx + ly <= (A-lza) + (B-lzb).
__device__ inline void adjoint_coef(CoefWs &w, const PairGeom &g, int func, const double *W,
                                    double *hab) {
    const CoefDims &d = w.d;
    const int L = d.L, lp = g.lp;
    // coset index -> lx | ly << 4 | lz << 8, read after the next barrier
    __shared__ int s_co[kNcoLocal];
    for (int i = threadIdx.x; i < max(d.nla, d.nlb); i += blockDim.x) {
        int x, y, z;
        coset_decode(i, x, y, z);
        s_co[i] = x | (y << 4) | (z << 8);
    }
    // Z^T: T2[lza][lzb][ly][lx] = sum_lz al_z[lza][lzb][lz] W[lz][ly][lx]
    for (int t = threadIdx.x; t < d.n_T2(); t += blockDim.x) {
        const int lx = t % L;
        const int ly = (t / L) % L;
        const int lzb = (t / (L * L)) % (d.B + 1);
        const int lza = t / (L * L * (d.B + 1));
        if (lx + ly > d.A + d.B - lza - lzb) continue;
        double s = 0.0;
        for (int lz = 0; lz <= lza + lzb && lz + ly + lx <= lp; lz++)
            s += w.AL(2, lza, lzb, lz) * W[pidx(lp, lz, ly, lx)];
        w.T2[t] = s;
    }
    __syncthreads();
    // Y^T: T1[ta][tb][lx] = sum_ly al_y[lya][lyb][ly] T2[lza][lzb][ly][lx]
    for (int t = threadIdx.x; t < d.n_T1(); t += blockDim.x) {
        const int lx = t % L;
        const int tb = (t / L) % d.nb2;
        const int ta = t / (L * d.nb2);
        int lya, lza, lyb, lzb;
        tri_decode(ta, lya, lza);
        tri_decode(tb, lyb, lzb);
        if (lx > (d.A - lya - lza) + (d.B - lyb - lzb)) continue;
        double s = 0.0;
        for (int ly = 0; ly <= lya + lyb; ly++)
            s += w.AL(1, lya, lyb, ly) * w.T2[((lza * (d.B + 1) + lzb) * L + ly) * L + lx];
        w.T1[t] = s;
    }
    __syncthreads();
    // X^T: P[b][a] = pref * sum_lx al_x[lxa][lxb][lx] T1[(lya,lza)][(lyb,lzb)][lx]
    for (int t = threadIdx.x; t < d.n_P(); t += blockDim.x) {
        const int jco = t / d.nla, ico = t - jco * d.nla;
        const int ca = s_co[ico], cb = s_co[jco];
        const int a[3] = {ca & 15, (ca >> 4) & 15, ca >> 8}, b[3] = {cb & 15, (cb >> 4) & 15, cb >> 8};
        const int la = a[0] + a[1] + a[2], lb = b[0] + b[1] + b[2];
        double s = 0.0;
        if (la >= g.la_min && la <= g.la_max && lb >= g.lb_min && lb <= g.lb_max) {
            const int ta = tri(a[1], a[2]), tb = tri(b[1], b[2]);
            for (int lx = 0; lx <= a[0] + b[0]; lx++)
                s += w.AL(0, a[0], b[0], lx) * w.T1[(ta * d.nb2 + tb) * L + lx];
        }
        w.P[t] = g.prefactor * s;
    }
    __syncthreads();
    // block map transposed, into hab (pairs may share hab entries: atomics)
    const int na0 = ncoset(g.la0_max), nb0 = ncoset(g.lb0_max);
    if (func == GPW_FUNC_AB) {
        // rho: the same coset order, the pair's shells only
        const int a_lo = ncoset(g.la0_min - 1), b_lo = ncoset(g.lb0_min - 1);
        for (int t = threadIdx.x; t < na0 * nb0; t += blockDim.x) {
            const int jco = t / na0, ico = t - jco * na0;
            if (ico >= a_lo && jco >= b_lo) atomicAdd(&hab[block_index(g, jco, ico)], w.P[jco * d.nla + ico]);
        }
        return;
    }
    for (int t = threadIdx.x; t < na0 * nb0; t += blockDim.x) {
        const int jco = t / na0, ico = t - jco * na0;
        const int ca = s_co[ico], cb = s_co[jco];
        const int a[3] = {ca & 15, (ca >> 4) & 15, ca >> 8}, b[3] = {cb & 15, (cb >> 4) & 15, cb >> 8};
        const int la = a[0] + a[1] + a[2], lb = b[0] + b[1] + b[2];
        if (la < g.la0_min || la > g.la0_max || lb < g.lb0_min || lb > g.lb0_max) continue;
        double s = 0.0;
        auto Pl = [&](const int at[3], const int bt[3]) {
            return w.P[coset(bt[0], bt[1], bt[2]) * d.nla + coset(at[0], at[1], at[2])];
        };
        if (func >= GPW_FUNC_ADBMDAB_X) {
            // the transpose of local_entry: source (a, b) feeds (a, b - e), (a, b + e),
            // (a - e, b) and (a + e, b)
            const int dd = func - GPW_FUNC_ADBMDAB_X;
            int at[3] = {a[0], a[1], a[2]}, bt[3] = {b[0], b[1], b[2]};
            if (b[dd] > 0) {
                bt[dd] = b[dd] - 1;
                s += (double)b[dd] * Pl(a, bt);
            }
            bt[dd] = b[dd] + 1;
            s -= 2.0 * g.zetb * Pl(a, bt);
            if (a[dd] > 0) {
                at[dd] = a[dd] - 1;
                s -= (double)a[dd] * Pl(at, b);
            }
            at[dd] = a[dd] + 1;
            s += 2.0 * g.zeta * Pl(at, b);
        } else {
            for (int dd = 0; dd < 3; dd++)
                for (int sa = 0; sa < 2; sa++) {
                    int at[3] = {a[0], a[1], a[2]};
                    double ca;
                    if (sa == 0) { if (a[dd] == 0) continue; ca = (double)a[dd]; at[dd] -= 1; }
                    else { ca = -2.0 * g.zeta; at[dd] += 1; }
                    for (int sb = 0; sb < 2; sb++) {
                        int bt[3] = {b[0], b[1], b[2]};
                        double cb;
                        if (sb == 0) { if (b[dd] == 0) continue; cb = (double)b[dd]; bt[dd] -= 1; }
                        else { cb = -2.0 * g.zetb; bt[dd] += 1; }
                        s += 0.5 * ca * cb * w.P[coset(bt[0], bt[1], bt[2]) * d.nla + coset(at[0], at[1], at[2])];
                    }
                }
        }
        atomicAdd(&hab[block_index(g, jco, ico)], s);
    }
}

}  // namespace gpw
