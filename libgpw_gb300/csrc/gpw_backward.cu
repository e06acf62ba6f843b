// Backward pass of E = sum over levels of <V, rho>: gradients with respect to
// the density blocks (the integrate path), the two centres and the two
// exponents of every pair, FP64.
//
// With phi_a = (x-ax)^lx (y-ay)^ly (z-az)^lz exp(-za |r-a|^2):
//   d phi_a / d ax  = -lx phi_{a-ex} + 2 za phi_{a+ex}
//   d phi_a / d za  = -(phi_{a+2ex} + phi_{a+2ey} + phi_{a+2ez})
// (the derivative rule the reference applies for tau, grid_base_ref_c.cc:77-140),
// so every gradient is a combination of pair integrals I(a', b) = <V, phi_a' phi_b>
// with |a'| <= la_max + 2.  Those come from the moments of V against the product
// Gaussian up to degree lp + 2 (one more integrate pass, the 1-D tables are
// recomputed), re-centred on a and b with the binomials of grid_base_ref_c.cc:195-231.
// The derivative functions (tau and phi_a d phi_b - d phi_a phi_b) are sums over
// their local block P'(a', b') of P' phi_a' phi_b' (shells l +- 1, coefficients
// that depend on the exponents): the same rule applies per local element, plus
// dP'/dzeta I(a', b') for the exponent gradients.
#include <cuda_runtime.h>

#include "gpw_coef.cuh"
#include "gpw_internal.h"

namespace gpw {

constexpr int kBI = kMaxL + 4;          // components up to l_max + 1 (local block) + 2
constexpr int kBK = 2 * kBI - 1;

struct BwdSmem {
    double al[3][kBI][kBI][kBK];
    double W[(kNPowB * (kNPowB + 1) * (kNPowB + 2)) / 6];  // moments up to degree lp + 2
    double red[8][4];
};

__device__ __forceinline__ double pair_integral(const BwdSmem &s, int lpe, const int a[3], const int b[3]) {
    double acc = 0.0;
    for (int lz = 0; lz <= a[2] + b[2]; lz++) {
        const double az = s.al[2][a[2]][b[2]][lz];
        for (int ly = 0; ly <= a[1] + b[1]; ly++) {
            const double ayz = az * s.al[1][a[1]][b[1]][ly];
            for (int lx = 0; lx <= a[0] + b[0]; lx++)
                acc += ayz * s.al[0][a[0]][b[0]][lx] * s.W[pidx(lpe, lz, ly, lx)];
        }
    }
    return acc;
}

__global__ void __launch_bounds__(128)
k_backward_epilogue(const PairGeom *__restrict__ geoms, const LevelDev *__restrict__ levels,
                    const double *__restrict__ tmat, const double *__restrict__ mom_ext, int func,
                    const double *__restrict__ pab, double *dra, double *drb, double *dza, double *dzb) {
    __shared__ BwdSmem s;
    const PairGeom g = geoms[blockIdx.x];
    const int tid = threadIdx.x;
    const int lpe = g.lp + 2;
    const int ia = g.la_max + 2, jb = g.lb_max + 2;  // local shells (after the function's shift)
    // re-centring binomials (x-a)^i (x-b)^j = sum_k al[i][j][k] (x-p)^k
    for (int t = tid; t < 3 * (ia + 1) * (jb + 1); t += blockDim.x) {
        const int j = t % (jb + 1), i = (t / (jb + 1)) % (ia + 1), ax = t / ((jb + 1) * (ia + 1));
        const double pa = g.rp[ax] - g.ra[ax], pb = g.rp[ax] - g.rb[ax];
        double *out = s.al[ax][i][j];
        for (int k = 0; k < kBK; k++) out[k] = 0.0;
        double ci = 1.0;
        for (int k1 = 0; k1 <= i; k1++) {
            double pai = 1.0;
            for (int e = 0; e < i - k1; e++) pai *= pa;
            double cj = 1.0;
            for (int k2 = 0; k2 <= j; k2++) {
                double pbj = 1.0;
                for (int e = 0; e < j - k2; e++) pbj *= pb;
                out[k1 + k2] += ci * pai * cj * pbj;
                cj = cj * (double)(j - k2) / (double)(k2 + 1);
            }
            ci = ci * (double)(i - k1) / (double)(k1 + 1);
        }
    }
    // Cartesian moments (general cells: transpose of the lattice transform)
    const int nc = ncoef(lpe);
    const double *Wsrc = mom_ext + g.mom_ext_off;
    for (int t = tid; t < nc; t += blockDim.x) {
        if (g.ortho) {
            s.W[t] = Wsrc[t];
            continue;
        }
        int lz = 0, ly = 0, lx = 0, r = t;
        for (lz = 0; lz <= lpe; lz++) {
            const int cnt = ((lpe - lz + 1) * (lpe - lz + 2)) / 2;
            if (r < cnt) break;
            r -= cnt;
        }
        const int q = lpe - lz;
        for (ly = 0; ly <= q; ly++) {
            if (r <= q - ly) break;
            r -= q - ly + 1;
        }
        lx = r;
        const int n = lx + ly + lz;
        const int NT = ncoef(kMaxLp);
        const double *Tm = tmat + levels[g.level].tmat_off;
        const int col = pidx(kMaxLp, lz, ly, lx);
        double acc = 0.0;
        for (int k = 0; k <= n; k++)
            for (int j = 0; j <= n - k; j++) acc += Tm[(int64_t)pidx(kMaxLp, k, j, n - k - j) * NT + col] * Wsrc[pidx(lpe, k, j, n - k - j)];
        s.W[t] = acc;
    }
    __syncthreads();
    double grad[8] = {0, 0, 0, 0, 0, 0, 0, 0};  // dRa[3], dRb[3], dza, dzb
    const int na = ncoset(g.la_max), nb = ncoset(g.lb_max);
    for (int t = tid; t < na * nb; t += blockDim.x) {
        const int jco = t / na, ico = t % na;
        int a[3], b[3];
        coset_decode(ico, a[0], a[1], a[2]);
        coset_decode(jco, b[0], b[1], b[2]);
        double dPa, dPb;  // dP'/dzeta, dP'/dzetb of the local element
        const double P = local_entry(g, func, pab, a, b, &dPa, &dPb);
        if (P == 0.0 && dPa == 0.0 && dPb == 0.0) continue;
        if (dPa != 0.0 || dPb != 0.0) {
            const double I0 = pair_integral(s, lpe, a, b);
            grad[6] += dPa * I0;
            grad[7] += dPb * I0;
        }
        if (P == 0.0) continue;
        for (int d = 0; d < 3; d++) {
            int a2[3] = {a[0], a[1], a[2]}, b2[3] = {b[0], b[1], b[2]};
            // centre a
            a2[d] = a[d] + 1;
            double v = 2.0 * g.zeta * pair_integral(s, lpe, a2, b);
            if (a[d] > 0) {
                a2[d] = a[d] - 1;
                v -= a[d] * pair_integral(s, lpe, a2, b);
            }
            grad[d] += P * v;
            a2[d] = a[d] + 2;
            grad[6] -= P * pair_integral(s, lpe, a2, b);
            a2[d] = a[d];
            // centre b
            b2[d] = b[d] + 1;
            v = 2.0 * g.zetb * pair_integral(s, lpe, a, b2);
            if (b[d] > 0) {
                b2[d] = b[d] - 1;
                v -= b[d] * pair_integral(s, lpe, a, b2);
            }
            grad[3 + d] += P * v;
            b2[d] = b[d] + 2;
            grad[7] -= P * pair_integral(s, lpe, a, b2);
        }
    }
    // block reduction of the eight gradients
    const int lane = tid & 31, warp = tid >> 5;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        double v = grad[k];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) s.red[k][warp] = v;
    }
    __syncthreads();
    if (tid < 8) {
        double v = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) v += s.red[tid][w];
        v *= g.prefactor;
        const int64_t t = g.task;
        if (tid < 3) {
            if (dra) dra[3 * t + tid] = v;
        } else if (tid < 6) {
            if (drb) drb[3 * t + tid - 3] = v;
        } else if (tid == 6) {
            if (dza) dza[t] = v;
        } else {
            if (dzb) dzb[t] = v;
        }
    }
}

cudaError_t launch_backward(const TaskSet &ts, const double *d_pab, const GridPtrs &g, double *d_hab,
                            double *d_dra, double *d_drb, double *d_dza, double *d_dzb, cudaStream_t s) {
    (void)d_hab;
    if (ts.ntasks == 0) return cudaSuccess;
    // orthorhombic moments go to degree lp + 2 <= kMaxLpB; general cells map them
    // through the lattice transform, which is built to degree kMaxLp
    for (int64_t k = ts.gen_first; k < ts.gen_first + ts.gen_count; k++)
        if (ts.h_geom[k].lp + 2 > kMaxLp) return cudaErrorNotSupported;
    if (ts.max_lp + 2 > kMaxLpB) return cudaErrorNotSupported;
    TaskSet &mts = const_cast<TaskSet &>(ts);
    if (!mts.d_mom_ext) {
        cudaError_t e = cudaMalloc(&mts.d_mom_ext, sizeof(double) * std::max<int64_t>(ts.mom_ext_len, 1));
        if (e != cudaSuccess) return e;
    }
    cudaError_t e = launch_moments_fp64(ts, g, 2, mts.d_mom_ext, s);
    if (e != cudaSuccess) return e;
    ts.n_kernels++;
    k_backward_epilogue<<<(unsigned)ts.ntasks, 128, 0, s>>>(ts.d_geom, ts.plan->d_levels, ts.plan->d_tmat,
                                                           mts.d_mom_ext, ts.tau, d_pab, d_dra, d_drb, d_dza,
                                                           d_dzb);
    return cudaGetLastError();
}

}  // namespace gpw
