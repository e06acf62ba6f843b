// Tensor-core self test: one kind::f16 MMA (M=128, N=32, K=16) on integer-valued
// fp16 operands laid out exactly as the tiled kernels lay them out, checked
// element by element against the exact integer products.  It exercises the
// descriptor encodings, TMEM allocation, the commit/mbarrier handshake and the
// TMEM load layout that the mixed path relies on.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <random>
#include <vector>

#include "gpw_ff.cuh"
#include "gpw_internal.h"
#include "gpw_tc.cuh"

namespace gpw {

namespace {
__device__ __forceinline__ int op_off(int r, int k) {
    return (r >> 3) * 256 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2;
}

struct alignas(128) SelfSmem {
    unsigned char buf[16384];  // operands at the start; every stride stays inside
    uint64_t mbar;
    uint32_t tmem;
    int timeout;
};

__global__ void __launch_bounds__(128) k_tc_selftest(const float *A, const float *B, float *D, int *status) {
    __shared__ SelfSmem sm;
    const int tid = threadIdx.x, warp = tid >> 5;
    __half *As = reinterpret_cast<__half *>(sm.buf);
    __half *Bs = reinterpret_cast<__half *>(sm.buf + 4096);
    for (int t = tid; t < 16384 / 4; t += 128) reinterpret_cast<uint32_t *>(sm.buf)[t] = 0u;
    __syncthreads();
    for (int k = 0; k < 16; k++) As[op_off(tid, k) >> 1] = __float2half_rn(A[tid * 16 + k]);
    if (tid < 32)
        for (int k = 0; k < 16; k++) Bs[op_off(tid, k) >> 1] = __float2half_rn(B[tid * 16 + k]);
    if (tid == 0) {
        tc::mbar_init(&sm.mbar, 1);
        tc::fence_mbar_init();
        sm.timeout = 0;
    }
    if (warp == 0) {
        tc::tmem_alloc(&sm.tmem, 32);
        tc::tmem_relinquish();
    }
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = sm.tmem;
    if (tid == 0) {
        tc::mma_f16(tmem, tc::desc_kmajor(As, 128, 256), tc::desc_kmajor(Bs, 128, 256), tc::idesc_f16_f32(128, 32), 0);
        tc::mma_commit(&sm.mbar);
    }
    if (!tc::mbar_wait_bounded(&sm.mbar, 0, 1u << 22)) {
        atomicOr(status, kStatTimeout);
        sm.timeout = 1;
    }
    __syncthreads();
    tc::fence_after_sync();
    if (!sm.timeout) {
#pragma unroll
        for (int c = 0; c < 4; c++) {
            uint32_t r[8];
            tc::tmem_ld8(tmem + ((uint32_t)(warp * 32) << 16) + 8 * c, r);
            tc::tmem_wait_ld8(r);
            for (int i = 0; i < 8; i++) D[tid * 32 + 8 * c + i] = __uint_as_float(r[i]);
        }
    } else {
        // give the tensor core a bounded second chance to finish before TMEM is freed
        tc::mbar_wait_bounded(&sm.mbar, 0, 1u << 22);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, 32);
}
}  // namespace

int tc_selftest(int64_t *mismatches, std::string &err) {
    std::mt19937 rng(12345);
    std::uniform_int_distribution<int> dist(-1024, 1024);
    std::vector<float> A(128 * 16), B(32 * 16), D(128 * 32, -1.f);
    for (auto &v : A) v = (float)dist(rng);
    for (auto &v : B) v = (float)dist(rng);
    float *dA = nullptr, *dB = nullptr, *dD = nullptr;
    int *dS = nullptr;
    cudaError_t e = cudaMalloc(&dA, A.size() * 4);
    if (e == cudaSuccess) e = cudaMalloc(&dB, B.size() * 4);
    if (e == cudaSuccess) e = cudaMalloc(&dD, D.size() * 4);
    if (e == cudaSuccess) e = cudaMalloc(&dS, 4);
    if (e == cudaSuccess) e = cudaMemcpy(dA, A.data(), A.size() * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dB, B.data(), B.size() * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(dS, 0, 4);
    if (e == cudaSuccess) {
        k_tc_selftest<<<1, 128>>>(dA, dB, dD, dS);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    int st = 0;
    if (e == cudaSuccess) e = cudaMemcpy(D.data(), dD, D.size() * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&st, dS, 4, cudaMemcpyDeviceToHost);
    cudaFree(dA);
    cudaFree(dB);
    cudaFree(dD);
    cudaFree(dS);
    if (e != cudaSuccess) {
        err = std::string("tensor-core self test: ") + cudaGetErrorString(e);
        return GPW_ERR_CUDA;
    }
    if (st & kStatTimeout) {
        err = "tensor-core self test: the MMA did not complete within the wait limit";
        return GPW_ERR_TIMEOUT;
    }
    int64_t bad = 0;
    for (int m = 0; m < 128; m++)
        for (int n = 0; n < 32; n++) {
            double s = 0.0;
            for (int k = 0; k < 16; k++) s += (double)A[m * 16 + k] * (double)B[n * 16 + k];
            if ((double)D[m * 32 + n] != s) bad++;
        }
    *mismatches = bad;
    return GPW_SUCCESS;
}

// ff_exp sweep: n arguments spread over [lo, hi) in float-float (a low part of up
// to half an ulp of the high part), each compared with the FP64 exp of the same
// value; every thread writes the largest error it saw (host reduction).
__global__ void k_ffexp_sweep(int64_t n, double lo, double hi, double *worst_out) {
    double worst = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double x = lo + (hi - lo) * ((double)i / (double)n);
        const float xh = __double2float_rn(x);
        // low part: a pseudo-random fraction of half an ulp of the high part
        const uint32_t h = (uint32_t)(i * 2654435761ull) >> 8;
        const float ulp = fabsf(__int_as_float(__float_as_int(xh) + 1) - xh);
        const float xl = ((float)h / 16777216.0f - 0.5f) * ulp;
        const ff v = ff_exp(ff{xh, xl});
        const double ref = exp((double)xh + (double)xl);
        // relative to exp, or to the smallest normal float where exp is below it
        // (results there are float subnormals with only a few significant bits)
        worst = fmax(worst, fabs(((double)v.hi + (double)v.lo) - ref) / fmax(ref, 0x1p-126));
    }
    worst_out[blockIdx.x * (int64_t)blockDim.x + threadIdx.x] = worst;
}

int ffexp_selftest(int64_t n, double *err_normal, double *err_low, std::string &err) {
    constexpr int kBlocks = 1024, kThreads = 256, kN = kBlocks * kThreads;
    double *d_w = nullptr;
    cudaError_t e = cudaMalloc(&d_w, 2 * sizeof(double) * kN);
    if (e == cudaSuccess) {
        // results with a normal low part (a > -60), then the range where it underflows gradually
        k_ffexp_sweep<<<kBlocks, kThreads>>>(n, -60.0, 88.0, d_w);
        k_ffexp_sweep<<<kBlocks, kThreads>>>(n / 4, -103.0, -60.0, d_w + kN);
        e = cudaGetLastError();
    }
    std::vector<double> w(2 * (size_t)kN, 0.0);
    if (e == cudaSuccess) e = cudaMemcpy(w.data(), d_w, sizeof(double) * w.size(), cudaMemcpyDeviceToHost);
    cudaFree(d_w);
    if (e != cudaSuccess) {
        err = std::string("ffexp_selftest: ") + cudaGetErrorString(e);
        return GPW_ERR_CUDA;
    }
    double a = 0.0, b = 0.0;
    for (int i = 0; i < kN; i++) {
        a = std::max(a, w[i]);
        b = std::max(b, w[kN + i]);
    }
    *err_normal = a;
    *err_low = b;
    return GPW_SUCCESS;
}

}  // namespace gpw
