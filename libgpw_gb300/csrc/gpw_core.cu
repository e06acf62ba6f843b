// Dense cube contractions of the factorised prototype (collocate.cc:438-623),
// FP64 on the device.  Used as known-answer kernels with the shapes of the
// reference's own tests (collocate_test.cc:35-140, called from collocate.cc:1185-1212).
#include <cuda_runtime.h>

#include "gpw_internal.h"

namespace gpw {

// out[z][y][x] = sum_{a,g,b} co[a][g][b] P0[g][z] P1[b][y] P2[a][x]; one CTA per z
__global__ void k_collocate_core(int nz, int ny, int nx, int L, const double *__restrict__ co,
                                 const double *__restrict__ pol, int ld, double *__restrict__ out) {
    extern __shared__ double sm[];
    double *C1 = sm;           // [a][b]
    double *C2 = C1 + L * L;   // [y][a]
    const int z = blockIdx.x;
    const double *P0 = pol, *P1 = pol + (size_t)L * ld, *P2 = pol + (size_t)2 * L * ld;
    for (int t = threadIdx.x; t < L * L; t += blockDim.x) {
        const int a = t / L, b = t % L;
        double s = 0.0;
        for (int g = 0; g < L; g++) s += co[(a * L + g) * L + b] * P0[g * ld + z];
        C1[t] = s;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < ny * L; t += blockDim.x) {
        const int y = t / L, a = t % L;
        double s = 0.0;
        for (int b = 0; b < L; b++) s += C1[a * L + b] * P1[b * ld + y];
        C2[t] = s;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < ny * nx; t += blockDim.x) {
        const int y = t / nx, x = t % nx;
        double s = 0.0;
        for (int a = 0; a < L; a++) s += C2[y * L + a] * P2[a * ld + x];
        out[((size_t)z * ny + y) * nx + x] = s;
    }
}

// co[g][b][a] = sum_{z,y,x} V[z][y][x] P0[g][z] P1[b][y] P2[a][x]; one CTA per output
__global__ void k_integrate_core(int nz, int ny, int nx, int L, const double *__restrict__ pol, int ld,
                                 const double *__restrict__ V, double *__restrict__ co) {
    __shared__ double red[32];
    const int a = blockIdx.x % L, b = (blockIdx.x / L) % L, g = blockIdx.x / (L * L);
    const double *P0 = pol + (size_t)g * ld, *P1 = pol + (size_t)(L + b) * ld, *P2 = pol + (size_t)(2 * L + a) * ld;
    double s = 0.0;
    const int n = nz * ny * nx;
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
        const int x = t % nx, y = (t / nx) % ny, z = t / (nx * ny);
        s += V[t] * P0[z] * P1[y] * P2[x];
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) co[((size_t)g * L + b) * L + a] = s;
    }
}

cudaError_t launch_collocate_core(const int length[3], int L, const double *co, const double *pol, int ld,
                                  double *out, cudaStream_t s) {
    const int smem = 8 * (L * L + length[1] * L);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute((const void *)k_collocate_core,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
    }
    k_collocate_core<<<length[0], 256, smem, s>>>(length[0], length[1], length[2], L, co, pol, ld, out);
    return cudaGetLastError();
}

cudaError_t launch_integrate_core(const int length[3], int L, const double *pol, int ld, const double *V,
                                  double *co, cudaStream_t s) {
    k_integrate_core<<<L * L * L, 256, 0, s>>>(length[0], length[1], length[2], L, pol, ld, V, co);
    return cudaGetLastError();
}

}  // namespace gpw
