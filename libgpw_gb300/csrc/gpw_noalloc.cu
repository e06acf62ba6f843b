// gpw_collocate_noalloc: collocation of a small batch of pairs that allocates
// no device memory.  Some callers cannot allocate on their call path -- their
// device memory belongs to their own pool allocator (an SCF code's offload
// buffers, a framework's caching allocator) and every other allocation is
// forbidden or too slow to risk.  This entry point works on the caller's input
// and output buffers only; the scratch it needs (the level, the pair
// geometry, the product-centre coefficients and a status word) lives in the
// file-scope device array below, which every GPU that loads the library holds
// until the process exits.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "gpw_internal.h"

namespace gpw {
namespace {

// Scratch capacity: GPW_NOALLOC_MAX_TASKS pairs with lp <= GPW_MAX_LP.
constexpr size_t kScratchBytes =
    256 + sizeof(LevelDev) + GPW_NOALLOC_MAX_TASKS * (sizeof(PairGeom) + sizeof(double) * 286) + 256;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_mu;
unsigned char *g_scratch_ptr[64] = {nullptr};  // device address per device id

// Set-up, once per device, with that device current: the device address of the
// scratch array (in host code its name is only a host-side handle).
int scratch_address(int dev, unsigned char **out) {
    if (dev < 0 || dev >= 64) {
        set_last_error("gpw_collocate_noalloc: device id out of range");
        return GPW_ERR_INVALID_ARG;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            set_last_error(std::string("gpw_collocate_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            return GPW_ERR_CUDA;
        }
        int smem_max = 0;
        cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        const cudaError_t e2 = fp64_kernel_attributes(smem_max);
        if (e2 != cudaSuccess) {
            set_last_error(std::string("gpw_collocate_noalloc: ") + cudaGetErrorString(e2));
            return GPW_ERR_CUDA;
        }
        g_scratch_ptr[dev] = static_cast<unsigned char *>(p);
    }
    *out = g_scratch_ptr[dev];
    return GPW_SUCCESS;
}

}  // namespace
}  // namespace gpw

using namespace gpw;

extern "C" int gpw_collocate_noalloc(const gpw_grid_desc *level, const gpw_task *tasks, int ntasks,
                                     int compute_tau, const double *d_pab, double *d_grid, void *stream) {
    if (!level || (ntasks > 0 && (!tasks || !d_pab)) || !d_grid || ntasks < 0) {
        set_last_error("gpw_collocate_noalloc: null argument or negative task count");
        return GPW_ERR_INVALID_ARG;
    }
    if (ntasks > GPW_NOALLOC_MAX_TASKS) {
        set_last_error("gpw_collocate_noalloc: at most GPW_NOALLOC_MAX_TASKS (" +
                       std::to_string(GPW_NOALLOC_MAX_TASKS) + ") pairs per call, got " + std::to_string(ntasks) +
                       "; use gpw_taskset_create / gpw_collocate for larger batches");
        return GPW_ERR_INVALID_ARG;
    }
    LevelDev lv;
    int st = level_from_desc(*level, lv);
    if (st) return st;
    if (!lv.ortho) {
        set_last_error("gpw_collocate_noalloc: orthorhombic grids only");
        return GPW_ERR_UNSUPPORTED;
    }
    if (ntasks == 0) return GPW_SUCCESS;
    // host geometry, checked exactly as gpw_taskset_create checks it
    std::vector<PairGeom> geo((size_t)ntasks);
    int max_A = 0, max_B = 0, smem_coll = 0;
    int64_t coef = 0;
    for (int i = 0; i < ntasks; i++) {
        if (tasks[i].level != 0 || tasks[i].sphere_offset >= 0) {
            set_last_error("gpw_collocate_noalloc: tasks must use level 0 and the radius rule (sphere_offset < 0)");
            return GPW_ERR_INVALID_ARG;
        }
        st = host_pair_geom(tasks[i], i, lv, compute_tau ? 1 : 0, geo[i]);
        if (st) return st;
        geo[i].coef_off = coef;
        coef += ncoef(geo[i].lp);
        max_A = std::max(max_A, geo[i].la_max);
        max_B = std::max(max_B, geo[i].lb_max);
        smem_coll = std::max(smem_coll, smem_ortho_fp64(geo[i]));
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        set_last_error("gpw_collocate_noalloc: no current CUDA device");
        return GPW_ERR_NO_DEVICE;
    }
    int smem_limit = 0;
    cudaDeviceGetAttribute(&smem_limit, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (smem_coll > smem_limit || smem_prep(max_A, max_B) > smem_limit) {
        set_last_error("gpw_collocate_noalloc: a cube is too large for one CTA");
        return GPW_ERR_UNSUPPORTED;
    }
    unsigned char *base = nullptr;
    st = scratch_address(dev, &base);
    if (st) return st;
    // scratch layout: status word | level | pair geometry | coefficients
    int *d_status = reinterpret_cast<int *>(base);
    LevelDev *d_level = reinterpret_cast<LevelDev *>(base + 256);
    PairGeom *d_geom = reinterpret_cast<PairGeom *>(base + 256 + sizeof(LevelDev));
    double *d_coef = reinterpret_cast<double *>(base + 256 + sizeof(LevelDev) + sizeof(PairGeom) * ntasks);
    const size_t used = 256 + sizeof(LevelDev) + sizeof(PairGeom) * ntasks + sizeof(double) * coef;
    if (used > kScratchBytes) {
        set_last_error("gpw_collocate_noalloc: pairs need more scratch than the fixed array holds");
        return GPW_ERR_INVALID_ARG;
    }
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaMemsetAsync(d_status, 0, sizeof(int), s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_level, &lv, sizeof(LevelDev), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_geom, geo.data(), sizeof(PairGeom) * ntasks, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = launch_pairs_fp64(d_geom, d_level, nullptr, d_coef, d_status, ntasks, compute_tau ? 1 : 0, max_A, max_B,
                              smem_coll, d_pab, d_grid, s);
    // the kernels' error bits, read into a stack variable (a copy, no allocation)
    int flags = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&flags, d_status, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);  // the host copies above read and write stack memory
    if (e != cudaSuccess) {
        set_last_error(std::string("gpw_collocate_noalloc: ") + cudaGetErrorString(e));
        return GPW_ERR_CUDA;
    }
    // the same meaning as in gpw_taskset_check
    if (flags & kStatOutOfWindow) {
        set_last_error("gpw_collocate_noalloc: a cube left the local grid window; its points outside were skipped");
        return GPW_ERR_OUT_OF_WINDOW;
    }
    if (flags & kStatTimeout) {
        set_last_error("gpw_collocate_noalloc: a bounded device wait gave up");
        return GPW_ERR_TIMEOUT;
    }
    if (flags) {
        set_last_error("gpw_collocate_noalloc: device status " + std::to_string(flags));
        return GPW_ERR_INVALID_ARG;
    }
    return GPW_SUCCESS;
}
