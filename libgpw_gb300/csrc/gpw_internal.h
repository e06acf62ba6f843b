// Internal host-side interfaces between the C ABI and the kernel files.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "gpw_common.cuh"

namespace gpw {

struct GridPtrs {
    double *p[GPW_MAX_LEVELS];
};

// A contiguous run of sorted tasks launched together (same kind, similar size).
struct Chunk {
    int first, count;
    int smem_bytes;
    int smem_ext;  // with two extra powers (backward moments)
    int kind;      // 0 ortho, 1 general
};

struct Plan {
    int device = 0;
    int nlevels = 0;
    LevelDev lv[GPW_MAX_LEVELS];
    LevelDev *d_levels = nullptr;
    double *d_tmat = nullptr;  // lattice transforms of general levels
    std::vector<double> h_tmat;
};

struct MixedState;  // tiled path, gpw_mixed.cu
constexpr int kDefaultTileLz = 3;  // tiles of 32 x 16 x 8 points until set or tuned
constexpr int kUntiled = -1;       // a general-cell level on the float-float kernel

struct TaskSet {
    Plan *plan = nullptr;
    int tau = 0;                   // gpw_function of the task set (0: rho, 1: tau, 2-4: ADBmDAB x/y/z)
    int64_t ntasks = 0;
    int64_t pab_extent = 0;
    int max_lp = 0;
    int max_A = 0, max_B = 0;
    std::vector<PairGeom> h_geom;  // sorted (stale after a device geometry update until refreshed)
    bool h_geom_stale = false;
    PairGeom *d_geom = nullptr;
    PairGeom *d_geom_next = nullptr;  // geometry updates are written here, then swapped in
    int *d_table = nullptr;        // random-access cube lists (explicit tables)
    double *d_coef = nullptr;      // packed coefficients, per call
    double *d_mom = nullptr;       // packed moments (integrate), per call
    int64_t coef_len = 0;
    int64_t mom_ext_len = 0;
    double *d_mom_ext = nullptr;   // backward: moments up to degree lp + 2
    int *d_status = nullptr;
    std::vector<Chunk> chunks;     // FP64 launches
    MixedState *mixed = nullptr;
    int tile_lz[GPW_MAX_LEVELS];   // tiled path: log2 of the tile's z extent per level
    int gen_first = 0, gen_count = 0, gen_smem = 0;  // general-cell pairs (float-float kernel)
    // profiling (gpw_taskset_profile / gpw_taskset_stats)
    bool profile = false;
    mutable std::vector<cudaEvent_t> ev_pool;
    mutable size_t ev_used = 0;
    mutable int64_t n_kernels = 0;
    mutable int64_t n_contract = 0;
};

// Brackets a contraction launch with events when profiling is on.
struct ProfScope {
    const TaskSet &ts;
    cudaStream_t s;
    ProfScope(const TaskSet &t, cudaStream_t st) : ts(t), s(st) {
        ts.n_kernels++;
        ts.n_contract++;
        if (ts.profile) record();
    }
    ~ProfScope() {
        if (ts.profile) record();
    }
    void record() {
        if (ts.ev_used == ts.ev_pool.size()) {
            cudaEvent_t e;
            if (cudaEventCreate(&e) != cudaSuccess) return;
            ts.ev_pool.push_back(e);
        }
        cudaEventRecord(ts.ev_pool[ts.ev_used++], s);
    }
};

// gpw_fp64.cu
cudaError_t launch_prep(const TaskSet &ts, const double *d_pab, cudaStream_t s);
cudaError_t launch_collocate_fp64(const TaskSet &ts, const GridPtrs &g, cudaStream_t s);
cudaError_t launch_integrate_fp64(const TaskSet &ts, const GridPtrs &g, cudaStream_t s);
// kind: 0 orthorhombic chunks, 1 general-cell chunks, -1 all
cudaError_t launch_fp64_kind(const TaskSet &ts, const GridPtrs &g, bool adj, int kind, cudaStream_t s);
cudaError_t launch_backtransform(const TaskSet &ts, const double *d_mom, double *d_hab,
                                 cudaStream_t s);
int smem_ortho_fp64(const PairGeom &g, int extra = 0);
int smem_general_fp64(const PairGeom &g, int extra = 0);
// moments <V | t^k...> up to degree lp + extra into out (offsets coef_off, or mom_ext_off when extra > 0)
cudaError_t launch_moments_fp64(const TaskSet &ts, const GridPtrs &g, int extra, double *out, cudaStream_t s);
int smem_prep(int A, int B);
cudaError_t fp64_kernel_attributes(int smem_max);

// gpw_core.cu
cudaError_t launch_collocate_core(const int length[3], int L, const double *co, const double *pol,
                                  int ld, double *out, cudaStream_t s);
cudaError_t launch_integrate_core(const int length[3], int L, const double *pol, int ld,
                                  const double *V, double *co, cudaStream_t s);

// gpw_mixed.cu
int mixed_build(TaskSet &ts, std::string &err);
int mixed_rebin(TaskSet &ts, std::string &err);  // records and bins from ts.d_geom
int64_t mixed_items(const TaskSet &ts);           // (tile, pair) items of the tiled path
int64_t mixed_units(const TaskSet &ts);           // its work units
void mixed_free(TaskSet &ts);
cudaError_t launch_collocate_mixed(const TaskSet &ts, const GridPtrs &g, cudaStream_t s);
cudaError_t launch_general_ff(const TaskSet &ts, const GridPtrs &g, bool adj, cudaStream_t s);
int smem_general_ff(const PairGeom &g);
cudaError_t launch_integrate_mixed(const TaskSet &ts, const GridPtrs &g, cudaStream_t s);

// gpw_capi.cu (host helpers)
int level_from_desc(const gpw_grid_desc &d, LevelDev &v);
int host_pair_geom(const gpw_task &t, int idx, const LevelDev &lv, int tau, PairGeom &g);
void set_last_error(const std::string &msg);

// gpw_fp64.cu: set-up + orthorhombic collocate of n pairs from raw device pointers
cudaError_t launch_pairs_fp64(const PairGeom *d_geoms, const LevelDev *d_levels, const double *d_tmat,
                              double *d_coef, int *d_status, int n, int tau, int max_A, int max_B,
                              int smem_coll, const double *d_pab, double *d_grid, cudaStream_t s);

// gpw_fp64.cu: one pair (the drop-in entry): set-up + collocation from raw device pointers
cudaError_t launch_one_fp64(const PairGeom &g, const PairGeom *d_geom, const LevelDev *d_levels, const double *d_tmat,
                            const int *d_table, double *d_coef, int *d_status, int func, const double *d_pab,
                            double *d_grid, cudaStream_t s);

// gpw_selftest.cu
int tc_selftest(int64_t *mismatches, std::string &err);
int ffexp_selftest(int64_t n, double *err_normal, double *err_low, std::string &err);

// gpw_backward.cu
cudaError_t launch_backward(const TaskSet &ts, const double *d_pab, const GridPtrs &g,
                            double *d_hab, double *d_dra, double *d_drb, double *d_dza,
                            double *d_dzb, cudaStream_t s);

}  // namespace gpw
