/*
 * gpw.h -- C ABI of libgpw_gb300: collocate / integrate of Gaussian-pair
 * densities on periodic real-space grids, on one NVIDIA GB300 (sm_103a).
 *
 * Every entry point takes plain pointers and sizes, returns an int status
 * (GPW_SUCCESS == 0) and never aborts or traps.  A failed call leaves a
 * message for gpw_last_error_string().  Device pointers are owned by the
 * caller; plans and task sets own their workspaces.
 *
 * Reference interfaces replaced (mtaillefumier/libgpw):
 *   grid_collocate_pgf_product_rspace   src/lib/grid_base_ref_c.h:40-67
 *                                       src/lib/grid_base_ref_c.cc:1018-1185
 *   collocate_core<T> / integrate_core<T> src/lib/collocate.cc:543-623, :438-541
 *   integrate<T> (grid -> matrix elements) src/lib/collocate.cc:626-679
 */
#ifndef GPW_H
#define GPW_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GPW_MAX_LEVELS 8
#define GPW_MAX_L 4          /* largest la_max / lb_max of one primitive    */
#define GPW_MAX_LP 10        /* la_max + lb_max (+2 for the derivative functions) */

enum gpw_status {
    GPW_SUCCESS = 0,
    GPW_ERR_INVALID_ARG = 1,   /* bad argument, caught on the host           */
    GPW_ERR_CUDA = 2,          /* CUDA runtime error                          */
    GPW_ERR_OUT_OF_WINDOW = 3, /* a non-periodic cube leaves the local grid   */
    GPW_ERR_UNSUPPORTED = 4,   /* valid input that this build does not handle */
    GPW_ERR_NO_DEVICE = 5,
    GPW_ERR_ALLOC = 6,
    GPW_ERR_TIMEOUT = 7        /* a bounded device wait gave up               */
};

/*
 * The function of each pair that collocate maps onto the grid (and integrate
 * takes the adjoint of), with phi_a, phi_b the pair's Cartesian Gaussians and
 * P the density block:
 *   GPW_FUNC_AB          sum P phi_a phi_b                 (rho, grid_base_ref_c.cc:158-192)
 *   GPW_FUNC_DADB        sum P 1/2 grad phi_a . grad phi_b (tau, grid_base_ref_c.cc:65-155;
 *                        compute_polynomial_coefficients_DADB, coefficient.hpp:67-196)
 *   GPW_FUNC_ADBMDAB_X   sum P (phi_a d_x phi_b - d_x phi_a phi_b), and _Y, _Z
 *                        (compute_polynomial_coefficients_ADBmDAB, coefficient.hpp:209-354,
 *                        restated with accumulation throughout)
 * The values 0 and 1 keep the meaning of the reference's compute_tau flag.
 */
enum gpw_function {
    GPW_FUNC_AB = 0,
    GPW_FUNC_DADB = 1,
    GPW_FUNC_ADBMDAB_X = 2,
    GPW_FUNC_ADBMDAB_Y = 3,
    GPW_FUNC_ADBMDAB_Z = 4
};

/* Arithmetic of the cube contraction. */
enum gpw_precision {
    GPW_PREC_FP64 = 0,   /* plain FP64 kernels, one CTA per pair, FP64 atomics   */
    GPW_PREC_MIXED = 1   /* tiled kernels: FP64 pair set-up, split-FP32 tables,   */
                         /* tensor-core cube contraction, compensated            */
                         /* accumulation, one FP64 write per grid point          */
};

/*
 * One grid level.  Mirrors the geometry arguments of
 * grid_collocate_pgf_product_rspace (grid_base_ref_c.h:20-27,49-56).
 * The grid array of a level is double[ngrid[2]][ngrid[1]][ngrid[0]] (x fastest),
 * as the reference's mdarray<double,3,CblasRowMajor> grid(k,j,i).
 * dh[i] is the step vector of grid axis i (Cartesian), dh_inv its inverse,
 * used transposed as in grid_base_ref_c.cc:539.
 */
typedef struct gpw_grid_desc {
    int npts[3];
    int ngrid[3];
    int lb_grid[3];
    int periodic[3];
    double dh[3][3];
    double dh_inv[3][3];
    int ortho;       /* 1: orthorhombic algorithm (use_ortho), 0: general cell */
    int pad_;
} gpw_grid_desc;

/*
 * One primitive pair (task).  Mirrors the per-call scalar arguments of
 * grid_collocate_pgf_product_rspace (grid_base_ref_c.h:40-66).
 * The density block element P(jco, ico) is pab[pab_offset + (o2+jco)*maxco + (o1+ico)]
 * with ico/jco the Cartesian (coset) indices of a and b, as pab(o2+jco, o1+ico)
 * in grid_base_ref_c.cc:185.  Integrate writes matrix elements to the same
 * place of its hab buffer.
 * Cube shape: sphere_offset < 0 takes the cube from `radius` by the library's
 * sphere rule (gpw_sphere_bounds); otherwise the cube is the CP2K-format
 * run-length list at sphere_table[sphere_offset...] with lb_cube/ub_cube
 * (grid_base_ref_c.cc:413-471).
 */
typedef struct gpw_task {
    double zeta, zetb, rscale;
    double ra[3];
    double rab[3];
    double radius;
    int64_t pab_offset;
    int64_t sphere_offset;
    int la_max, la_min, lb_max, lb_min;
    int level;
    int maxco;
    int o1, o2;
    int lb_cube[3];
    int ub_cube[3];
} gpw_task;

typedef struct gpw_plan gpw_plan;       /* grid levels bound to one device   */
typedef struct gpw_taskset gpw_taskset; /* uploaded, sorted and binned pairs */

/* Last error message of the calling thread ("" if none). */
const char *gpw_last_error_string(void);

/* Library version string. */
const char *gpw_version(void);

/*
 * The library's cube rule.  For a sphere of `radius` on an orthorhombic grid
 * with steps dh[0][0], dh[1][1], dh[2][2], writes lb_cube/ub_cube and the
 * CP2K-format run-length list (kgmin, then per kg: jgmin, then per jg: igmin)
 * that grid_collocate_core consumes (grid_base_ref_c.cc:413-471).  Returns the
 * list length, or -needed if cap is too small, or 0 on a bad argument.
 * Pure host function.
 */
int gpw_sphere_bounds(double radius, const double dh[3][3], int lb_cube[3],
                      int ub_cube[3], int *sphere_bounds, int cap);

/* Plans ---------------------------------------------------------------- */
int gpw_plan_create(gpw_plan **plan, int nlevels, const gpw_grid_desc *levels,
                    int device);
int gpw_plan_destroy(gpw_plan *plan);

/*
 * Uploads and analyses a task list (host memory) for repeated collocate /
 * integrate calls: validation, sorting by level and grid tile, per-tile work
 * lists.  func (enum gpw_function) selects the collocated function; 0 and 1
 * are the reference's compute_tau = false / true (grid_base_ref_c.cc:889-900).
 * sphere_table (host, may be NULL) holds the CP2K-format lists that tasks with
 * sphere_offset >= 0 index.  Allocates device memory; synchronous.
 */
int gpw_taskset_create(gpw_plan *plan, const gpw_task *tasks, int64_t ntasks,
                       int func, const int *sphere_table,
                       int64_t sphere_table_len, gpw_taskset **out);
int gpw_taskset_destroy(gpw_taskset *ts);
/* Number of elements the pab / hab buffer must hold for this task set. */
int64_t gpw_taskset_pab_extent(const gpw_taskset *ts);

/*
 * grid[level] += sum over tasks of the pair density (grid_base_ref_c.cc:1018).
 * d_pab and d_grids[l] are device pointers; asynchronous on `stream`
 * (a cudaStream_t, NULL = legacy default); no allocation, so the call can be
 * captured in a CUDA graph.  A task set's work buffers (coefficients, moments,
 * work queues) serve one call at a time: calls on one task set that could
 * overlap on the GPU belong on one stream; different task sets are independent.
 */
int gpw_collocate(gpw_taskset *ts, int precision, const double *d_pab,
                  double *const *d_grids, void *stream);

/*
 * d_hab += <V | pair basis functions>: the adjoint of gpw_collocate with respect
 * to the density block (the role of integrate<T>, collocate.cc:626-679).
 */
int gpw_integrate(gpw_taskset *ts, int precision, double *const *d_grids,
                  double *d_hab, void *stream);

/*
 * Backward pass of E = sum_levels <V_level, rho_level>: with V given per level,
 * accumulates dE/dpab into d_hab (== gpw_integrate), and per task dE/dRa,
 * dE/dRb (double[3*ntasks], task order as given) and dE/dzeta, dE/dzetb
 * (double[ntasks]).  Any of the gradient outputs may be NULL.  Recomputes the
 * 1-D tables; stores nothing between forward and backward.
 */
int gpw_backward(gpw_taskset *ts, const double *d_pab, double *const *d_grids,
                 double *d_hab, double *d_dra, double *d_drb, double *d_dzeta,
                 double *d_dzetb, void *stream);

/*
 * Waits for `stream` and reports device-side error flags raised since the
 * last check (e.g. GPW_ERR_OUT_OF_WINDOW, GPW_ERR_TIMEOUT).
 */
int gpw_taskset_check(gpw_taskset *ts, void *stream);

/*
 * New centres and exponents for the same pairs (a geometry step of a force or
 * molecular-dynamics loop), without rebuilding the task set: d_ra and d_rab
 * (double[3 * ntasks]) and d_zeta, d_zetb (double[ntasks]) are device arrays in
 * the task order given to gpw_taskset_create; a NULL array keeps the current
 * values.  The pair set-up (zeta_p, prefactor, product centre, cube or box
 * placement; grid_base_ref_c.cc:878-886) runs on the device in FP64 and the
 * tiled path's bins are rebuilt on the device.  Radii, shells, cube lists and
 * the density-block layout stay as created.  Synchronous; no launch of the task
 * set may be in flight.  On an error (non-finite or non-positive inputs, a cube
 * that would leave a non-periodic window) the task set is left unchanged.
 * No reference counterpart: the reference sets a pair up on every call.
 */
int gpw_taskset_update_geometry(gpw_taskset *ts, const double *d_ra, const double *d_rab,
                                const double *d_zeta, const double *d_zetb, void *stream);

/*
 * Profiling counters of a task set, for benchmarks.  With enable != 0 the
 * library brackets each cube-contraction launch with CUDA events on the
 * launching stream.  gpw_taskset_stats waits for the device, returns the
 * accumulated device time of those launches (ms) and their number, and the
 * number of kernels the library launched for this task set, then resets all
 * three.  Any output pointer may be NULL.
 */
int gpw_taskset_profile(gpw_taskset *ts, int enable);
/* Diagnostics of the tiled path: its (tile, pair) items and work units (0 and
 * 0 when the task set has no tiled pairs). */
int gpw_taskset_bins(const gpw_taskset *ts, int64_t *items, int64_t *units);
int gpw_taskset_stats(gpw_taskset *ts, double *contraction_ms,
                      int64_t *contraction_launches, int64_t *kernel_launches);

/*
 * Tile shapes of the mixed-precision (tiled) path.  A level is cut into tiles
 * of 32 x (128 / tz) x tz grid points (x, y, z), tz = 4 or 8; the shape sets
 * how many tiles a cube touches and how much per-tile work a pair costs.  A
 * general-cell level may also take tz = 0 (its default): no tiles, its pairs
 * run on the float-float kernel, one CTA per pair.  No reference counterpart:
 * the reference has no tiled path; the shapes change the speed, not the
 * results beyond rounding.
 *
 * gpw_taskset_set_tiles takes tz per level (nlevels entries) and re-bins the
 * task set; gpw_taskset_get_tiles returns the current tz per level.  Both wait
 * for the device: call them when no launch of this task set is in flight.
 *
 * gpw_taskset_autotune times one mixed collocate + integrate of the task set on
 * `stream` for each candidate tz of each level that holds tasks (one level at
 * a time, the others at their best so far), keeps the fastest and writes tz
 * per level to tile_z (may be NULL) and the measured ms to ms[3 * level + c]
 * for the candidates tz = 8, 4, 0 (tz = 0 on general-cell levels only; -1
 * where not timed; may be NULL).  d_pab is a density buffer as for
 * gpw_collocate.  The timed calls run on scratch grids and matrix elements
 * allocated here; the caller's buffers are not written.
 */
int gpw_taskset_set_tiles(gpw_taskset *ts, const int *tile_z);
int gpw_taskset_get_tiles(const gpw_taskset *ts, int *tile_z);
int gpw_taskset_autotune(gpw_taskset *ts, const double *d_pab, int *tile_z, double *ms, void *stream);

/*
 * Tensor-core self test on the current device: one fp16 MMA with FP32
 * accumulation (M=128, N=32, K=16) on integer-valued operands in the operand
 * layout the mixed path uses, compared exactly with the integer products.
 * *mismatches receives the number of wrong elements (0 when the path works).
 */
int gpw_selftest_tensorcore(int64_t *mismatches);

/*
 * Self test of the float-float exponential of the mixed path (no reference
 * counterpart): npoints arguments over [-60, 88) and npoints / 4 over [-103, -60),
 * each a float-float value (a low part of up to half an ulp), against the FP64
 * exp of the same value on the current device.  *max_rel_err receives the
 * largest relative error where the result has a normal low part (a > -60),
 * *max_rel_err_low the largest error below, relative to max(exp(a), 2^-126):
 * there the low part, and below a = -87.3 the high part too, are subnormal.
 */
int gpw_selftest_ff_exp(int64_t npoints, double *max_rel_err, double *max_rel_err_low);

/*
 * Collocation that allocates no device memory (no counterpart in the
 * reference).  For callers that cannot allocate on their call path, because
 * their device memory belongs to their own pool allocator.  Collocates up to
 * GPW_NOALLOC_MAX_TASKS pairs on one orthorhombic level: d_grid (device,
 * double[ngrid[2]][ngrid[1]][ngrid[0]]) += rho, with the density blocks in
 * d_pab (device, addressed as in gpw_task).  Tasks use level 0 and the radius
 * rule (sphere_offset < 0).  FP64 arithmetic, the plain FP64 kernels.
 * The scratch (level, pair geometry, coefficients, about 200 KB) is one
 * fixed device array in the library, held by every GPU that loads it until
 * the process exits; its device address is looked up on the first call on
 * each device (make that first call with the device current, and before any
 * stream capture begins).  All calls
 * share it: calls that overlap on the GPU (different streams or threads
 * without ordering) race.  Waits for `stream` before returning and reports
 * the kernels' error flags as gpw_taskset_check does (GPW_ERR_OUT_OF_WINDOW
 * when a cube left a non-periodic window).
 * Larger batches: gpw_taskset_create / gpw_collocate.
 */
#define GPW_NOALLOC_MAX_TASKS 64
int gpw_collocate_noalloc(const gpw_grid_desc *level, const gpw_task *tasks,
                          int ntasks, int compute_tau, const double *d_pab,
                          double *d_grid, void *stream);

/* Host-buffer convenience calls (copies inside, synchronous) -------------
 * The same accumulation as gpw_collocate / gpw_integrate from host arrays
 * (pinned or pageable).  Device staging buffers are allocated on a task set's
 * first host-buffer call and kept until gpw_taskset_destroy; calls on one task
 * set from several host threads must be serialised by the caller. */
int gpw_collocate_host(gpw_taskset *ts, int precision, const double *h_pab,
                       double *const *h_grids);
int gpw_integrate_host(gpw_taskset *ts, int precision, double *const *h_grids,
                       double *h_hab);

/*
 * Drop-in form of grid_collocate_pgf_product_rspace (grid_base_ref_c.h:40-67)
 * with mdarray arguments replaced by raw row-major arrays:
 *   dh, dh_inv   double[3][3]
 *   pab          double[maxco][maxco]
 *   grid         double[ngrid[2]][ngrid[1]][ngrid[0]]  (host, accumulated)
 * Runs the FP64 GPU path on the current device (default 0).  lb_cube, ub_cube
 * and sphere_bounds are read only when use_ortho != 0, as in the reference.
 */
int gpw_collocate_pgf_product_rspace(
    int compute_tau, int use_ortho, int la_max, int la_min, int lb_max,
    int lb_min, double zeta, double zetb, double rscale, const double dh[3][3],
    const double dh_inv[3][3], const double ra[3], const double rab[3],
    const int npts[3], const int ngrid[3], const int lb_grid[3],
    const int periodic[3], int lmax, double radius, const int lb_cube[3],
    const int ub_cube[3], int nspheres, const int *sphere_bounds, int maxco,
    int o1, int o2, const double *pab, double *grid);

/*
 * Dense cube contraction of the factorised prototype, on the device:
 *   collocate_core: out[z][y][x] = sum co[a][g][b] * pol[0][g][z] * pol[1][b][y] * pol[2][a][x]
 *     (collocate.cc:543-623; naive form collocate_test.cc:11-33)
 *   integrate_core: co[g][b][a] = sum V[z][y][x] * pol[0][g][z] * pol[1][b][y] * pol[2][a][x]
 *     (collocate.cc:438-541; naive form collocate_test.cc:77-99)
 * length = {nz, ny, nx}; pol is double[3][L][ld_pol] with ld_pol >= max(length);
 * co is double[L][L][L].  All pointers are device pointers; FP64.
 */
int gpw_collocate_core(const int length[3], int L, const double *d_co,
                       const double *d_pol, int ld_pol, double *d_out,
                       void *stream);
int gpw_integrate_core(const int length[3], int L, const double *d_pol,
                       int ld_pol, const double *d_V, double *d_co,
                       void *stream);

#ifdef __cplusplus
}
#endif
#endif /* GPW_H */
