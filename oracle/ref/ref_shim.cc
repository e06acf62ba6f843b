// C entry point over the reference's own FP64 collocate
// (grid_collocate_pgf_product_rspace, src/lib/grid_base_ref_c.cc:1018), compiled
// from the reference sources where they lie.  Test infrastructure only: it wraps
// caller arrays in the reference's mdarray (no copies) and calls it unchanged.
#include <vector>
#include "grid_base_ref_c.h"
#include "grid_base_ref_replay.h"
#include "rt_graph.hpp"

rt_graph::Timer timer;  // the reference expects the caller to define it (grid_base_ref_miniapp.cc:13)

extern "C" int gpwref_collocate(
    int compute_tau, int use_ortho, int la_max, int la_min, int lb_max, int lb_min,
    double zeta, double zetb, double rscale, const double *dh9, const double *dh_inv9,
    const double *ra, const double *rab, const int *npts, const int *ngrid,
    const int *lb_grid, const int *periodic_i, int lmax, double radius,
    const int *lb_cube, const int *ub_cube, int nspheres, const int *sphere_bounds,
    int maxco, int o1, int o2, const double *pab_ptr, double *grid_ptr) {
    double dh[3][3], dh_inv[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            dh[i][j] = dh9[3 * i + j];
            dh_inv[i][j] = dh_inv9[3 * i + j];
        }
    bool periodic[3] = {periodic_i[0] != 0, periodic_i[1] != 0, periodic_i[2] != 0};
    std::vector<int> sb(sphere_bounds, sphere_bounds + (nspheres > 0 ? nspheres : 0));
    mdarray<double, 2, CblasRowMajor> pab(const_cast<double *>(pab_ptr), maxco, maxco);
    mdarray<double, 3, CblasRowMajor> grid(grid_ptr, ngrid[2], ngrid[1], ngrid[0]);
    grid_collocate_pgf_product_rspace(compute_tau != 0, use_ortho != 0, la_max, la_min, lb_max,
                                      lb_min, zeta, zetb, rscale, dh, dh_inv, ra, rab, npts,
                                      ngrid, lb_grid, periodic, lmax, radius,
                                      use_ortho ? lb_cube : nullptr,
                                      use_ortho ? ub_cube : nullptr, nspheres, sb, maxco, o1,
                                      o2, pab, grid);
    return 0;
}

// The reference's own task-file replay (grid_collocate_replay,
// src/lib/grid_base_ref_replay.cc:18-274): parses a "Grid collocate task v1"
// file with the reference's reader, collocates it `cycles` times and returns
// the largest difference to the grid values the file pins.  A malformed file
// fails the reader's asserts (the process aborts), so callers run it in a
// child process.
extern "C" double gpwref_replay(const char *path, int cycles) { return grid_collocate_replay(path, cycles); }
