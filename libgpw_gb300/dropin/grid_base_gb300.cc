// Drop-in replacement for the reference's FP64 collocate
// (mtaillefumier/libgpw src/lib/grid_base_ref_c.cc): the same C++ function,
// with the same signature as src/lib/grid_base_ref_c.h:40-67, running on the
// GB300 through the C ABI (gpw_collocate_pgf_product_rspace, include/gpw.h).
//
// Build it in the caller's tree in place of grid_base_ref_c.cc, with the
// caller's mdarray.hpp / grid_base_ref_c.h on the include path, and link
// libgpw_gb300.so.  Like the reference it accumulates into `grid`; an error
// from the library is reported on stderr and aborts, as the reference's
// assertions do.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "gpw.h"
#include "grid_base_ref_c.h"

void grid_collocate_pgf_product_rspace(const bool compute_tau, const bool use_ortho, const int la_max,
                                       const int la_min, const int lb_max, const int lb_min, const double zeta,
                                       const double zetb, const double rscale, const double dh[3][3],
                                       const double dh_inv[3][3], const double ra[3], const double rab[3],
                                       const int npts[3], const int ngrid[3], const int lb_grid[3],
                                       const bool periodic[3], const int lmax, const double radius,
                                       const int lb_cube[3], const int ub_cube[3], const int nspheres,
                                       const std::vector<int> &sphere_bounds, const int maxco, const int o1,
                                       const int o2, const mdarray<double, 2, CblasRowMajor> &pab,
                                       mdarray<double, 3, CblasRowMajor> &grid) {
    const int per[3] = {periodic[0] ? 1 : 0, periodic[1] ? 1 : 0, periodic[2] ? 1 : 0};
    const int st = gpw_collocate_pgf_product_rspace(
        compute_tau ? 1 : 0, use_ortho ? 1 : 0, la_max, la_min, lb_max, lb_min, zeta, zetb, rscale, dh, dh_inv,
        ra, rab, npts, ngrid, lb_grid, per, lmax, radius, use_ortho ? lb_cube : nullptr,
        use_ortho ? ub_cube : nullptr, nspheres, sphere_bounds.data(), maxco, o1, o2,
        pab.template at<CPU>(), grid.template at<CPU>());
    if (st != GPW_SUCCESS) {
        std::fprintf(stderr, "grid_collocate_pgf_product_rspace (libgpw_gb300): %s\n", gpw_last_error_string());
        std::abort();
    }
}
