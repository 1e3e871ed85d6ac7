// C entry point around the reference's own tricubic multi-spline VGH evaluation
// (spline2::evaluate_vgh_impl, src/spline2/MultiBsplineVGLH.hpp:120-230, and
// computeLocationAndFractional, src/spline2/MultiBsplineEval_helper.hpp:65-95),
// compiled in place from the reference sources by oracle/build_ref.sh.  Test
// infrastructure only: it cross-checks the oracle's restatement.
#include <cstdint>
#include <cstring>
#include <vector>

#include "spline2/MultiBsplineEval_helper.hpp"
#include "spline2/MultiBsplineVGLH.hpp"

extern "C" int ref_spline_vgh(const int* grid, int npad, const double* coefs, int norb, const double* u, double* v,
                              double* g, double* h)
{
  multi_UBspline_3d_d sp;
  std::memset(&sp, 0, sizeof(sp));
  sp.coefs    = const_cast<double*>(coefs);
  sp.z_stride = npad;
  sp.y_stride = (intptr_t)(grid[2] + 3) * npad;
  sp.x_stride = (intptr_t)(grid[1] + 3) * sp.y_stride;
  Ugrid* gs[3] = {&sp.x_grid, &sp.y_grid, &sp.z_grid};
  for (int d = 0; d < 3; d++)
  {
    gs[d]->start     = 0.0;
    gs[d]->end       = 1.0;
    gs[d]->num       = grid[d];
    gs[d]->delta     = 1.0 / grid[d];
    gs[d]->delta_inv = grid[d];
  }
  sp.num_splines = npad;
  spline2::evaluate_vgh_impl<double>(&sp, u[0], u[1], u[2], v, g, h, norb, 0, norb);
  return 0;
}
