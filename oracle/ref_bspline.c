/* Test infrastructure: the reference's einspline coefficient solve (set_multi_UBspline_3d_d,
 * src/einspline/multi_bspline_create.c) compiled in place, behind one C entry for ctypes.
 * ref_multi_spline_3d_d: data [norb][nx][ny][nz] -> coefs [nx+3][ny+3][nz+3][norb_padded]
 * exactly as the reference stores them (periodic boundaries). */
#include <stdlib.h>
#include <string.h>

#include "multi_bspline_create.h"

void init_sse_data(void) {}

int ref_multi_spline_3d_d(const int* n, int norb, const double* data, double* coefs, int* padded)
{
  Ugrid g[3];
  for (int d = 0; d < 3; d++)
  {
    g[d].start = 0.0;
    g[d].end   = 1.0;
    g[d].num   = n[d];
  }
  BCtype_d bc;
  bc.lCode = bc.rCode = PERIODIC;
  bc.lVal = bc.rVal = 0.0;
  multi_UBspline_3d_d* s = create_multi_UBspline_3d_d(g[0], g[1], g[2], bc, bc, bc, norb);
  if (!s)
    return -1;
  const size_t vol = (size_t)n[0] * n[1] * n[2];
  for (int o = 0; o < norb; o++)
    set_multi_UBspline_3d_d(s, o, (double*)(data + (size_t)o * vol));
  const size_t N = (size_t)(n[0] + 3) * (n[1] + 3) * (n[2] + 3);
  *padded = (int)s->z_stride;
  memcpy(coefs, s->coefs, N * s->z_stride * sizeof(double));
  free(s->coefs);
  free(s);
  return 0;
}
