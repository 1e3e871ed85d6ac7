// Tricubic multi-orbital B-spline evaluation shared by the move and recompute kernels
// (spline2::evaluate_vgh_impl, src/spline2/MultiBsplineVGLH.hpp:120-230, and
// SplineR2R::assign_vgl, src/QMCWaveFunctions/BsplineFactory/SplineR2R.cpp:338-374,
// restricted to orthorhombic cells where the Laplacian only needs hxx, hyy, hzz).
#pragma once
#include "common.cuh"

namespace qmcg
{
template<typename T>
struct Vec;
// FP32 coefficients are read as float2: with 128-512 threads per walker and 192-768
// orbitals this gives a whole number of (column, x-plane) units per thread (measured
// 4% faster at 192 orbitals than float4, which left half the threads idle in the
// last pass over the units)
template<>
struct Vec<float>
{
  using type            = float2;
  static constexpr int W = 2;
  static __device__ __forceinline__ void load(const float* p, float (&o)[2])
  {
    const float2 v = __ldg(reinterpret_cast<const float2*>(p));
    o[0] = v.x;
    o[1] = v.y;
  }
};
template<>
struct Vec<double>
{
  using type            = double2;
  static constexpr int W = 2;
  static __device__ __forceinline__ void load(const double* p, double (&o)[2])
  {
    const double2 v = __ldg(reinterpret_cast<const double2*>(p));
    o[0] = v.x;
    o[1] = v.y;
  }
};

// fractional coordinates of pos in [0, 1): the FP64 part of a spline evaluation, which
// one thread can do for a whole CTA (FP64 arithmetic is slow on this GPU)
template<typename T>
__device__ __forceinline__ void spline_frac(const DevState<T>& s, const double pos[3], T ru[3])
{
#pragma unroll
  for (int d = 0; d < 3; d++)
  {
    T u = static_cast<T>(pos[d] * s.G[d]); // CrystalLattice::toUnit: r . G
    if (-Eps<T>::v < u && u < T(0))
      u = T(0);
    else
      u -= floor(u);
    ru[d] = u;
  }
}

// ---------------------------------------------------------------------------
// Tricubic spline VGL of all orbitals at one position, split over the block:
// a work unit is (orbital vector c, x-offset i); it reads the 16 (y,z) rows of
// its x-plane with vector loads that are contiguous over orbitals, and writes
// 7 partial sums (v, gx, gy, gz, hxx, hyy, hzz) to part[i][7][lda].
// ---------------------------------------------------------------------------
// Units [u_lo, u_hi) are handed to threads t, t + nt, ... (t = the caller's rank).
template<typename T>
__device__ __forceinline__ void spline_partials_frac(const DevState<T>& s, const T ru[3], T* part,
                                                     int t = threadIdx.x, int nt = blockDim.x, int u_lo = 0,
                                                     int u_hi = 1 << 30);

template<typename T>
__device__ __forceinline__ void spline_partials(const DevState<T>& s, const double pos[3], T* part,
                                                int t = threadIdx.x, int nt = blockDim.x, int u_lo = 0,
                                                int u_hi = 1 << 30)
{
  T ru[3];
  spline_frac(s, pos, ru);
  spline_partials_frac(s, ru, part, t, nt, u_lo, u_hi);
}

template<typename T>
__device__ __forceinline__ void spline_partials_frac(const DevState<T>& s, const T ru[3], T* part, int t, int nt,
                                                     int u_lo, int u_hi)
{
  constexpr int W = Vec<T>::W;
  int ix, iy, iz;
  T tx, ty, tz;
  spline_bound(ru[0] * T(s.gx), s.gx - 1, ix, tx);
  spline_bound(ru[1] * T(s.gy), s.gy - 1, iy, ty);
  spline_bound(ru[2] * T(s.gz), s.gz - 1, iz, tz);
  T a[4], da[4], d2a[4], b[4], db[4], d2b[4], c[4], dc[4], d2c[4];
  bspline_weights(tx, a, da, d2a);
  bspline_weights(ty, b, db, d2b);
  bspline_weights(tz, c, dc, d2c);
  const int ncol  = s.lda / W;
  const T* origin = s.coefs + ix * s.xs + iy * s.ys + iz * s.zs;
  const int u_end = min(4 * ncol, u_hi);
  for (int unit = u_lo + t; unit < u_end; unit += nt)
  {
    const int col = unit % ncol;
    const int i   = unit / ncol;
    const T* bi   = origin + i * s.xs + col * W;
    T acc[7][W];
#pragma unroll
    for (int q = 0; q < 7; q++)
#pragma unroll
      for (int w = 0; w < W; w++)
        acc[q][w] = T(0);
    T ai = a[0], dai = da[0], d2ai = d2a[0];
#pragma unroll
    for (int q = 1; q < 4; q++)
      if (i == q)
      {
        ai   = a[q];
        dai  = da[q];
        d2ai = d2a[q];
      }
    T vall[4][4][W];
#pragma unroll
    for (int j = 0; j < 4; j++)
#pragma unroll
      for (int kk = 0; kk < 4; kk++)
        Vec<T>::load(bi + j * s.ys + kk * s.zs, vall[j][kk]);
#pragma unroll
    for (int j = 0; j < 4; j++)
    {
      T(&v)[4][W] = vall[j];
      const T pre00 = ai * b[j], pre10 = dai * b[j], pre01 = ai * db[j], pre20 = d2ai * b[j], pre02 = ai * d2b[j];
#pragma unroll
      for (int w = 0; w < W; w++)
      {
        const T s0 = c[0] * v[0][w] + c[1] * v[1][w] + c[2] * v[2][w] + c[3] * v[3][w];
        const T s1 = dc[0] * v[0][w] + dc[1] * v[1][w] + dc[2] * v[2][w] + dc[3] * v[3][w];
        const T s2 = d2c[0] * v[0][w] + d2c[1] * v[1][w] + d2c[2] * v[2][w] + d2c[3] * v[3][w];
        acc[0][w] += pre00 * s0;
        acc[1][w] += pre10 * s0;
        acc[2][w] += pre01 * s0;
        acc[3][w] += pre00 * s1;
        acc[4][w] += pre20 * s0;
        acc[5][w] += pre02 * s0;
        acc[6][w] += pre00 * s2;
      }
    }
#pragma unroll
    for (int q = 0; q < 7; q++)
#pragma unroll
      for (int w = 0; w < W; w++)
        part[(i * 7 + q) * s.lda + col * W + w] = acc[q][w];
  }
}

// combine the four x-plane partials of orbital o into Cartesian v, grad, laplacian
template<typename T>
__device__ __forceinline__ void spline_combine(const DevState<T>& s, const T* part, int o, T out[5])
{
  T r[7];
#pragma unroll
  for (int q = 0; q < 7; q++)
    r[q] = part[(0 * 7 + q) * s.lda + o] + part[(1 * 7 + q) * s.lda + o] + part[(2 * 7 + q) * s.lda + o] +
        part[(3 * 7 + q) * s.lda + o];
  const T fx = s.grid_scale[0], fy = s.grid_scale[1], fz = s.grid_scale[2];
  out[0] = r[0];
  out[1] = r[1] * fx;
  out[2] = r[2] * fy;
  out[3] = r[3] * fz;
  out[4] = r[4] * (fx * fx) + r[5] * (fy * fy) + r[6] * (fz * fz);
}

} // namespace qmcg
