// Ratios of the trial wavefunction for virtual moves: psi(R with electron e at r') /
// psi(R), the quadrature points of a non-local pseudopotential
// (TrialWaveFunction::mw_evaluateRatios, src/QMCWaveFunctions/TrialWaveFunction.cpp:1079-1110,
// over VirtualParticleSets).  Per virtual move, the three factors:
//   determinant  Ainv[row(e)] . phi(r')  with orbital values only
//                (SplineR2R::mw_evaluateDetRatios, SplineR2R.cpp:204-335,
//                 spline2 evaluate_v: 4x4x4 coefficient rows weighted by a_i b_j c_k)
//   J2           exp(Uat[e] - sum_{j != e} u(|r_j - r'|))
//                (TwoBodyJastrow::mw_evaluateRatios, TwoBodyJastrow.cpp:174-206, with
//                 BsplineFunctor::mw_evaluateV, BsplineFunctor.cpp:135-201)
//   J1           exp(Vat[e] - sum_I u1(|R_I - r'|))  (J1OrbitalSoA::evaluateRatios, J1OrbitalSoA.h:295-299)
// One warp per virtual move: each lane owns 16-byte vectors of consecutive orbitals,
// reads that vector from each of the 64 coefficient rows of the move's grid cell
// (coalesced along the orbital index across the warp), forms the orbital values and
// their product with the inverse row; the Jastrow sums run over the lanes and every sum
// is a warp shuffle reduction.  The walker's delayed updates must be flushed.
#include <cuda_runtime.h>

#include "common.cuh"
#include "launch.h"
#include "spline.cuh"

namespace qmcg
{

template<typename T>
struct VpVec;
template<>
struct VpVec<float>
{
  static constexpr int W = 4;
  static __device__ __forceinline__ void load(const float* p, float (&o)[4])
  {
    const float4 v = __ldg(reinterpret_cast<const float4*>(p));
    o[0] = v.x;
    o[1] = v.y;
    o[2] = v.z;
    o[3] = v.w;
  }
};
template<>
struct VpVec<double>
{
  static constexpr int W = 2;
  static __device__ __forceinline__ void load(const double* p, double (&o)[2])
  {
    const double2 v = __ldg(reinterpret_cast<const double2*>(p));
    o[0] = v.x;
    o[1] = v.y;
  }
};

// cubic B-spline value weights of one axis (MultiBsplineData::compute_prefactors, values)
template<typename T>
__device__ __forceinline__ void bspline_values(T t, T a[4])
{
  a[0] = ((T(-1.0 / 6.0) * t + T(3.0 / 6.0)) * t + T(-3.0 / 6.0)) * t + T(1.0 / 6.0);
  a[1] = ((T(3.0 / 6.0) * t + T(-1.0)) * t + T(0.0)) * t + T(4.0 / 6.0);
  a[2] = ((T(-3.0 / 6.0) * t + T(3.0 / 6.0)) * t + T(3.0 / 6.0)) * t + T(1.0 / 6.0);
  a[3] = ((T(1.0 / 6.0) * t + T(0.0)) * t + T(0.0)) * t + T(0.0);
}

constexpr int VP_NT = 256; // 8 virtual moves per CTA

template<typename T>
__global__ void __launch_bounds__(VP_NT) vp_ratio_kernel(DevState<T> s, int nvp, const int* __restrict__ vp_walker,
                                                         const int* __restrict__ vp_elec,
                                                         const double* __restrict__ vp_pos,
                                                         double* __restrict__ out, int* __restrict__ bad)
{
  constexpr int W = VpVec<T>::W;
  const int lane = threadIdx.x & 31;
  const int v    = blockIdx.x * (VP_NT / 32) + (threadIdx.x >> 5);
  if (v >= nvp)
    return;
  const int w = vp_walker[v], e = vp_elec[v];
  const double pos[3] = {vp_pos[3 * v], vp_pos[3 * v + 1], vp_pos[3 * v + 2]};
  // the arguments are checked here, not on the host: an invalid move reads nothing
  if (w < 0 || w >= s.nw || e < 0 || e >= s.ne || !isfinite(pos[0]) || !isfinite(pos[1]) || !isfinite(pos[2]))
  {
    if (lane == 0)
    {
      out[v] = nan("");
      atomicMin(bad, v);
    }
    return;
  }
  const int spin = e >= s.nup ? 1 : 0, row = e - spin * s.nup;
  // ---------------- determinant: orbital values at r' against the inverse row
  T ru[3];
  spline_frac(s, pos, ru);
  int ix, iy, iz;
  T tx, ty, tz;
  spline_bound(ru[0] * T(s.gx), s.gx - 1, ix, tx);
  spline_bound(ru[1] * T(s.gy), s.gy - 1, iy, ty);
  spline_bound(ru[2] * T(s.gz), s.gz - 1, iz, tz);
  T a[4], b[4], c[4];
  bspline_values(tx, a);
  bspline_values(ty, b);
  bspline_values(tz, c);
  const T* origin = s.coefs + ix * s.xs + iy * s.ys + iz * s.zs;
  const T* inv    = s.Ainv + (((size_t)spin * s.nw + w) * s.norb + row) * s.lda;
  const int nchunk = s.lda / W;
  T det = T(0);
  for (int ch = lane; ch < nchunk; ch += 32)
  {
    T val[W];
#pragma unroll
    for (int q = 0; q < W; q++)
      val[q] = T(0);
#pragma unroll
    for (int i = 0; i < 4; i++)
    {
      T rows[4][4][W];
#pragma unroll
      for (int j = 0; j < 4; j++)
#pragma unroll
        for (int k = 0; k < 4; k++)
          VpVec<T>::load(origin + i * s.xs + j * s.ys + k * s.zs + ch * W, rows[j][k]);
#pragma unroll
      for (int j = 0; j < 4; j++)
      {
        const T ab = a[i] * b[j];
#pragma unroll
        for (int q = 0; q < W; q++)
          val[q] += ab * (c[0] * rows[j][0][q] + c[1] * rows[j][1][q] + c[2] * rows[j][2][q] + c[3] * rows[j][3][q]);
      }
    }
#pragma unroll
    for (int q = 0; q < W; q++)
      if (ch * W + q < s.norb)
        det += val[q] * inv[ch * W + q];
  }
  det = warp_sum(det);
  // ---------------- Jastrow factors
  const T x0 = static_cast<T>(pos[0]), y0 = static_cast<T>(pos[1]), z0 = static_cast<T>(pos[2]);
  const T L0 = T(s.L[0]), L1 = T(s.L[1]), L2 = T(s.L[2]);
  const T Li0 = T(s.G[0]), Li1 = T(s.G[1]), Li2 = T(s.G[2]);
  T u2 = T(0), u1 = T(0);
  if (s.has_j2)
  {
    const T* R = s.Rt + (size_t)w * 3 * s.ne_pad;
    const int same_lo = spin ? s.nup : 0, same_hi = spin ? s.ne : s.nup;
    for (int j = lane; j < s.ne; j += 32)
    {
      if (j == e)
        continue;
      const T dx = min_image(R[j] - x0, L0, Li0);
      const T dy = min_image(R[s.ne_pad + j] - y0, L1, Li1);
      const T dz = min_image(R[2 * s.ne_pad + j] - z0, L2, Li2);
      const T r  = sqrt(dx * dx + dy * dy + dz * dz);
      if (r < s.j2_rcut)
      {
        const int same = j >= same_lo && j < same_hi;
        T du, d2u;
        u2 += functor_eval(s.j2c + (same ? 0 : s.j2_ncoef), s.j2_dri, s.j2_maxidx, r, du, d2u);
      }
    }
    u2 = warp_sum(u2);
  }
  if (s.has_j1)
  {
    for (int I = lane; I < s.nions; I += 32)
    {
      const T dx = min_image(s.ions[I] - x0, L0, Li0);
      const T dy = min_image(s.ions[s.nions_pad + I] - y0, L1, Li1);
      const T dz = min_image(s.ions[2 * s.nions_pad + I] - z0, L2, Li2);
      const T r  = sqrt(dx * dx + dy * dy + dz * dz);
      if (r < s.j1_rcut)
      {
        T du, d2u;
        u1 += functor_eval(s.j1c + (size_t)s.ion_species[I] * s.j1_ncoef, s.j1_dri, s.j1_maxidx, r, du, d2u);
      }
    }
    u1 = warp_sum(u1);
  }
  if (lane == 0)
  {
    T logj = T(0);
    if (s.has_j2)
      logj += s.J2[(size_t)w * 5 * s.ne_pad + e] - u2;
    if (s.has_j1)
      logj += s.J1[(size_t)w * 5 * s.ne_pad + e] - u1;
    // in the move-loop precision, as the move loop forms its ratios: one FP64 exp per move
    // would cost the FP32 kernel a large share of its time on this GPU's FP64 pipe
    out[v] = static_cast<double>(det * exp(logj));
  }
}

template<typename T>
cudaError_t launch_vp_ratios(const DevState<T>& s, int nvp, const int* walker, const int* elec, const double* pos,
                             double* out, int* bad, cudaStream_t st)
{
  if (nvp <= 0)
    return cudaSuccess;
  const int grid = (nvp + VP_NT / 32 - 1) / (VP_NT / 32);
  vp_ratio_kernel<T><<<grid, VP_NT, 0, st>>>(s, nvp, walker, elec, pos, out, bad);
  return cudaGetLastError();
}

template cudaError_t launch_vp_ratios<float>(const DevState<float>&, int, const int*, const int*, const double*,
                                             double*, int*, cudaStream_t);
template cudaError_t launch_vp_ratios<double>(const DevState<double>&, int, const int*, const int*, const double*,
                                              double*, int*, cudaStream_t);

} // namespace qmcg
