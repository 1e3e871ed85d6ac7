// Diffusion Monte Carlo on the device: the branch weight of every walker after a
// fixed-node sweep, and the walker copies of population control.
//
// The sweep itself is the walker-resident kernel with DevState::dmc set (moves that
// change the sign of psi rejected, tau |xi|^2 summed over proposed and accepted
// moves).  After it and the local energy, one kernel applies
//   SFNBranch::branchWeight (src/QMCDrivers/SFNBranch.h:199-208):
//     x = max(E_ref - E_new, E_ref - E_old)
//     t = tau_eff / 2, scaled by 1 - (x - cutoff) / (max - cutoff) above the cutoff,
//         0 above max
//     w *= exp(t (2 E_trial - E_new - E_old))
// with the walker's age (DMCBatched.cpp:269-275) and the ensemble sums population
// control reads (WalkerControl::computeCurData, WalkerControl.cpp:243-270):
// sum w, sum w E, sum w E^2, sum r2_accepted, sum r2_proposed, all FP64 in a fixed
// reduction order.  Population control itself decides on the host which walkers
// are copied where; copy_walkers_kernel moves the device state
// (Walker::makeCopy for the MCPopulation of a crowd).
#include <cuda_runtime.h>

#include "common.cuh"
#include "launch.h"

namespace qmcg
{

constexpr int DMC_NT = 1024;

// par: [0] E_trial, [1] E_ref, [2] tau_eff, [3] branch cutoff, [4] branch max
// sums: [0] sum w, [1] sum w E, [2] sum w E^2, [3] sum r2 accepted, [4] sum r2 proposed
__global__ void __launch_bounds__(DMC_NT) dmc_branch_kernel(int nw, const double* __restrict__ e_new,
                                                              double* __restrict__ e_old, double* __restrict__ weight,
                                                              int* __restrict__ age, double* __restrict__ rr,
                                                              const double* __restrict__ par, double* __restrict__ sums,
                                                              double* __restrict__ w_out)
{
  __shared__ double red[5][DMC_NT / 32];
  const double etrial = par[0], eref = par[1], taueff = par[2], bcut = par[3], bmax = par[4];
  const double bfilter = 1.0 / (bmax - bcut);
  double acc[5] = {0, 0, 0, 0, 0};
  for (int iw = threadIdx.x; iw < nw; iw += DMC_NT)
  {
    const double en = e_new[iw], eo = e_old[iw];
    double t       = 0.5 * taueff;
    const double x = fmax(eref - en, eref - eo);
    if (x > bmax)
      t = 0.0;
    else if (x > bcut)
      t *= 1.0 - (x - bcut) * bfilter;
    const double w = weight[iw] * exp(t * (2.0 * etrial - en - eo));
    weight[iw]     = w;
    w_out[iw]      = w;
    e_old[iw]      = en;
    const double rp = rr[2 * iw], ra = rr[2 * iw + 1];
    age[iw]         = rp > 0 ? 0 : age[iw] + 1;
    rr[2 * iw]      = 0.0;
    rr[2 * iw + 1]  = 0.0;
    acc[0] += w;
    acc[1] += w * en;
    acc[2] += w * en * en;
    acc[3] += ra;
    acc[4] += rp;
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < 5; q++)
  {
    double v = acc[q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
      v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0)
      red[q][wid] = v;
  }
  __syncthreads();
  if (wid == 0)
#pragma unroll
    for (int q = 0; q < 5; q++)
    {
      double v = red[q][lane];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0)
        sums[q] = v;
    }
}

cudaError_t launch_dmc_branch(int nw, const double* e_new, double* e_old, double* weight, int* age, double* rr,
                              const double* par, double* sums, double* w_out, cudaStream_t st)
{
  dmc_branch_kernel<<<1, DMC_NT, 0, st>>>(nw, e_new, e_old, weight, age, rr, par, sums, w_out);
  return cudaGetLastError();
}

// 16-byte copies of one contiguous block (sizes and addresses are multiples of 16 bytes)
__device__ __forceinline__ void copy16(void* dst, const void* src, size_t bytes)
{
  int4* d       = static_cast<int4*>(dst);
  const int4* s = static_cast<const int4*>(src);
  for (size_t i = threadIdx.x; i < bytes / 16; i += blockDim.x)
    d[i] = s[i];
}

// Walker w takes the state of walker src[w] (nothing happens where src[w] == w).  Every
// source walker keeps its own state (src[src[w]] == src[w], checked on the host), so
// the copies of one launch never read a walker another block writes.  Delayed updates
// must be flushed (only the inverse, not U, V or Binv, is copied).  Weights of every
// walker are set to 1 (WalkerControl::branch, WalkerControl.cpp:224-231).
template<typename T>
__global__ void __launch_bounds__(256) copy_walkers_kernel(DevState<T> s, const int* __restrict__ src,
                                                           double* __restrict__ weight, double* __restrict__ e_old,
                                                           int* __restrict__ age)
{
  const int w = blockIdx.x, f = src[w];
  if (threadIdx.x == 0)
    weight[w] = 1.0;
  if (f == w)
    return;
  const size_t N = s.norb, lda = s.lda, np = s.ne_pad, nw = s.nw;
  copy16(s.R + (size_t)w * 3 * np, s.R + (size_t)f * 3 * np, 3 * np * sizeof(double));
  copy16(s.Rt + (size_t)w * 3 * np, s.Rt + (size_t)f * 3 * np, 3 * np * sizeof(T));
  copy16(s.J2 + (size_t)w * 5 * np, s.J2 + (size_t)f * 5 * np, 5 * np * sizeof(T));
  copy16(s.J1 + (size_t)w * 5 * np, s.J1 + (size_t)f * 5 * np, 5 * np * sizeof(T));
  for (int spin = 0; spin < 2; spin++)
  {
    const size_t dw = (size_t)spin * nw + w, fw = (size_t)spin * nw + f;
    copy16(s.Ainv + dw * N * lda, s.Ainv + fw * N * lda, N * lda * sizeof(T));
    copy16(s.dgrad + dw * N * 3 * lda, s.dgrad + fw * N * 3 * lda, N * 3 * lda * sizeof(T));
    copy16(s.dlap + dw * N * lda, s.dlap + fw * N * lda, N * lda * sizeof(T));
    copy16(s.psiv + dw * N * lda, s.psiv + fw * N * lda, N * lda * sizeof(T));
  }
  if (threadIdx.x == 0)
  {
    for (int spin = 0; spin < 2; spin++)
    {
      s.log_abs[(size_t)spin * nw + w] = s.log_abs[(size_t)spin * nw + f];
      s.sign[(size_t)spin * nw + w]    = s.sign[(size_t)spin * nw + f];
    }
    e_old[w]    = e_old[f];
    age[w]      = age[f];
    s.status[w] = 0;
  }
}

template<typename T>
cudaError_t launch_copy_walkers(const DevState<T>& s, const int* src, double* weight, double* e_old, int* age,
                                cudaStream_t st)
{
  copy_walkers_kernel<T><<<s.nw, 256, 0, st>>>(s, src, weight, e_old, age);
  return cudaGetLastError();
}

template cudaError_t launch_copy_walkers<float>(const DevState<float>&, const int*, double*, double*, int*,
                                                cudaStream_t);
template cudaError_t launch_copy_walkers<double>(const DevState<double>&, const int*, double*, double*, int*,
                                                 cudaStream_t);

} // namespace qmcg
