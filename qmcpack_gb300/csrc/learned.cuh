// Device pieces of the learned MH proposal shared by the staged kernels (learned.cu)
// and the walker-resident sweep (sweep_kernel.cu): nearest-neighbour selection and a
// SIMT evaluation of the network by one CTA for one walker.
//
// The SIMT weight image holds W1, W2, W3 as BF16 pairs along the input index,
// pairs[kp][j] = (W[j][2kp], W[j][2kp+1]), so thread j (an output neuron) reads one
// coalesced 4-byte word per two inputs, and W4 row-major [6][128].  Activations are
// rounded to BF16 after every tanh, as in the tensor-core forward pass.
#pragma once
#include <cuda_bf16.h>

#include "common.cuh"
#include "launch.h"

namespace qmcg
{

constexpr int MS_P1 = 0;                        // [32][128] pairs
constexpr int MS_P2 = MS_P1 + (ML_IN / 2) * ML_H; // [64][128] pairs
constexpr int MS_P3 = MS_P2 + (ML_H / 2) * ML_H;
constexpr int MS_NPAIRS = MS_P3 + (ML_H / 2) * ML_H;
constexpr int MS_BYTES  = MS_NPAIRS * 4 + ML_NOUT * ML_H * 2; // + W4 [6][128] BF16
constexpr float ML_MU_MAX = 4.f, ML_S_MIN = -3.f, ML_S_MAX = 2.f, ML_LSCALE = 2.f;

__device__ __forceinline__ float bf16_round(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }
__device__ __forceinline__ float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }

// sorted insertion into a register list of the 8 smallest (d2, index)
__device__ __forceinline__ void top8_insert(float (&bd)[8], int (&bj)[8], float v, int id)
{
#pragma unroll
  for (int q = 0; q < 8; q++)
    if (v < bd[q])
    {
      const float tv = bd[q];
      const int ti   = bj[q];
      bd[q]          = v;
      bj[q]          = id;
      v              = tv;
      id             = ti;
    }
}

// 8 rounds of warp argmin over the lanes' list heads; lane q gets the q-th nearest index
__device__ __forceinline__ int top8_merge(float (&bd)[8], int (&bj)[8], int lane)
{
  int mine = -1;
#pragma unroll
  for (int q = 0; q < 8; q++)
  {
    float v = bd[0];
    int who = lane;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
    {
      const float v2 = __shfl_xor_sync(0xffffffffu, v, o);
      const int w2   = __shfl_xor_sync(0xffffffffu, who, o);
      if (v2 < v || (v2 == v && w2 < who))
      {
        v   = v2;
        who = w2;
      }
    }
    const int j = __shfl_sync(0xffffffffu, bj[0], who);
    if (lane == q)
      mine = (v < 3.0e38f) ? j : -1;
    if (lane == who)
    {
#pragma unroll
      for (int t = 0; t < 7; t++)
      {
        bd[t] = bd[t + 1];
        bj[t] = bj[t + 1];
      }
      bd[7] = 3.4e38f;
      bj[7] = -1;
    }
  }
  return mine;
}

// Features of electron iat at position p for one walker, written to x[64] (shared
// memory, BF16-rounded floats) by warps 0 (electrons), 1 (ions) and 2 (drift, padding).
// Rs: the walker's positions [3][ne_pad] in shared memory; g: gradient of log psi at p.
template<typename T>
__device__ __noinline__ void features_cta(const DevState<T>& s, const T* Rs, int iat, const T p[3], const T g[3],
                                             float* x)
{
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const T L[3]  = {T(s.L[0]), T(s.L[1]), T(s.L[2])};
  const T Li[3] = {T(s.G[0]), T(s.G[1]), T(s.G[2])};
  if (wid < 2)
  {
    float bd[8];
    int bj[8];
#pragma unroll
    for (int q = 0; q < 8; q++)
    {
      bd[q] = 3.4e38f;
      bj[q] = -1;
    }
    const int n = wid == 0 ? s.ne : s.nions;
    auto coord  = [&](int j, int d) -> T {
      return wid == 0 ? Rs[d * s.ne_pad + j] : s.ions[d * s.nions_pad + j];
    };
    for (int j = lane; j < n; j += 32)
      if (wid == 1 || j != iat)
      {
        T r2 = 0;
#pragma unroll
        for (int d = 0; d < 3; d++)
        {
          const T dd = min_image(coord(j, d) - p[d], L[d], Li[d]);
          r2 += dd * dd;
        }
        top8_insert(bd, bj, (float)r2, j);
      }
    const int jn = top8_merge(bd, bj, lane);
    if (lane < 8)
#pragma unroll
      for (int d = 0; d < 3; d++)
        x[wid * 24 + 3 * lane + d] =
            jn >= 0 ? bf16_round((float)(min_image(coord(jn, d) - p[d], L[d], Li[d]) / T(ML_LSCALE))) : 0.f;
  }
  else if (wid == 2 && lane == 0)
  {
    T dr[3];
    const T tau = T(s.tau);
    unr_drift_t(tau, g, dr);
    const T st = sqrt(tau);
#pragma unroll
    for (int d = 0; d < 3; d++)
      x[48 + d] = bf16_round((float)(dr[d] / st));
  }
  else if (wid == 2 && lane >= 1 && lane <= ML_IN - ML_NIN)
    x[ML_NIN + lane - 1] = 0.f;
}

// The network for one walker by a CTA of exactly 128 threads (one per hidden neuron).
// x: [64] inputs, h: [2][128] scratch, red: [6 * 4] scratch, out: [6] (all shared).
// Contains __syncthreads(): every thread of the CTA must call it.
static __device__ __noinline__ void mlp_eval_cta(const __nv_bfloat162* __restrict__ pairs,
                                             const __nv_bfloat16* __restrict__ w4, const float* __restrict__ prm,
                                             const float* x, float* h, float* red, float* out)
{
  const int j = threadIdx.x, lane = j & 31, wid = j >> 5;
  // the weights come from L2: a layer's loads are issued in batches of MB words
  // before their FMAs so that many are in flight at once
  constexpr int MB = 32;
  const unsigned* pw = reinterpret_cast<const unsigned*>(pairs);
  auto layer = [&](int base, int npairs, const float* in, float bias) {
    float a = bias;
    for (int k0 = 0; k0 < npairs; k0 += MB)
    {
      unsigned wv[MB];
#pragma unroll
      for (int q = 0; q < MB; q++)
        wv[q] = k0 + q < npairs ? __ldg(pw + base + (k0 + q) * ML_H + j) : 0u;
#pragma unroll
      for (int q = 0; q < MB; q++)
      {
        __nv_bfloat162 b2;
        *reinterpret_cast<unsigned*>(&b2) = wv[q];
        const float2 w = __bfloat1622float2(b2);
        if (k0 + q < npairs)
          a += w.x * in[2 * (k0 + q)] + w.y * in[2 * (k0 + q) + 1];
      }
    }
    return a;
  };
  h[j] = bf16_round(tanhf(layer(MS_P1, (ML_NIN + 1) / 2, x, prm[MP_B1 + j])));
  __syncthreads();
  h[ML_H + j] = bf16_round(tanhf(layer(MS_P2, ML_H / 2, h, prm[MP_B2 + j])));
  __syncthreads();
  const float h3 = bf16_round(tanhf(layer(MS_P3, ML_H / 2, h + ML_H, prm[MP_B3 + j])));
  float o[ML_NOUT];
#pragma unroll
  for (int q = 0; q < ML_NOUT; q++)
    o[q] = warp_sum(h3 * __bfloat162float(w4[q * ML_H + j]));
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < ML_NOUT; q++)
      red[q * 4 + wid] = o[q];
  __syncthreads();
  if (j < ML_NOUT)
    out[j] = prm[MP_B4 + j] + ((red[j * 4] + red[j * 4 + 1]) + (red[j * 4 + 2] + red[j * 4 + 3]));
  __syncthreads();
}

} // namespace qmcg
