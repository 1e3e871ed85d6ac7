// Learned Metropolis-Hastings proposal for the particle-by-particle move (no
// counterpart in the reference; it replaces the drift-diffusion proposal of
// VMCBatched::advanceWalkers, VMCBatched.cpp:106-177, inside the same exact MH test).
//
// For electron i of a walker at configuration R, a per-electron MLP maps 51 features
//   8 nearest other electrons: displacement (3) / 2 bohr, nearest first
//   8 nearest ions:            displacement (3) / 2 bohr, nearest first
//   UNR drift d(R) / sqrt(tau)
// through 3 tanh layers of width 128 to (mu, s) in R^3 x R^3 and proposes
//   r' = r + d(R) + sqrt(tau) mu + sigma . xi,  sigma = sqrt(tau) exp(s),  xi ~ N(0, 1)
// (mu clipped to [-4, 4], s to [-3, 2]).  With the last layer zero this is exactly the
// drift-diffusion proposal.  The MH probability uses the forward and reverse densities
//   p = |psi(R')/psi(R)|^2 q(r | R') / q(r' | R),
//   log q(r' | R) = -sum s - |xi|^2 / 2,  log q(r | R') = -sum s' - |z|^2 / 2,
//   z = (r - r' - d(R') - sqrt(tau) mu(R')) / sigma(R')
// (the common -3/2 log(2 pi tau) cancels), so the sampled distribution stays |psi|^2.
//
// Inference: BF16 weights and activations, FP32 accumulation on the tensor cores
// (tcgen05.mma kind::f16, accumulators in TMEM), 128 walkers per CTA; the proposal or
// the MH probability is computed in the epilogue of the last layer.
// Training (hand-written, FP32): the expected squared jump j = alpha |r' - r|^2 of every
// walker's move is pushed up through the objective mean(lambda^4 / j - j) (large jumps
// rewarded, walkers that do not move penalised), by reparameterised gradients through
// (mu, s) of both evaluations,
// backpropagated through the three layers by SIMT kernels, with Adam on FP32 master
// weights that are re-packed into the BF16 tensor-core image after every step.
#include <cuda_bf16.h>

#include "common.cuh"
#include "launch.h"
#include "learned.cuh"
#include "tc.cuh"

namespace qmcg
{

// packed BF16 weight image (core-matrix K-major tiles): W1 [128][64], W2, W3 [128][128], W4 [16][128]
constexpr int ML_W1 = 0;
constexpr int ML_W2 = ML_W1 + ML_H * ML_IN * 2;
constexpr int ML_W3 = ML_W2 + ML_H * ML_H * 2;
constexpr int ML_W4 = ML_W3 + ML_H * ML_H * 2;
constexpr int ML_WBYTES = ML_W4 + ML_OUT * ML_H * 2;
constexpr int ML_A      = ML_WBYTES;               // activation tile 128 x 128 BF16
constexpr int ML_BIAS   = ML_A + ML_M * ML_H * 2;  // 400 floats
constexpr int ML_BAR    = ML_BIAS + 400 * 4;
constexpr int ML_SMEM   = ML_BAR + 64;

// ---------------------------------------------------------------------------
// weight packing and parameter layout
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool mp_structural_zero(int i)
{
  if (i < MP_B1)
    return (i % ML_IN) >= ML_NIN; // W1 columns beyond the 51 features
  if (i >= MP_W4 && i < MP_B4)
    return (i - MP_W4) / ML_H >= ML_NOUT; // W4 rows beyond the 6 outputs
  if (i >= MP_B4)
    return (i - MP_B4) >= ML_NOUT;
  return false;
}

__global__ void mlp_pack_kernel(const float* __restrict__ p, unsigned char* __restrict__ img,
                                unsigned char* __restrict__ simt)
{
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  int base, n, k, K, src;
  if (e < ML_H * ML_IN)
  {
    base = ML_W1; K = ML_IN; n = e / K; k = e % K; src = MP_W1 + e;
  }
  else if (e < ML_H * ML_IN + ML_H * ML_H)
  {
    const int q = e - ML_H * ML_IN;
    base = ML_W2; K = ML_H; n = q / K; k = q % K; src = MP_W2 + q;
  }
  else if (e < ML_H * ML_IN + 2 * ML_H * ML_H)
  {
    const int q = e - ML_H * ML_IN - ML_H * ML_H;
    base = ML_W3; K = ML_H; n = q / K; k = q % K; src = MP_W3 + q;
  }
  else if (e < ML_H * ML_IN + 2 * ML_H * ML_H + ML_OUT * ML_H)
  {
    const int q = e - ML_H * ML_IN - 2 * ML_H * ML_H;
    base = ML_W4; K = ML_H; n = q / K; k = q % K; src = MP_W4 + q;
  }
  else
    return;
  const __nv_bfloat16 v = __float2bfloat16_rn(p[src]);
  *reinterpret_cast<__nv_bfloat16*>(img + base + cm_off_b(n, k, K, 2)) = v;
  // SIMT image: W1..W3 as pairs along k, W4 rows 0..5 row-major
  __nv_bfloat16* sp = reinterpret_cast<__nv_bfloat16*>(simt);
  if (base == ML_W4)
  {
    if (n < ML_NOUT)
      sp[2 * MS_NPAIRS + n * ML_H + k] = v;
  }
  else
  {
    const int off = base == ML_W1 ? MS_P1 : base == ML_W2 ? MS_P2 : MS_P3;
    sp[2 * (off + (k >> 1) * ML_H + n) + (k & 1)] = v;
  }
}

// ---------------------------------------------------------------------------
// features: one warp per walker
// ---------------------------------------------------------------------------
template<typename T>
__global__ void features_kernel(DevState<T> s, int iat, int at_proposed, __nv_bfloat16* __restrict__ X)
{
  const int iw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (iw >= s.nw)
    return;
  double p[3];
#pragma unroll
  for (int d = 0; d < 3; d++)
    p[d] = at_proposed ? s.active_pos[iw * 3 + d] : s.R[((size_t)iw * 3 + d) * s.ne_pad + iat];
  auto disp = [&](double x, double y, double z, double (&dv)[3]) {
    const double q[3] = {x - p[0], y - p[1], z - p[2]};
#pragma unroll
    for (int d = 0; d < 3; d++)
      dv[d] = q[d] - s.L[d] * rint(q[d] / s.L[d]);
  };
  const double* Rw = s.R + (size_t)iw * 3 * s.ne_pad;
  float bd[8];
  int bj[8];
#pragma unroll
  for (int q = 0; q < 8; q++)
  {
    bd[q] = 3.4e38f;
    bj[q] = -1;
  }
  for (int j = lane; j < s.ne; j += 32)
    if (j != iat)
    {
      double dv[3];
      disp(Rw[j], Rw[s.ne_pad + j], Rw[2 * s.ne_pad + j], dv);
      top8_insert(bd, bj, (float)(dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2]), j);
    }
  const int je = top8_merge(bd, bj, lane);
#pragma unroll
  for (int q = 0; q < 8; q++)
  {
    bd[q] = 3.4e38f;
    bj[q] = -1;
  }
  for (int I = lane; I < s.nions; I += 32)
  {
    double dv[3];
    disp(s.ions[I], s.ions[s.nions_pad + I], s.ions[2 * s.nions_pad + I], dv);
    top8_insert(bd, bj, (float)(dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2]), I);
  }
  const int ji = top8_merge(bd, bj, lane);
  __nv_bfloat16* xr = X + (size_t)iw * ML_IN;
  if (lane < 8)
  {
    double dv[3] = {0, 0, 0};
    if (je >= 0)
      disp(Rw[je], Rw[s.ne_pad + je], Rw[2 * s.ne_pad + je], dv);
#pragma unroll
    for (int d = 0; d < 3; d++)
      xr[3 * lane + d] = __float2bfloat16_rn((float)(dv[d] / ML_LSCALE));
    double di[3] = {0, 0, 0};
    if (ji >= 0)
      disp(s.ions[ji], s.ions[s.nions_pad + ji], s.ions[2 * s.nions_pad + ji], di);
#pragma unroll
    for (int d = 0; d < 3; d++)
      xr[24 + 3 * lane + d] = __float2bfloat16_rn((float)(di[d] / ML_LSCALE));
  }
  else if (lane == 8)
  {
    const double* g = at_proposed ? s.grads_new + iw * 3 : s.grads_now + iw * 3;
    double dr[3];
    unr_drift(s.tau, g, dr);
    const double st = sqrt(s.tau);
#pragma unroll
    for (int d = 0; d < 3; d++)
      xr[48 + d] = __float2bfloat16_rn((float)(dr[d] / st));
  }
  else if (lane >= 9 && lane < 9 + (ML_IN - ML_NIN))
    xr[ML_NIN + lane - 9] = __float2bfloat16_rn(0.f);
}

// ---------------------------------------------------------------------------
// forward pass on the tensor cores, 128 rows per CTA
// ---------------------------------------------------------------------------
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, int accum)
{
  asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
               "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
               "l"(a), "l"(b), "r"(idesc), "r"(accum)
               : "memory");
}

// kind::f16 instruction descriptor: BF16 A and B, FP32 accumulate, K-major operands
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n)
{
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

// MODE 0: raw outputs; 1: proposal at the current position; 2: MH probability at the proposed one
template<typename T, int MODE>
__global__ void __launch_bounds__(128) mlp_forward_kernel(MlpArgs a, DevState<T> s, int iat)
{
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ int s_fail;
  __shared__ uint32_t s_tmem;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int r = warp * 32 + lane, grow = blockIdx.x * ML_M + r;
  const bool valid = grow < a.rows;
  unsigned char* W = sm;
  unsigned char* A = sm + ML_A;
  float* bs        = reinterpret_cast<float*>(sm + ML_BIAS);
  const uint32_t bar = smem_u32(sm + ML_BAR);
  if (tid == 0)
  {
    s_fail = 0;
    mbar_init(bar);
  }
  if (warp == 0)
    tmem_alloc(smem_u32(&s_tmem), 256);
  {
    const uint4* src = reinterpret_cast<const uint4*>(a.wimg);
    uint4* dst       = reinterpret_cast<uint4*>(W);
    for (int e = tid; e < ML_WBYTES / 16; e += 128)
      dst[e] = src[e];
    for (int e = tid; e < 400; e += 128)
      bs[e] = e < 384 ? a.params[(e >> 7) == 0 ? MP_B1 + e : (e >> 7) == 1 ? MP_B2 + e - 128 : MP_B3 + e - 256]
                      : a.params[MP_B4 + e - 384];
    const uint4* xr = reinterpret_cast<const uint4*>(a.x + (size_t)(valid ? grow : 0) * ML_IN);
#pragma unroll
    for (int c = 0; c < ML_IN / 8; c++)
    {
      const uint4 v = valid ? xr[c] : make_uint4(0, 0, 0, 0);
      *reinterpret_cast<uint4*>(A + cm_off_b(r, 8 * c, ML_IN, 2)) = v;
    }
  }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = s_tmem;
  uint32_t phase      = 0;
  for (int l = 0; l < 4; l++)
  {
    const int K = l == 0 ? ML_IN : ML_H, N = l == 3 ? ML_OUT : ML_H;
    const int woff = l == 0 ? ML_W1 : l == 1 ? ML_W2 : l == 2 ? ML_W3 : ML_W4;
    const uint32_t dcol = l == 3 ? 128u : 0u;
    if (tid == 0)
    {
      tc_fence_after();
      const uint32_t id = idesc_bf16(ML_M, N);
      const uint32_t ab = smem_u32(A), wb = smem_u32(W + woff);
      for (int ks = 0; ks < K / 16; ks++)
        mma_bf16(tmem + dcol, smem_desc_b(ab + ks * 256, K * 2), smem_desc_b(wb + ks * 256, K * 2), id, ks > 0);
      mma_commit(bar);
    }
    if (!mbar_wait(bar, phase))
      atomicExch(&s_fail, 1);
    phase ^= 1;
    tc_fence_after();
    __syncthreads();
    if (s_fail)
      break;
    if (l < 3)
    {
#pragma unroll 1
      for (int c0 = 0; c0 < ML_H; c0 += 32)
      {
        float v[32];
        tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + c0, v);
        uint32_t pk[16];
#pragma unroll
        for (int q = 0; q < 16; q++)
        {
          const float h0 = tanhf(v[2 * q] + bs[l * 128 + c0 + 2 * q]);
          const float h1 = tanhf(v[2 * q + 1] + bs[l * 128 + c0 + 2 * q + 1]);
          const __nv_bfloat162 b2 = __floats2bfloat162_rn(h0, h1);
          pk[q] = *reinterpret_cast<const uint32_t*>(&b2);
        }
#pragma unroll
        for (int j = 0; j < 4; j++)
        {
          const uint4 v4 = make_uint4(pk[4 * j], pk[4 * j + 1], pk[4 * j + 2], pk[4 * j + 3]);
          *reinterpret_cast<uint4*>(A + cm_off_b(r, c0 + 8 * j, ML_H, 2)) = v4;
          if (a.hid && valid)
            *reinterpret_cast<uint4*>(a.hid + ((size_t)l * a.hid_rows + a.hid_row0 + grow) * ML_H + c0 + 8 * j) = v4;
        }
      }
      fence_async_smem();
      tc_fence_before();
      __syncthreads();
      tc_fence_after();
    }
    else
    {
      float v[32];
      tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + 128, v);
      float o[ML_NOUT];
#pragma unroll
      for (int q = 0; q < ML_NOUT; q++)
        o[q] = v[q] + bs[384 + q];
      if (valid && a.out)
#pragma unroll
        for (int q = 0; q < ML_NOUT; q++)
          a.out[(size_t)grow * 8 + q] = o[q];
      if (MODE != 0 && valid)
      {
        const int iw    = grow;
        const double st = sqrt(s.tau);
        float* ax       = a.aux + (size_t)iw * ML_AUX;
        double mu[3], sg[3], sum_s = 0;
#pragma unroll
        for (int d = 0; d < 3; d++)
        {
          mu[d] = clampf(o[d], -ML_MU_MAX, ML_MU_MAX);
          const double sd = clampf(o[3 + d], ML_S_MIN, ML_S_MAX);
          sum_s += sd;
          sg[d] = st * exp(sd);
        }
        if (MODE == 1)
        {
          double g[3] = {s.grads_now[iw * 3], s.grads_now[iw * 3 + 1], s.grads_now[iw * 3 + 2]}, dr[3], xi[3];
          unr_drift(s.tau, g, dr);
          const uint32_t sw = static_cast<uint32_t>(*s.sweep_counter);
          gaussians<double>((uint32_t)iw, (uint32_t)iat, sw, static_cast<uint32_t>(s.seed),
                            static_cast<uint32_t>(s.seed >> 32), xi);
          double x2 = 0;
#pragma unroll
          for (int d = 0; d < 3; d++)
          {
            const double dd = dr[d] + st * mu[d] + sg[d] * xi[d];
            s.disp[iw * 3 + d]       = dd;
            s.active_pos[iw * 3 + d] = s.R[((size_t)iw * 3 + d) * s.ne_pad + iat] + dd;
            x2 += xi[d] * xi[d];
            ax[d]     = o[d];
            ax[3 + d] = o[3 + d];
            ax[6 + d] = (float)xi[d];
          }
          s.log_gf[iw] = -sum_s - 0.5 * x2;
        }
        else
        {
          double g[3] = {s.grads_new[iw * 3], s.grads_new[iw * 3 + 1], s.grads_new[iw * 3 + 2]}, dr[3];
          unr_drift(s.tau, g, dr);
          double z2 = 0;
#pragma unroll
          for (int d = 0; d < 3; d++)
          {
            const double rp = s.active_pos[iw * 3 + d];
            const double r0 = s.R[((size_t)iw * 3 + d) * s.ne_pad + iat];
            const double z  = (r0 - rp - dr[d] - st * mu[d]) / sg[d];
            z2 += z * z;
            ax[9 + d]  = o[d];
            ax[12 + d] = o[3 + d];
            ax[15 + d] = (float)z;
          }
          const double log_gb = -sum_s - 0.5 * z2;
          const double ratio  = s.ratios[iw];
          const double p      = ratio * ratio;
          s.flag[iw]          = (p >= static_cast<double>(Eps<T>::v)) ? 1 : 0;
          s.prob[iw]          = p * exp(log_gb - s.log_gf[iw]);
        }
      }
    }
  }
  if (s_fail && tid == 0)
    atomicExch(a.err, 1);
  tc_fence_before();
  __syncthreads();
  if (warp == 0)
    tmem_dealloc(tmem, 256);
}

// ---------------------------------------------------------------------------
// training: loss gradient, backward, Adam
// ---------------------------------------------------------------------------
// dL/d(raw outputs) of the forward row iw and the reverse row nw + iw for
// L = (1/nw) sum_w (lambda^4 / j_w - j_w), j_w = alpha_w |r'_w - r_w|^2 the expected
// squared jump of walker w's move, alpha = min(1, e^Delta) (0 when p < eps); the
// objective of Levy, Hoffman, Sohl-Dickstein (ICLR 2018) for learned MCMC kernels
template<typename T>
__global__ void mlp_loss_grad_kernel(DevState<T> s, const float* __restrict__ aux, float* __restrict__ g4,
                                     double* __restrict__ stats)
{
  const int iw = blockIdx.x * blockDim.x + threadIdx.x;
  if (iw >= s.nw)
    return;
  const float* ax = aux + (size_t)iw * ML_AUX;
  const double st = sqrt(s.tau);
  const double pr = s.prob[iw];
  const double alpha = s.flag[iw] ? fmin(1.0, pr) : 0.0;
  const double ad    = (s.flag[iw] && pr < 1.0) ? alpha : 0.0; // d alpha / d Delta
  double dr[3], j2 = 0;
#pragma unroll
  for (int d = 0; d < 3; d++)
  {
    dr[d] = s.disp[iw * 3 + d];
    j2 += dr[d] * dr[d];
  }
  // per-walker weight of the jump objective L_w = lambda^4 / j_w - j_w, j_w = alpha |dr|^2,
  // lambda^2 = 3 tau (the jump of drift-diffusion): dL/dtheta = -(lambda^4 / j^2 + 1) dj/dtheta.
  // The first term keeps every walker moving instead of favouring rare long jumps.
  const double lam2  = 3.0 * s.tau;
  const double jw    = fmax(alpha * j2, 0.01 * lam2);
  const double inv_n = (lam2 * lam2 / (jw * jw) + 1.0) / s.nw;
  float* gf = g4 + (size_t)iw * 8;
  float* gr = g4 + (size_t)(s.nw + iw) * 8;
  // a walker whose move produced a non-finite value (a proposal at a node of psi gives an
  // infinite gradient of log psi) contributes nothing: one such value would otherwise
  // reach every weight through the backward pass and the optimizer
  bool finite = isfinite(alpha) && isfinite(j2);
#pragma unroll
  for (int d = 0; d < 3; d++)
  {
    const double muf = ax[d], sf = ax[3 + d], xi = ax[6 + d];
    const double mur = ax[9 + d], sr = ax[12 + d], z = ax[15 + d];
    const double sgf = st * exp((double)clampf((float)sf, ML_S_MIN, ML_S_MAX));
    const double sgr = st * exp((double)clampf((float)sr, ML_S_MIN, ML_S_MAX));
    const double dlp = 2.0 * s.grads_new[iw * 3 + d] + z / sgr; // dDelta/dr'
    double g_mu = -(j2 * ad * st * dlp + alpha * 2.0 * dr[d] * st) * inv_n;
    double g_s  = -(j2 * ad * (sgf * xi * dlp + 1.0) + alpha * 2.0 * dr[d] * sgf * xi) * inv_n;
    double g_mr = -(j2 * ad * z * st / sgr) * inv_n;
    double g_sr = -(j2 * ad * (z * z - 1.0)) * inv_n;
    if (fabs(muf) >= ML_MU_MAX)
      g_mu = 0;
    if (sf <= ML_S_MIN || sf >= ML_S_MAX)
      g_s = 0;
    if (fabs(mur) >= ML_MU_MAX)
      g_mr = 0;
    if (sr <= ML_S_MIN || sr >= ML_S_MAX)
      g_sr = 0;
    gf[d]     = (float)g_mu;
    gf[3 + d] = (float)g_s;
    gr[d]     = (float)g_mr;
    gr[3 + d] = (float)g_sr;
    finite    = finite && isfinite(gf[d]) && isfinite(gf[3 + d]) && isfinite(gr[d]) && isfinite(gr[3 + d]);
  }
  gf[6] = gf[7] = gr[6] = gr[7] = 0.f;
  if (!finite)
  {
#pragma unroll
    for (int q = 0; q < 6; q++)
      gf[q] = gr[q] = 0.f;
    return;
  }
  atomicAdd(stats, alpha * j2);
  atomicAdd(stats + 1, alpha);
  atomicAdd(stats + 2, lam2 * lam2 / jw - alpha * j2);
}

__device__ __forceinline__ float bf(const __nv_bfloat16 x) { return __bfloat162float(x); }

// delta_prev[b][j] = (sum_o delta[b][o] W[o][j]) (1 - h[b][j]^2); W FP32 master [no][128]
__global__ void mlp_delta_kernel(const float* __restrict__ dn, int ldn, int no, const float* __restrict__ Wm,
                                 const __nv_bfloat16* __restrict__ h, int rows, float* __restrict__ dout)
{
  __shared__ float ws[32][129];
  const int b0 = blockIdx.x * 32;
  const int j  = threadIdx.x; // 128 threads
  float acc[32];
#pragma unroll
  for (int q = 0; q < 32; q++)
    acc[q] = 0.f;
  for (int o0 = 0; o0 < no; o0 += 32)
  {
    const int oc = min(32, no - o0);
    __syncthreads();
    for (int e = threadIdx.x; e < oc * 128; e += 128)
      ws[e / 128][e % 128] = Wm[(size_t)(o0 + e / 128) * ML_H + e % 128];
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 32; q++)
    {
      const int b = min(b0 + q, rows - 1);
      float a = 0.f;
      for (int o = 0; o < oc; o++)
        a += dn[(size_t)b * ldn + o0 + o] * ws[o][j];
      acc[q] += a;
    }
  }
#pragma unroll
  for (int q = 0; q < 32; q++)
  {
    const int b = b0 + q;
    if (b < rows)
    {
      const float hv = bf(h[(size_t)b * ML_H + j]);
      dout[(size_t)b * ML_H + j] = acc[q] * (1.f - hv * hv);
    }
  }
}

// gW[o][k] += sum_b delta[b][o] in[b][k] (k < kin), gb[o] += sum_b delta[b][o]
__global__ void mlp_wgrad_kernel(const float* __restrict__ dl, int ldd, int no, const __nv_bfloat16* __restrict__ in,
                                 int ldi, int kin, int rows, float* __restrict__ gW, int ldw, float* __restrict__ gb)
{
  const int o = blockIdx.x;
  const int k = threadIdx.x; // blockDim = ldw (64 or 128)
  if (o >= no)
    return;
  float a = 0.f, bsum = 0.f;
  for (int b = 0; b < rows; b++)
  {
    const float d = dl[(size_t)b * ldd + o];
    if (k < kin)
      a += d * bf(in[(size_t)b * ldi + k]);
    bsum += d;
  }
  gW[(size_t)o * ldw + k] = k < kin ? a : 0.f;
  if (k == 0)
    gb[o] = bsum;
}

// Adam on the FP32 master parameters (structural zeros stay zero); the step count
// lives on the device and is advanced by mlp_step_kernel
__global__ void mlp_adam_kernel(float* __restrict__ p, float* __restrict__ m, float* __restrict__ v,
                                const float* __restrict__ g, const int* __restrict__ step, float lr)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= MP_N)
    return;
  if (mp_structural_zero(i))
  {
    p[i] = 0.f;
    return;
  }
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const int t    = *step + 1;
  const float gi = isfinite(g[i]) ? g[i] : 0.f; // a non-finite gradient counts as zero
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i]           = mi;
  v[i]           = vi;
  const float mh = mi / (1.f - powf(b1, (float)t));
  const float vh = vi / (1.f - powf(b2, (float)t));
  p[i] -= lr * mh / (sqrtf(vh) + eps);
}

__global__ void mlp_step_kernel(int* step) { step[0] += 1; }

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------
template<typename T>
cudaError_t setup_learned()
{
  cudaError_t e = cudaFuncSetAttribute(mlp_forward_kernel<T, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, ML_SMEM);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(mlp_forward_kernel<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, ML_SMEM);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(mlp_forward_kernel<T, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, ML_SMEM);
  return e;
}

cudaError_t launch_mlp_pack(const float* params, unsigned char* img, unsigned char* simt, cudaStream_t st)
{
  const int n = ML_H * ML_IN + 2 * ML_H * ML_H + ML_OUT * ML_H;
  mlp_pack_kernel<<<(n + 255) / 256, 256, 0, st>>>(params, img, simt);
  return cudaGetLastError();
}

template<typename T>
cudaError_t launch_features(const DevState<T>& s, int iat, int at_proposed, __nv_bfloat16* X, cudaStream_t st)
{
  const int warps = 4;
  features_kernel<T><<<(s.nw + warps - 1) / warps, 32 * warps, 0, st>>>(s, iat, at_proposed, X);
  return cudaGetLastError();
}

template<typename T>
cudaError_t launch_mlp_forward(const MlpArgs& a, const DevState<T>& s, int iat, int mode, cudaStream_t st)
{
  const int grid = (a.rows + ML_M - 1) / ML_M;
  if (grid == 0)
    return cudaSuccess;
  if (mode == 0)
    mlp_forward_kernel<T, 0><<<grid, 128, ML_SMEM, st>>>(a, s, iat);
  else if (mode == 1)
    mlp_forward_kernel<T, 1><<<grid, 128, ML_SMEM, st>>>(a, s, iat);
  else
    mlp_forward_kernel<T, 2><<<grid, 128, ML_SMEM, st>>>(a, s, iat);
  return cudaGetLastError();
}

template<typename T>
cudaError_t launch_mlp_loss_grad(const DevState<T>& s, const float* aux, float* g4, double* stats, cudaStream_t st)
{
  mlp_loss_grad_kernel<T><<<(s.nw + 127) / 128, 128, 0, st>>>(s, aux, g4, stats);
  return cudaGetLastError();
}

cudaError_t launch_mlp_backward(const MlpTrain& t, int rows, cudaStream_t st)
{
  const int rb = (rows + 31) / 32;
  const __nv_bfloat16* h1 = t.hid;
  const __nv_bfloat16* h2 = t.hid + (size_t)rows * ML_H;
  const __nv_bfloat16* h3 = t.hid + (size_t)2 * rows * ML_H;
  float* d3 = t.delta;
  float* d2 = t.delta + (size_t)rows * ML_H;
  float* d1 = t.delta + (size_t)2 * rows * ML_H;
  mlp_delta_kernel<<<rb, 128, 0, st>>>(t.g4, 8, ML_NOUT, t.params + MP_W4, h3, rows, d3);
  mlp_delta_kernel<<<rb, 128, 0, st>>>(d3, ML_H, ML_H, t.params + MP_W3, h2, rows, d2);
  mlp_delta_kernel<<<rb, 128, 0, st>>>(d2, ML_H, ML_H, t.params + MP_W2, h1, rows, d1);
  mlp_wgrad_kernel<<<ML_OUT, ML_H, 0, st>>>(t.g4, 8, ML_NOUT, h3, ML_H, ML_H, rows, t.grad + MP_W4, ML_H,
                                            t.grad + MP_B4);
  mlp_wgrad_kernel<<<ML_H, ML_H, 0, st>>>(d3, ML_H, ML_H, h2, ML_H, ML_H, rows, t.grad + MP_W3, ML_H, t.grad + MP_B3);
  mlp_wgrad_kernel<<<ML_H, ML_H, 0, st>>>(d2, ML_H, ML_H, h1, ML_H, ML_H, rows, t.grad + MP_W2, ML_H, t.grad + MP_B2);
  mlp_wgrad_kernel<<<ML_H, ML_IN, 0, st>>>(d1, ML_H, ML_H, t.x, ML_IN, ML_NIN, rows, t.grad + MP_W1, ML_IN,
                                           t.grad + MP_B1);
  return cudaGetLastError();
}

cudaError_t launch_mlp_adam(const MlpTrain& t, float lr, cudaStream_t st)
{
  mlp_adam_kernel<<<(MP_N + 255) / 256, 256, 0, st>>>(t.params, t.m, t.v, t.grad, t.step, lr);
  mlp_step_kernel<<<1, 1, 0, st>>>(t.step);
  return launch_mlp_pack(t.params, t.wimg, t.wsimt, st);
}

template cudaError_t setup_learned<float>();
template cudaError_t setup_learned<double>();
template cudaError_t launch_features<float>(const DevState<float>&, int, int, __nv_bfloat16*, cudaStream_t);
template cudaError_t launch_features<double>(const DevState<double>&, int, int, __nv_bfloat16*, cudaStream_t);
template cudaError_t launch_mlp_forward<float>(const MlpArgs&, const DevState<float>&, int, int, cudaStream_t);
template cudaError_t launch_mlp_forward<double>(const MlpArgs&, const DevState<double>&, int, int, cudaStream_t);
template cudaError_t launch_mlp_loss_grad<float>(const DevState<float>&, const float*, float*, double*, cudaStream_t);
template cudaError_t launch_mlp_loss_grad<double>(const DevState<double>&, const float*, float*, double*,
                                                  cudaStream_t);

} // namespace qmcg
