// Walker-resident sweep: one CTA owns one walker for a segment of up to k
// electrons of one spin group (k = delay rank; the whole spin group with rank-1
// updates).
//
// With counter-based random numbers every walker's Markov chain is independent
// of the others, so the body of VMCBatched::advanceWalkers
// (src/QMCDrivers/VMC/VMCBatched.cpp:106-177) for one walker runs inside one CTA:
// for every electron the proposal (mw_evalGrad + drift-diffusion), the evaluation
// at the proposed position (mw_makeMove + mw_calcRatioGrad), the accept test and
// the state update (mw_accept_rejectMove).  Segments end where the delayed
// update fills its window (DelayedUpdateBatched::mw_updateInvMat,
// DelayedUpdateBatched.h:675-738); that flush runs batched over all walkers in
// flush_kernels.cu.
//
// Per CTA the walker's positions, two-body Jastrow state and the delayed-update
// matrix Binv stay in shared memory for the segment; the next electron's inverse
// row, orbital-gradient rows and orbital values are prefetched with cp.async
// while the current electron is evaluated.  Driver arithmetic (Box-Muller
// Gaussians, drift, Green's functions) runs in the move-loop precision, as the
// reference's mixed-precision build does in RealType.
#include <algorithm>
#include <type_traits>

#include "common.cuh"
#include "launch.h"
#include "learned.cuh"
#include "spline.cuh"

namespace qmcg
{

template<typename T>
struct SweepCfg
{
  static constexpr int NT   = 128;
  static constexpr int MINB = sizeof(T) == 4 ? 4 : 2;
};

template<typename T>
static size_t sweep_smem_elems(const DevState<T>& s)
{
  return (size_t)28 * s.lda    // spline partials
      + (size_t)10 * s.lda     // prefetch double buffer (inverse row, dgrad xyz, orbital values)
      + 2 * (size_t)s.lda      // up-to-date inverse row, spare row (keeps 16-byte alignment)
      + 5 * (size_t)s.lda      // orbital VGL at the proposed position
      + 8 * (size_t)s.ne_pad   // positions, J2 state
      + (size_t)s.k * s.k      // Binv
      + 3 * (size_t)s.k        // p, t, y
      + 16 * 32                // block reductions
      + (size_t)s.k * (s.k - 1) / 2; // U_c . Ainv[row_x] of the segment, c < x
}

// cp.async of n_elems elements (a multiple of 16 bytes) from global to shared
template<typename T>
__device__ __forceinline__ void async_copy(T* dst, const T* src, int n_elems, int tid, int nt)
{
  const int chunks = n_elems * (int)sizeof(T) / 16;
  for (int c = tid; c < chunks; c += nt)
  {
    const unsigned sa = static_cast<unsigned>(__cvta_generic_to_shared(reinterpret_cast<char*>(dst) + 16 * c));
    const char* ga    = reinterpret_cast<const char*>(src) + 16 * c;
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(ga) : "memory");
  }
}
__device__ __forceinline__ void async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// rows of electron `row` of spin slot into pre[5][lda]: inverse row, dgrad xyz, orbital values
template<typename T>
__device__ __forceinline__ void prefetch_rows(const DevState<T>& s, size_t slot, int row, T* pre, int tid, int nt)
{
  const int n = s.norb;
  async_copy(pre, s.Ainv + (slot * n + row) * s.lda, s.lda, tid, nt);
  async_copy(pre + s.lda, s.dgrad + ((slot * n + row) * 3) * s.lda, 3 * s.lda, tid, nt);
  async_copy(pre + 4 * s.lda, s.psiv + (slot * n + row) * s.lda, s.lda, tid, nt);
  async_commit();
}

// out[c] = scale * (rows[c] . x) for c < nrows (rows in global memory, stride ld,
// x in shared memory): every warp owns up to 8 rows and issues the loads of four
// 32-column strips of all of them (32 loads in flight) before the first product
template<typename T, int NT>
__device__ __forceinline__ void rows_dot(const T* rows, int ld, int nrows, const T* x, int n, T* out, T scale)
{
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  constexpr int NW = NT / 32;
  constexpr int JB = 4; // 32-column strips per batch of loads
  for (int c0 = wid; c0 < nrows; c0 += 8 * NW)
  {
    T a[8];
#pragma unroll
    for (int q = 0; q < 8; q++)
      a[q] = T(0);
    for (int jb = lane; jb < n; jb += 32 * JB)
    {
      T v[JB][8], xv[JB];
#pragma unroll
      for (int u = 0; u < JB; u++)
      {
        const int j = jb + 32 * u;
        xv[u]       = j < n ? x[j] : T(0);
#pragma unroll
        for (int q = 0; q < 8; q++)
        {
          const int c = c0 + q * NW;
          v[u][q]     = (c < nrows && j < n) ? rows[(size_t)c * ld + j] : T(0);
        }
      }
#pragma unroll
      for (int u = 0; u < JB; u++)
#pragma unroll
        for (int q = 0; q < 8; q++)
          a[q] += v[u][q] * xv[u];
    }
#pragma unroll
    for (int q = 0; q < 8; q++)
    {
      const T v = warp_sum(a[q]);
      const int c = c0 + q * NW;
      if (lane == 0 && c < nrows)
        out[c] = scale * v;
    }
  }
}

// shared scratch of the learned proposal (empty for the drift-diffusion kernel)
template<typename T, bool LEARNED>
struct LearnedSmem
{
};
template<typename T>
struct LearnedSmem<T, true>
{
  T g[3];
  T p;
};
// the network's features, activations, reduction scratch and outputs live in the spline
// partials buffer, which is free while the network runs (before the spline partials of
// the proposed position are formed, and after they are combined)
constexpr int ML_SCRATCH_FLOATS = ML_IN + 2 * ML_H + ML_NOUT * 4 + 8;
static_assert(ML_SCRATCH_FLOATS * 4 <= 28 * 16 * 4, "the network scratch fits the partials of the smallest padding");

// per-CTA scalars of the resident sweep in shared memory
template<typename T, bool LEARNED>
struct SweepShared
{
  double pos[3];
  T posT[3]; // the proposed position in the move-loop precision
  T ru[3];   // its fractional coordinates (spline_frac)
  T disp[3];
  T rgauss[32][3]; // Gaussians of the proposals of a block of 32 electrons
  T runif[32];     // uniforms of their acceptance tests
  T loggf;
  int acc;
  T det;
  T cur[10];
  LearnedSmem<T, LEARNED> lsm;
};

// The segment [i0, i1) of walker w by one CTA: the body of the resident sweep.
template<typename T, int NT, bool LEARNED>
__device__ __forceinline__ void sweep_walker(const DevState<T>& s, int i0, int i1, int w, unsigned char* smem_raw,
                                             SweepShared<T, LEARNED>& sh, unsigned long long& n_acc,
                                             unsigned long long& n_rej)
{
  const int lda = s.lda, n = s.norb, K = s.k;
  T* part   = reinterpret_cast<T*>(smem_raw); // 28 x lda
  T* pre    = part + 28 * lda;                // 2 x 5 x lda prefetch buffers
  T* invrow = pre + 10 * lda;                 // lda
  T* spare  = invrow + lda;                   // lda
  T* phi    = spare + lda;                    // 5 x lda
  T* Rs     = phi + 5 * lda;                  // 3 x ne_pad
  T* J2s    = Rs + 3 * s.ne_pad;              // 5 x ne_pad
  T* Bs     = J2s + 5 * s.ne_pad;             // K x K
  T* pv     = Bs + K * K;                     // K
  T* tv     = pv + K;                         // K
  T* yv     = tv + K;                         // K
  T* red    = yv + K;                         // 16 x 32
  T* tri    = red + 16 * 32;                  // K (K - 1) / 2: entry x (x - 1) / 2 + c = U_c . Ainv[row_x]
  const __nv_bfloat162* ml_pairs = reinterpret_cast<const __nv_bfloat162*>(s.mlp_simt);
  const __nv_bfloat16* ml_w4 = reinterpret_cast<const __nv_bfloat16*>(ml_pairs + MS_NPAIRS);
  float* ml_x   = reinterpret_cast<float*>(part); // ML_SCRATCH_FLOATS <= 28 * lda elements of part
  float* ml_h   = ml_x + ML_IN;
  float* ml_red = ml_h + 2 * ML_H;
  float* ml_out = ml_red + ML_NOUT * 4;

  const uint32_t sweep = static_cast<uint32_t>(*s.sweep_counter);
  const uint32_t k0 = static_cast<uint32_t>(s.seed), k1 = static_cast<uint32_t>(s.seed >> 32);
  const T L0 = T(s.L[0]), L1 = T(s.L[1]), L2 = T(s.L[2]);
  const T Li0 = T(s.G[0]), Li1 = T(s.G[1]), Li2 = T(s.G[2]);
  const T tau       = T(s.tau);
  const int spin    = i0 >= s.nup ? 1 : 0;
  const int first   = spin ? s.nup : 0;
  const int lane    = threadIdx.x & 31, wid = threadIdx.x >> 5;
  (void)spare;
  (void)ml_w4;
  (void)ml_out;

  {
    const size_t slot = (size_t)spin * s.nw + w;
    for (int e = threadIdx.x; e < 3 * s.ne_pad; e += NT)
      Rs[e] = s.Rt[(size_t)w * 3 * s.ne_pad + e];
    for (int e = threadIdx.x; e < 5 * s.ne_pad; e += NT)
      J2s[e] = s.J2[(size_t)w * 5 * s.ne_pad + e];
    prefetch_rows(s, slot, i0 - first, pre, threadIdx.x, NT);
    int dc = 0;
    // DMC: tau |xi|^2 of this segment's proposed and accepted moves (thread 0)
    double rr_prop = 0, rr_acc = 0;
    // product of the accepted determinant ratios (thread 0), one log per segment
    double det_mant = 1.0;
    int det_exp     = 0;
    int det_neg     = 0;
    for (int iat = i0; iat < i1; iat++)
    {
      const int row = iat - first;
      T* arow       = pre + ((iat - i0) & 1) * 5 * lda; // this electron's prefetched rows
      const T* dg   = arow + lda;
      const T* pv0  = arow + 4 * lda;
      // the random numbers of the next 32 electrons, one electron per thread (counter-based:
      // the same values the single-electron calls would draw)
      const int jj = (iat - i0) & 31;
      if (jj == 0 && threadIdx.x < 32 && iat + threadIdx.x < i1)
      {
        const uint32_t e = (uint32_t)(iat + threadIdx.x);
        gaussians<T>((uint32_t)w, e, sweep, k0, k1, sh.rgauss[threadIdx.x]);
        const u4 r2            = philox4x32_10(u4{(uint32_t)w, e, sweep, 2u}, k0, k1);
        sh.runif[threadIdx.x]  = T(u01(r2.x, r2.y));
      }
      // thread 0's operands of the proposal and the decision, loaded ahead of their use
      double r_now[3] = {0, 0, 0};
      T j1_now[4]     = {0, 0, 0, 0}; // Vat, Grad xyz of this electron
      if (threadIdx.x == 0)
      {
        for (int d = 0; d < 3; d++)
          r_now[d] = s.R[((size_t)w * 3 + d) * s.ne_pad + iat];
        if (s.has_j1)
          for (int q = 0; q < 4; q++)
            j1_now[q] = s.J1[((size_t)w * 5 + q) * s.ne_pad + iat];
      }
      async_wait_all();
      __syncthreads();
      // ------------------------------------------------ up-to-date inverse row, fused with
      // the gradient and self-ratio sums of the same elements
      const T* inv = arow;
      T g[4]       = {0, 0, 0, 0};
      if (K > 1 && dc > 0)
      {
        const T* V = s.V + slot * K * lda;
        // pv_c = U_c . Ainv[row] of the earlier slots of this segment, formed when slot c
        // was decided (zero for a rejected move), read straight from the table
        const T* pvt = tri + dc * (dc - 1) / 2;
        for (int i = threadIdx.x; i < dc; i += NT)
        {
          T a = 0;
          for (int c = 0; c < dc; c++)
            a += Bs[c * K + i] * pvt[c];
          tv[i]          = -a;
          Bs[dc * K + i] = -a;
        }
        __syncthreads();
        // the next electron's rows arrive while this one is evaluated
        if (iat + 1 < i1)
          prefetch_rows(s, slot, row + 1, pre + ((iat + 1 - i0) & 1) * 5 * lda, threadIdx.x, NT);
        for (int j = threadIdx.x; j < n; j += NT)
        {
          T a[4] = {0, 0, 0, 0};
          int c  = 0;
          for (; c + 4 <= dc; c += 4)
          {
            const T v0 = V[(size_t)c * lda + j], v1 = V[(size_t)(c + 1) * lda + j];
            const T v2 = V[(size_t)(c + 2) * lda + j], v3 = V[(size_t)(c + 3) * lda + j];
            a[0] += v0 * tv[c];
            a[1] += v1 * tv[c + 1];
            a[2] += v2 * tv[c + 2];
            a[3] += v3 * tv[c + 3];
          }
          for (; c < dc; c++)
            a[0] += V[(size_t)c * lda + j] * tv[c];
          const T x = arow[j] + ((a[0] + a[1]) + (a[2] + a[3]));
          invrow[j] = x;
          g[0] += x * dg[j];
          g[1] += x * dg[lda + j];
          g[2] += x * dg[2 * lda + j];
          g[3] += x * pv0[j];
        }
        inv = invrow;
      }
      else
      {
        if (iat + 1 < i1)
          prefetch_rows(s, slot, row + 1, pre + ((iat + 1 - i0) & 1) * 5 * lda, threadIdx.x, NT);
        for (int j = threadIdx.x; j < n; j += NT)
        {
          const T x = arow[j];
          g[0] += x * dg[j];
          g[1] += x * dg[lda + j];
          g[2] += x * dg[2 * lda + j];
          g[3] += x * pv0[j];
        }
      }
      // ------------------------------------------------ gradient, health check, proposal
      {
        block_sum_to0<T, 4>(g, red); // thread 0 uses the sums
        if constexpr (LEARNED)
        {
          // the network at the current position: (mu, s) of the proposal
          if (threadIdx.x == 0)
          {
            if (!(fabs(g[3] - T(1)) <= HealthTol<T>::v))
              atomicOr(s.status + w, spin ? ST_ILLCOND_DN : ST_ILLCOND_UP);
            for (int d = 0; d < 3; d++)
            {
              T gs = g[d];
              if (s.has_j1)
                gs += j1_now[1 + d];
              if (s.has_j2)
                gs += J2s[(1 + d) * s.ne_pad + iat];
              sh.lsm.g[d] = gs;
            }
          }
          __syncthreads();
          const T pc[3] = {Rs[iat], Rs[s.ne_pad + iat], Rs[2 * s.ne_pad + iat]};
          features_cta(s, Rs, iat, pc, sh.lsm.g, ml_x);
          __syncthreads();
          mlp_eval_cta(ml_pairs, ml_w4, s.mlp_params, ml_x, ml_h, ml_red, ml_out);
          if (threadIdx.x == 0)
          {
            const T st = sqrt(tau);
            T drift[3];
            unr_drift_t(tau, sh.lsm.g, drift);
            T sum_s = 0, x2 = 0;
            for (int d = 0; d < 3; d++)
            {
              const T mu = T(clampf(ml_out[d], -ML_MU_MAX, ML_MU_MAX));
              const T sd = T(clampf(ml_out[3 + d], ML_S_MIN, ML_S_MAX));
              sum_s += sd;
              x2 += sh.rgauss[jj][d] * sh.rgauss[jj][d];
              const T dd = drift[d] + st * mu + st * exp(sd) * sh.rgauss[jj][d];
              sh.disp[d]  = dd;
              sh.pos[d]   = r_now[d] + static_cast<double>(dd);
              sh.posT[d]  = static_cast<T>(sh.pos[d]);
            }
            spline_frac(s, sh.pos, sh.ru);
            sh.loggf = -sum_s - T(0.5) * x2;
          }
          __syncthreads();
        }
        else
        {
        if (threadIdx.x == 0)
        {
          if (!(fabs(g[3] - T(1)) <= HealthTol<T>::v))
            atomicOr(s.status + w, spin ? ST_ILLCOND_DN : ST_ILLCOND_UP);
          T gn[3];
          for (int d = 0; d < 3; d++)
          {
            T gs = g[d];
            if (s.has_j1)
              gs += j1_now[1 + d];
            if (s.has_j2)
              gs += J2s[(1 + d) * s.ne_pad + iat];
            gn[d] = gs;
          }
          if (s.trace)
          {
            double* tr = s.trace + ((size_t)iat * s.nw + w) * TRACE_FIELDS;
            for (int d = 0; d < 3; d++)
              tr[TR_GRAD_NOW + d] = static_cast<double>(gn[d]);
            tr[TR_SELF] = static_cast<double>(g[3]);
          }
          const T sqrttau = sqrt(tau);
          T delta[3], drift[3];
          for (int d = 0; d < 3; d++)
            delta[d] = sh.rgauss[jj][d] * sqrttau;
          if (s.use_drift)
          {
            unr_drift_t(tau, gn, drift);
            for (int d = 0; d < 3; d++)
              drift[d] += delta[d];
          }
          else
            for (int d = 0; d < 3; d++)
              drift[d] = delta[d];
          for (int d = 0; d < 3; d++)
          {
            sh.disp[d] = drift[d];
            sh.pos[d]  = r_now[d] + static_cast<double>(drift[d]);
            sh.posT[d] = static_cast<T>(sh.pos[d]);
          }
          spline_frac(s, sh.pos, sh.ru);
          sh.loggf = s.use_drift
              ? -(T(0.5) / tau) * (delta[0] * delta[0] + delta[1] * delta[1] + delta[2] * delta[2])
              : T(0);
        }
        __syncthreads();
        }
      }
      // ------------------------------------------------ evaluation at the proposed position
      // the FP64 position and its fractional coordinates were converted once, by thread 0
      T acc[14];
#pragma unroll
      for (int q = 0; q < 14; q++)
        acc[q] = T(0);
      const T x0 = sh.posT[0], y0 = sh.posT[1], z0 = sh.posT[2];
      // Jastrow rows against the positions in shared memory, threads t0, t0 + stride, ...
      auto jastrow_rows = [&](int t0, int stride) {
        if (s.has_j2)
          for (int j = t0; j < s.ne; j += stride)
          {
            if (j == iat)
              continue;
            const T dx = min_image(Rs[j] - x0, L0, Li0);
            const T dy = min_image(Rs[s.ne_pad + j] - y0, L1, Li1);
            const T dz = min_image(Rs[2 * s.ne_pad + j] - z0, L2, Li2);
            const T r  = sqrt(dx * dx + dy * dy + dz * dz);
            if (r < s.j2_rcut)
            {
              const int same = (j < s.nup) == (iat < s.nup);
              T du, d2u;
              const T u = functor_eval(s.j2c + (same ? 0 : s.j2_ncoef), s.j2_dri, s.j2_maxidx, r, du, d2u);
              du *= T(1) / r;
              acc[5] += u;
              acc[6] += du * dx;
              acc[7] += du * dy;
              acc[8] += du * dz;
              acc[9] += d2u + T(2) * du;
            }
          }
        if (s.has_j1)
          for (int j = t0; j < s.nions; j += stride)
          {
            const T dx = min_image(s.ions[j] - x0, L0, Li0);
            const T dy = min_image(s.ions[s.nions_pad + j] - y0, L1, Li1);
            const T dz = min_image(s.ions[2 * s.nions_pad + j] - z0, L2, Li2);
            const T r  = sqrt(dx * dx + dy * dy + dz * dz);
            if (r < s.j1_rcut)
            {
              T du, d2u;
              const T u =
                  functor_eval(s.j1c + (size_t)s.ion_species[j] * s.j1_ncoef, s.j1_dri, s.j1_maxidx, r, du, d2u);
              du *= T(1) / r;
              acc[10] += u;
              acc[11] += du * dx;
              acc[12] += du * dy;
              acc[13] += du * dz;
              acc[4] += d2u + T(2) * du;
            }
          }
      };
      spline_partials_frac(s, sh.ru, part);
      jastrow_rows(threadIdx.x, NT);
      __syncthreads();
      for (int o = threadIdx.x; o < n; o += NT)
      {
        T vgl[5];
        spline_combine(s, part, o, vgl);
#pragma unroll
        for (int q = 0; q < 5; q++)
          phi[q * lda + o] = vgl[q];
        const T x = inv[o];
        acc[0] += x * vgl[0];
        acc[1] += x * vgl[1];
        acc[2] += x * vgl[2];
        acc[3] += x * vgl[3];
      }
      block_sum_to0<T, 14>(acc, red);
      if (threadIdx.x == 0)
      {
        const T detr = acc[0];
        T g[3]       = {acc[1] / detr, acc[2] / detr, acc[3] / detr};
        T logj       = T(0);
        if (s.has_j1)
        {
          logj += j1_now[0] - acc[10];
          g[0] += acc[11];
          g[1] += acc[12];
          g[2] += acc[13];
        }
        if (s.has_j2)
        {
          logj += J2s[iat] - acc[5];
          g[0] += acc[6];
          g[1] += acc[7];
          g[2] += acc[8];
        }
        // |ratio|^2 = det^2 exp(2 log J)
        const T p = detr * detr * exp(T(2) * logj);
        if (!isfinite(p) || (p != T(0) && (!isfinite(g[0]) || !isfinite(g[1]) || !isfinite(g[2]))))
          atomicOr(s.status + w, ST_NONFINITE);
        sh.det    = detr;
        sh.cur[0] = acc[10];
        sh.cur[1] = acc[11];
        sh.cur[2] = acc[12];
        sh.cur[3] = acc[13];
        sh.cur[4] = acc[4];
        sh.cur[5] = acc[5];
        sh.cur[6] = acc[6];
        sh.cur[7] = acc[7];
        sh.cur[8] = acc[8];
        sh.cur[9] = -acc[9];
        if constexpr (LEARNED)
        {
          sh.lsm.p = p;
          for (int d = 0; d < 3; d++)
            sh.lsm.g[d] = g[d];
        }
        else
        {
        T log_gb = T(0);
        if (s.use_drift)
        {
          T dr[3];
          unr_drift_t(tau, g, dr);
          for (int d = 0; d < 3; d++)
            dr[d] += sh.disp[d];
          log_gb = -(T(0.5) / tau) * (dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2]);
        }
        int a = 0;
        // DMC: a move that changes the sign of psi is rejected (fixed node,
        // DMCBatched.cpp:203-210 with SFNBranch::phaseChanged for real ratios)
        if (p >= Eps<T>::v && (!s.dmc || detr > T(0)))
        {
          a = sh.runif[jj] < p * exp(log_gb - sh.loggf) ? 1 : 0;
        }
        if (s.dmc)
        {
          const double r2 = static_cast<double>(tau) *
              static_cast<double>(sh.rgauss[jj][0] * sh.rgauss[jj][0] + sh.rgauss[jj][1] * sh.rgauss[jj][1] +
                                  sh.rgauss[jj][2] * sh.rgauss[jj][2]);
          rr_prop += r2;
          if (a)
            rr_acc += r2;
        }
        if (a)
        {
          n_acc++;
          int ex;
          det_mant = frexp(det_mant * fabs(static_cast<double>(detr)), &ex);
          det_exp += ex;
          if (detr < T(0))
            det_neg ^= 1;
        }
        else
          n_rej++;
        sh.acc = a;
        if (s.trace)
        {
          double* tr = s.trace + ((size_t)iat * s.nw + w) * TRACE_FIELDS;
          for (int d = 0; d < 3; d++)
          {
            tr[TR_POS + d]      = sh.pos[d];
            tr[TR_GRAD_NEW + d] = static_cast<double>(g[d]);
          }
          tr[TR_RATIO]  = static_cast<double>(detr) * exp(static_cast<double>(logj));
          tr[TR_ACCEPT] = a;
        }
        }
      }
      __syncthreads();
      if constexpr (LEARNED)
      {
        // the network at the proposed position: the reverse density q(r | R')
        const T pn[3] = {sh.posT[0], sh.posT[1], sh.posT[2]};
        features_cta(s, Rs, iat, pn, sh.lsm.g, ml_x);
        __syncthreads();
        mlp_eval_cta(ml_pairs, ml_w4, s.mlp_params, ml_x, ml_h, ml_red, ml_out);
        if (threadIdx.x == 0)
        {
          const T st = sqrt(tau);
          T drift[3];
          unr_drift_t(tau, sh.lsm.g, drift);
          T sum_s = 0, z2 = 0;
          for (int d = 0; d < 3; d++)
          {
            const T mu = T(clampf(ml_out[d], -ML_MU_MAX, ML_MU_MAX));
            const T sd = T(clampf(ml_out[3 + d], ML_S_MIN, ML_S_MAX));
            sum_s += sd;
            const T z = (-sh.disp[d] - drift[d] - st * mu) / (st * exp(sd));
            z2 += z * z;
          }
          const T log_gb = -sum_s - T(0.5) * z2;
          const T p      = sh.lsm.p;
          const T detr   = sh.det;
          int a          = 0;
          if (p >= Eps<T>::v)
          {
            a = sh.runif[jj] < p * exp(log_gb - sh.loggf) ? 1 : 0;
          }
          if (a)
          {
            n_acc++;
            int ex;
            det_mant = frexp(det_mant * fabs(static_cast<double>(detr)), &ex);
            det_exp += ex;
            if (detr < T(0))
              det_neg ^= 1;
          }
          else
            n_rej++;
          sh.acc = a;
        }
        __syncthreads();
      }
      // ------------------------------------------------ accept / reject
      const bool accd = sh.acc != 0;
      if (K > 1)
      {
        T* U       = s.U + slot * K * lda;
        T* V       = s.V + slot * K * lda;
        int* dlist = s.delay_list + slot * K;
        for (int j = threadIdx.x; j < n; j += NT)
          V[(size_t)dc * lda + j] = arow[j];
        const int m = i1 - i0; // slots of this segment
        if (accd)
        {
          const T sigma = T(1) / sh.det;
          // phi . Ainv[row_x] for every electron x of the segment: x < dc are the V_x . phi
          // of the Binv update (V_x is Ainv[row_x]), x > dc the U . invRow terms of later slots
          rows_dot<T, NT>(s.Ainv + (slot * n + (i0 - first)) * lda, lda, m, phi, n, pv, T(1));
          __syncthreads();
          for (int x = dc + 1 + threadIdx.x; x < m; x += NT)
            tri[x * (x - 1) / 2 + dc] = pv[x];
          for (int i = threadIdx.x; i < dc; i += NT)
          {
            T a = 0;
            for (int c = 0; c < dc; c++)
              a += Bs[i * K + c] * pv[c];
            yv[i] = -sigma * a;
          }
          __syncthreads();
          for (int e = threadIdx.x; e < dc * dc; e += NT)
          {
            const int i = e / dc, j = e % dc;
            Bs[i * K + j] += Bs[dc * K + j] * yv[i];
          }
          __syncthreads();
          for (int i = threadIdx.x; i < dc; i += NT)
          {
            Bs[i * K + dc] = yv[i];
            Bs[dc * K + i] *= sigma;
          }
          if (threadIdx.x == 0)
          {
            Bs[dc * K + dc] = sigma;
            dlist[dc]       = row;
          }
          for (int j = threadIdx.x; j < n; j += NT)
            U[(size_t)dc * lda + j] = phi[j];
        }
        else
        {
          for (int x = dc + 1 + threadIdx.x; x < m; x += NT)
            tri[x * (x - 1) / 2 + dc] = T(0);
          for (int j = threadIdx.x; j < n; j += NT)
            U[(size_t)dc * lda + j] = T(0);
          for (int i = threadIdx.x; i < dc; i += NT)
            Bs[i * K + dc] = T(0);
          if (threadIdx.x == 0)
          {
            Bs[dc * K + dc] = T(1);
            dlist[dc]       = -1;
          }
        }
      }
      else if (accd)
      {
        // rank-1 Sherman-Morrison on the whole inverse (arow holds the old row)
        T* Aw  = s.Ainv + slot * n * lda;
        T* tmp = part;
        for (int j = wid; j < n; j += NT / 32)
        {
          T a = 0;
          for (int i = lane; i < n; i += 32)
            a += Aw[(size_t)j * lda + i] * phi[i];
          a = warp_sum(a);
          if (lane == 0)
            tmp[j] = (j == row) ? a - T(1) : a;
        }
        __syncthreads();
        const T c = T(-1) / sh.det;
        for (int e = threadIdx.x; e < n * n; e += NT)
        {
          const int j = e / n, i = e % n;
          Aw[(size_t)j * lda + i] += c * arow[i] * tmp[j];
        }
        // the prefetched rows of the next electron predate this update: fetch them again
        __syncthreads();
        if (iat + 1 < i1)
        {
          async_wait_all();
          __syncthreads();
          prefetch_rows(s, slot, row + 1, pre + ((iat + 1 - i0) & 1) * 5 * lda, threadIdx.x, NT);
        }
      }
      if (accd)
      {
        T* dgo = s.dgrad + ((slot * n + row) * 3) * lda;
        T* dlo = s.dlap + (slot * n + row) * lda;
        T* pvo = s.psiv + (slot * n + row) * lda;
        for (int j = threadIdx.x; j < n; j += NT)
        {
          pvo[j]           = phi[j];
          dgo[j]           = phi[1 * lda + j];
          dgo[lda + j]     = phi[2 * lda + j];
          dgo[2 * lda + j] = phi[3 * lda + j];
          dlo[j]           = phi[4 * lda + j];
        }
        if (s.has_j2)
        {
          const T xo = Rs[iat], yo = Rs[s.ne_pad + iat], zo = Rs[2 * s.ne_pad + iat];
          for (int j = threadIdx.x; j < s.ne; j += NT)
          {
            if (j == iat)
              continue;
            const int same = (j < s.nup) == (iat < s.nup);
            const T* fc    = s.j2c + (same ? 0 : s.j2_ncoef);
            const T xj = Rs[j], yj = Rs[s.ne_pad + j], zj = Rs[2 * s.ne_pad + j];
            const T odx = min_image(xj - xo, L0, Li0), ody = min_image(yj - yo, L1, Li1),
                    odz = min_image(zj - zo, L2, Li2);
            const T ndx = min_image(xj - x0, L0, Li0), ndy = min_image(yj - y0, L1, Li1),
                    ndz = min_image(zj - z0, L2, Li2);
            const T ro = sqrt(odx * odx + ody * ody + odz * odz);
            const T rn = sqrt(ndx * ndx + ndy * ndy + ndz * ndz);
            T u = 0, du = 0, d2u = 0, cu = 0, cdu = 0, cd2u = 0;
            if (ro < s.j2_rcut)
            {
              u = functor_eval(fc, s.j2_dri, s.j2_maxidx, ro, du, d2u);
              du *= T(1) / ro;
            }
            if (rn < s.j2_rcut)
            {
              cu = functor_eval(fc, s.j2_dri, s.j2_maxidx, rn, cdu, cd2u);
              cdu *= T(1) / rn;
            }
            J2s[j] += cu - u;
            J2s[1 * s.ne_pad + j] -= ndx * cdu - odx * du;
            J2s[2 * s.ne_pad + j] -= ndy * cdu - ody * du;
            J2s[3 * s.ne_pad + j] -= ndz * cdu - odz * du;
            J2s[4 * s.ne_pad + j] -= cd2u + T(2) * cdu - (d2u + T(2) * du);
          }
        }
        __syncthreads();
        if (threadIdx.x == 0)
        {
          if (s.has_j2)
            for (int q = 0; q < 5; q++)
              J2s[q * s.ne_pad + iat] = sh.cur[5 + q];
          if (s.has_j1)
            for (int q = 0; q < 5; q++)
              s.J1[((size_t)w * 5 + q) * s.ne_pad + iat] = sh.cur[q];
          for (int d = 0; d < 3; d++)
          {
            s.R[((size_t)w * 3 + d) * s.ne_pad + iat] = sh.pos[d];
            Rs[d * s.ne_pad + iat]                    = static_cast<T>(sh.pos[d]);
          }
        }
      }
      __syncthreads();
      if (K > 1)
        dc++;
    }
    async_wait_all();
    if (threadIdx.x == 0)
    {
      s.log_abs[slot] += log(det_mant) + det_exp * 0.69314718055994530942;
      if (det_neg)
        s.sign[slot] = -s.sign[slot];
      if (s.dmc)
      {
        s.rr[2 * w] += rr_prop;
        s.rr[2 * w + 1] += rr_acc;
      }
    }
    // hand the segment's Binv to the batched flush, positions and J2 state back to HBM
    if (K > 1)
    {
      T* Binv = s.Binv + slot * K * K;
      for (int e = threadIdx.x; e < dc * K; e += NT)
        Binv[e] = Bs[e];
    }
    for (int e = threadIdx.x; e < 3 * s.ne_pad; e += NT)
      s.Rt[(size_t)w * 3 * s.ne_pad + e] = Rs[e];
    for (int e = threadIdx.x; e < 5 * s.ne_pad; e += NT)
      s.J2[(size_t)w * 5 * s.ne_pad + e] = J2s[e];
    __syncthreads();
  }
}

template<typename T, int NT, int MINB, bool LEARNED>
__global__ void __launch_bounds__(NT, MINB) sweep_kernel(DevState<T> s, int i0, int i1)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ SweepShared<T, LEARNED> sh;
  unsigned long long n_acc = 0, n_rej = 0;
  for (int w = blockIdx.x; w < s.nw; w += gridDim.x)
    sweep_walker<T, NT, LEARNED>(s, i0, i1, w, smem_raw, sh, n_acc, n_rej);
  if (threadIdx.x == 0)
  {
    atomicAdd(s.counters + 0, n_acc);
    atomicAdd(s.counters + 1, n_rej);
  }
}

// ---------------------------------------------------------------------------
// Uneven crowds: one persistent launch covers one stage (the st-th segment of every
// crowd that has one).  Work items are (crowd, walker) pairs, ordered with the most
// expensive crowd first and handed out dynamically through a global counter, so CTAs
// that finish cheap walkers pick up the next item; each CTA loads a crowd's state
// descriptor into shared memory when it switches crowds.
// ---------------------------------------------------------------------------
template<typename T, int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB) sweep_multi_kernel(const DevState<T>* __restrict__ table, MultiStage st,
                                                               int* __restrict__ work)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ SweepShared<T, false> sh;
  __shared__ __align__(16) DevState<T> ds;
  __shared__ int s_item;
  unsigned long long n_acc = 0, n_rej = 0;
  int cur = -1;
  const int total = st.begin[st.nactive];
  for (;;)
  {
    if (threadIdx.x == 0)
      s_item = atomicAdd(work, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= total)
      break;
    int a = 0;
    while (a + 1 < st.nactive && item >= st.begin[a + 1])
      a++;
    const int c = st.crowd[a];
    if (c != cur)
    {
      if (cur >= 0 && threadIdx.x == 0)
      {
        atomicAdd(ds.counters + 0, n_acc);
        atomicAdd(ds.counters + 1, n_rej);
      }
      n_acc = n_rej = 0;
      __syncthreads();
      const int* src = reinterpret_cast<const int*>(table + c);
      int* dst       = reinterpret_cast<int*>(&ds);
      for (int e = threadIdx.x; e < (int)(sizeof(DevState<T>) / sizeof(int)); e += NT)
        dst[e] = src[e];
      __syncthreads();
      cur = c;
    }
    sweep_walker<T, NT, false>(ds, st.i0[a], st.i1[a], item - st.begin[a], smem_raw, sh, n_acc, n_rej);
    __syncthreads();
  }
  if (cur >= 0 && threadIdx.x == 0)
  {
    atomicAdd(ds.counters + 0, n_acc);
    atomicAdd(ds.counters + 1, n_rej);
  }
}

// threads per walker of the group launch: 128 or 256
template<typename T>
cudaError_t launch_sweep_multi(const DevState<T>* table, const MultiStage& st, size_t smem, int grid, int* work,
                               cudaStream_t stm, int nt)
{
  if (st.nactive <= 0)
    return cudaSuccess;
  if (nt == 256)
    sweep_multi_kernel<T, 256, sizeof(T) == 4 ? 2 : 1><<<grid, 256, smem, stm>>>(table, st, work);
  else
    sweep_multi_kernel<T, 128, sizeof(T) == 4 ? 4 : 2><<<grid, 128, smem, stm>>>(table, st, work);
  return cudaGetLastError();
}

template<typename T>
cudaError_t sweep_multi_grid(size_t smem, int* grid, int nt)
{
  int dev = 0, sms = 0, per_sm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess)
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  auto occ = [&](auto kern, int threads) {
    cudaError_t r = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    if (r == cudaSuccess)
      r = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem);
    return r;
  };
  if (e == cudaSuccess)
    e = nt == 256 ? occ(sweep_multi_kernel<T, 256, sizeof(T) == 4 ? 2 : 1>, 256)
                  : occ(sweep_multi_kernel<T, 128, sizeof(T) == 4 ? 4 : 2>, 128);
  if (e != cudaSuccess)
    return e;
  if (per_sm < 1)
    return cudaErrorInvalidConfiguration;
  *grid = per_sm * sms;
  return cudaSuccess;
}

// threads per walker of the drift-diffusion kernel: 128, 256 or 512 (FP64: up to 256);
// the registers per thread stay at 128 (255 for FP64) whatever the CTA size
template<typename T, int NT>
struct SweepMinb
{
  static constexpr int v = sizeof(T) == 4 ? (NT == 128 ? 4 : NT == 256 ? 2 : 1) : (NT == 128 ? 2 : 1);
};

bool sweep_threads_ok(int nt, int tsize) { return nt == 128 || nt == 256 || (nt == 512 && tsize == 4); }

template<typename T, typename F>
static cudaError_t with_threads(int nt, F&& f)
{
  if (nt == 128)
    return f(std::integral_constant<int, 128>{});
  if (nt == 256)
    return f(std::integral_constant<int, 256>{});
  if constexpr (sizeof(T) == 4)
    if (nt == 512)
      return f(std::integral_constant<int, 512>{});
  return cudaErrorInvalidValue;
}

template<typename T>
cudaError_t setup_sweep_kernel()
{
  cudaError_t e = cudaFuncSetAttribute(sweep_kernel<T, SweepCfg<T>::NT, SweepCfg<T>::MINB, true>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
  for (int nt : {128, 256, 512})
    if (e == cudaSuccess && sweep_threads_ok(nt, sizeof(T)))
      e = with_threads<T>(nt, [](auto c) {
        constexpr int NT = decltype(c)::value;
        return cudaFuncSetAttribute(sweep_kernel<T, NT, SweepMinb<T, NT>::v, false>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
      });
  return e;
}

template<typename T>
size_t sweep_smem_bytes(const DevState<T>& s)
{
  return sizeof(T) * sweep_smem_elems(s);
}

// electrons [i0, i1) of every walker, inside one spin group; with delayed updates
// i1 - i0 <= k and the host flushes after the launch.  The learned proposal needs 128
// threads (one per hidden neuron).
template<typename T>
cudaError_t launch_sweep_segment(const DevState<T>& s, int grid, int i0, int i1, cudaStream_t st, bool learned,
                                 int nt)
{
  if (i0 < 0 || i1 > s.ne || i1 <= i0 || (i0 < s.nup) != (i1 - 1 < s.nup) || (s.k > 1 && i1 - i0 > s.k))
    return cudaErrorInvalidValue;
  if (learned)
  {
    constexpr int NT = SweepCfg<T>::NT, MINB = SweepCfg<T>::MINB;
    if (!s.mlp_simt || !s.mlp_params)
      return cudaErrorInvalidValue;
    sweep_kernel<T, NT, MINB, true><<<grid, NT, sweep_smem_bytes(s), st>>>(s, i0, i1);
    return cudaGetLastError();
  }
  return with_threads<T>(nt, [&](auto c) {
    constexpr int NT = decltype(c)::value;
    sweep_kernel<T, NT, SweepMinb<T, NT>::v, false><<<grid, NT, sweep_smem_bytes(s), st>>>(s, i0, i1);
    return cudaGetLastError();
  });
}

template<typename T>
cudaError_t sweep_grid(const DevState<T>& s, int* grid, bool learned, int nt)
{
  int dev = 0, sms = 0, per_sm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess)
    return e;
  e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess)
    return e;
  if (learned)
  {
    constexpr int NT = SweepCfg<T>::NT, MINB = SweepCfg<T>::MINB;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sweep_kernel<T, NT, MINB, true>, NT,
                                                      sweep_smem_bytes(s));
  }
  else
    e = with_threads<T>(nt, [&](auto c) {
      constexpr int NT = decltype(c)::value;
      return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sweep_kernel<T, NT, SweepMinb<T, NT>::v, false>,
                                                           NT, sweep_smem_bytes(s));
    });
  if (e != cudaSuccess)
    return e;
  if (per_sm < 1)
    return cudaErrorInvalidConfiguration;
  *grid = std::min(s.nw, per_sm * sms);
  return cudaSuccess;
}

// default threads per walker: enough warps per SM when shared memory allows few CTAs
template<typename T>
int sweep_default_threads(const DevState<T>& s)
{
  const size_t sm = sweep_smem_bytes(s);
  if (sm > 114 * 1024)
    return sizeof(T) == 4 ? 512 : 256;
  if (sm > 76 * 1024)
    return 256;
  return 128;
}

template cudaError_t setup_sweep_kernel<float>();
template cudaError_t setup_sweep_kernel<double>();
template size_t sweep_smem_bytes<float>(const DevState<float>&);
template size_t sweep_smem_bytes<double>(const DevState<double>&);
template cudaError_t launch_sweep_segment<float>(const DevState<float>&, int, int, int, cudaStream_t, bool, int);
template cudaError_t launch_sweep_segment<double>(const DevState<double>&, int, int, int, cudaStream_t, bool, int);
template cudaError_t sweep_grid<float>(const DevState<float>&, int*, bool, int);
template cudaError_t sweep_grid<double>(const DevState<double>&, int*, bool, int);
template int sweep_default_threads<float>(const DevState<float>&);
template int sweep_default_threads<double>(const DevState<double>&);

template cudaError_t launch_sweep_multi<float>(const DevState<float>*, const MultiStage&, size_t, int, int*,
                                               cudaStream_t, int);
template cudaError_t launch_sweep_multi<double>(const DevState<double>*, const MultiStage&, size_t, int, int*,
                                                cudaStream_t, int);
template cudaError_t sweep_multi_grid<float>(size_t, int*, int);
template cudaError_t sweep_multi_grid<double>(size_t, int*, int);

} // namespace qmcg
