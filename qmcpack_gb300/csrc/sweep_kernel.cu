// Walker-resident sweep: one CTA owns one walker for a whole VMC sweep.
//
// With counter-based random numbers every walker's Markov chain is independent
// of the others (no cross-walker random-number cursor), so the whole body of
// VMCBatched::advanceWalkers (src/QMCDrivers/VMC/VMCBatched.cpp:106-177) for one
// walker runs inside one CTA: for every electron the proposal (mw_evalGrad +
// drift-diffusion), the evaluation at the proposed position (mw_makeMove +
// mw_calcRatioGrad), the accept test and the state update
// (mw_accept_rejectMove), and every k moves the delayed-update flush
// (DelayedUpdateBatched::mw_updateInvMat, DelayedUpdateBatched.h:675-738).
// The walker's positions and two-body Jastrow state stay in shared memory for
// the whole sweep; the inverse, U, V, Binv and the orbital-gradient rows stay in
// HBM/L2.  The arithmetic is the staged kernels' (same device routines), so the
// two paths agree to rounding.
#include <algorithm>

#include "common.cuh"
#include "launch.h"
#include "spline.cuh"

namespace qmcg
{

template<typename T>
struct SweepSmem
{
  // sizes in elements of T
  static size_t bytes(const DevState<T>& s, int rb)
  {
    const size_t part  = (size_t)28 * s.lda;
    const size_t flush = (size_t)rb * s.lda + (size_t)rb * s.k;
    return sizeof(T) * (std::max(part, flush) + 7 * (size_t)s.lda + 8 * (size_t)s.ne_pad + 3 * (size_t)s.k + 16 * 32);
  }
};

// Ainv -= (Ainv U^T - E)(Binv V) for one walker and spin, by the whole CTA.
template<typename T, int NT, int RB>
__device__ void flush_walker(const DevState<T>& s, int w, int spin, int dc, T* W, T* rows, T* t1)
{
  const size_t slot = (size_t)spin * s.nw + w;
  const int n       = s.norb;
  T* A              = s.Ainv + slot * n * s.lda;
  const T* U        = s.U + slot * s.k * s.lda;
  const T* V        = s.V + slot * s.k * s.lda;
  const T* Binv     = s.Binv + slot * s.k * s.k;
  const int* dlist  = s.delay_list + slot * s.k;
  for (int e = threadIdx.x; e < dc * n; e += NT)
  {
    const int l = e / n, i = e % n;
    T a         = 0;
    for (int c = 0; c < dc; c++)
      a += Binv[(size_t)l * s.k + c] * V[(size_t)c * s.lda + i];
    W[(size_t)l * s.lda + i] = a;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int r0 = 0; r0 < n; r0 += RB)
  {
    const int nr = min(RB, n - r0);
    for (int e = threadIdx.x; e < nr * n; e += NT)
    {
      const int r = e / n, i = e % n;
      rows[r * s.lda + i] = A[(size_t)(r0 + r) * s.lda + i];
    }
    __syncthreads();
    for (int e = wid; e < nr * dc; e += NT / 32)
    {
      const int r = e / dc, c = e % dc;
      T a         = 0;
      for (int i = lane; i < n; i += 32)
        a += rows[r * s.lda + i] * U[(size_t)c * s.lda + i];
      a = warp_sum(a);
      if (lane == 0)
        t1[r * s.k + c] = (dlist[c] == r0 + r) ? a - T(1) : a;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < nr * n; e += NT)
    {
      const int r = e / n, i = e % n;
      T a         = 0;
      for (int c = 0; c < dc; c++)
        a += t1[r * s.k + c] * W[(size_t)c * s.lda + i];
      A[(size_t)(r0 + r) * s.lda + i] = rows[r * s.lda + i] - a;
    }
    __syncthreads();
  }
}

template<typename T, int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB) sweep_kernel(DevState<T> s, T* Wbuf, int i0, int i1, int dc0, int inline_flush)
{
  constexpr int RB = 16;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* part   = reinterpret_cast<T*>(smem_raw);
  const size_t big = std::max((size_t)28 * s.lda, (size_t)RB * s.lda + (size_t)RB * s.k);
  T* arow   = part + big;
  T* invrow = arow + s.lda;
  T* phi    = invrow + s.lda; // 5 x lda
  T* Rs     = phi + 5 * s.lda; // 3 x ne_pad
  T* J2s    = Rs + 3 * s.ne_pad; // 5 x ne_pad
  T* pv     = J2s + 5 * s.ne_pad; // k
  T* tv     = pv + s.k;          // k
  T* yv     = tv + s.k;          // k
  T* red    = yv + s.k;          // 16 x 32
  T* rows   = part;
  T* t1     = part + RB * s.lda;
  __shared__ double s_pos[3];
  __shared__ double s_disp[3];
  __shared__ double s_loggf;
  __shared__ int s_acc;
  __shared__ T s_det;
  __shared__ T s_cur[10];

  const unsigned long long sweep = *s.sweep_counter;
  const uint32_t k0 = static_cast<uint32_t>(s.seed), k1 = static_cast<uint32_t>(s.seed >> 32);
  const int n = s.norb;
  unsigned long long n_acc = 0, n_rej = 0;
  const T L0 = T(s.L[0]), L1 = T(s.L[1]), L2 = T(s.L[2]);
  const T Li0 = T(1.0 / s.L[0]), Li1 = T(1.0 / s.L[1]), Li2 = T(1.0 / s.L[2]);

  for (int w = blockIdx.x; w < s.nw; w += gridDim.x)
  {
    T* Wg = Wbuf + (size_t)w * s.k * s.lda;
    for (int e = threadIdx.x; e < 3 * s.ne_pad; e += NT)
      Rs[e] = s.Rt[(size_t)w * 3 * s.ne_pad + e];
    for (int e = threadIdx.x; e < 5 * s.ne_pad; e += NT)
      J2s[e] = s.J2[(size_t)w * 5 * s.ne_pad + e];
    __syncthreads();
    int dc = dc0;
    for (int iat = i0; iat < i1; iat++)
    {
      const int spin = iat >= s.nup ? 1 : 0;
      const int row  = iat - (spin ? s.nup : 0);
      if (inline_flush && iat == s.nup && s.k > 1 && dc > 0)
      {
        // the up-spin delays are complete: flush them now (same result as at the sweep end)
        flush_walker<T, NT, RB>(s, w, 0, dc, Wg, rows, t1);
        dc = 0;
      }
      const size_t slot = (size_t)spin * s.nw + w;
      const T* A        = s.Ainv + (slot * n + row) * s.lda;
      // ------------------------------------------------ proposal
      for (int j = threadIdx.x; j < n; j += NT)
        arow[j] = A[j];
      __syncthreads();
      const T* inv = arow;
      if (s.k > 1 && dc > 0)
      {
        const T* U = s.U + slot * s.k * s.lda;
        const T* V = s.V + slot * s.k * s.lda;
        T* Binv    = s.Binv + slot * s.k * s.k;
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        for (int c = wid; c < dc; c += NT / 32)
        {
          T a = 0;
          for (int j = lane; j < n; j += 32)
            a += U[(size_t)c * s.lda + j] * arow[j];
          a = warp_sum(a);
          if (lane == 0)
            pv[c] = a;
        }
        __syncthreads();
        for (int i = threadIdx.x; i < dc; i += NT)
        {
          T a = 0;
          for (int c = 0; c < dc; c++)
            a += Binv[(size_t)c * s.k + i] * pv[c];
          tv[i]                      = -a;
          Binv[(size_t)dc * s.k + i] = -a;
        }
        __syncthreads();
        for (int j = threadIdx.x; j < n; j += NT)
        {
          T a = 0;
          for (int c = 0; c < dc; c++)
            a += V[(size_t)c * s.lda + j] * tv[c];
          invrow[j] = arow[j] + a;
        }
        __syncthreads();
        inv = invrow;
      }
      {
        const T* dg  = s.dgrad + ((slot * n + row) * 3) * s.lda;
        const T* pv0 = s.psiv + (slot * n + row) * s.lda;
        T g[4]       = {0, 0, 0, 0};
        for (int j = threadIdx.x; j < n; j += NT)
        {
          const T x = inv[j];
          g[0] += x * dg[j];
          g[1] += x * dg[s.lda + j];
          g[2] += x * dg[2 * s.lda + j];
          g[3] += x * pv0[j];
        }
        block_sum<T, 4>(g, red);
        if (threadIdx.x == 0)
        {
          if (!(fabs(g[3] - T(1)) <= HealthTol<T>::v))
            atomicOr(s.status + w, ST_ILLCOND);
          double gn[3];
          for (int d = 0; d < 3; d++)
          {
            double gs = static_cast<double>(g[d]);
            if (s.has_j1)
              gs += static_cast<double>(s.J1[((size_t)w * 5 + 1 + d) * s.ne_pad + iat]);
            if (s.has_j2)
              gs += static_cast<double>(J2s[(1 + d) * s.ne_pad + iat]);
            gn[d] = gs;
          }
          const u4 r0 = philox4x32_10(u4{(uint32_t)w, (uint32_t)iat, (uint32_t)sweep, 0u}, k0, k1);
          const u4 r1 = philox4x32_10(u4{(uint32_t)w, (uint32_t)iat, (uint32_t)sweep, 1u}, k0, k1);
          const double one_m = 1.0 - 2.2204460492503131e-16;
          const double t1_   = sqrt(-2.0 * log(1.0 - one_m * u01(r0.x, r0.y)));
          const double t2_   = 2.0 * 3.14159265358979323846 * u01(r0.z, r0.w);
          const double t3_   = sqrt(-2.0 * log(1.0 - one_m * u01(r1.x, r1.y)));
          const double t4_   = 2.0 * 3.14159265358979323846 * u01(r1.z, r1.w);
          double delta[3]    = {t1_ * cos(t2_), t1_ * sin(t2_), t3_ * cos(t4_)};
          const double sqrttau = sqrt(s.tau);
          for (int d = 0; d < 3; d++)
            delta[d] *= sqrttau;
          double drift[3];
          if (s.use_drift)
          {
            unr_drift(s.tau, gn, drift);
            for (int d = 0; d < 3; d++)
              drift[d] += delta[d];
          }
          else
            for (int d = 0; d < 3; d++)
              drift[d] = delta[d];
          for (int d = 0; d < 3; d++)
          {
            s_disp[d] = drift[d];
            s_pos[d]  = s.R[((size_t)w * 3 + d) * s.ne_pad + iat] + drift[d];
          }
          s_loggf = s.use_drift ? -(0.5 / s.tau) * (delta[0] * delta[0] + delta[1] * delta[1] + delta[2] * delta[2])
                                : 0.0;
        }
        __syncthreads();
      }
      // ------------------------------------------------ evaluation at the proposed position
      const double pos[3] = {s_pos[0], s_pos[1], s_pos[2]};
      spline_partials(s, pos, part);
      T acc[14];
#pragma unroll
      for (int q = 0; q < 14; q++)
        acc[q] = T(0);
      const T x0 = static_cast<T>(pos[0]), y0 = static_cast<T>(pos[1]), z0 = static_cast<T>(pos[2]);
      if (s.has_j2)
        for (int j = threadIdx.x; j < s.ne; j += NT)
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
        for (int j = threadIdx.x; j < s.nions; j += NT)
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
      __syncthreads();
      for (int o = threadIdx.x; o < n; o += NT)
      {
        T vgl[5];
        spline_combine(s, part, o, vgl);
#pragma unroll
        for (int q = 0; q < 5; q++)
          phi[q * s.lda + o] = vgl[q];
        const T x = inv[o];
        acc[0] += x * vgl[0];
        acc[1] += x * vgl[1];
        acc[2] += x * vgl[2];
        acc[3] += x * vgl[3];
      }
      block_sum<T, 14>(acc, red);
      if (threadIdx.x == 0)
      {
        const T detr = acc[0];
        double ratio = static_cast<double>(detr);
        double g[3]  = {static_cast<double>(acc[1] / detr), static_cast<double>(acc[2] / detr),
                        static_cast<double>(acc[3] / detr)};
        if (s.has_j1)
        {
          ratio *= exp(static_cast<double>(s.J1[((size_t)w * 5) * s.ne_pad + iat] - acc[10]));
          g[0] += static_cast<double>(acc[11]);
          g[1] += static_cast<double>(acc[12]);
          g[2] += static_cast<double>(acc[13]);
        }
        if (s.has_j2)
        {
          ratio *= exp(static_cast<double>(J2s[iat] - acc[5]));
          g[0] += static_cast<double>(acc[6]);
          g[1] += static_cast<double>(acc[7]);
          g[2] += static_cast<double>(acc[8]);
        }
        if (!isfinite(ratio) || (ratio != 0.0 && (!isfinite(g[0]) || !isfinite(g[1]) || !isfinite(g[2]))))
          atomicOr(s.status + w, ST_NONFINITE);
        const double p = ratio * ratio;
        double log_gb  = 0.0;
        if (s.use_drift)
        {
          double dr[3];
          unr_drift(s.tau, g, dr);
          for (int d = 0; d < 3; d++)
            dr[d] += s_disp[d];
          log_gb = -(0.5 / s.tau) * (dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2]);
        }
        int a = 0;
        if (p >= static_cast<double>(Eps<T>::v))
        {
          const u4 r2    = philox4x32_10(u4{(uint32_t)w, (uint32_t)iat, (uint32_t)sweep, 2u}, k0, k1);
          const double u = u01(r2.x, r2.y);
          a              = u < p * exp(log_gb - s_loggf) ? 1 : 0;
        }
        if (a)
        {
          n_acc++;
          if (detr == T(0))
            atomicOr(s.status + w, ST_ZERO_RATIO);
          s.log_abs[slot] += log(fabs(static_cast<double>(detr)));
          if (detr < T(0))
            s.sign[slot] = -s.sign[slot];
        }
        else
          n_rej++;
        s_acc = a;
        s_det = detr;
        s_cur[0] = acc[10];
        s_cur[1] = acc[11];
        s_cur[2] = acc[12];
        s_cur[3] = acc[13];
        s_cur[4] = acc[4];
        s_cur[5] = acc[5];
        s_cur[6] = acc[6];
        s_cur[7] = acc[7];
        s_cur[8] = acc[8];
        s_cur[9] = -acc[9];
      }
      __syncthreads();
      // ------------------------------------------------ accept / reject
      const bool accd = s_acc != 0;
      if (s.k > 1)
      {
        T* U       = s.U + slot * s.k * s.lda;
        T* V       = s.V + slot * s.k * s.lda;
        T* Binv    = s.Binv + slot * s.k * s.k;
        int* dlist = s.delay_list + slot * s.k;
        for (int j = threadIdx.x; j < n; j += NT)
          V[(size_t)dc * s.lda + j] = arow[j];
        if (accd)
        {
          const T sigma = T(1) / s_det;
          const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
          for (int c = wid; c < dc; c += NT / 32)
          {
            T a = 0;
            for (int j = lane; j < n; j += 32)
              a += V[(size_t)c * s.lda + j] * phi[j];
            a = warp_sum(a);
            if (lane == 0)
              pv[c] = -a;
          }
          __syncthreads();
          for (int i = threadIdx.x; i < dc; i += NT)
          {
            T a = 0;
            for (int c = 0; c < dc; c++)
              a += Binv[(size_t)i * s.k + c] * pv[c];
            yv[i] = sigma * a;
          }
          __syncthreads();
          for (int e = threadIdx.x; e < dc * dc; e += NT)
          {
            const int i = e / dc, j = e % dc;
            Binv[(size_t)i * s.k + j] += Binv[(size_t)dc * s.k + j] * yv[i];
          }
          __syncthreads();
          for (int i = threadIdx.x; i < dc; i += NT)
          {
            Binv[(size_t)i * s.k + dc] = yv[i];
            Binv[(size_t)dc * s.k + i] *= sigma;
          }
          if (threadIdx.x == 0)
          {
            Binv[(size_t)dc * s.k + dc] = sigma;
            dlist[dc]                   = row;
          }
          for (int j = threadIdx.x; j < n; j += NT)
            U[(size_t)dc * s.lda + j] = phi[j];
        }
        else
        {
          for (int j = threadIdx.x; j < n; j += NT)
            U[(size_t)dc * s.lda + j] = T(0);
          for (int i = threadIdx.x; i < dc; i += NT)
            Binv[(size_t)i * s.k + dc] = T(0);
          if (threadIdx.x == 0)
          {
            Binv[(size_t)dc * s.k + dc] = T(1);
            dlist[dc]                   = -1;
          }
        }
      }
      else if (accd)
      {
        // rank-1 Sherman-Morrison on the whole inverse (arow holds the old row)
        T* Aw = s.Ainv + slot * n * s.lda;
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        T* tmp = part; // n
        for (int j = wid; j < n; j += NT / 32)
        {
          T a = 0;
          for (int i = lane; i < n; i += 32)
            a += Aw[(size_t)j * s.lda + i] * phi[i];
          a = warp_sum(a);
          if (lane == 0)
            tmp[j] = (j == row) ? a - T(1) : a;
        }
        __syncthreads();
        const T c = T(-1) / s_det;
        for (int e = threadIdx.x; e < n * n; e += NT)
        {
          const int j = e / n, i = e % n;
          Aw[(size_t)j * s.lda + i] += c * arow[i] * tmp[j];
        }
      }
      if (accd)
      {
        T* dg  = s.dgrad + ((slot * n + row) * 3) * s.lda;
        T* dl  = s.dlap + (slot * n + row) * s.lda;
        T* pv0 = s.psiv + (slot * n + row) * s.lda;
        for (int j = threadIdx.x; j < n; j += NT)
        {
          pv0[j]            = phi[j];
          dg[j]             = phi[1 * s.lda + j];
          dg[s.lda + j]     = phi[2 * s.lda + j];
          dg[2 * s.lda + j] = phi[3 * s.lda + j];
          dl[j]             = phi[4 * s.lda + j];
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
              J2s[q * s.ne_pad + iat] = s_cur[5 + q];
          if (s.has_j1)
            for (int q = 0; q < 5; q++)
              s.J1[((size_t)w * 5 + q) * s.ne_pad + iat] = s_cur[q];
          for (int d = 0; d < 3; d++)
          {
            s.R[((size_t)w * 3 + d) * s.ne_pad + iat] = s_pos[d];
            Rs[d * s.ne_pad + iat]                    = static_cast<T>(s_pos[d]);
          }
        }
      }
      __syncthreads();
      if (s.k > 1)
      {
        dc++;
        if (inline_flush && dc == s.k)
        {
          flush_walker<T, NT, RB>(s, w, spin, dc, Wg, rows, t1);
          dc = 0;
        }
      }
    }
    if (inline_flush && s.k > 1 && dc > 0 && i1 == s.ne)
      flush_walker<T, NT, RB>(s, w, 1, dc, Wg, rows, t1);
    for (int e = threadIdx.x; e < 3 * s.ne_pad; e += NT)
      s.Rt[(size_t)w * 3 * s.ne_pad + e] = Rs[e];
    for (int e = threadIdx.x; e < 5 * s.ne_pad; e += NT)
      s.J2[(size_t)w * 5 * s.ne_pad + e] = J2s[e];
    __syncthreads();
  }
  if (threadIdx.x == 0)
  {
    atomicAdd(s.counters + 0, n_acc);
    atomicAdd(s.counters + 1, n_rej);
  }
}

template<typename T>
cudaError_t setup_sweep_kernel()
{
  return cudaFuncSetAttribute(sweep_kernel<T, 128, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
}

template<typename T>
size_t sweep_smem_bytes(const DevState<T>& s)
{
  return SweepSmem<T>::bytes(s, 16);
}

template<typename T>
cudaError_t launch_sweep(const DevState<T>& s, T* W, int grid, cudaStream_t st)
{
  sweep_kernel<T, 128, 4><<<grid, 128, sweep_smem_bytes(s), st>>>(s, W, 0, s.ne, 0, 1);
  return cudaGetLastError();
}

// electrons [i0, i1) of every walker starting at delay count dc0; a segment that
// would fill the delay window is cut by the host so the flush runs batched
template<typename T>
cudaError_t launch_sweep_segment(const DevState<T>& s, T* W, int grid, int i0, int i1, int dc0, cudaStream_t st)
{
  sweep_kernel<T, 128, 4><<<grid, 128, sweep_smem_bytes(s), st>>>(s, W, i0, i1, dc0, 0);
  return cudaGetLastError();
}

template<typename T>
cudaError_t sweep_grid(const DevState<T>& s, int* grid)
{
  int dev = 0, sms = 0, per_sm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess)
    return e;
  e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess)
    return e;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sweep_kernel<T, 128, 4>, 128, sweep_smem_bytes(s));
  if (e != cudaSuccess)
    return e;
  if (per_sm < 1)
    return cudaErrorInvalidConfiguration;
  *grid = std::min(s.nw, per_sm * sms);
  return cudaSuccess;
}

template cudaError_t setup_sweep_kernel<float>();
template cudaError_t setup_sweep_kernel<double>();
template size_t sweep_smem_bytes<float>(const DevState<float>&);
template size_t sweep_smem_bytes<double>(const DevState<double>&);
template cudaError_t launch_sweep<float>(const DevState<float>&, float*, int, cudaStream_t);
template cudaError_t launch_sweep<double>(const DevState<double>&, double*, int, cudaStream_t);
template cudaError_t launch_sweep_segment<float>(const DevState<float>&, float*, int, int, int, int, cudaStream_t);
template cudaError_t launch_sweep_segment<double>(const DevState<double>&, double*, int, int, int, int,
                                                  cudaStream_t);
template cudaError_t sweep_grid<float>(const DevState<float>&, int*);
template cudaError_t sweep_grid<double>(const DevState<double>&, int*);

} // namespace qmcg
