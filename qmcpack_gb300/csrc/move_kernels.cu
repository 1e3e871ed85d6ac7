// Kernels of one particle-by-particle move, batched over the walkers of a crowd.
//
// Per electron iat the sweep runs three launches (plus a flush every k moves):
//   propose_kernel  <- DelayedUpdateBatched::mw_prepareInvRow + mw_evalGrad
//                      (DelayedUpdateBatched.h:174-235, 354-400), J1/J2 evalGrad,
//                      drift-diffusion proposal (VMCBatched.cpp:119-133)
//   ratio_kernel    <- SoaDistanceTableAA/AB mw_move (SoaDistanceTableAAOMPTarget.h:265-380),
//                      J1/J2 ratioGrad (J1OrbitalSoA.h:441-450, BsplineFunctor.cpp:26-133),
//                      SplineR2R::mw_evaluateVGLandDetRatioGrads (SplineR2R.cpp:414-582),
//                      Green's function and acceptance argument (VMCBatched.cpp:135-155)
//   accept_kernel   <- accept test (VMCBatched.cpp:156-167), DiracDeterminantBatched::
//                      mw_accept_rejectMove + DelayedUpdateBatched::mw_accept_rejectRow
//                      (DelayedUpdateBatched.h:542-670), J2 mw_updateVGL (BsplineFunctor.cpp:203-320),
//                      J1 acceptMove, position accept (RealSpacePositionsOMPTarget.h:110-170)
//   flush           <- DelayedUpdateBatched::mw_updateInvMat (DelayedUpdateBatched.h:675-738)
// One CTA owns one walker in the first three, so every walker's move is
// independent and the only cross-walker data is the random-number cursor.
#include "common.cuh"
#include "launch.h"
#include "spline.cuh"

namespace qmcg
{

// ---------------------------------------------------------------------------
// propose_kernel: prepare the up-to-date inverse row, gradient of log psi of
// the current position and (driver mode) the drift-diffusion proposal.
// ---------------------------------------------------------------------------
template<typename T, int NT>
__global__ void __launch_bounds__(NT) propose_kernel(DevState<T> s, int iat, int dc, int driver)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* arow   = reinterpret_cast<T*>(smem_raw);  // lda
  T* pvec   = arow + s.lda;                    // k
  T* tvec   = pvec + s.k;                      // k
  __shared__ T red[4 * 32];
  const int iw   = blockIdx.x;
  const int spin = iat >= s.nup ? 1 : 0;
  const int row  = iat - (spin ? s.nup : 0);
  const int n    = s.norb;
  const size_t wslot = (size_t)spin * s.nw + iw;
  const T* A     = s.Ainv + (wslot * n + row) * s.lda;
  for (int j = threadIdx.x; j < n; j += blockDim.x)
    arow[j] = A[j];
  __syncthreads();
  const T* inv = arow;
  if (s.k > 1)
  {
    T* invRow = s.invRow + (size_t)iw * s.lda;
    if (dc > 0)
    {
      const size_t set0 = wslot * s.nsets; // set 0 of this slot
      const T* U = s.U + set0 * s.k * s.lda;
      const T* V = s.V + set0 * s.k * s.lda;
      T* Binv    = s.Binv + set0 * s.k * s.k;
      const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
      // p[c] = U[c] . Ainv[row]
      for (int c = wid; c < dc; c += NT / 32)
      {
        T acc = 0;
        for (int j = lane; j < n; j += 32)
          acc += U[(size_t)c * s.lda + j] * arow[j];
        acc = warp_sum(acc);
        if (lane == 0)
          pvec[c] = acc;
      }
      __syncthreads();
      // t[i] = -sum_c Binv[c][i] p[c], kept in Binv row dc for the accept step
      for (int i = threadIdx.x; i < dc; i += blockDim.x)
      {
        T acc = 0;
        for (int c = 0; c < dc; c++)
          acc += Binv[(size_t)c * s.k + i] * pvec[c];
        tvec[i]                    = -acc;
        Binv[(size_t)dc * s.k + i] = -acc;
      }
      __syncthreads();
      for (int j = threadIdx.x; j < n; j += blockDim.x)
      {
        T acc = 0;
        for (int c = 0; c < dc; c++)
          acc += V[(size_t)c * s.lda + j] * tvec[c];
        const T v = arow[j] + acc;
        invRow[j] = v;
        arow[j]   = v;
      }
      __syncthreads();
    }
    else
    {
      for (int j = threadIdx.x; j < n; j += blockDim.x)
        invRow[j] = arow[j];
    }
  }
  // gradient of the determinant part: invRow . dgrad[row]; self ratio invRow . psiv[row] (= 1)
  const T* dg = s.dgrad + ((wslot * n + row) * 3) * s.lda;
  const T* pv0 = s.psiv + (wslot * n + row) * s.lda;
  T g[4]      = {0, 0, 0, 0};
  for (int j = threadIdx.x; j < n; j += blockDim.x)
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
      atomicOr(s.status + iw, ST_ILLCOND);
    double gn[3];
    for (int d = 0; d < 3; d++)
    {
      double gs = static_cast<double>(g[d]);
      if (s.has_j1)
        gs += static_cast<double>(s.J1[((size_t)iw * 5 + 1 + d) * s.ne_pad + iat]);
      if (s.has_j2)
        gs += static_cast<double>(s.J2[((size_t)iw * 5 + 1 + d) * s.ne_pad + iat]);
      gn[d]                 = gs;
      s.grads_now[iw * 3 + d] = gs;
    }
    if (driver)
    {
      // driver arithmetic in the move-loop precision (RealType of the reference)
      T gt[3];
      for (int d = 0; d < 3; d++)
      {
        T gs = g[d];
        if (s.has_j1)
          gs += s.J1[((size_t)iw * 5 + 1 + d) * s.ne_pad + iat];
        if (s.has_j2)
          gs += s.J2[((size_t)iw * 5 + 1 + d) * s.ne_pad + iat];
        gt[d] = gs;
      }
      (void)gn;
      const T tau = T(s.tau);
      T delta[3];
      if (s.rng_mode == 0)
      {
        const double* gz = s.gauss + ((size_t)iat * s.nw + iw) * 3;
        for (int d = 0; d < 3; d++)
          delta[d] = T(gz[d]);
      }
      else
      {
        const uint32_t sw = static_cast<uint32_t>(*s.sweep_counter);
        gaussians<T>((uint32_t)iw, (uint32_t)iat, sw, static_cast<uint32_t>(s.seed),
                     static_cast<uint32_t>(s.seed >> 32), delta);
      }
      const T sqrttau = sqrt(tau);
      for (int d = 0; d < 3; d++)
        delta[d] *= sqrttau;
      T drift[3];
      if (s.use_drift)
      {
        unr_drift_t(tau, gt, drift);
        for (int d = 0; d < 3; d++)
          drift[d] += delta[d];
      }
      else
        for (int d = 0; d < 3; d++)
          drift[d] = delta[d];
      for (int d = 0; d < 3; d++)
      {
        s.disp[iw * 3 + d]       = static_cast<double>(drift[d]);
        s.active_pos[iw * 3 + d] = s.R[((size_t)iw * 3 + d) * s.ne_pad + iat] + static_cast<double>(drift[d]);
      }
      s.log_gf[iw] = s.use_drift
          ? static_cast<double>(-(T(0.5) / tau) * (delta[0] * delta[0] + delta[1] * delta[1] + delta[2] * delta[2]))
          : 0.0;
    }
  }
}

// active position from a caller displacement (ParticleSet::mw_makeMove)
template<typename T>
__global__ void make_move_kernel(DevState<T> s, int iat)
{
  const int iw = blockIdx.x * blockDim.x + threadIdx.x;
  if (iw >= s.nw)
    return;
  for (int d = 0; d < 3; d++)
    s.active_pos[iw * 3 + d] = s.R[((size_t)iw * 3 + d) * s.ne_pad + iat] + s.disp[iw * 3 + d];
}

// ---------------------------------------------------------------------------
// ratio_kernel: everything evaluated at the proposed position.
// ---------------------------------------------------------------------------
template<typename T, int NT>
__global__ void __launch_bounds__(NT) ratio_kernel(DevState<T> s, int iat, int driver)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* part = reinterpret_cast<T*>(smem_raw); // [4][7][lda]
  __shared__ T red[14 * 32];
  const int iw   = blockIdx.x;
  const int spin = iat >= s.nup ? 1 : 0;
  const int row  = iat - (spin ? s.nup : 0);
  const int n    = s.norb;
  const size_t wslot = (size_t)spin * s.nw + iw;
  double pos[3];
  for (int d = 0; d < 3; d++)
    pos[d] = s.active_pos[iw * 3 + d];

  spline_partials(s, pos, part);

  // two-body Jastrow over all other electrons and one-body over the ions,
  // computed while the spline loads are in flight in other warps
  T acc[14];
#pragma unroll
  for (int q = 0; q < 14; q++)
    acc[q] = T(0);
  const T x0 = static_cast<T>(pos[0]), y0 = static_cast<T>(pos[1]), z0 = static_cast<T>(pos[2]);
  const T L0 = T(s.L[0]), L1 = T(s.L[1]), L2 = T(s.L[2]);
  const T Li0 = T(s.G[0]), Li1 = T(s.G[1]), Li2 = T(s.G[2]);
  if (s.has_j2)
  {
    const T* Rx = s.Rt + ((size_t)iw * 3) * s.ne_pad;
    for (int j = threadIdx.x; j < s.ne; j += blockDim.x)
    {
      if (j == iat)
        continue;
      const T dx = min_image(Rx[j] - x0, L0, Li0);
      const T dy = min_image(Rx[s.ne_pad + j] - y0, L1, Li1);
      const T dz = min_image(Rx[2 * s.ne_pad + j] - z0, L2, Li2);
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
  }
  if (s.has_j1)
  {
    for (int j = threadIdx.x; j < s.nions; j += blockDim.x)
    {
      const T dx = min_image(s.ions[j] - x0, L0, Li0);
      const T dy = min_image(s.ions[s.nions_pad + j] - y0, L1, Li1);
      const T dz = min_image(s.ions[2 * s.nions_pad + j] - z0, L2, Li2);
      const T r  = sqrt(dx * dx + dy * dy + dz * dz);
      if (r < s.j1_rcut)
      {
        T du, d2u;
        const T u = functor_eval(s.j1c + (size_t)s.ion_species[j] * s.j1_ncoef, s.j1_dri, s.j1_maxidx, r, du, d2u);
        du *= T(1) / r;
        acc[10] += u;
        acc[11] += du * dx;
        acc[12] += du * dy;
        acc[13] += du * dz;
        acc[0 + 4] += d2u + T(2) * du; // J1 laplacian kept in slot 4
      }
    }
  }
  __syncthreads();
  // orbital VGL, saved for the accept step, and the determinant ratio / gradient
  const T* inv = (s.k > 1) ? s.invRow + (size_t)iw * s.lda : s.Ainv + (wslot * n + row) * s.lda;
  T* phi       = s.phi + (size_t)iw * 5 * s.lda;
  for (int o = threadIdx.x; o < n; o += blockDim.x)
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
    s.cur_det[iw] = detr;
    double ratio  = static_cast<double>(detr);
    double g[3]   = {static_cast<double>(acc[1] / detr), static_cast<double>(acc[2] / detr),
                     static_cast<double>(acc[3] / detr)};
    T* cj         = s.cur_j + (size_t)iw * 10;
    if (s.has_j1)
    {
      cj[0] = acc[10];
      cj[1] = acc[11];
      cj[2] = acc[12];
      cj[3] = acc[13];
      cj[4] = acc[4];
      ratio *= exp(static_cast<double>(s.J1[((size_t)iw * 5) * s.ne_pad + iat] - acc[10]));
      g[0] += static_cast<double>(acc[11]);
      g[1] += static_cast<double>(acc[12]);
      g[2] += static_cast<double>(acc[13]);
    }
    if (s.has_j2)
    {
      cj[5] = acc[5];
      cj[6] = acc[6];
      cj[7] = acc[7];
      cj[8] = acc[8];
      cj[9] = -acc[9];
      ratio *= exp(static_cast<double>(s.J2[((size_t)iw * 5) * s.ne_pad + iat] - acc[5]));
      g[0] += static_cast<double>(acc[6]);
      g[1] += static_cast<double>(acc[7]);
      g[2] += static_cast<double>(acc[8]);
    }
    s.ratios[iw] = ratio;
    for (int d = 0; d < 3; d++)
      s.grads_new[iw * 3 + d] = g[d];
    if (!isfinite(ratio) || (ratio != 0.0 && (!isfinite(g[0]) || !isfinite(g[1]) || !isfinite(g[2]))))
      atomicOr(s.status + iw, ST_NONFINITE);
    if (driver)
    {
      // driver arithmetic in the move-loop precision: |ratio|^2 = det^2 exp(2 log J)
      T logj = T(0);
      T gt[3] = {acc[1] / detr, acc[2] / detr, acc[3] / detr};
      if (s.has_j1)
      {
        logj += s.J1[((size_t)iw * 5) * s.ne_pad + iat] - acc[10];
        gt[0] += acc[11];
        gt[1] += acc[12];
        gt[2] += acc[13];
      }
      if (s.has_j2)
      {
        logj += s.J2[((size_t)iw * 5) * s.ne_pad + iat] - acc[5];
        gt[0] += acc[6];
        gt[1] += acc[7];
        gt[2] += acc[8];
      }
      const T tau = T(s.tau);
      const T p   = detr * detr * exp(T(2) * logj);
      T log_gb    = T(0);
      if (s.use_drift)
      {
        T dr[3];
        unr_drift_t(tau, gt, dr);
        for (int d = 0; d < 3; d++)
          dr[d] += T(s.disp[iw * 3 + d]);
        log_gb = -(T(0.5) / tau) * (dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2]);
      }
      s.flag[iw] = (p >= Eps<T>::v) ? 1 : 0;
      s.prob[iw] = static_cast<double>(p * exp(log_gb - T(s.log_gf[iw])));
    }
  }
}

// ---------------------------------------------------------------------------
// accept_kernel: accept/reject decision (driver mode) and every state update.
// ---------------------------------------------------------------------------
template<typename T, int NT>
__global__ void __launch_bounds__(NT) accept_kernel(DevState<T> s, int iat, int dc, int driver)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* pv  = reinterpret_cast<T*>(smem_raw); // k
  T* yv  = pv + s.k;                       // k
  __shared__ int s_acc;
  __shared__ int s_before;
  __shared__ int s_total;
  const int iw   = blockIdx.x;
  const int spin = iat >= s.nup ? 1 : 0;
  const int row  = iat - (spin ? s.nup : 0);
  const int n    = s.norb;
  const size_t wslot = (size_t)spin * s.nw + iw;

  if (driver)
  {
    // walkers before this one that consume a uniform (valid && p >= eps)
    int before = 0, total = 0;
    for (int j = threadIdx.x; j < s.nw; j += blockDim.x)
    {
      const int f = s.flag[j];
      total += f;
      if (j < iw)
        before += f;
    }
    before = __reduce_add_sync(0xffffffffu, before);
    total  = __reduce_add_sync(0xffffffffu, total);
    if (threadIdx.x == 0)
    {
      s_before = 0;
      s_total  = 0;
    }
    __syncthreads();
    if ((threadIdx.x & 31) == 0)
    {
      atomicAdd(&s_before, before);
      atomicAdd(&s_total, total);
    }
    __syncthreads();
    if (threadIdx.x == 0)
    {
      int acc = 0;
      if (s.flag[iw])
      {
        T u;
        if (s.rng_mode == 0)
          u = T(s.uniform[s.ucursor[iat & 1] + s_before]);
        else
        {
          const uint32_t sw = static_cast<uint32_t>(*s.sweep_counter);
          const uint32_t k0 = static_cast<uint32_t>(s.seed), k1 = static_cast<uint32_t>(s.seed >> 32);
          const u4 r2 = philox4x32_10(u4{(uint32_t)iw, (uint32_t)iat, sw, 2u}, k0, k1);
          u           = T(u01(r2.x, r2.y));
        }
        acc = u < T(s.prob[iw]) ? 1 : 0;
      }
      s.accepted[iw] = acc;
      if (iw == 0 && s.rng_mode == 0)
        s.ucursor[(iat + 1) & 1] = s.ucursor[iat & 1] + s_total;
      atomicAdd(s.counters + (acc ? 0 : 1), 1ull);
      s_acc = acc;
    }
    __syncthreads();
  }
  else
  {
    if (threadIdx.x == 0)
      s_acc = s.accepted[iw];
    __syncthreads();
  }
  const bool acc = s_acc != 0;
  const T* phi   = s.phi + (size_t)iw * 5 * s.lda;
  T* A           = s.Ainv + (wslot * n + row) * s.lda;

  // ---------------- determinant
  if (acc && threadIdx.x == 0)
  {
    const T detr = s.cur_det[iw];
    if (detr == T(0))
      atomicOr(s.status + iw, ST_ZERO_RATIO);
    s.log_abs[wslot] += log(fabs(static_cast<double>(detr)));
    if (detr < T(0))
      s.sign[wslot] = -s.sign[wslot];
  }
  if (s.k > 1)
  {
    const size_t set0 = wslot * s.nsets; // set 0 of this slot
    T* U       = s.U + set0 * s.k * s.lda;
    T* V       = s.V + set0 * s.k * s.lda;
    T* Binv    = s.Binv + set0 * s.k * s.k;
    int* dlist = s.delay_list + set0 * s.k;
    for (int j = threadIdx.x; j < n; j += blockDim.x)
      V[(size_t)dc * s.lda + j] = A[j];
    if (acc)
    {
      const T sigma = T(1) / s.cur_det[iw];
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
      for (int i = threadIdx.x; i < dc; i += blockDim.x)
      {
        T a = 0;
        for (int c = 0; c < dc; c++)
          a += Binv[(size_t)i * s.k + c] * pv[c];
        yv[i] = sigma * a;
      }
      __syncthreads();
      for (int e = threadIdx.x; e < dc * dc; e += blockDim.x)
      {
        const int i = e / dc, j = e % dc;
        Binv[(size_t)i * s.k + j] += Binv[(size_t)dc * s.k + j] * yv[i];
      }
      __syncthreads();
      for (int i = threadIdx.x; i < dc; i += blockDim.x)
      {
        Binv[(size_t)i * s.k + dc] = yv[i];
        Binv[(size_t)dc * s.k + i] *= sigma;
      }
      if (threadIdx.x == 0)
      {
        Binv[(size_t)dc * s.k + dc] = sigma;
        dlist[dc]                   = row;
      }
      for (int j = threadIdx.x; j < n; j += blockDim.x)
        U[(size_t)dc * s.lda + j] = phi[j];
    }
    else
    {
      for (int j = threadIdx.x; j < n; j += blockDim.x)
        U[(size_t)dc * s.lda + j] = T(0);
      for (int i = threadIdx.x; i < dc; i += blockDim.x)
        Binv[(size_t)i * s.k + dc] = T(0);
      if (threadIdx.x == 0)
      {
        Binv[(size_t)dc * s.k + dc] = T(1);
        dlist[dc]                   = -1;
      }
    }
  }
  else if (acc)
  {
    // rank-1 path: keep a copy of the old row for the Sherman-Morrison kernel
    T* rc = s.rcopy + (size_t)iw * s.lda;
    for (int j = threadIdx.x; j < n; j += blockDim.x)
      rc[j] = A[j];
  }
  if (acc)
  {
    T* dg = s.dgrad + ((wslot * n + row) * 3) * s.lda;
    T* dl = s.dlap + (wslot * n + row) * s.lda;
    T* pv0 = s.psiv + (wslot * n + row) * s.lda;
    for (int j = threadIdx.x; j < n; j += blockDim.x)
    {
      pv0[j]            = phi[j];
      dg[j]             = phi[1 * s.lda + j];
      dg[s.lda + j]     = phi[2 * s.lda + j];
      dg[2 * s.lda + j] = phi[3 * s.lda + j];
      dl[j]             = phi[4 * s.lda + j];
    }
  }
  if (!acc)
    return;

  // ---------------- two-body Jastrow state (new minus old pair terms)
  const T* cj = s.cur_j + (size_t)iw * 10;
  if (s.has_j2)
  {
    T* J2  = s.J2 + (size_t)iw * 5 * s.ne_pad;
    const T* Rx = s.Rt + ((size_t)iw * 3) * s.ne_pad;
    const T xn = static_cast<T>(s.active_pos[iw * 3 + 0]), yn = static_cast<T>(s.active_pos[iw * 3 + 1]),
            zn = static_cast<T>(s.active_pos[iw * 3 + 2]);
    const T xo = Rx[iat], yo = Rx[s.ne_pad + iat], zo = Rx[2 * s.ne_pad + iat];
    const T L0 = T(s.L[0]), L1 = T(s.L[1]), L2 = T(s.L[2]);
    const T Li0 = T(s.G[0]), Li1 = T(s.G[1]), Li2 = T(s.G[2]);
    for (int j = threadIdx.x; j < s.ne; j += blockDim.x)
    {
      if (j == iat)
        continue;
      const int same = (j < s.nup) == (iat < s.nup);
      const T* fc    = s.j2c + (same ? 0 : s.j2_ncoef);
      const T xj = Rx[j], yj = Rx[s.ne_pad + j], zj = Rx[2 * s.ne_pad + j];
      const T odx = min_image(xj - xo, L0, Li0), ody = min_image(yj - yo, L1, Li1), odz = min_image(zj - zo, L2, Li2);
      const T ndx = min_image(xj - xn, L0, Li0), ndy = min_image(yj - yn, L1, Li1), ndz = min_image(zj - zn, L2, Li2);
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
      J2[j] += cu - u;
      J2[1 * s.ne_pad + j] -= ndx * cdu - odx * du;
      J2[2 * s.ne_pad + j] -= ndy * cdu - ody * du;
      J2[3 * s.ne_pad + j] -= ndz * cdu - odz * du;
      J2[4 * s.ne_pad + j] -= cd2u + T(2) * cdu - (d2u + T(2) * du);
    }
    if (threadIdx.x == 0)
      for (int q = 0; q < 5; q++)
        J2[q * s.ne_pad + iat] = cj[5 + q];
  }
  __syncthreads();
  if (threadIdx.x == 0)
  {
    if (s.has_j1)
    {
      T* J1 = s.J1 + (size_t)iw * 5 * s.ne_pad;
      for (int q = 0; q < 5; q++)
        J1[q * s.ne_pad + iat] = cj[q];
    }
    for (int d = 0; d < 3; d++)
    {
      const double x                               = s.active_pos[iw * 3 + d];
      s.R[((size_t)iw * 3 + d) * s.ne_pad + iat]  = x;
      s.Rt[((size_t)iw * 3 + d) * s.ne_pad + iat] = static_cast<T>(x);
    }
  }
}

// Fahy SM-1 for accepted walkers: Ainv -= (1/ratio) (Ainv phi - e_row) (x) rcopy.
// grid (nw, ceil(N/RB)); each CTA owns RB rows of one walker's inverse.
template<typename T, int RB>
__global__ void sm1_kernel(DevState<T> s, int iat)
{
  const int iw = blockIdx.x;
  if (!s.accepted[iw])
    return;
  __shared__ T tmp[RB];
  const int spin = iat >= s.nup ? 1 : 0;
  const int row  = iat - (spin ? s.nup : 0);
  const int n    = s.norb;
  const size_t wslot = (size_t)spin * s.nw + iw;
  T* A         = s.Ainv + wslot * n * s.lda;
  const T* phi = s.phi + (size_t)iw * 5 * s.lda;
  const T* rc  = s.rcopy + (size_t)iw * s.lda;
  const int r0 = blockIdx.y * RB;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  for (int r = wid; r < RB; r += nwarp)
  {
    const int j = r0 + r;
    T a         = 0;
    if (j < n)
      for (int i = lane; i < n; i += 32)
        a += A[(size_t)j * s.lda + i] * phi[i];
    a = warp_sum(a);
    if (lane == 0)
      tmp[r] = (j == row) ? a - T(1) : a;
  }
  __syncthreads();
  const T c = T(-1) / s.cur_det[iw];
  for (int e = threadIdx.x; e < RB * n; e += blockDim.x)
  {
    const int r = e / n, i = e % n;
    const int j = r0 + r;
    if (j < n)
      A[(size_t)j * s.lda + i] += c * rc[i] * tmp[r];
  }
}

// ---------------------------------------------------------------------------
// Delayed-update flush, SIMT form: W = Binv V, then per row block
// Ainv[rows] -= (Ainv[rows] U^T - E[rows]) W.  Works on any batch of walkers
// through FlushArgs (crowd buffers or caller device buffers).
// ---------------------------------------------------------------------------
template<typename T>
__global__ void flush_w_kernel(FlushArgs<T> f)
{
  const int iw  = blockIdx.x;
  const T* Binv = f.binv + (size_t)iw * f.sB;
  const T* V    = f.v + (size_t)iw * f.sU;
  T* Wi         = f.w + (size_t)iw * f.k * f.lda;
  for (int e = threadIdx.x; e < f.dc * f.n; e += blockDim.x)
  {
    const int l = e / f.n, i = e % f.n;
    T a         = 0;
    for (int c = 0; c < f.dc; c++)
      a += Binv[(size_t)l * f.k + c] * V[(size_t)c * f.lda + i];
    Wi[(size_t)l * f.lda + i] = a;
  }
}

template<typename T, int RB>
__global__ void flush_update_kernel(FlushArgs<T> f)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* arows = reinterpret_cast<T*>(smem_raw); // RB x lda
  T* t1    = arows + RB * f.lda;             // RB x k
  const int iw = blockIdx.x;
  const int r0 = blockIdx.y * RB;
  const int n  = f.n;
  T* A         = f.ainv + (size_t)iw * f.sA;
  const T* U   = f.u + (size_t)iw * f.sU;
  const T* Wi  = f.w + (size_t)iw * f.k * f.lda;
  const int* dlist = f.delay_list + (size_t)iw * f.sD;
  const int nr = min(RB, n - r0);
  for (int e = threadIdx.x; e < nr * n; e += blockDim.x)
  {
    const int r = e / n, i = e % n;
    arows[r * f.lda + i] = A[(size_t)(r0 + r) * f.lda + i];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  for (int e = wid; e < nr * f.dc; e += nwarp)
  {
    const int r = e / f.dc, c = e % f.dc;
    T a         = 0;
    for (int i = lane; i < n; i += 32)
      a += arows[r * f.lda + i] * U[(size_t)c * f.lda + i];
    a = warp_sum(a);
    if (lane == 0)
      t1[r * f.k + c] = (dlist[c] == r0 + r) ? a - T(1) : a;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < nr * n; e += blockDim.x)
  {
    const int r = e / n, i = e % n;
    T a         = 0;
    for (int c = 0; c < f.dc; c++)
      a += t1[r * f.k + c] * Wi[(size_t)c * f.lda + i];
    A[(size_t)(r0 + r) * f.lda + i] = arows[r * f.lda + i] - a;
  }
}

template<typename T>
cudaError_t launch_flush_args(const FlushArgs<T>& f, cudaStream_t st)
{
  if (f.dc <= 0 || f.nw <= 0)
    return cudaSuccess;
  flush_w_kernel<T><<<f.nw, 256, 0, st>>>(f);
  constexpr int RB = 16;
  const size_t sm = sizeof(T) * ((size_t)RB * f.lda + (size_t)RB * f.k);
  dim3 grid(f.nw, (f.n + RB - 1) / RB);
  flush_update_kernel<T, RB><<<grid, 256, sm, st>>>(f);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------
constexpr int MOVE_NT = 256;

template<typename T>
size_t ratio_smem(const DevState<T>& s)
{
  return sizeof(T) * 4 * 7 * (size_t)s.lda;
}

template<typename T>
cudaError_t launch_propose(const DevState<T>& s, int iat, int dc, int driver, cudaStream_t st)
{
  const size_t sm = sizeof(T) * ((size_t)s.lda + 2 * (size_t)s.k);
  propose_kernel<T, MOVE_NT><<<s.nw, MOVE_NT, sm, st>>>(s, iat, dc, driver);
  return cudaGetLastError();
}

template<typename T>
cudaError_t launch_make_move(const DevState<T>& s, int iat, cudaStream_t st)
{
  make_move_kernel<T><<<(s.nw + 127) / 128, 128, 0, st>>>(s, iat);
  return cudaGetLastError();
}

template<typename T>
cudaError_t launch_ratio(const DevState<T>& s, int iat, int driver, cudaStream_t st)
{
  const size_t sm = ratio_smem(s);
  ratio_kernel<T, MOVE_NT><<<s.nw, MOVE_NT, sm, st>>>(s, iat, driver);
  return cudaGetLastError();
}

template<typename T>
cudaError_t launch_accept(const DevState<T>& s, int iat, int dc, int driver, cudaStream_t st)
{
  const size_t sm = sizeof(T) * 2 * (size_t)s.k;
  accept_kernel<T, MOVE_NT><<<s.nw, MOVE_NT, sm, st>>>(s, iat, dc, driver);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || s.k > 1)
    return e;
  constexpr int RB = 16;
  dim3 grid(s.nw, (s.norb + RB - 1) / RB);
  sm1_kernel<T, RB><<<grid, 128, 0, st>>>(s, iat);
  return cudaGetLastError();
}

template<typename T>
cudaError_t launch_flush_simt(const DevState<T>& s, int spin, int dc, T* W, cudaStream_t st)
{
  FlushArgs<T> f;
  f.nw         = s.nw;
  f.n          = s.norb;
  f.lda        = s.lda;
  f.k          = s.k;
  f.dc         = dc;
  f.sA         = (long long)s.norb * s.lda;
  f.sU         = (long long)s.nsets * s.k * s.lda;
  f.sB         = (long long)s.nsets * s.k * s.k;
  f.sD         = s.nsets * s.k;
  f.ainv       = s.Ainv + (size_t)spin * s.nw * f.sA;
  f.u          = s.U + (size_t)spin * s.nw * f.sU;
  f.v          = s.V + (size_t)spin * s.nw * f.sU;
  f.binv       = s.Binv + (size_t)spin * s.nw * f.sB;
  f.delay_list = s.delay_list + (size_t)spin * s.nw * f.sD;
  f.w          = W;
  return launch_flush_args(f, st);
}

template<typename T>
cudaError_t setup_move_kernels()
{
  cudaError_t e = cudaFuncSetAttribute(ratio_kernel<T, MOVE_NT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       200 * 1024);
  if (e != cudaSuccess)
    return e;
  return cudaFuncSetAttribute(flush_update_kernel<T, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
}

#define INSTANTIATE(T)                                                                                                 \
  template cudaError_t setup_move_kernels<T>();                                                                        \
  template cudaError_t launch_propose<T>(const DevState<T>&, int, int, int, cudaStream_t);                             \
  template cudaError_t launch_make_move<T>(const DevState<T>&, int, cudaStream_t);                                     \
  template cudaError_t launch_ratio<T>(const DevState<T>&, int, int, cudaStream_t);                                    \
  template cudaError_t launch_accept<T>(const DevState<T>&, int, int, int, cudaStream_t);                              \
  template cudaError_t launch_flush_simt<T>(const DevState<T>&, int, int, T*, cudaStream_t);                        \
  template cudaError_t launch_flush_args<T>(const FlushArgs<T>&, cudaStream_t);
INSTANTIATE(float)
INSTANTIATE(double)
#undef INSTANTIATE

} // namespace qmcg
