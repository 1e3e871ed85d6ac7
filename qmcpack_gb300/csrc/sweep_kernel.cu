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
// flush_kernels.cu / flush_tc.cu.
//
// Per CTA the walker's positions, two-body Jastrow state and the delayed-update
// matrix Binv stay in shared memory for the segment.  Where it does not enlarge the
// kernel's shared-memory footprint, the segment's inverse rows (the rows of its k
// electrons, which the delayed update reads as V and the accepted moves read against
// the new orbital row) arrive in shared memory at the start of the segment by one
// bulk asynchronous copy completing on an mbarrier; the next electron's orbital
// gradient and value rows are prefetched with cp.async while the current one is
// evaluated.  The evaluation at the proposed position is split by warps: the first
// warps own orbital pairs and read all 64 coefficient rows of the grid cell for them
// (8-byte loads contiguous over orbitals, the value, gradient and Laplacian formed in
// registers), the remaining warp(s) compute the one- and two-body Jastrow rows at the
// same time.  Driver arithmetic (Box-Muller Gaussians, drift, Green's functions) runs
// in the move-loop precision, as the reference's mixed-precision build does in RealType.
#include <algorithm>
#include <type_traits>

#include "common.cuh"
#include "launch.h"
#include "learned.cuh"
#include "spline.cuh"
#include "tc.cuh"

namespace qmcg
{

template<typename T>
struct SweepCfg
{
  static constexpr int NT   = 128;
  static constexpr int MINB = sizeof(T) == 4 ? 4 : 2;
};

// network scratch of the learned proposal: features, activations, reduction scratch, outputs
constexpr int ML_SCRATCH_FLOATS = ML_IN + 2 * ML_H + ML_NOUT * 4 + 8;

// shared-memory layout of the resident sweep (offsets in elements of T, every region on a
// 16-byte boundary)
struct SweepLayout
{
  int npre; // rows per prefetch buffer: dgrad xyz, values (+ the inverse row when the segment rows are not staged)
  int pre, invrow, phi, Rs, J2s, Bs, pv, tv, yv, red, tri, seg, ml, coef, total;
  // delayed updates with unstaged rows: the orbital values at the proposed position are
  // written over the current electron's prefetch buffer (five rows, spent by then)
  int phi_in_pre;
};

template<typename T>
__host__ __device__ inline SweepLayout sweep_layout(int lda, int ne_pad, int K, bool seg_smem, bool learned,
                                                   int ncoef)
{
  constexpr int a = 16 / (int)sizeof(T);
  auto up         = [](int x) { return (x + a - 1) / a * a; };
  SweepLayout L;
  int o    = 0;
  L.npre       = seg_smem ? 4 : 5;
  L.phi_in_pre = !seg_smem && K > 1 && !learned;
  L.pre        = o, o += up(2 * L.npre * lda);
  L.invrow     = o, o += up(lda);
  L.phi        = o, o += L.phi_in_pre ? 0 : up(5 * lda);
  L.Rs     = o, o += up(3 * ne_pad);
  L.J2s    = o, o += up(5 * ne_pad);
  L.Bs     = o, o += up(K * K);
  L.pv     = o, o += up(K);
  L.tv     = o, o += up(K);
  L.yv     = o, o += up(K);
  L.red    = o, o += up(16 * 16); // block reductions of up to 16 values over up to 16 warps
  L.tri    = o, o += up(K * (K - 1) / 2);
  L.seg    = o, o += up(seg_smem ? K * lda : (K == 1 ? lda : 0)); // the segment's rows, or the rank-1 scratch
  L.ml     = o, o += learned ? up((ML_SCRATCH_FLOATS * 4 + (int)sizeof(T) - 1) / (int)sizeof(T)) : 0;
  L.coef   = o, o += up(ncoef); // the J2 (same, opposite spin) and J1 (per species) functor coefficients
  L.total  = o;
  return L;
}

// the footprint of the previous design (spline partials in shared memory, every row
// from global memory): the segment rows are staged only where they fit inside it
template<typename T>
static size_t sweep_smem_reference(int lda, int ne_pad, int K)
{
  return sizeof(T) * ((size_t)45 * lda + 8 * (size_t)ne_pad + (size_t)K * K + 3 * (size_t)K + 512 +
                      (size_t)K * (K - 1) / 2);
}

// functor coefficients staged per CTA
template<typename T>
__host__ __device__ inline int sweep_ncoef(const DevState<T>& s)
{
  return (s.has_j2 ? 2 * s.j2_ncoef : 0) + (s.has_j1 ? s.j1_nspecies * s.j1_ncoef : 0);
}

template<typename T>
bool sweep_seg_smem(const DevState<T>& s)
{
  if (s.k <= 1)
    return false;
  const SweepLayout L = sweep_layout<T>(s.lda, s.ne_pad, s.k, true, false, sweep_ncoef(s));
  return sizeof(T) * (size_t)L.total <= sweep_smem_reference<T>(s.lda, s.ne_pad, s.k);
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

// rows of electron `row` of spin slot into pre: [inverse row,] dgrad xyz, orbital values
template<typename T>
__device__ __forceinline__ void prefetch_rows(const DevState<T>& s, size_t slot, int row, T* pre, bool with_inv,
                                              int tid, int nt)
{
  const int n = s.norb;
  if (with_inv)
  {
    async_copy(pre, s.Ainv + (slot * n + row) * s.lda, s.lda, tid, nt);
    pre += s.lda;
  }
  async_copy(pre, s.dgrad + ((slot * n + row) * 3) * s.lda, 3 * s.lda, tid, nt);
  async_copy(pre + 3 * s.lda, s.psiv + (slot * n + row) * s.lda, s.lda, tid, nt);
  async_commit();
}

// bulk asynchronous copy global -> shared completing on an mbarrier (16-byte aligned, size a
// multiple of 16); issued by one thread after it announced the byte count on the barrier
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint32_t mbar)
{
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(mbar), "r"(bytes) : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(mbar)
               : "memory");
}

// out[c] = scale * (rows[c] . x) for c < nrows (rows in shared or global memory, stride
// ld, x in shared memory): every warp owns up to 8 rows, a lane sums its columns of all of
// them, and one transposed reduction (9 shuffles for the 8 sums) finishes them.  The loop
// is kept short: the walker-resident kernel's speed depends on how much of its loop body
// the SM's instruction cache holds.
template<typename T, int NT>
__device__ __forceinline__ void rows_dot(const T* rows, int ld, int nrows, const T* x, int n, T* out, T scale)
{
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  constexpr int NW = NT / 32;
  for (int c0 = wid; c0 < nrows; c0 += 8 * NW)
  {
    T a[8];
#pragma unroll
    for (int q = 0; q < 8; q++)
      a[q] = T(0);
#pragma unroll 1
    for (int j = lane; j < n; j += 32)
    {
      const T xv = x[j];
#pragma unroll
      for (int q = 0; q < 8; q++)
      {
        const int c = c0 + q * NW;
        a[q] += (c < nrows ? rows[(size_t)c * ld + j] : T(0)) * xv;
      }
    }
    // transposed reduction: distances 16, 8, 4 halve the values, 2 and 1 finish the sums;
    // lane l ends with the sum of row value (l >> 2) & 7
#pragma unroll
    for (int h = 4; h >= 1; h >>= 1)
    {
      const bool up = (lane & (4 * h)) != 0;
#pragma unroll
      for (int q = 0; q < h; q++)
      {
        const T send = up ? a[q] : a[q + h];
        const T recv = __shfl_xor_sync(0xffffffffu, send, 4 * h);
        a[q]         = (up ? a[q + h] : a[q]) + recv;
      }
    }
    a[0] += __shfl_xor_sync(0xffffffffu, a[0], 2);
    a[0] += __shfl_xor_sync(0xffffffffu, a[0], 1);
    const int q = (lane >> 2) & 7, c = c0 + q * NW;
    if ((lane & 3) == 0 && c < nrows)
      out[c] = scale * a[0];
  }
}

// Orbital values, gradients and Laplacians of the orbital pair starting at orbital o0 at
// the grid cell (ix, iy, iz): all 64 coefficient rows of the cell for these two orbitals,
// read plane by plane (16 loads in flight), the tricubic sums in registers
// (spline2::evaluate_vgh_impl, MultiBsplineVGLH.hpp:120-230, and SplineR2R::assign_vgl,
// SplineR2R.cpp:338-374, for an orthorhombic cell).  out[q][w]: q = value, gradient xyz,
// Laplacian of orbital o0 + w.
template<typename T>
__device__ __forceinline__ void spline_pair_vgl(const DevState<T>& s, const T* origin, int o0, const T a[4],
                                                const T da[4], const T d2a[4], const T b[4], const T db[4],
                                                const T d2b[4], const T c[4], const T dc[4], const T d2c[4],
                                                T (&out)[5][2])
{
  T acc[7][2];
#pragma unroll
  for (int q = 0; q < 7; q++)
    acc[q][0] = acc[q][1] = T(0);
  const T* base = origin + o0;
#pragma unroll 1
  for (int i = 0; i < 4; i++)
  {
    T v[4][4][2];
#pragma unroll
    for (int j = 0; j < 4; j++)
#pragma unroll
      for (int k = 0; k < 4; k++)
        Vec<T>::load(base + i * s.xs + j * s.ys + k * s.zs, v[j][k]);
    // z sums of every (j, orbital), then y sums, then this plane's x weights
    T t0[2] = {T(0), T(0)}, t1[2] = {T(0), T(0)}, t2[2] = {T(0), T(0)}, u1[2] = {T(0), T(0)}, u2[2] = {T(0), T(0)};
#pragma unroll
    for (int j = 0; j < 4; j++)
    {
#pragma unroll
      for (int w = 0; w < 2; w++)
      {
        const T s0 = c[0] * v[j][0][w] + c[1] * v[j][1][w] + c[2] * v[j][2][w] + c[3] * v[j][3][w];
        const T s1 = dc[0] * v[j][0][w] + dc[1] * v[j][1][w] + dc[2] * v[j][2][w] + dc[3] * v[j][3][w];
        const T s2 = d2c[0] * v[j][0][w] + d2c[1] * v[j][1][w] + d2c[2] * v[j][2][w] + d2c[3] * v[j][3][w];
        t0[w] += b[j] * s0;
        t1[w] += db[j] * s0;
        t2[w] += d2b[j] * s0;
        u1[w] += b[j] * s1;
        u2[w] += b[j] * s2;
      }
    }
    // this plane's x weights by selection: indexing the weight arrays with the loop counter
    // would place them in local memory
    const T ai   = i == 0 ? a[0] : (i == 1 ? a[1] : (i == 2 ? a[2] : a[3]));
    const T dai  = i == 0 ? da[0] : (i == 1 ? da[1] : (i == 2 ? da[2] : da[3]));
    const T d2ai = i == 0 ? d2a[0] : (i == 1 ? d2a[1] : (i == 2 ? d2a[2] : d2a[3]));
#pragma unroll
    for (int w = 0; w < 2; w++)
    {
      acc[0][w] += ai * t0[w];
      acc[1][w] += dai * t0[w];
      acc[2][w] += ai * t1[w];
      acc[3][w] += ai * u1[w];
      acc[4][w] += d2ai * t0[w];
      acc[5][w] += ai * t2[w];
      acc[6][w] += ai * u2[w];
    }
  }
  const T fx = s.grid_scale[0], fy = s.grid_scale[1], fz = s.grid_scale[2];
#pragma unroll
  for (int w = 0; w < 2; w++)
  {
    out[0][w] = acc[0][w];
    out[1][w] = acc[1][w] * fx;
    out[2][w] = acc[2][w] * fy;
    out[3][w] = acc[3][w] * fz;
    out[4][w] = acc[4][w] * (fx * fx) + acc[5][w] * (fy * fy) + acc[6][w] * (fz * fz);
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
  unsigned long long seg_bar; // mbarrier of the segment rows' bulk copy
  int seg_phase;              // its parity
};

template<typename T, bool LEARNED>
__device__ __forceinline__ void sweep_shared_init(SweepShared<T, LEARNED>& sh)
{
  if (threadIdx.x == 0)
  {
    mbar_init(smem_u32(&sh.seg_bar));
    sh.seg_phase = 0;
  }
  __syncthreads();
}

// The segment [i0, i1) of walker w by one CTA: the body of the resident sweep.  FORM 1
// compiles the delayed-update form with the segment's inverse rows in shared memory and
// nothing else (the rank-1 and unstaged branches drop out of the loop body, which the
// instruction cache then holds better), FORM 2 the same for plain VMC sweeps (no DMC
// sign rule or sums, no move records); FORM 0, the generic form, decides all at run time.
template<typename T, int NT, bool LEARNED, int FORM>
__device__ __forceinline__ void sweep_walker(const DevState<T>& s, int i0, int i1, int w, unsigned char* smem_raw,
                                             SweepShared<T, LEARNED>& sh, unsigned long long& n_acc,
                                             unsigned long long& n_rej)
{
  constexpr bool STAGED = FORM >= 1, PLAIN = FORM == 2;
  const int lda = s.lda, n = s.norb, K = s.k;
  const bool delayed   = STAGED || K > 1;
  const bool seg_smem  = STAGED || (K > 1 && s.seg_smem != 0);
  const bool dmc       = !PLAIN && s.dmc != 0;
  double* const trace  = PLAIN ? nullptr : s.trace;
  const SweepLayout Ly = sweep_layout<T>(lda, s.ne_pad, K, seg_smem, LEARNED, sweep_ncoef(s));
  T* sm     = reinterpret_cast<T*>(smem_raw);
  T* pre    = sm + Ly.pre;    // 2 x npre x lda prefetch buffers
  T* invrow = sm + Ly.invrow; // lda
  T* const phi_own = sm + Ly.phi; // 5 x lda (unless phi_in_pre)
  T* Rs     = sm + Ly.Rs;     // 3 x ne_pad
  T* J2s    = sm + Ly.J2s;    // 5 x ne_pad
  T* Bs     = sm + Ly.Bs;     // K x K
  T* pv     = sm + Ly.pv;     // K
  T* tv     = sm + Ly.tv;     // K
  T* yv     = sm + Ly.yv;     // K
  T* red    = sm + Ly.red;    // 16 x NT/32
  T* tri    = sm + Ly.tri;    // K (K - 1) / 2: entry x (x - 1) / 2 + c = U_c . Ainv[row_x]
  T* seg    = sm + Ly.seg;    // the segment's inverse rows (K x lda), or the rank-1 scratch
  constexpr int NW = NT / 32;
  const __nv_bfloat162* ml_pairs = reinterpret_cast<const __nv_bfloat162*>(s.mlp_simt);
  const __nv_bfloat16* ml_w4 = reinterpret_cast<const __nv_bfloat16*>(ml_pairs + MS_NPAIRS);
  float* ml_x   = reinterpret_cast<float*>(sm + Ly.ml);
  float* ml_h   = ml_x + ML_IN;
  float* ml_red = ml_h + 2 * ML_H;
  float* ml_out = ml_red + ML_NOUT * 4;
  (void)ml_w4;
  (void)ml_out;

  const uint32_t sweep = static_cast<uint32_t>(*s.sweep_counter);
  const uint32_t k0 = static_cast<uint32_t>(s.seed), k1 = static_cast<uint32_t>(s.seed >> 32);
  const T L0 = T(s.L[0]), L1 = T(s.L[1]), L2 = T(s.L[2]);
  const T Li0 = T(s.G[0]), Li1 = T(s.G[1]), Li2 = T(s.G[2]);
  const T tau       = T(s.tau);
  const int spin    = i0 >= s.nup ? 1 : 0;
  const int first   = spin ? s.nup : 0;
  const int lane    = threadIdx.x & 31, wid = threadIdx.x >> 5;
  // warps [0, spw) evaluate the orbitals (orbital pairs, one or more per thread), the others the
  // Jastrow rows; every thread reads the functor coefficients from shared memory
  const int pairs   = lda / 2;
  const int spw     = max(1, min(NW - 1, (pairs + 31) / 32));
  const bool spline_thread = wid < spw;
  T* coef           = sm + Ly.coef;
  const T* j2c      = coef;                                   // [2][j2_ncoef]
  const T* j1c      = coef + (s.has_j2 ? 2 * s.j2_ncoef : 0); // [species][j1_ncoef]

  {
    const size_t slot = (size_t)spin * s.nw + w;
    const T* ainv_seg = s.Ainv + (slot * n + (i0 - first)) * lda; // rows of this segment's electrons
    // this segment's delayed-update set: its own one when the crowd keeps a set per segment
    const size_t dset = slot * s.nsets + (s.nsets > 1 ? (i0 - first) / K : 0);
    if (seg_smem && threadIdx.x == 0)
    {
      // the previous walker's reads of seg (generic proxy) precede this copy (async proxy)
      fence_async_smem();
      bulk_copy_g2s(seg, ainv_seg, (uint32_t)((i1 - i0) * lda * sizeof(T)), smem_u32(&sh.seg_bar));
    }
    for (int e = threadIdx.x; e < 3 * s.ne_pad; e += NT)
      Rs[e] = s.Rt[(size_t)w * 3 * s.ne_pad + e];
    for (int e = threadIdx.x; e < 5 * s.ne_pad; e += NT)
      J2s[e] = s.J2[(size_t)w * 5 * s.ne_pad + e];
    if (s.has_j2)
      for (int e = threadIdx.x; e < 2 * s.j2_ncoef; e += NT)
        coef[e] = s.j2c[e];
    if (s.has_j1)
      for (int e = threadIdx.x; e < s.j1_nspecies * s.j1_ncoef; e += NT)
        coef[(s.has_j2 ? 2 * s.j2_ncoef : 0) + e] = s.j1c[e];
    prefetch_rows(s, slot, i0 - first, pre, !seg_smem, threadIdx.x, NT);
    if (seg_smem)
    {
      const int phase = sh.seg_phase;
      bool ok         = mbar_wait(smem_u32(&sh.seg_bar), (uint32_t)phase);
      if (__syncthreads_or(!ok))
      {
        // a copy that did not complete in time: record it, let the copy finish (bounded)
        // before the shared memory is used again, and skip this walker's segment
        if (!ok)
          mbar_wait(smem_u32(&sh.seg_bar), (uint32_t)phase);
        if (threadIdx.x == 0)
        {
          atomicOr(s.status + w, ST_TIMEOUT);
          sh.seg_phase = phase ^ 1;
        }
        async_wait_all();
        __syncthreads();
        return;
      }
      __syncthreads();
      if (threadIdx.x == 0)
        sh.seg_phase = phase ^ 1;
    }
    // the segment's rows: V (the inverse rows of the earlier electrons, fixed during a
    // segment) and the rows the accepted moves are multiplied with
    const T* segrows = seg_smem ? seg : ainv_seg;
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
      T* pb         = pre + ((iat - i0) & 1) * Ly.npre * lda; // this electron's prefetched rows
      const T* arow = seg_smem ? segrows + (size_t)(iat - i0) * lda : pb;
      const T* dg   = seg_smem ? pb : pb + lda;
      const T* pv0  = dg + 3 * lda;
      T* pnext      = pre + ((iat + 1 - i0) & 1) * Ly.npre * lda;
      T* const phi  = Ly.phi_in_pre ? pb : phi_own;
      // with phi over the prefetch buffer the inverse row (V of this slot) is stored before
      // the evaluation overwrites it
      T* const vrow = s.V + (dset * K + dc) * lda;
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
      // operands of the proposal (lanes 0-2 of warp 0: component `lane` of the position and of
      // the one-body gradient) and of the decision (thread 0: the one-body value), loaded
      // ahead of their use
      double r_me = 0;
      T j1g_me = 0, j1v_now = 0;
      if (threadIdx.x < 3)
      {
        r_me = s.R[((size_t)w * 3 + threadIdx.x) * s.ne_pad + iat];
        if (s.has_j1)
        {
          j1g_me  = s.J1[((size_t)w * 5 + 1 + threadIdx.x) * s.ne_pad + iat];
          j1v_now = s.J1[((size_t)w * 5) * s.ne_pad + iat];
        }
      }
      async_wait_all();
      __syncthreads();
      // ------------------------------------------------ up-to-date inverse row, fused with
      // the gradient and self-ratio sums of the same elements
      const T* inv = arow;
      T g[4]       = {0, 0, 0, 0};
      if (delayed && dc > 0)
      {
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
          prefetch_rows(s, slot, row + 1, pnext, !seg_smem, threadIdx.x, NT);
        const T* V = segrows;
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
          if (Ly.phi_in_pre)
            vrow[j] = arow[j];
          g[0] += x * dg[j];
          g[1] += x * dg[lda + j];
          g[2] += x * dg[2 * lda + j];
          g[3] += x * pv0[j];
        }
        inv = invrow;
      }
      else
      {
        if (iat + 1 < i1 && delayed)
          prefetch_rows(s, slot, row + 1, pnext, !seg_smem, threadIdx.x, NT);
        for (int j = threadIdx.x; j < n; j += NT)
        {
          const T x = arow[j];
          g[0] += x * dg[j];
          g[1] += x * dg[lda + j];
          g[2] += x * dg[2 * lda + j];
          g[3] += x * pv0[j];
          if (Ly.phi_in_pre)
          {
            invrow[j] = x;
            vrow[j]   = x;
          }
        }
        if (Ly.phi_in_pre)
          inv = invrow;
        // rank-1 updates: the next rows are fetched after this electron's update
      }
      // ------------------------------------------------ gradient, health check, proposal
      {
        block_sum_to0<T, 4>(g, red, NW); // thread 0 uses the sums
        if constexpr (LEARNED)
        {
          // the network at the current position: (mu, s) of the proposal
          if (threadIdx.x == 0)
          {
            if (!(fabs(g[3] - T(1)) <= HealthTol<T>::v))
              atomicOr(s.status + w, spin ? ST_ILLCOND_DN : ST_ILLCOND_UP);
          }
          if (threadIdx.x < 3)
          {
            const int d = threadIdx.x;
            T gs        = d == 0 ? g[0] : (d == 1 ? g[1] : g[2]);
            if (s.has_j1)
              gs += j1g_me;
            if (s.has_j2)
              gs += J2s[(1 + d) * s.ne_pad + iat];
            sh.lsm.g[d] = gs;
            sh.pos[d]   = r_me; // the current position, read back by thread 0 below
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
              sh.pos[d]   = sh.pos[d] + static_cast<double>(dd);
              sh.posT[d]  = static_cast<T>(sh.pos[d]);
            }
            spline_frac(s, sh.pos, sh.ru);
            sh.loggf = -sum_s - T(0.5) * x2;
          }
          __syncthreads();
        }
        else
        {
        if (threadIdx.x < 32)
        {
          // drift-diffusion proposal (DriftModifierUNR::getDrift and the Gaussian step of
          // VMCBatched::advanceWalkers): lane d < 3 forms component d; |grad|^2 and |delta|^2
          // are gathered across the three lanes
          const int d = lane < 3 ? lane : 0;
          T gs = d == 0 ? g[0] : (d == 1 ? g[1] : g[2]);
          if (s.has_j1)
            gs += j1g_me;
          if (s.has_j2)
            gs += J2s[(1 + d) * s.ne_pad + iat];
          const T g2  = gs * gs;
          const T vsq = __shfl_sync(0xffffffffu, g2, 0) + __shfl_sync(0xffffffffu, g2, 1) +
              __shfl_sync(0xffffffffu, g2, 2);
          const T delta = sh.rgauss[jj][d] * sqrt(tau);
          T drift       = delta;
          if (s.use_drift)
          {
            const T sc = vsq < Eps<T>::v ? tau : ((T(-1) + sqrt(T(1) + T(2) * tau * vsq)) / vsq);
            drift      = gs * sc + delta;
          }
          const T d2  = delta * delta;
          const T dsq = __shfl_sync(0xffffffffu, d2, 0) + __shfl_sync(0xffffffffu, d2, 1) +
              __shfl_sync(0xffffffffu, d2, 2);
          if (lane < 3)
          {
            const double pos = r_me + static_cast<double>(drift);
            sh.disp[d]       = drift;
            sh.pos[d]        = pos;
            sh.posT[d]       = static_cast<T>(pos);
            // fractional coordinate (spline_frac) of this component
            const double Gd = d == 0 ? s.G[0] : (d == 1 ? s.G[1] : s.G[2]);
            T u             = static_cast<T>(pos * Gd);
            if (-Eps<T>::v < u && u < T(0))
              u = T(0);
            else
              u -= floor(u);
            sh.ru[d] = u;
            if (trace)
              trace[((size_t)iat * s.nw + w) * TRACE_FIELDS + TR_GRAD_NOW + d] = static_cast<double>(gs);
          }
          if (lane == 0)
          {
            if (!(fabs(g[3] - T(1)) <= HealthTol<T>::v))
              atomicOr(s.status + w, spin ? ST_ILLCOND_DN : ST_ILLCOND_UP);
            if (trace)
              trace[((size_t)iat * s.nw + w) * TRACE_FIELDS + TR_SELF] = static_cast<double>(g[3]);
            sh.loggf = s.use_drift ? -(T(0.5) / tau) * dsq : T(0);
          }
        }
        __syncthreads();
        }
      }
      // ------------------------------------------------ evaluation at the proposed position
      // the FP64 position and its fractional coordinates were converted once, by thread 0;
      // spline warps: orbital pairs; the other warps: Jastrow rows
      T acc[14];
#pragma unroll
      for (int q = 0; q < 14; q++)
        acc[q] = T(0);
      const T x0 = sh.posT[0], y0 = sh.posT[1], z0 = sh.posT[2];
      if (spline_thread)
      {
        int ix, iy, iz;
        T tx, ty, tz;
        spline_bound(sh.ru[0] * T(s.gx), s.gx - 1, ix, tx);
        spline_bound(sh.ru[1] * T(s.gy), s.gy - 1, iy, ty);
        spline_bound(sh.ru[2] * T(s.gz), s.gz - 1, iz, tz);
        T a[4], da[4], d2a[4], b[4], db[4], d2b[4], c[4], dcw[4], d2c[4];
        bspline_weights(tx, a, da, d2a);
        bspline_weights(ty, b, db, d2b);
        bspline_weights(tz, c, dcw, d2c);
        const T* origin = s.coefs + ix * s.xs + iy * s.ys + iz * s.zs;
        for (int p = threadIdx.x; p < pairs; p += spw * 32)
        {
          T vgl[5][2];
          spline_pair_vgl(s, origin, 2 * p, a, da, d2a, b, db, d2b, c, dcw, d2c, vgl);
#pragma unroll
          for (int w2 = 0; w2 < 2; w2++)
          {
            const int o = 2 * p + w2;
#pragma unroll
            for (int q = 0; q < 5; q++)
              phi[q * lda + o] = vgl[q][w2];
            if (o < n)
            {
              const T x = inv[o];
              acc[0] += x * vgl[0][w2];
              acc[1] += x * vgl[1][w2];
              acc[2] += x * vgl[2][w2];
              acc[3] += x * vgl[3][w2];
            }
          }
        }
      }
      else
      {
        const int t0 = threadIdx.x - spw * 32, stride = NT - spw * 32;
        if (s.has_j2)
          for (int j = t0; j < s.ne; j += stride)
          {
            if (j == iat)
              continue;
            const T dx   = min_image(Rs[j] - x0, L0, Li0);
            const T dy   = min_image(Rs[s.ne_pad + j] - y0, L1, Li1);
            const T dz   = min_image(Rs[2 * s.ne_pad + j] - z0, L2, Li2);
            const T r2   = dx * dx + dy * dy + dz * dz;
            const T rinv = inv_sqrt(r2);
            const T r    = r2 * rinv;
            if (r < s.j2_rcut)
            {
              const int same = (j < s.nup) == (iat < s.nup);
              T du, d2u;
              const T u = functor_eval(j2c + (same ? 0 : s.j2_ncoef), s.j2_dri, s.j2_maxidx, r, du, d2u);
              du *= rinv;
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
            const T dx   = min_image(s.ions[j] - x0, L0, Li0);
            const T dy   = min_image(s.ions[s.nions_pad + j] - y0, L1, Li1);
            const T dz   = min_image(s.ions[2 * s.nions_pad + j] - z0, L2, Li2);
            const T r2   = dx * dx + dy * dy + dz * dz;
            const T rinv = inv_sqrt(r2);
            const T r    = r2 * rinv;
            if (r < s.j1_rcut)
            {
              T du, d2u;
              const T u =
                  functor_eval(j1c + (size_t)s.ion_species[j] * s.j1_ncoef, s.j1_dri, s.j1_maxidx, r, du, d2u);
              du *= rinv;
              acc[10] += u;
              acc[11] += du * dx;
              acc[12] += du * dy;
              acc[13] += du * dz;
              acc[4] += d2u + T(2) * du;
            }
          }
      }
      block_sum_to0<T, 14>(acc, red, NW);
      if (threadIdx.x == 0)
      {
        const T detr = acc[0];
        T g[3]       = {acc[1] / detr, acc[2] / detr, acc[3] / detr};
        T logj       = T(0);
        if (s.has_j1)
        {
          logj += j1v_now - acc[10];
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
        if (p >= Eps<T>::v && (!dmc || detr > T(0)))
        {
          a = sh.runif[jj] < p * exp(log_gb - sh.loggf) ? 1 : 0;
        }
        if (dmc)
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
        if (trace)
        {
          double* tr = trace + ((size_t)iat * s.nw + w) * TRACE_FIELDS;
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
      if (delayed)
      {
        T* U       = s.U + dset * K * lda;
        T* V       = s.V + dset * K * lda;
        int* dlist = s.delay_list + dset * K;
        if (!Ly.phi_in_pre)
          for (int j = threadIdx.x; j < n; j += NT)
            V[(size_t)dc * lda + j] = arow[j];
        const int m = i1 - i0; // slots of this segment
        if (accd)
        {
          const T sigma = T(1) / sh.det;
          // phi . Ainv[row_x] for every electron x of the segment: x < dc are the V_x . phi
          // of the Binv update (V_x is Ainv[row_x]), x > dc the U . invRow terms of later slots
          rows_dot<T, NT>(segrows, lda, m, phi, n, pv, T(1));
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
        T* tmp = seg;
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
        __syncthreads();
      }
      if (!delayed && iat + 1 < i1)
      {
        // rank-1 updates change the whole inverse: the next electron's rows are read after it
        __syncthreads();
        prefetch_rows(s, slot, row + 1, pnext, true, threadIdx.x, NT);
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
          // not unrolled: a smaller loop body keeps more of the kernel in the instruction cache
#pragma unroll 1
          for (int j = threadIdx.x; j < s.ne; j += NT)
          {
            if (j == iat)
              continue;
            const int same = (j < s.nup) == (iat < s.nup);
            const T* fc    = j2c + (same ? 0 : s.j2_ncoef);
            const T xj = Rs[j], yj = Rs[s.ne_pad + j], zj = Rs[2 * s.ne_pad + j];
            const T odx = min_image(xj - xo, L0, Li0), ody = min_image(yj - yo, L1, Li1),
                    odz = min_image(zj - zo, L2, Li2);
            const T ndx = min_image(xj - x0, L0, Li0), ndy = min_image(yj - y0, L1, Li1),
                    ndz = min_image(zj - z0, L2, Li2);
            const T ro2 = odx * odx + ody * ody + odz * odz, rn2 = ndx * ndx + ndy * ndy + ndz * ndz;
            const T roinv = inv_sqrt(ro2), rninv = inv_sqrt(rn2);
            const T ro = ro2 * roinv, rn = rn2 * rninv;
            T u = 0, du = 0, d2u = 0, cu = 0, cdu = 0, cd2u = 0;
            if (ro < s.j2_rcut)
            {
              u = functor_eval(fc, s.j2_dri, s.j2_maxidx, ro, du, d2u);
              du *= roinv;
            }
            if (rn < s.j2_rcut)
            {
              cu = functor_eval(fc, s.j2_dri, s.j2_maxidx, rn, cdu, cd2u);
              cdu *= rninv;
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
      if (delayed)
        dc++;
    }
    async_wait_all();
    if (threadIdx.x == 0)
    {
      s.log_abs[slot] += log(det_mant) + det_exp * 0.69314718055994530942;
      if (det_neg)
        s.sign[slot] = -s.sign[slot];
      if (dmc)
      {
        s.rr[2 * w] += rr_prop;
        s.rr[2 * w + 1] += rr_acc;
      }
    }
    // hand the segment's Binv to the batched flush, positions and J2 state back to HBM
    if (delayed)
    {
      T* Binv = s.Binv + dset * K * K;
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

template<typename T, int NT, int MINB, bool LEARNED, int FORM>
__global__ void __launch_bounds__(NT, MINB) sweep_kernel(DevState<T> s, int i0, int i1)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ SweepShared<T, LEARNED> sh;
  sweep_shared_init(sh);
  unsigned long long n_acc = 0, n_rej = 0;
  for (int w = blockIdx.x; w < s.nw; w += gridDim.x)
    sweep_walker<T, NT, LEARNED, FORM>(s, i0, i1, w, smem_raw, sh, n_acc, n_rej);
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
  sweep_shared_init(sh);
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
    sweep_walker<T, NT, false, 0>(ds, st.i0[a], st.i1[a], item - st.begin[a], smem_raw, sh, n_acc, n_rej);
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

// the forms of the kernel: 0 generic, 1 delayed updates with the segment rows staged,
// 2 the same for plain VMC sweeps (no DMC, no move records; FP32 only)
template<typename T, typename F>
static cudaError_t with_form(int form, F&& f)
{
  if constexpr (sizeof(T) == 4)
    if (form == 2)
      return f(std::integral_constant<int, 2>{});
  if (form >= 1)
    return f(std::integral_constant<int, 1>{});
  return f(std::integral_constant<int, 0>{});
}

template<typename T>
static int sweep_form(const DevState<T>& s)
{
  if (s.k <= 1 || s.seg_smem == 0)
    return 0;
  return sizeof(T) == 4 && !s.dmc && !s.trace ? 2 : 1;
}

template<typename T>
cudaError_t setup_sweep_kernel()
{
  cudaError_t e = cudaSuccess;
  for (int form : {0, 1, 2})
  {
    if (e == cudaSuccess)
      e = with_form<T>(form, [](auto g) {
        return cudaFuncSetAttribute(sweep_kernel<T, SweepCfg<T>::NT, SweepCfg<T>::MINB, true, decltype(g)::value>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
      });
    for (int nt : {128, 256, 512})
      if (e == cudaSuccess && sweep_threads_ok(nt, sizeof(T)))
        e = with_form<T>(form, [&](auto g) {
          return with_threads<T>(nt, [](auto c) {
            constexpr int NT = decltype(c)::value;
            return cudaFuncSetAttribute(sweep_kernel<T, NT, SweepMinb<T, NT>::v, false, decltype(g)::value>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
          });
        });
  }
  return e;
}

template<typename T>
size_t sweep_smem_bytes(const DevState<T>& s, bool learned)
{
  return sizeof(T) * (size_t)sweep_layout<T>(s.lda, s.ne_pad, s.k, s.k > 1 && s.seg_smem, learned, sweep_ncoef(s))
                         .total;
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
    return with_form<T>(sweep_form(s), [&](auto g) {
      sweep_kernel<T, NT, MINB, true, decltype(g)::value><<<grid, NT, sweep_smem_bytes(s, true), st>>>(s, i0, i1);
      return cudaGetLastError();
    });
  }
  return with_form<T>(sweep_form(s), [&](auto g) {
    return with_threads<T>(nt, [&](auto c) {
      constexpr int NT = decltype(c)::value;
      sweep_kernel<T, NT, SweepMinb<T, NT>::v, false, decltype(g)::value>
          <<<grid, NT, sweep_smem_bytes(s, false), st>>>(s, i0, i1);
      return cudaGetLastError();
    });
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
    e = with_form<T>(sweep_form(s), [&](auto g) {
      return cudaOccupancyMaxActiveBlocksPerMultiprocessor(
          &per_sm, sweep_kernel<T, NT, MINB, true, decltype(g)::value>, NT, sweep_smem_bytes(s, true));
    });
  }
  else
    e = with_form<T>(sweep_form(s), [&](auto g) {
      return with_threads<T>(nt, [&](auto c) {
        constexpr int NT = decltype(c)::value;
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &per_sm, sweep_kernel<T, NT, SweepMinb<T, NT>::v, false, decltype(g)::value>, NT,
            sweep_smem_bytes(s, false));
      });
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
  const size_t sm = sweep_smem_bytes<T>(s, false);
  if (sm > 114 * 1024)
    return sizeof(T) == 4 ? 512 : 256;
  if (sm > 76 * 1024)
    return 256;
  return 128;
}

template cudaError_t setup_sweep_kernel<float>();
template cudaError_t setup_sweep_kernel<double>();
template size_t sweep_smem_bytes<float>(const DevState<float>&, bool);
template size_t sweep_smem_bytes<double>(const DevState<double>&, bool);
template bool sweep_seg_smem<float>(const DevState<float>&);
template bool sweep_seg_smem<double>(const DevState<double>&);
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
