// From-scratch evaluation of the wave-function state of every walker:
//   * all-electron orbital VGL    <- SPOSet::mw_evaluate_notranspose (SPOSet.h:453-459)
//   * FP64 inverse and log|det|   <- DiracMatrixInverterCUDA::mw_computeInvertAndLog
//                                    (DiracMatrixInverterCUDA.hpp:112-180), DiracMatrix::invert_transpose
//                                    (DiracMatrix.h:189-230), computeLogDet (DiracMatrix.h:100-110)
//   * two-body Jastrow state      <- TwoBodyJastrow::recompute (TwoBodyJastrow.cpp:662-714)
//   * one-body Jastrow state      <- J1OrbitalSoA::recompute (J1OrbitalSoA.h:240-250)
// This is the initial mw_evaluateLog and the periodic FP64 recompute of the
// mixed-precision move loop.  The inverse is a Gauss-Jordan elimination with
// partial pivoting (same pivots as LU with partial pivoting), one CTA per matrix,
// in FP64 whatever the move-loop precision.
#include <algorithm>
#include <type_traits>

#include "common.cuh"
#include "launch.h"
#include "spline.cuh"

namespace qmcg
{

// log|det| as the product of the pivots kept as an FP64 mantissa and a binary exponent:
// one multiply per pivot and one log at the end, instead of a log per pivot (FP64
// transcendentals are slow on this GPU and sit on the elimination's critical path)
struct LogAbsProduct
{
  double m = 1.0;
  int e    = 0;
  __device__ void mul(double x)
  {
    int ex;
    m = frexp(m * fabs(x), &ex);
    e += ex;
  }
  __device__ double value() const { return log(m) + e * 0.69314718055994530942; }
};

// A walker takes part in a masked (repair) recompute only if its status has a
// repair bit; an unmasked recompute takes every walker.
template<typename T>
__device__ __forceinline__ bool skip_walker(const DevState<T>& s, int iw, int masked)
{
  return masked && !(s.status[iw] & ST_REPAIR_MASK);
}

// the same for the inverse of one spin slot (spin * nw + iw): a walker whose check failed
// in one determinant only has only that one inverted again
template<typename T>
__device__ __forceinline__ bool skip_slot(const DevState<T>& s, int slot, int masked)
{
  return masked && !(s.status[slot % s.nw] & st_repair_spin(slot / s.nw));
}

constexpr int VGL_EPB = 8; // electrons per CTA of the all-electron VGL

// Work items (walker, block of VGL_EPB electrons): orbital VGL of the block into the FP64
// Slater matrix (stored transposed: Mt[slot][o][row]) and the psiv / dgrad / dlap rows.
// Unmasked: one item per CTA over every walker.  Masked: the walkers of repair_list,
// handed to a small grid in strides.
template<typename T, int NT>
__global__ void __launch_bounds__(NT) vgl_all_kernel(DevState<T> s, double* Mt, int masked)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* part          = reinterpret_cast<T*>(smem_raw);
  const int nblk   = (s.ne + VGL_EPB - 1) / VGL_EPB;
  const int nitems = (masked ? s.repair_list[0] : s.nw) * nblk;
  for (int item = blockIdx.x; item < nitems; item += gridDim.x)
  {
  const int iw = masked ? s.repair_list[1 + item / nblk] : item / nblk;
  const int e0 = (item % nblk) * VGL_EPB;
  for (int e = e0; e < min(e0 + VGL_EPB, s.ne); e++)
  {
  const int spin = e >= s.nup ? 1 : 0;
  const int row  = e - (spin ? s.nup : 0);
  const int n    = s.norb;
  const size_t slot = (size_t)spin * s.nw + iw;
  double pos[3];
  for (int d = 0; d < 3; d++)
    pos[d] = s.R[((size_t)iw * 3 + d) * s.ne_pad + e];
  spline_partials(s, pos, part);
  __syncthreads();
  double* M = Mt + slot * (size_t)n * n;
  T* dg     = s.dgrad + ((slot * n + row) * 3) * s.lda;
  T* dl     = s.dlap + (slot * n + row) * s.lda;
  T* pv     = s.psiv + (slot * n + row) * s.lda;
  for (int o = threadIdx.x; o < n; o += blockDim.x)
  {
    T vgl[5];
    spline_combine(s, part, o, vgl);
    M[(size_t)o * n + row] = static_cast<double>(vgl[0]);
    pv[o]                  = vgl[0];
    dg[o]                  = vgl[1];
    dg[s.lda + o]          = vgl[2];
    dg[2 * s.lda + o]      = vgl[3];
    dl[o]                  = vgl[4];
  }
  __syncthreads();
  }
  }
}

// the walkers with a repair bit: repair_list[0] = count, repair_list[1..] = walkers (one CTA)
template<typename T>
__global__ void __launch_bounds__(1024) repair_list_kernel(DevState<T> s)
{
  __shared__ int cnt;
  if (threadIdx.x == 0)
    cnt = 0;
  __syncthreads();
  for (int iw = threadIdx.x; iw < s.nw; iw += blockDim.x)
    if (s.status[iw] & ST_REPAIR_MASK)
      s.repair_list[1 + atomicAdd(&cnt, 1)] = iw;
  __syncthreads();
  if (threadIdx.x == 0)
    s.repair_list[0] = cnt;
}

// grid (2 * nw): in-place FP64 Gauss-Jordan inverse of Mt[slot] (n x n), log|det|
// and sign; writes Ainv = Mt^-1 = (M^-1)^T in the move-loop precision.
template<typename T, int NT>
__global__ void __launch_bounds__(NT) gj_inverse_kernel(DevState<T> s, double* Mt, int masked)
{
  if (skip_slot(s, blockIdx.x, masked))
    return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n = s.norb;
  double* prow = reinterpret_cast<double*>(smem_raw); // n
  double* pcol = prow + n;                           // n
  int* perm    = reinterpret_cast<int*>(pcol + n);   // n
  __shared__ double bval[32];
  __shared__ int bidx[32];
  __shared__ int s_piv;
  __shared__ int s_bad;
  const int slot = blockIdx.x;
  double* a      = Mt + (size_t)slot * n * n;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  LogAbsProduct logabs;
  int sgn       = 1;
  if (threadIdx.x == 0)
    s_bad = 0;
  __syncthreads();
  for (int k = 0; k < n; k++)
  {
    // pivot: first row of maximal |a[i][k]|, i >= k
    double bv = -1.0;
    int bi    = n;
    for (int i = k + threadIdx.x; i < n; i += NT)
    {
      const double v = fabs(a[(size_t)i * n + k]);
      if (v > bv || (v == bv && i < bi))
      {
        bv = v;
        bi = i;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
    {
      const double ov = __shfl_xor_sync(0xffffffffu, bv, o);
      const int oi    = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ov > bv || (ov == bv && oi < bi))
      {
        bv = ov;
        bi = oi;
      }
    }
    if (lane == 0)
    {
      bval[wid] = bv;
      bidx[wid] = bi;
    }
    __syncthreads();
    if (threadIdx.x == 0)
    {
      double b = bval[0];
      int p    = bidx[0];
      for (int w = 1; w < NT / 32; w++)
        if (bval[w] > b || (bval[w] == b && bidx[w] < p))
        {
          b = bval[w];
          p = bidx[w];
        }
      if (!(b > 0.0))
      {
        s_bad = 1;
        p     = k;
      }
      s_piv   = p;
      perm[k] = p;
    }
    __syncthreads();
    if (s_bad)
      break;
    const int p = s_piv;
    if (p != k)
      for (int j = threadIdx.x; j < n; j += NT)
      {
        const double t          = a[(size_t)k * n + j];
        a[(size_t)k * n + j]    = a[(size_t)p * n + j];
        a[(size_t)p * n + j]    = t;
      }
    __syncthreads();
    const double d = a[(size_t)k * n + k];
    for (int j = threadIdx.x; j < n; j += NT)
    {
      const double v       = (j == k ? 1.0 : a[(size_t)k * n + j]) / d;
      prow[j]              = v;
      a[(size_t)k * n + j] = v;
    }
    for (int i = threadIdx.x; i < n; i += NT)
      pcol[i] = (i == k) ? 0.0 : a[(size_t)i * n + k];
    if (threadIdx.x == 0)
    {
      logabs.mul(d);
      if (d < 0.0)
        sgn = -sgn;
      if (p != k)
        sgn = -sgn;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < n * n; e += NT)
    {
      const int i = e / n, j = e % n;
      if (i == k)
        continue;
      const double base = (j == k) ? 0.0 : a[e];
      a[e]              = base - pcol[i] * prow[j];
    }
    __syncthreads();
  }
  const size_t iw_spin = slot;
  if (s_bad)
  {
    if (threadIdx.x == 0)
    {
      atomicOr(s.status + (slot % s.nw), ST_SINGULAR);
      s.log_abs[iw_spin] = -INFINITY;
      s.sign[iw_spin]    = 0;
    }
    return;
  }
  // undo the row interchanges as column interchanges, in reverse order
  for (int k = n - 1; k >= 0; k--)
  {
    const int p = perm[k];
    if (p != k)
      for (int i = threadIdx.x; i < n; i += NT)
      {
        const double t       = a[(size_t)i * n + k];
        a[(size_t)i * n + k] = a[(size_t)i * n + p];
        a[(size_t)i * n + p] = t;
      }
    __syncthreads();
  }
  T* A = s.Ainv + (size_t)slot * n * s.lda;
  for (int e = threadIdx.x; e < n * n; e += NT)
  {
    const int i = e / n, j = e % n;
    A[(size_t)i * s.lda + j] = static_cast<T>(a[e]);
  }
  if (threadIdx.x == 0)
  {
    s.log_abs[iw_spin] = logabs.value();
    s.sign[iw_spin]    = sgn;
  }
}

// ---------------------------------------------------------------------------
// The same FP64 Gauss-Jordan inverse spread over a cluster of GJ_CL CTAs per matrix
// (one SM each), for the masked repair of a few walkers where one SM's FP64 rate is
// the latency: CTA r owns a contiguous block of columns.  Per pivot step the owner of
// column k finds the pivot and publishes (pivot row, pivot value, column k with rows k
// and p exchanged) in a double-buffered global scratch; one cluster barrier
// (release/acquire) later every CTA swaps, scales and eliminates its own columns.
// ---------------------------------------------------------------------------
constexpr int GJ_CL = 8;
constexpr int GJ_NT = 256;
constexpr int GJ_SMEM_MAX = 200 * 1024; // dynamic shared memory of the resident-block variant

__device__ __forceinline__ void cluster_sync_all()
{
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}

__device__ __forceinline__ unsigned cluster_rank()
{
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;\n" : "=r"(r));
  return r;
}

__host__ __device__ size_t gj_scratch_doubles(int n) { return 3 * (size_t)n + 8; }

template<typename T>
__global__ void __launch_bounds__(GJ_NT) gj_cluster_kernel(DevState<T> s, double* Mt, int masked)
{
  const int slot = blockIdx.x / GJ_CL;
  if (skip_slot(s, slot, masked)) // uniform over the cluster
    return;
  extern __shared__ __align__(16) unsigned char gsm[];
  const int n = s.norb, r = (int)cluster_rank();
  const int cw = (n + GJ_CL - 1) / GJ_CL, c0 = r * cw, c1 = min(n, c0 + cw), ncw = max(0, c1 - c0);
  double* prow = reinterpret_cast<double*>(gsm);  // cw
  int* cmap    = reinterpret_cast<int*>(prow + cw); // n
  __shared__ double bval[GJ_NT / 32];
  __shared__ int bidx[GJ_NT / 32];
  double* a   = Mt + (size_t)slot * n * n;
  double* scr = s.gj_scratch + (size_t)slot * gj_scratch_doubles(n);
  double* pdv = scr + 2 * (size_t)n;                  // [2][2] pivot row, pivot value
  int* perm   = reinterpret_cast<int*>(scr + 2 * (size_t)n + 4);
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  LogAbsProduct logabs;
  int sgn = 1, bad = 0;
  for (int k = 0; k < n; k++)
  {
    const int b     = k & 1;
    double* pc      = scr + (size_t)b * n;
    if (k / cw == r)
    {
      double bv = -1.0;
      int bi    = n;
      for (int i = k + tid; i < n; i += GJ_NT)
      {
        const double v = fabs(a[(size_t)i * n + k]);
        if (v > bv || (v == bv && i < bi))
        {
          bv = v;
          bi = i;
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1)
      {
        const double ov = __shfl_xor_sync(0xffffffffu, bv, o);
        const int oi    = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ov > bv || (ov == bv && oi < bi))
        {
          bv = ov;
          bi = oi;
        }
      }
      if (lane == 0)
      {
        bval[wid] = bv;
        bidx[wid] = bi;
      }
      __syncthreads();
      double pb = bval[0];
      int p     = bidx[0];
      for (int w = 1; w < GJ_NT / 32; w++)
        if (bval[w] > pb || (bval[w] == pb && bidx[w] < p))
        {
          pb = bval[w];
          p  = bidx[w];
        }
      if (!(pb > 0.0))
        p = k;
      for (int i = tid; i < n; i += GJ_NT)
      {
        const int src = (i == p) ? k : i;
        pc[i]         = (i == k) ? 0.0 : a[(size_t)src * n + k];
      }
      if (tid == 0)
      {
        pdv[2 * b]     = (double)p;
        pdv[2 * b + 1] = pb > 0.0 ? a[(size_t)p * n + k] : 0.0;
        perm[k]        = p;
      }
    }
    cluster_sync_all();
    const int p    = (int)__ldcg(pdv + 2 * b);
    const double d = __ldcg(pdv + 2 * b + 1);
    if (!(fabs(d) > 0.0))
    {
      bad = 1;
      break;
    }
    if (r == 0 && tid == 0) // the one thread that writes log|det| (FP64 log is slow on this GPU)
    {
      logabs.mul(d);
      if (d < 0.0)
        sgn = -sgn;
      if (p != k)
        sgn = -sgn;
    }
    if (p != k)
      for (int j = c0 + tid; j < c1; j += GJ_NT)
      {
        const double t        = a[(size_t)k * n + j];
        a[(size_t)k * n + j]  = a[(size_t)p * n + j];
        a[(size_t)p * n + j]  = t;
      }
    __syncthreads();
    for (int jj = tid; jj < ncw; jj += GJ_NT)
    {
      const int j = c0 + jj;
      const double v = (j == k ? 1.0 : a[(size_t)k * n + j]) / d;
      prow[jj]             = v;
      a[(size_t)k * n + j] = v;
    }
    __syncthreads();
    for (int i = wid; i < n; i += GJ_NT / 32)
    {
      if (i == k)
        continue;
      const double f = __ldcg(pc + i);
      double* ai     = a + (size_t)i * n + c0;
      for (int jj = lane; jj < ncw; jj += 32)
      {
        const double base = (c0 + jj == k) ? 0.0 : ai[jj];
        ai[jj]            = base - f * prow[jj];
      }
    }
    __syncthreads();
  }
  cluster_sync_all();
  if (bad)
  {
    if (r == 0 && tid == 0)
    {
      atomicOr(s.status + (slot % s.nw), ST_SINGULAR);
      s.log_abs[slot] = -INFINITY;
      s.sign[slot]    = 0;
    }
    return;
  }
  // the row interchanges become column interchanges applied in reverse order:
  // output column j holds working column cmap[j]
  if (tid == 0)
  {
    for (int j = 0; j < n; j++)
      cmap[j] = j;
    for (int k = n - 1; k >= 0; k--)
    {
      const int p = __ldcg(perm + k);
      const int t = cmap[k];
      cmap[k]     = cmap[p];
      cmap[p]     = t;
    }
  }
  __syncthreads();
  T* A = s.Ainv + (size_t)slot * n * s.lda;
  for (int i = wid; i < n; i += GJ_NT / 32)
    for (int jj = lane; jj < ncw; jj += 32)
      A[(size_t)i * s.lda + c0 + jj] = static_cast<T>(__ldcg(a + (size_t)i * n + cmap[c0 + jj]));
  if (r == 0 && tid == 0)
  {
    s.log_abs[slot] = logabs.value();
    s.sign[slot]    = sgn;
  }
}

// Variant with the CTA's column block resident in shared memory (when it fits): the
// pivot search, row swap, scaling and elimination touch only shared memory, and the
// other CTAs read the owner's pivot data from its shared memory over the cluster
// (distributed shared memory).  Global memory is touched once to load the block and
// once to write the result.
__device__ __forceinline__ unsigned dsm_map(const void* p, unsigned rank)
{
  unsigned r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;\n" : "=r"(r) : "r"((unsigned)__cvta_generic_to_shared(p)), "r"(rank));
  return r;
}
__device__ __forceinline__ double dsm_ld(unsigned addr)
{
  double v;
  asm volatile("ld.shared::cluster.f64 %0, [%1];\n" : "=d"(v) : "r"(addr) : "memory");
  return v;
}
__device__ __forceinline__ float dsm_ldf(unsigned addr)
{
  float v;
  asm volatile("ld.shared::cluster.f32 %0, [%1];\n" : "=f"(v) : "r"(addr) : "memory");
  return v;
}
__device__ __forceinline__ int dsm_ldi(unsigned addr)
{
  int v;
  asm volatile("ld.shared::cluster.s32 %0, [%1];\n" : "=r"(v) : "r"(addr) : "memory");
  return v;
}
template<typename W>
__device__ __forceinline__ W dsm_ldw(unsigned addr);
template<>
__device__ __forceinline__ double dsm_ldw<double>(unsigned addr) { return dsm_ld(addr); }
template<>
__device__ __forceinline__ float dsm_ldw<float>(unsigned addr) { return dsm_ldf(addr); }

// shared memory of the cluster Gauss-Jordan: pivot (row, value) [2][2] in FP64, the
// CTA's column block [n][cw + 1], the published pivot column [2][n] and the local copy
// of the current one [n] in the working type, pivot rows and the column map [n] each
__host__ __device__ inline size_t gj_smem_bytes(int n, int cl, int wsize)
{
  const int cw = (n + cl - 1) / cl;
  return 4 * sizeof(double) + (size_t)wsize * ((size_t)n * (cw + 1) + 3 * (size_t)n) + sizeof(int) * 2 * (size_t)n;
}

// W = working precision of the elimination (the log|det| sums are FP64 either way);
// CL = CTAs per matrix.  FP32 crowds repair in FP32: GB300's FP64 rate is a small
// fraction of its FP32 rate, and the repaired inverse is stored in FP32.
template<typename T, typename W, int CL>
__global__ void __launch_bounds__(GJ_NT) gj_cluster_smem_kernel(DevState<T> s, double* Mt, int masked)
{
  const int slot = blockIdx.x / CL;
  if (skip_slot(s, slot, masked)) // uniform over the cluster
    return;
  extern __shared__ __align__(16) unsigned char gsm[];
  const int n = s.norb, r = (int)cluster_rank();
  const int cw = (n + CL - 1) / CL, ld = cw + 1;
  const int c0 = r * cw, c1 = min(n, c0 + cw), ncw = max(0, c1 - c0);
  double* pds = reinterpret_cast<double*>(gsm);        // [2][2] published pivot row, value
  W* blk      = reinterpret_cast<W*>(pds + 4);         // [n][ld] own columns
  W* pcs      = blk + (size_t)n * ld;                  // [2][n] published pivot column
  W* pcl      = pcs + 2 * (size_t)n;                   // [n] this step's pivot column, local copy
  int* perm   = reinterpret_cast<int*>(pcl + n);       // [n] pivot rows of the columns this CTA owns
  int* cmap   = perm + n;                              // [n]
  __shared__ W bval[GJ_NT / 32];
  __shared__ int bidx[GJ_NT / 32];
  double* a = Mt + (size_t)slot * n * n;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  for (int i = wid; i < n; i += GJ_NT / 32)
    for (int jj = lane; jj < ncw; jj += 32)
      blk[(size_t)i * ld + jj] = static_cast<W>(a[(size_t)i * n + c0 + jj]);
  __syncthreads();
  LogAbsProduct logabs;
  int sgn = 1, bad = 0;
  for (int k = 0; k < n; k++)
  {
    const int b     = k & 1;
    const int owner = k / cw;
    if (owner == r)
    {
      const int kk = k - c0;
      W bv         = W(-1);
      int bi       = n;
      for (int i = k + tid; i < n; i += GJ_NT)
      {
        const W v = fabs(blk[(size_t)i * ld + kk]);
        if (v > bv || (v == bv && i < bi))
        {
          bv = v;
          bi = i;
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1)
      {
        const W ov   = __shfl_xor_sync(0xffffffffu, bv, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ov > bv || (ov == bv && oi < bi))
        {
          bv = ov;
          bi = oi;
        }
      }
      if (lane == 0)
      {
        bval[wid] = bv;
        bidx[wid] = bi;
      }
      __syncthreads();
      W pb  = bval[0];
      int p = bidx[0];
      for (int w = 1; w < GJ_NT / 32; w++)
        if (bval[w] > pb || (bval[w] == pb && bidx[w] < p))
        {
          pb = bval[w];
          p  = bidx[w];
        }
      if (!(pb > W(0)))
        p = k;
      for (int i = tid; i < n; i += GJ_NT)
      {
        const int src          = (i == p) ? k : i;
        pcs[(size_t)b * n + i] = (i == k) ? W(0) : blk[(size_t)src * ld + kk];
      }
      if (tid == 0)
      {
        pds[2 * b]     = (double)p;
        pds[2 * b + 1] = pb > W(0) ? static_cast<double>(blk[(size_t)p * ld + kk]) : 0.0;
        perm[k]        = p;
      }
    }
    cluster_sync_all();
    const unsigned rpd = dsm_map(pds + 2 * b, (unsigned)owner);
    const int p        = (int)dsm_ld(rpd);
    const double dd    = dsm_ld(rpd + 8);
    if (!(fabs(dd) > 0.0))
    {
      bad = 1;
      break;
    }
    if (r == 0 && tid == 0) // the one thread that writes log|det| (FP64 log is slow on this GPU)
    {
      logabs.mul(dd);
      if (dd < 0.0)
        sgn = -sgn;
      if (p != k)
        sgn = -sgn;
    }
    const W d = static_cast<W>(dd);
    if (p != k)
      for (int jj = tid; jj < ncw; jj += GJ_NT)
      {
        const W t                = blk[(size_t)k * ld + jj];
        blk[(size_t)k * ld + jj] = blk[(size_t)p * ld + jj];
        blk[(size_t)p * ld + jj] = t;
      }
    // the owner's pivot column into local shared memory: one round trip over the cluster
    // for all rows instead of one per row
    const unsigned rpc = dsm_map(pcs + (size_t)b * n, (unsigned)owner);
    for (int i = tid; i < n; i += GJ_NT)
      pcl[i] = dsm_ldw<W>(rpc + (unsigned)sizeof(W) * (unsigned)i);
    __syncthreads();
    for (int jj = tid; jj < ncw; jj += GJ_NT)
      blk[(size_t)k * ld + jj] = (c0 + jj == k ? W(1) : blk[(size_t)k * ld + jj]) / d;
    __syncthreads();
    // elimination over (rows x own columns) with 16 threads along a row
    {
      const int tx = tid & 15, ty = tid >> 4;
      const W* bk  = blk + (size_t)k * ld;
      for (int i = ty; i < n; i += GJ_NT / 16)
      {
        if (i == k)
          continue;
        const W f = pcl[i];
        W* bi     = blk + (size_t)i * ld;
        for (int jj = tx; jj < ncw; jj += 16)
        {
          const W base = (c0 + jj == k) ? W(0) : bi[jj];
          bi[jj]       = base - f * bk[jj];
        }
      }
    }
    __syncthreads();
  }
  // results back to global memory, then the column interchanges (column j holds working
  // column cmap[j], possibly of another CTA)
  for (int i = wid; i < n; i += GJ_NT / 32)
    for (int jj = lane; jj < ncw; jj += 32)
      a[(size_t)i * n + c0 + jj] = static_cast<double>(blk[(size_t)i * ld + jj]);
  cluster_sync_all();
  if (bad)
  {
    if (r == 0 && tid == 0)
    {
      atomicOr(s.status + (slot % s.nw), ST_SINGULAR);
      s.log_abs[slot] = -INFINITY;
      s.sign[slot]    = 0;
    }
    cluster_sync_all(); // the owners' shared memory stays valid until every CTA is done
    return;
  }
  if (tid == 0)
  {
    for (int j = 0; j < n; j++)
      cmap[j] = j;
    for (int k = n - 1; k >= 0; k--)
    {
      const int p = dsm_ldi(dsm_map(perm + k, (unsigned)(k / cw)));
      const int t = cmap[k];
      cmap[k]     = cmap[p];
      cmap[p]     = t;
    }
  }
  __syncthreads();
  T* A = s.Ainv + (size_t)slot * n * s.lda;
  for (int i = wid; i < n; i += GJ_NT / 32)
    for (int jj = lane; jj < ncw; jj += 32)
      A[(size_t)i * s.lda + c0 + jj] = static_cast<T>(__ldcg(a + (size_t)i * n + cmap[c0 + jj]));
  if (r == 0 && tid == 0)
  {
    s.log_abs[slot] = logabs.value();
    s.sign[slot]    = sgn;
  }
  cluster_sync_all(); // the owners' shared memory stays valid until every CTA is done
}

// ---------------------------------------------------------------------------
// Gauss-Jordan inverse with partial pivoting (FP32 elimination, FP64 log|det| sums) of
// one n x n matrix held in registers, n <= min(TY * NAR, 16 * NB): thread (ty, tx) of a
// TY x 16 block owns rows ty + TY a (a < NAR) and columns tx + 16 b (b < NB).  Per pivot step the column
// and the two interchanged rows pass through shared memory and every thread applies
// the rank-1 elimination to its own elements.  For the repair of small determinants
// (FP32 crowds), where a cluster's barrier would be the latency of every step.
// ---------------------------------------------------------------------------
template<typename T, int TY, int NAR, int NB>
__global__ void __launch_bounds__(16 * TY) gj_reg_kernel(DevState<T> s, const double* Mt, int masked)
{
  const int slot = blockIdx.x;
  if (skip_slot(s, slot, masked))
    return;
  constexpr int NMAX = 16 * NB > TY * NAR ? 16 * NB : TY * NAR;
  // rows and columns beyond n hold zeros throughout (their factors and pivot-row
  // entries are zero), so the staging below needs no bounds checks
  __shared__ float colk[2][NMAX]; // column k before the interchange (double-buffered: the
                                  // owners of column k + 1 write it during step k)
  __shared__ float rowk[NMAX];    // row k before the interchange
  __shared__ float rowp[NMAX];    // the pivot row before the interchange
  __shared__ int perm[NMAX];      // pivot row of every step
  __shared__ int cinv[NMAX];      // output column of every working column
  const int n = s.norb, tid = threadIdx.x, tx = tid & 15, ty = tid >> 4, lane = tid & 31;
  const double* M = Mt + (size_t)slot * n * n;
  float a[NAR][NB];
#pragma unroll
  for (int ia = 0; ia < NAR; ia++)
#pragma unroll
    for (int ib = 0; ib < NB; ib++)
    {
      const int i = ty + TY * ia, j = tx + 16 * ib;
      a[ia][ib]   = (i < n && j < n) ? static_cast<float>(M[(size_t)i * n + j]) : 0.f;
    }
  if (tx == 0)
#pragma unroll
    for (int ia = 0; ia < NAR; ia++)
      colk[0][ty + TY * ia] = a[ia][0];
  __syncthreads();
  LogAbsProduct logabs;
  int sgn = 1, bad = 0;
  for (int k = 0; k < n; k++)
  {
    const float* ck = colk[k & 1];
    const int kt = k & 15, kb = k >> 4;       // owners of column k
    const int kr = k % TY, ka = k / TY;       // owners of row k
    // every warp finds the pivot (same result, no broadcast)
    float bv = -1.f;
    int bi   = n;
    for (int i = k + lane; i < n; i += 32)
    {
      const float v = fabsf(ck[i]);
      if (v > bv || (v == bv && i < bi))
      {
        bv = v;
        bi = i;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
    {
      const float ov = __shfl_xor_sync(0xffffffffu, bv, o);
      const int oi   = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ov > bv || (ov == bv && oi < bi))
      {
        bv = ov;
        bi = oi;
      }
    }
    if (!(bv > 0.f))
    {
      bad = 1;
      break;
    }
    const int p = bi;
    if (tid == 0)
      perm[k] = p;
    const float d = ck[p];
    if (tid == 0) // the one thread that writes log|det| (FP64 log is slow on this GPU)
    {
      logabs.mul(static_cast<double>(d));
      if (d < 0.f)
        sgn = -sgn;
      if (p != k)
        sgn = -sgn;
    }
    const int pr = p % TY, pa = p / TY;       // owners of row p
    if (ty == kr)
#pragma unroll
      for (int c = 0; c < NAR; c++)
        if (c == ka)
#pragma unroll
          for (int ib = 0; ib < NB; ib++)
            rowk[tx + 16 * ib] = a[c][ib];
    if (ty == pr)
#pragma unroll
      for (int c = 0; c < NAR; c++)
        if (c == pa)
#pragma unroll
          for (int ib = 0; ib < NB; ib++)
            rowp[tx + 16 * ib] = a[c][ib];
    __syncthreads();
    // new pivot row rk = (old row p with 1 at column k) / d; factors f = column k after
    // the interchange, 0 at row k
    const float rinv = 1.f / d;
    float rk[NB], f[NAR];
#pragma unroll
    for (int ib = 0; ib < NB; ib++)
    {
      const int j = tx + 16 * ib;
      rk[ib]      = j < n ? (j == k ? 1.f : rowp[j]) * rinv : 0.f;
    }
#pragma unroll
    for (int ia = 0; ia < NAR; ia++)
    {
      const int i = ty + TY * ia;
      f[ia]       = (i < n && i != k) ? ck[i == p ? k : i] : 0.f;
    }
    // the interchange: row p takes row k's old values
    if (ty == pr && p != k)
#pragma unroll
      for (int c = 0; c < NAR; c++)
        if (c == pa)
#pragma unroll
          for (int ib = 0; ib < NB; ib++)
            a[c][ib] = rowk[tx + 16 * ib];
    // elimination of every element, then row k and column k set to their new values
#pragma unroll
    for (int ia = 0; ia < NAR; ia++)
#pragma unroll
      for (int ib = 0; ib < NB; ib++)
        a[ia][ib] = fmaf(-f[ia], rk[ib], a[ia][ib]);
    if (tx == kt)
#pragma unroll
      for (int c = 0; c < NB; c++)
        if (c == kb)
#pragma unroll
          for (int ia = 0; ia < NAR; ia++)
            a[ia][c] = -f[ia] * rinv;
    if (ty == kr)
#pragma unroll
      for (int c = 0; c < NAR; c++)
        if (c == ka)
#pragma unroll
          for (int ib = 0; ib < NB; ib++)
            a[c][ib] = rk[ib];
    // column k + 1 for the next step's pivot search, by its owners
    const int k1 = k + 1, k1t = k1 & 15, k1b = k1 >> 4;
    if (k1 < n && tx == k1t)
#pragma unroll
      for (int c = 0; c < NB; c++)
        if (c == k1b)
#pragma unroll
          for (int ia = 0; ia < NAR; ia++)
            colk[k1 & 1][ty + TY * ia] = a[ia][c];
    __syncthreads(); // rowk, rowp and the other column buffer are rewritten by the next step
  }
  if (bad)
  {
    if (tid == 0)
    {
      atomicOr(s.status + (slot % s.nw), ST_SINGULAR);
      s.log_abs[slot] = -INFINITY;
      s.sign[slot]    = 0;
    }
    return;
  }
  // the row interchanges become column interchanges applied in reverse order: output
  // column c holds working column cmap[c]; cinv is its inverse
  if (tid == 0)
  {
    int* cmap = reinterpret_cast<int*>(rowk); // rowk is free now (same size as an int array)
    for (int j = 0; j < n; j++)
      cmap[j] = j;
    for (int k = n - 1; k >= 0; k--)
    {
      const int p = perm[k];
      const int t = cmap[k];
      cmap[k]     = cmap[p];
      cmap[p]     = t;
    }
    for (int c = 0; c < n; c++)
      cinv[cmap[c]] = c;
  }
  __syncthreads();
  T* A = s.Ainv + (size_t)slot * n * s.lda;
#pragma unroll
  for (int ia = 0; ia < NAR; ia++)
#pragma unroll
    for (int ib = 0; ib < NB; ib++)
    {
      const int i = ty + TY * ia, j = tx + 16 * ib;
      if (i < n && j < n)
        A[(size_t)i * s.lda + cinv[j]] = static_cast<T>(a[ia][ib]);
    }
  if (tid == 0)
  {
    s.log_abs[slot] = logabs.value();
    s.sign[slot]    = sgn;
  }
}

// ---------------------------------------------------------------------------
// Register-resident Gauss-Jordan over a cluster of CL CTAs (FP32 elimination, FP64
// log|det| product), for determinants too large for one CTA's registers: CTA r owns the
// columns [r cw, r cw + cw); inside it thread (ty, tx) owns rows ty + TY a (a < NAR) and
// local columns tx + 16 b (b < NB).  Rows k and p and the pivot value are local to every
// CTA (each holds its slice of every row); only the pivot column crosses CTAs: its owner
// finds the pivot and publishes the column in shared memory (double-buffered), one
// cluster barrier later every CTA copies it once over distributed shared memory and
// eliminates its block in registers.
// ---------------------------------------------------------------------------
template<typename T, int CL, int TY, int NAR, int NB>
__global__ void __launch_bounds__(16 * TY) gj_regcl_kernel(DevState<T> s, const double* Mt, int masked)
{
  const int slot = blockIdx.x / CL;
  if (skip_slot(s, slot, masked)) // uniform over the cluster
    return;
  constexpr int NMAX = TY * NAR;   // rows
  constexpr int CWMAX = 16 * NB;   // columns per CTA
  __shared__ float colp[2][NMAX];  // published pivot column (before the interchange), owner CTA
  __shared__ int pub[2];           // published pivot row (-1: singular)
  __shared__ float colk[NMAX];     // this CTA's copy of the step's pivot column
  __shared__ float rowk[CWMAX];    // this CTA's slice of row k before the interchange
  __shared__ float rowp[CWMAX];    // this CTA's slice of the pivot row before the interchange
  __shared__ int perm[NMAX];       // pivot row of every step
  __shared__ int cinv[NMAX];       // output column of every working column
  const int n = s.norb, r = (int)cluster_rank();
  const int cw = (n + CL - 1) / CL, c0 = r * cw, ncw = max(0, min(n, c0 + cw) - c0);
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4, lane = tid & 31;
  const double* M = Mt + (size_t)slot * n * n;
  float a[NAR][NB];
#pragma unroll
  for (int ia = 0; ia < NAR; ia++)
#pragma unroll
    for (int ib = 0; ib < NB; ib++)
    {
      const int i = ty + TY * ia, jl = tx + 16 * ib;
      a[ia][ib]   = (i < n && jl < ncw) ? static_cast<float>(M[(size_t)i * n + c0 + jl]) : 0.f;
    }
  LogAbsProduct logabs;
  int sgn = 1, bad = 0;
  for (int k = 0; k < n; k++)
  {
    const int b = k & 1;
    const int owner = k / cw, kl = k - owner * cw; // owning CTA and its local column
    const int kt = kl & 15, kb = kl >> 4;
    if (owner == r)
    {
      // column k to shared memory, then every warp finds the pivot; warp 0 publishes it
      if (tx == kt)
#pragma unroll
        for (int c = 0; c < NB; c++)
          if (c == kb)
#pragma unroll
            for (int ia = 0; ia < NAR; ia++)
              colp[b][ty + TY * ia] = a[ia][c];
      __syncthreads();
      float bv = -1.f;
      int bi   = n;
      for (int i = k + lane; i < n; i += 32)
      {
        const float v = fabsf(colp[b][i]);
        if (v > bv || (v == bv && i < bi))
        {
          bv = v;
          bi = i;
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1)
      {
        const float ov = __shfl_xor_sync(0xffffffffu, bv, o);
        const int oi   = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ov > bv || (ov == bv && oi < bi))
        {
          bv = ov;
          bi = oi;
        }
      }
      if (tid == 0)
        pub[b] = bv > 0.f ? bi : -1;
    }
    cluster_sync_all();
    const int p = dsm_ldi(dsm_map(&pub[b], (unsigned)owner));
    if (p < 0)
    {
      bad = 1;
      break;
    }
    // the pivot column from the owner, this CTA's slices of rows k and p
    const unsigned rc = dsm_map(&colp[b][0], (unsigned)owner);
    for (int i = tid; i < n; i += 16 * TY)
      colk[i] = dsm_ldf(rc + 4u * (unsigned)i);
    const int kr = k % TY, ka = k / TY, pr = p % TY, pa = p / TY;
    if (ty == kr)
#pragma unroll
      for (int c = 0; c < NAR; c++)
        if (c == ka)
#pragma unroll
          for (int ib = 0; ib < NB; ib++)
            rowk[tx + 16 * ib] = a[c][ib];
    if (ty == pr)
#pragma unroll
      for (int c = 0; c < NAR; c++)
        if (c == pa)
#pragma unroll
          for (int ib = 0; ib < NB; ib++)
            rowp[tx + 16 * ib] = a[c][ib];
    __syncthreads();
    const float d = colk[p];
    if (tid == 0)
      perm[k] = p;
    if (r == 0 && tid == 0) // the one thread that writes log|det|
    {
      logabs.mul(static_cast<double>(d));
      if (d < 0.f)
        sgn = -sgn;
      if (p != k)
        sgn = -sgn;
    }
    const float rinv = 1.f / d;
    // new pivot row slice rk = (old row p with 1 at column k) / d
    float rk[NB];
#pragma unroll
    for (int ib = 0; ib < NB; ib++)
    {
      const int jl = tx + 16 * ib;
      rk[ib]       = jl < ncw ? (c0 + jl == k ? 1.f : rowp[jl]) * rinv : 0.f;
    }
    // the interchange: row p takes row k's old values
    if (ty == pr && p != k)
#pragma unroll
      for (int c = 0; c < NAR; c++)
        if (c == pa)
#pragma unroll
          for (int ib = 0; ib < NB; ib++)
            a[c][ib] = rowk[tx + 16 * ib];
    // elimination with the factors of column k after the interchange (0 at row k)
#pragma unroll
    for (int ia = 0; ia < NAR; ia++)
    {
      const int i   = ty + TY * ia;
      const float f = (i < n && i != k) ? colk[i == p ? k : i] : 0.f;
#pragma unroll
      for (int ib = 0; ib < NB; ib++)
        a[ia][ib] = fmaf(-f, rk[ib], a[ia][ib]);
      if (owner == r && tx == kt)
#pragma unroll
        for (int c = 0; c < NB; c++)
          if (c == kb)
            a[ia][c] = -f * rinv;
    }
    if (ty == kr)
#pragma unroll
      for (int c = 0; c < NAR; c++)
        if (c == ka)
#pragma unroll
          for (int ib = 0; ib < NB; ib++)
            a[c][ib] = rk[ib];
    __syncthreads(); // colk, rowk and rowp are rewritten by the next step
  }
  if (bad)
  {
    if (r == 0 && tid == 0)
    {
      atomicOr(s.status + (slot % s.nw), ST_SINGULAR);
      s.log_abs[slot] = -INFINITY;
      s.sign[slot]    = 0;
    }
    cluster_sync_all(); // the owners' shared memory stays valid until every CTA is done
    return;
  }
  // output column c holds working column cmap[c] (built in colk's storage); cinv is its
  // inverse.  Every CTA holds perm.
  if (tid == 0)
  {
    int* cmap = reinterpret_cast<int*>(colk);
    for (int j = 0; j < n; j++)
      cmap[j] = j;
    for (int k = n - 1; k >= 0; k--)
    {
      const int p = perm[k];
      const int t = cmap[k];
      cmap[k]     = cmap[p];
      cmap[p]     = t;
    }
    for (int c = 0; c < n; c++)
      cinv[cmap[c]] = c;
  }
  __syncthreads();
  T* A = s.Ainv + (size_t)slot * n * s.lda;
#pragma unroll
  for (int ia = 0; ia < NAR; ia++)
#pragma unroll
    for (int ib = 0; ib < NB; ib++)
    {
      const int i = ty + TY * ia, jl = tx + 16 * ib;
      if (i < n && jl < ncw)
        A[(size_t)i * s.lda + cinv[c0 + jl]] = static_cast<T>(a[ia][ib]);
    }
  if (r == 0 && tid == 0)
  {
    s.log_abs[slot] = logabs.value();
    s.sign[slot]    = sgn;
  }
  cluster_sync_all(); // the owners' shared memory stays valid until every CTA is done
}

// Work items (walker, block of NT / 32 electrons), one warp per electron i with its lanes
// over the partners: Uat, dUat, d2Uat of electron i over all j != i, and Vat, Grad, Lap
// over the ions.  Unmasked: every walker; masked: the walkers of repair_list.
template<typename T, int NT>
__global__ void __launch_bounds__(NT) jastrow_full_kernel(DevState<T> s, int masked)
{
  constexpr int EPB = NT / 32;
  const int lane   = threadIdx.x & 31;
  const int nbj    = (s.ne + EPB - 1) / EPB;
  const int nitems = (masked ? s.repair_list[0] : s.nw) * nbj;
  for (int item = blockIdx.x; item < nitems; item += gridDim.x)
  {
  const int iw = masked ? s.repair_list[1 + item / nbj] : item / nbj;
  const int i  = (item % nbj) * EPB + (threadIdx.x >> 5);
  if (i >= s.ne) // uniform over the warp
    continue;
  const T* Rx = s.Rt + ((size_t)iw * 3) * s.ne_pad;
  const T xi = Rx[i], yi = Rx[s.ne_pad + i], zi = Rx[2 * s.ne_pad + i];
  const T L0 = T(s.L[0]), L1 = T(s.L[1]), L2 = T(s.L[2]);
  const T Li0 = T(s.G[0]), Li1 = T(s.G[1]), Li2 = T(s.G[2]);
  {
    T v[5] = {0, 0, 0, 0, 0}; // u, grad xyz, lap
    if (s.has_j2)
      for (int j = lane; j < s.ne; j += 32)
      {
        if (j == i)
          continue;
        const T dx = min_image(Rx[j] - xi, L0, Li0);
        const T dy = min_image(Rx[s.ne_pad + j] - yi, L1, Li1);
        const T dz = min_image(Rx[2 * s.ne_pad + j] - zi, L2, Li2);
        const T r  = sqrt(dx * dx + dy * dy + dz * dz);
        if (r < s.j2_rcut)
        {
          const int same = (j < s.nup) == (i < s.nup);
          T du, d2u;
          v[0] += functor_eval(s.j2c + (same ? 0 : s.j2_ncoef), s.j2_dri, s.j2_maxidx, r, du, d2u);
          du *= T(1) / r;
          v[1] += du * dx;
          v[2] += du * dy;
          v[3] += du * dz;
          v[4] += d2u + T(2) * du;
        }
      }
#pragma unroll
    for (int q = 0; q < 5; q++)
      v[q] = warp_sum(v[q]);
    if (lane == 0)
    {
      T* J2                = s.J2 + (size_t)iw * 5 * s.ne_pad;
      J2[i]                = v[0];
      J2[s.ne_pad + i]     = v[1];
      J2[2 * s.ne_pad + i] = v[2];
      J2[3 * s.ne_pad + i] = v[3];
      J2[4 * s.ne_pad + i] = -v[4];
    }
  }
  {
    T v[5] = {0, 0, 0, 0, 0};
    if (s.has_j1)
      for (int j = lane; j < s.nions; j += 32)
      {
        const T dx = min_image(s.ions[j] - xi, L0, Li0);
        const T dy = min_image(s.ions[s.nions_pad + j] - yi, L1, Li1);
        const T dz = min_image(s.ions[2 * s.nions_pad + j] - zi, L2, Li2);
        const T r  = sqrt(dx * dx + dy * dy + dz * dz);
        if (r < s.j1_rcut)
        {
          T du, d2u;
          v[0] += functor_eval(s.j1c + (size_t)s.ion_species[j] * s.j1_ncoef, s.j1_dri, s.j1_maxidx, r, du, d2u);
          du *= T(1) / r;
          v[1] += du * dx;
          v[2] += du * dy;
          v[3] += du * dz;
          v[4] += d2u + T(2) * du;
        }
      }
#pragma unroll
    for (int q = 0; q < 5; q++)
      v[q] = warp_sum(v[q]);
    if (lane == 0)
    {
      T* J1                = s.J1 + (size_t)iw * 5 * s.ne_pad;
      J1[i]                = v[0];
      J1[s.ne_pad + i]     = v[1];
      J1[2 * s.ne_pad + i] = v[2];
      J1[3 * s.ne_pad + i] = v[3];
      J1[4 * s.ne_pad + i] = v[4];
    }
  }
  }
}

// after a masked recompute: count and clear the repaired walkers' repair bits
template<typename T>
__global__ void finish_repair_kernel(DevState<T> s)
{
  const int iw = blockIdx.x * blockDim.x + threadIdx.x;
  if (iw >= s.nw)
    return;
  const int st = s.status[iw];
  if (st & ST_REPAIR_MASK)
  {
    s.status[iw] = st & ~ST_REPAIR_MASK;
    atomicAdd(s.counters + 2, 1ull);
  }
}

static bool gj_cluster16_ok();

template<typename T>
cudaError_t launch_recompute(const DevState<T>& s, double* Mt, int masked, cudaStream_t st)
{
  constexpr int NT = 128;
  const size_t sm  = sizeof(T) * 4 * 7 * (size_t)s.lda;
  const int nblk   = (s.ne + VGL_EPB - 1) / VGL_EPB;
  static int sms   = 0;
  if (sms == 0)
  {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                  cudaSuccess || sms <= 0)
      sms = 1;
  }
  // a repair touches a few walkers: their work items go to a grid of one wave
  const int small = 8 * sms;
  if (masked)
  {
    repair_list_kernel<T><<<1, 1024, 0, st>>>(s);
    vgl_all_kernel<T, NT><<<std::min(small, s.nw * nblk), NT, sm, st>>>(s, Mt, masked);
  }
  else
    vgl_all_kernel<T, NT><<<s.nw * nblk, NT, sm, st>>>(s, Mt, masked);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess)
    return e;
  if (masked && s.gj_scratch)
  {
    // the few flagged matrices: a cluster of SMs each
    const int n            = s.norb;
    cudaLaunchConfig_t cfg = {};
    cfg.blockDim           = dim3(GJ_NT);
    cfg.stream             = st;
    cudaLaunchAttribute attr[1];
    attr[0].id               = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs                = attr;
    cfg.numAttrs             = 1;
    auto with_cluster = [&](int cl, size_t smem, int threads = GJ_NT) {
      cfg.gridDim              = dim3(2 * s.nw * cl);
      cfg.blockDim             = dim3(threads);
      attr[0].val.clusterDim.x = cl;
      cfg.dynamicSmemBytes     = smem;
    };
    bool done = false;
    if constexpr (std::is_same<T, float>::value)
    {
      if (n <= 192)
      {
        // register-resident, one CTA per matrix
        if (n <= 32)
          gj_reg_kernel<float, 16, 2, 2><<<2 * s.nw, 256, 0, st>>>(s, Mt, masked);
        else if (n <= 64)
          gj_reg_kernel<float, 16, 4, 4><<<2 * s.nw, 256, 0, st>>>(s, Mt, masked);
        else if (n <= 128)
          gj_reg_kernel<float, 32, 4, 8><<<2 * s.nw, 512, 0, st>>>(s, Mt, masked);
        else
          gj_reg_kernel<float, 24, 8, 12><<<2 * s.nw, 384, 0, st>>>(s, Mt, masked);
        e    = cudaGetLastError();
        done = true;
      }
      else if (n <= 384)
      {
        // register-resident over a cluster of 8 CTAs (48 columns each)
        with_cluster(8, 0, 16 * 32);
        e    = cudaLaunchKernelEx(&cfg, gj_regcl_kernel<float, 8, 32, 12, 3>, s, static_cast<const double*>(Mt),
                                  masked);
        done = true;
      }
      else if (n <= 768 && gj_cluster16_ok())
      {
        // register-resident over a cluster of 16 CTAs (48 columns each)
        with_cluster(16, 0, 16 * 48);
        e    = cudaLaunchKernelEx(&cfg, gj_regcl_kernel<float, 16, 48, 16, 3>, s, static_cast<const double*>(Mt),
                                  masked);
        done = true;
      }
      else if (gj_smem_bytes(n, 8, 4) <= GJ_SMEM_MAX)
      {
        with_cluster(8, gj_smem_bytes(n, 8, 4));
        e    = cudaLaunchKernelEx(&cfg, gj_cluster_smem_kernel<float, float, 8>, s, Mt, masked);
        done = true;
      }
      else if (gj_smem_bytes(n, 16, 4) <= GJ_SMEM_MAX && gj_cluster16_ok())
      {
        with_cluster(16, gj_smem_bytes(n, 16, 4));
        e    = cudaLaunchKernelEx(&cfg, gj_cluster_smem_kernel<float, float, 16>, s, Mt, masked);
        done = true;
      }
    }
    if (!done && gj_smem_bytes(n, GJ_CL, 8) <= GJ_SMEM_MAX)
    {
      with_cluster(GJ_CL, gj_smem_bytes(n, GJ_CL, 8));
      e = cudaLaunchKernelEx(&cfg, gj_cluster_smem_kernel<T, double, GJ_CL>, s, Mt, masked);
    }
    else if (!done)
    {
      with_cluster(GJ_CL, (size_t)((n + GJ_CL - 1) / GJ_CL) * sizeof(double) + (size_t)n * sizeof(int));
      e = cudaLaunchKernelEx(&cfg, gj_cluster_kernel<T>, s, Mt, masked);
    }
  }
  else
  {
    // every matrix in FP64: for larger matrices a column block per CTA in shared memory
    // over a cluster of 8 CTAs when it fits (the same eliminations as one CTA per matrix,
    // without the global-memory traffic of every pivot step; 18% faster at 384 x 384, no
    // gain at 192 x 192), else one CTA per matrix
    const int n            = s.norb;
    cudaLaunchConfig_t cfg = {};
    cfg.blockDim           = dim3(GJ_NT);
    cfg.stream             = st;
    cudaLaunchAttribute attr[1];
    attr[0].id               = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs                = attr;
    cfg.numAttrs             = 1;
    if (n > 256 && gj_smem_bytes(n, GJ_CL, 8) <= GJ_SMEM_MAX)
    {
      cfg.gridDim              = dim3(2 * s.nw * GJ_CL);
      attr[0].val.clusterDim.x = GJ_CL;
      cfg.dynamicSmemBytes     = gj_smem_bytes(n, GJ_CL, 8);
      e = cudaLaunchKernelEx(&cfg, gj_cluster_smem_kernel<T, double, GJ_CL>, s, Mt, masked);
    }
    else
    {
      constexpr int NTG = 512;
      const size_t smg  = (size_t)s.norb * (2 * sizeof(double) + sizeof(int));
      gj_inverse_kernel<T, NTG><<<2 * s.nw, NTG, smg, st>>>(s, Mt, masked);
      e = cudaGetLastError();
    }
  }
  if (e != cudaSuccess)
    return e;
  const int jitems = s.nw * ((s.ne + 3) / 4);
  jastrow_full_kernel<T, 128><<<masked ? std::min(small, jitems) : jitems, 128, 0, st>>>(s, masked);
  e = cudaGetLastError();
  if (e != cudaSuccess || !masked)
    return e;
  finish_repair_kernel<T><<<(s.nw + 127) / 128, 128, 0, st>>>(s);
  return cudaGetLastError();
}

template<typename T>
cudaError_t setup_recompute_kernels()
{
  cudaError_t e = cudaFuncSetAttribute(vgl_all_kernel<T, 128>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(gj_cluster_smem_kernel<T, double, GJ_CL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             GJ_SMEM_MAX);

  if constexpr (std::is_same<T, float>::value)
  {
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(gj_cluster_smem_kernel<float, float, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               GJ_SMEM_MAX);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(gj_cluster_smem_kernel<float, float, 16>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, GJ_SMEM_MAX);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(gj_cluster_smem_kernel<float, float, 16>,
                               cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(gj_regcl_kernel<float, 16, 48, 16, 3>,
                               cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  }
  return e;
}

// whether a cluster of 16 CTAs with the largest column block can be resident on this
// GPU (16 is above the portable cluster size); asked once per process
static bool gj_cluster16_ok()
{
  static int ok = -1;
  if (ok < 0)
  {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim            = dim3(16);
    cfg.blockDim           = dim3(GJ_NT);
    cfg.dynamicSmemBytes   = GJ_SMEM_MAX;
    cudaLaunchAttribute attr[1];
    attr[0].id               = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 16;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs                = attr;
    cfg.numAttrs             = 1;
    int nc                   = 0;
    const cudaError_t e      = cudaOccupancyMaxActiveClusters(&nc, gj_cluster_smem_kernel<float, float, 16>, &cfg);
    if (e != cudaSuccess)
      (void)cudaGetLastError();
    ok = (e == cudaSuccess && nc >= 1) ? 1 : 0;
  }
  return ok == 1;
}

template cudaError_t setup_recompute_kernels<float>();
template cudaError_t setup_recompute_kernels<double>();
template cudaError_t launch_recompute<float>(const DevState<float>&, double*, int, cudaStream_t);
template cudaError_t launch_recompute<double>(const DevState<double>&, double*, int, cudaStream_t);

} // namespace qmcg
