// Block-lazy delayed updates of the walker-resident sweep.
//
// DelayedUpdateBatched::mw_updateInvMat (DelayedUpdateBatched.h:675-738) brings every row
// of the inverse up to date after each k moves of a spin group:
//   Ainv -= (Ainv U^T - E) Binv V,   E[r][c] = 1 where r is the row moved in slot c.
// A segment of the walker-resident sweep reads only the inverse rows of its own k
// electrons.  Here every segment's (U, V, Binv, delay list) is kept as a set, and a block
// of k rows receives the sets it has not yet seen right before the segment that reads
// it; one pass at the end of the spin group gives every block the sets from its own on,
// so the inverse is complete after each spin group, as after mw_completeUpdates.  Every
// row receives the same rank-k updates in the same order as with a flush after every
// segment, but the inverse is read and written about twice per spin group instead of
// once per segment.
//
// A rejected (pseudo-accepted) slot has a zero U row, no delay-list row and an identity
// column of Binv (mw_accept_rejectRow), so its column of (Ainv U^T - E) is zero and its
// column of (Ainv U^T - E) Binv is zero too: only the accepted slots of a set enter the
// products, which at VMC acceptance rates is a fraction of k.
//
// One CTA per (walker, row block of up to 32 rows), eight warps: warp w keeps rows
// 4w..4w+3 of the block in registers for all sets (lane l holds columns l + 32 i).  Per
// set the accepted U and V rows and Binv restricted to them arrive in shared memory (one
// barrier); T1 = rows U^T - E is formed by the lanes over the columns and finished by a
// transposed warp reduction, X = T1 Binv and rows -= X V stay inside the warp.  The
// delay lists of all pending sets are compacted at the start, one warp per set.
#include <type_traits>

#include "common.cuh"
#include "launch.h"

namespace qmcg
{

// E[r][c] of the accepted slot c: 1 where slot c moved row r
__device__ __forceinline__ bool acrq_is(const int* acr, int c, int row) { return acr[c] == row; }

constexpr int BU_NT   = 256;
constexpr int BU_NW   = BU_NT / 32;
constexpr int BU_RPW  = 4;  // rows per warp
constexpr int BU_MAXK = 32; // rows per block = delay rank
constexpr int BU_JN   = 8;  // columns per lane: lda <= 256

struct BuLayout
{
  int ldu;                       // row stride of Us and Vs: 32 x columns per lane, zero beyond lda
  int us, vs, t1, xs, bs, total; // offsets in elements of T
  int ac_bytes;                  // the compacted delay lists (ints), after total
};

// rows of Us and Vs: the delay rank rounded up to the 8-column chunks of T1 (rows beyond a
// set's accepted count are zero)
__host__ __device__ inline int bu_urows(int k) { return (k + 7) / 8 * 8; }

__host__ __device__ inline BuLayout bu_layout(int lda, int k, int nsets)
{
  BuLayout L;
  L.ldu = (lda + 31) / 32 * 32;
  int o = 0;
  L.us       = o, o += bu_urows(k) * L.ldu;
  L.vs       = o, o += bu_urows(k) * L.ldu;
  L.t1       = o, o += BU_MAXK * (k + 1);
  L.xs       = o, o += BU_MAXK * (k + 1);
  L.bs       = o, o += k * (k + 1);
  L.total    = o;
  L.ac_bytes = (2 * nsets * k + nsets) * (int)sizeof(int);
  return L;
}

template<typename T>
static size_t bu_smem(int lda, int k, int nsets)
{
  const BuLayout L = bu_layout(lda, k, nsets);
  return sizeof(T) * (size_t)L.total + L.ac_bytes;
}

// cp.async of one row of lda elements (a multiple of 16 bytes) into shared memory by one warp
template<typename T>
__device__ __forceinline__ void row_async(T* dst, const T* src, int lda, int lane)
{
  const int chunks = lda * (int)sizeof(T) / 16;
  for (int c = lane; c < chunks; c += 32)
  {
    const unsigned sa = static_cast<unsigned>(__cvta_generic_to_shared(reinterpret_cast<char*>(dst) + 16 * c));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(reinterpret_cast<const char*>(src) +
                                                                          16 * c)
                 : "memory");
  }
}

// T1 columns [c0, c0 + CW) of this warp's four rows: every lane forms its columns'
// partial dot products of the 4 x CW values, a transposed warp reduction finishes them
// (lane l ends with value l / (32 / (4 CW)), row-major over the 4 x CW), and the values
// minus E land in t1w.  Us rows beyond the set's accepted count and columns beyond lda
// are zero, so the loads need no guard.
template<typename T, int JN, int CW>
__device__ __forceinline__ void t1_chunk(const T (&a)[BU_RPW][JN], const T* Us, int ldu, int m, int c0,
                                         const int* acrq, int r0w, T* t1w, int ldk, int lane)
{
  constexpr int NV = BU_RPW * CW; // 32 or 16 values
  T acc[NV];
#pragma unroll
  for (int v = 0; v < NV; v++)
    acc[v] = T(0);
#pragma unroll
  for (int i = 0; i < JN; i++)
  {
    const T* up = Us + c0 * ldu + lane + 32 * i;
#pragma unroll
    for (int cc = 0; cc < CW; cc++)
    {
      const T u = up[cc * ldu];
#pragma unroll
      for (int rr = 0; rr < BU_RPW; rr++)
        acc[rr * CW + cc] += a[rr][i] * u;
    }
  }
  // halve the values at distances 16, 8, ...: after the stage at distance h lane l keeps
  // the values whose index bit (h / (32 / NV)) matches its lane bit
#pragma unroll
  for (int h = NV / 2; h >= 1; h >>= 1)
  {
    const int d    = h * (32 / NV);
    const bool up  = (lane & d) != 0;
#pragma unroll
    for (int v = 0; v < h; v++)
    {
      const T send = up ? acc[v] : acc[v + h];
      const T recv = __shfl_xor_sync(0xffffffffu, send, d);
      acc[v]       = (up ? acc[v + h] : acc[v]) + recv;
    }
  }
  if (NV == 16)
    acc[0] += __shfl_xor_sync(0xffffffffu, acc[0], 1);
  // value index held by this lane: (lane / (32 / NV)) = rr * CW + cc
  const int idx = lane / (32 / NV), rr = idx / CW, c = c0 + idx % CW;
  if (c < m && lane % (32 / NV) == 0)
    t1w[rr * ldk + c] = acrq_is(acrq, c, r0w + rr) ? acc[0] - T(1) : acc[0];
}

// JN = columns per lane (lda <= 32 JN)
template<typename T, int JN>
__global__ void __launch_bounds__(BU_NT, sizeof(T) == 4 ? 2 : 1) block_update_kernel(DevState<T> s, int spin,
                                                                                     int block0, int set_hi,
                                                                                     int complete)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int w = blockIdx.x, b = block0 + blockIdx.y;
  const int K = s.k, n = s.norb, lda = s.lda;
  const int nspin = spin ? s.ne - s.nup : s.nup;
  const int r0 = b * K, rb = min(K, nspin - r0);
  const int lo = complete ? b : 0, hi = set_hi, nq = hi - lo;
  if (rb <= 0 || nq <= 0)
    return;
  const BuLayout L = bu_layout(lda, K, s.nsets);
  const int ldu    = L.ldu;
  T* sm   = reinterpret_cast<T*>(smem_raw);
  T* Us   = sm + L.us;
  T* Vs   = sm + L.vs;
  T* t1   = sm + L.t1;
  T* xs   = sm + L.xs;
  T* bs   = sm + L.bs;
  int* ac  = reinterpret_cast<int*>(sm + L.total); // [nq][K] accepted slots of each pending set
  int* acr = ac + s.nsets * K;                      // [nq][K] their rows
  int* ms  = acr + s.nsets * K;                     // [nq] accepted counts
  const int ldk = K + 1;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const size_t slot = (size_t)spin * s.nw + w;
  T* A = s.Ainv + (slot * n + r0) * lda;

  // the delay lists of the pending sets, one warp per set
  for (int q = wid; q < nq; q += BU_NW)
  {
    const int set = lo + q, len = min(K, nspin - set * K);
    const int* dl = s.delay_list + (slot * s.nsets + set) * K;
    const int row = lane < len ? dl[lane] : -1;
    const unsigned bal = __ballot_sync(0xffffffffu, row >= 0);
    if (row >= 0)
    {
      const int p     = __popc(bal & ((1u << lane) - 1u));
      ac[q * K + p]   = lane;
      acr[q * K + p]  = row;
    }
    if (lane == 0)
      ms[q] = __popc(bal);
  }
  // columns [lda, ldu) of Us and Vs stay zero for the whole CTA
  if (ldu > lda)
    for (int e = threadIdx.x; e < 2 * bu_urows(K) * (ldu - lda); e += BU_NT)
    {
      const int r = e / (ldu - lda), j = lda + e % (ldu - lda);
      (r < bu_urows(K) ? Us : Vs)[(r % bu_urows(K)) * ldu + j] = T(0);
    }
  // this warp's rows in registers, lane l holding columns l + 32 i (columns beyond n are zero)
  T a[BU_RPW][JN];
#pragma unroll
  for (int rr = 0; rr < BU_RPW; rr++)
  {
    const int r = BU_RPW * wid + rr;
#pragma unroll
    for (int i = 0; i < JN; i++)
    {
      const int j = lane + 32 * i;
      a[rr][i]    = (r < rb && j < n) ? A[(size_t)r * lda + j] : T(0);
    }
  }
  __syncthreads();

  bool touched = false; // a set with accepted slots was applied (uniform over the CTA)
  T* t1w = t1 + BU_RPW * wid * ldk;
  T* xw  = xs + BU_RPW * wid * ldk;
  for (int q = 0; q < nq; q++)
  {
    const int m = ms[q];
    if (m == 0)
      continue;
    touched         = true;
    const size_t ds = slot * s.nsets + lo + q;
    const T* U      = s.U + ds * K * lda;
    const T* V      = s.V + ds * K * lda;
    const T* B      = s.Binv + ds * K * K;
    const int* acq  = ac + q * K;
    for (int c = wid; c < m; c += BU_NW)
    {
      row_async(Us + c * ldu, U + (size_t)acq[c] * lda, lda, lane);
      row_async(Vs + c * ldu, V + (size_t)acq[c] * lda, lda, lane);
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    // U rows [m, 8-column boundary) read as zero by the last chunk of T1
    for (int e = threadIdx.x; e < (bu_urows(m) - m) * lda; e += BU_NT)
      Us[(m + e / lda) * ldu + e % lda] = T(0);
    for (int e = threadIdx.x; e < m * m; e += BU_NT)
    {
      const int c = e / m, c2 = e % m;
      bs[c * ldk + c2] = B[acq[c] * K + acq[c2]];
    }
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    __syncthreads();

    // T1 = rows U^T - E, eight columns at a time, four for a remainder of at most four
    for (int c0 = 0; c0 < m;)
      if (m - c0 > 4)
      {
        t1_chunk<T, JN, 8>(a, Us, ldu, m, c0, acr + q * K, r0 + BU_RPW * wid, t1w, ldk, lane);
        c0 += 8;
      }
      else
      {
        t1_chunk<T, JN, 4>(a, Us, ldu, m, c0, acr + q * K, r0 + BU_RPW * wid, t1w, ldk, lane);
        c0 += 4;
      }
    __syncwarp();
    // X = T1 Binv for this warp's rows
    for (int e = lane; e < BU_RPW * m; e += 32)
    {
      const int rr = e / m, c2 = e % m;
      T x = 0;
      for (int c = 0; c < m; c++)
        x += t1w[rr * ldk + c] * bs[c * ldk + c2];
      xw[rr * ldk + c2] = x;
    }
    __syncwarp();
    // rows -= X V (columns beyond n of the rows are never stored)
    for (int c = 0; c < m; c++)
    {
      T x[BU_RPW];
#pragma unroll
      for (int rr = 0; rr < BU_RPW; rr++)
        x[rr] = xw[rr * ldk + c];
      const T* vp = Vs + c * ldu + lane;
#pragma unroll
      for (int i = 0; i < JN; i++)
      {
        const T v = vp[32 * i];
#pragma unroll
        for (int rr = 0; rr < BU_RPW; rr++)
          a[rr][i] -= x[rr] * v;
      }
    }
    // the next set's rows overwrite Us, Vs and bs
    __syncthreads();
  }
  if (!touched)
    return;
#pragma unroll
  for (int rr = 0; rr < BU_RPW; rr++)
  {
    const int r = BU_RPW * wid + rr;
#pragma unroll
    for (int i = 0; i < JN; i++)
    {
      const int j = lane + 32 * i;
      if (r < rb && j < n)
        A[(size_t)r * lda + j] = a[rr][i];
    }
  }
}

// the kernel instantiation for lda (columns per lane 1..8)
template<typename T, typename F>
static cudaError_t with_columns(int lda, F&& f)
{
  switch ((lda + 31) / 32)
  {
  case 1: return f(std::integral_constant<int, 1>{});
  case 2: return f(std::integral_constant<int, 2>{});
  case 3: return f(std::integral_constant<int, 3>{});
  case 4: return f(std::integral_constant<int, 4>{});
  case 5: return f(std::integral_constant<int, 5>{});
  case 6: return f(std::integral_constant<int, 6>{});
  case 7: return f(std::integral_constant<int, 7>{});
  case 8: return f(std::integral_constant<int, 8>{});
  default: return cudaErrorInvalidValue;
  }
}

template<typename T>
bool block_update_supported(const DevState<T>& s)
{
  return s.k > 1 && s.k <= BU_MAXK && s.nsets > 1 && s.lda <= 32 * BU_JN && s.lda * sizeof(T) % 16 == 0 &&
         bu_smem<T>(s.lda, s.k, s.nsets) <= 200 * 1024;
}

template<typename T>
cudaError_t setup_block_update()
{
  cudaError_t e = cudaSuccess;
  for (int jn = 1; jn <= BU_JN && e == cudaSuccess; jn++)
    e = with_columns<T>(32 * jn, [](auto c) {
      return cudaFuncSetAttribute(block_update_kernel<T, decltype(c)::value>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    });
  return e;
}

template<typename T>
cudaError_t launch_block_update(const DevState<T>& s, int spin, int block, int nblocks, int set_hi, bool complete,
                                cudaStream_t st)
{
  if (!block_update_supported(s) || nblocks < 1)
    return cudaErrorInvalidValue;
  const dim3 grid(s.nw, nblocks);
  return with_columns<T>(s.lda, [&](auto c) {
    block_update_kernel<T, decltype(c)::value>
        <<<grid, BU_NT, bu_smem<T>(s.lda, s.k, s.nsets), st>>>(s, spin, block, set_hi, complete ? 1 : 0);
    return cudaGetLastError();
  });
}

template bool block_update_supported<float>(const DevState<float>&);
template bool block_update_supported<double>(const DevState<double>&);
template cudaError_t setup_block_update<float>();
template cudaError_t setup_block_update<double>();
template cudaError_t launch_block_update<float>(const DevState<float>&, int, int, int, int, bool, cudaStream_t);
template cudaError_t launch_block_update<double>(const DevState<double>&, int, int, int, int, bool, cudaStream_t);

} // namespace qmcg
