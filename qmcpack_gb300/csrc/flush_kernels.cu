// Batched delayed-update flush, one CTA per (walker, block of R inverse rows):
//   W  = Binv V                     (dc x n, recomputed per CTA from Binv and V)
//   T1 = Ainv[rows] U^T - E[rows]   (R x dc)
//   Ainv[rows] -= T1 W
// DelayedUpdateBatched::mw_updateInvMat (DelayedUpdateBatched.h:675-738).  The row
// block, U^T, W and Binv are staged in shared memory; both products are register
// tiled with a warp owning 8 rows and its lanes owning columns, so shared-memory
// reads of the row block are warp-wide broadcasts and reads of U^T / W are
// contiguous.  The inverse is read and written once per flush (HBM bound at the
// algorithmic 2 x n x lda per walker, plus U, V, Binv).
#include <algorithm>

#include "common.cuh"
#include "launch.h"

namespace qmcg
{

constexpr int FLUSH_R  = 64;  // inverse rows per CTA
constexpr int FLUSH_NT = 256; // 8 warps x 8 rows
constexpr int FLUSH_MAXK = 64; // largest delay rank of the fused kernel

template<typename T>
static size_t flush_fused_smem(int n, int k)
{
  const size_t lds = (size_t)n + 1, ldu = (size_t)k + 1;
  return sizeof(T) * (FLUSH_R * lds + (size_t)n * ldu + (size_t)k * n + (size_t)FLUSH_R * k + (size_t)k * k);
}

template<typename T>
__global__ void __launch_bounds__(FLUSH_NT) flush_fused_kernel(FlushArgs<T> f)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n = f.n, k = f.k, dc = f.dc;
  const int lds = n + 1, ldu = k + 1;
  T* rows = reinterpret_cast<T*>(smem_raw); // R x lds
  T* Ut   = rows + FLUSH_R * lds;           // n x ldu   Ut[i][c] = U[c][i]
  T* Ws   = Ut + (size_t)n * ldu;           // k x n     W[c][i]
  T* t1   = Ws + (size_t)k * n;             // R x k
  T* Bs   = t1 + FLUSH_R * k;               // k x k
  const int iw = blockIdx.x;
  const int r0 = blockIdx.y * FLUSH_R;
  const int nr = min(FLUSH_R, n - r0);
  T* A             = f.ainv + (size_t)iw * f.sA;
  const T* U       = f.u + (size_t)iw * f.sU;
  const T* V       = f.v + (size_t)iw * f.sU;
  const T* Binv    = f.binv + (size_t)iw * f.sB;
  const int* dlist = f.delay_list + (size_t)iw * f.sD;

  for (int e = threadIdx.x; e < dc * dc; e += FLUSH_NT)
  {
    const int l = e / dc, c = e % dc;
    Bs[l * k + c] = Binv[(size_t)l * k + c];
  }
  for (int e = threadIdx.x; e < dc * n; e += FLUSH_NT)
  {
    const int c = e / n, i = e % n;
    Ut[i * ldu + c] = U[(size_t)c * f.lda + i];
  }
  for (int e = threadIdx.x; e < nr * n; e += FLUSH_NT)
  {
    const int r = e / n, i = e % n;
    rows[r * lds + i] = A[(size_t)(r0 + r) * f.lda + i];
  }
  // V staged in the W buffer
  for (int e = threadIdx.x; e < dc * n; e += FLUSH_NT)
  {
    const int c = e / n, i = e % n;
    Ws[c * n + i] = V[(size_t)c * f.lda + i];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  // W = Binv V in registers (warp w: rows l = lb + 4w..4w+3 of every 32-row chunk lb,
  // lanes: columns of a 128-column chunk), written over V once the chunk is complete
  for (int cb = 0; cb < n; cb += 128)
  {
    T wacc[FLUSH_MAXK / 32][4][4];
#pragma unroll
    for (int b = 0; b < FLUSH_MAXK / 32; b++)
#pragma unroll
      for (int q = 0; q < 4; q++)
#pragma unroll
        for (int j = 0; j < 4; j++)
          wacc[b][q][j] = T(0);
    for (int c = 0; c < dc; c++)
    {
      T vv[4];
#pragma unroll
      for (int j = 0; j < 4; j++)
      {
        const int i = cb + lane + 32 * j;
        vv[j]       = i < n ? Ws[c * n + i] : T(0);
      }
#pragma unroll
      for (int b = 0; b < FLUSH_MAXK / 32; b++)
#pragma unroll
        for (int q = 0; q < 4; q++)
        {
          const int l = 32 * b + wid * 4 + q;
          const T bl  = l < dc ? Bs[l * k + c] : T(0);
#pragma unroll
          for (int j = 0; j < 4; j++)
            wacc[b][q][j] += bl * vv[j];
        }
    }
    __syncthreads();
#pragma unroll
    for (int b = 0; b < FLUSH_MAXK / 32; b++)
#pragma unroll
      for (int q = 0; q < 4; q++)
      {
        const int l = 32 * b + wid * 4 + q;
        if (l < dc)
#pragma unroll
          for (int j = 0; j < 4; j++)
          {
            const int i = cb + lane + 32 * j;
            if (i < n)
              Ws[l * n + i] = wacc[b][q][j];
          }
      }
    __syncthreads();
  }
  const int rw   = wid * 8; // this warp's first row in the block
  // T1 = rows U^T - E
  for (int cb = 0; cb < dc; cb += 32)
  {
    const int c = cb + lane;
    T acc[8];
#pragma unroll
    for (int r = 0; r < 8; r++)
      acc[r] = T(0);
    if (c < dc)
      for (int i = 0; i < n; i++)
      {
        const T u = Ut[i * ldu + c];
#pragma unroll
        for (int r = 0; r < 8; r++)
          acc[r] += rows[(rw + r) * lds + i] * u;
      }
    if (c < dc)
#pragma unroll
      for (int r = 0; r < 8; r++)
        if (rw + r < nr)
          t1[(rw + r) * k + c] = (dlist[c] == r0 + rw + r) ? acc[r] - T(1) : acc[r];
  }
  __syncthreads();
  // rows -= T1 W, 8 rows x 4 columns per thread per 128-column chunk
  for (int cb = 0; cb < n; cb += 128)
  {
    T acc[8][4];
#pragma unroll
    for (int r = 0; r < 8; r++)
#pragma unroll
      for (int j = 0; j < 4; j++)
        acc[r][j] = T(0);
    for (int c = 0; c < dc; c++)
    {
      T wv[4];
#pragma unroll
      for (int j = 0; j < 4; j++)
      {
        const int i = cb + lane + 32 * j;
        wv[j]       = i < n ? Ws[c * n + i] : T(0);
      }
#pragma unroll
      for (int r = 0; r < 8; r++)
      {
        const T t = t1[(rw + r) * k + c];
#pragma unroll
        for (int j = 0; j < 4; j++)
          acc[r][j] += t * wv[j];
      }
    }
#pragma unroll
    for (int r = 0; r < 8; r++)
      if (rw + r < nr)
#pragma unroll
        for (int j = 0; j < 4; j++)
        {
          const int i = cb + lane + 32 * j;
          if (i < n)
            A[(size_t)(r0 + rw + r) * f.lda + i] = rows[(rw + r) * lds + i] - acc[r][j];
        }
  }
}

template<typename T>
bool flush_fused_fits(int n, int k)
{
  return flush_fused_smem<T>(n, k) <= 200 * 1024 && k <= FLUSH_MAXK;
}

template<typename T>
cudaError_t setup_flush_fused()
{
  return cudaFuncSetAttribute(flush_fused_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
}

template<typename T>
cudaError_t launch_flush_fused(const FlushArgs<T>& f, cudaStream_t st)
{
  if (f.dc <= 0 || f.nw <= 0)
    return cudaSuccess;
  const size_t sm = flush_fused_smem<T>(f.n, f.k);
  if (sm > 200 * 1024 || f.k > FLUSH_MAXK)
    return launch_flush_args(f, st);
  dim3 grid(f.nw, (f.n + FLUSH_R - 1) / FLUSH_R);
  flush_fused_kernel<T><<<grid, FLUSH_NT, sm, st>>>(f);
  return cudaGetLastError();
}

template bool flush_fused_fits<float>(int, int);
template bool flush_fused_fits<double>(int, int);
template cudaError_t setup_flush_fused<float>();
template cudaError_t setup_flush_fused<double>();
template cudaError_t launch_flush_fused<float>(const FlushArgs<float>&, cudaStream_t);
template cudaError_t launch_flush_fused<double>(const FlushArgs<double>&, cudaStream_t);

} // namespace qmcg
