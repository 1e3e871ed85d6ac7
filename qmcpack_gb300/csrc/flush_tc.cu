// Delayed-update flush on the 5th-generation tensor cores (tcgen05, kind::tf32):
//   T1 = Ainv[rows] U^T            (128 x k,   K = n)   -> TMEM columns [0, 32..64)
//   P  = (T1 - E) W,  W = Binv V   (128 x n,   K = k)   -> TMEM columns [64, 64+n)
//   Ainv[rows] -= P
// DelayedUpdateBatched::mw_updateInvMat (DelayedUpdateBatched.h:675-738) for one
// walker and a block of 128 inverse rows per CTA.  Operands are staged in shared
// memory in the no-swizzle K-major core-matrix layout (8 rows x 16 bytes per core
// matrix), the MMAs are issued by one thread, accumulate in TMEM and are read
// back with tcgen05.ld for the epilogue.
//
// Split precision (3xTF32): every FP32 operand x is split as hi = rna_tf32(x),
// lo = x - hi, and each product is accumulated as hi*hi + hi*lo + lo*hi in FP32,
// which keeps the flush close to FP32 accuracy; with one term (TF32) the products
// carry the 2^-11 relative error of TF32.
//
// Every wait on an mbarrier is bounded; on timeout the CTA records an error in
// *err, skips its epilogue, frees its TMEM and returns.
#include <cstdint>

#include "common.cuh"
#include "launch.h"
#include "tc.cuh"

namespace qmcg
{

constexpr int TC_M     = 128; // rows per CTA (TMEM lanes)
constexpr int TC_NT    = 128; // 4 warps: warp w owns TMEM lanes 32w..32w+31
constexpr int TC_KC    = 64;  // K chunk of the first product
// TMEM columns allocated: T1 in [0, 32), P in [64, 64 + n_pad); a power of two
__host__ __device__ constexpr int tc_cols(int npad) { return 64 + npad <= 256 ? 256 : 512; }
// byte offset of element (r, k) of an R x KC tile in the K-major core-matrix layout
__device__ __forceinline__ uint32_t cm_off(int r, int k, int kc)
{
  return (uint32_t)(((r >> 3) * (kc >> 2) + (k >> 2)) * 128 + (r & 7) * 16 + (k & 3) * 4);
}

// shared-memory matrix descriptor: no swizzle, K-major, LBO = 128 B (next core
// matrix along K), SBO = (kc/4)*128 B (next 8-row group), descriptor version 1
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, int kc)
{
  const uint64_t lbo = 128 >> 4;
  const uint64_t sbo = (uint64_t)((kc >> 2) * 128) >> 4;
  return (uint64_t)((saddr >> 4) & 0x3FFF) | (lbo << 16) | (sbo << 32) | (1ull << 46);
}

// instruction descriptor: kind::tf32, FP32 accumulate, both operands K-major
__host__ __device__ constexpr uint32_t idesc_tf32(int m, int n)
{
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ float tf32_hi(float x)
{
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, int accum)
{
  asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
               "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
               "l"(a), "l"(b), "r"(idesc), "r"(accum)
               : "memory");
}

// shared memory plan (bytes), all tiles 1024-byte aligned
struct TcPlan
{
  int n, k1, kc;   // n = orbitals, k1 = delay rank padded to 32, kc = K chunk
  uint32_t a_hi, a_lo, b_hi, b_lo; // first product: 128 x kc and k1 x kc tiles
  uint32_t a2_hi, a2_lo, w_hi, w_lo; // second product: 128 x k1 and n_pad x k1 tiles
  uint32_t v, binv, dl, bar, tslot, total;
  int npad;        // n padded to 16 (N of the second product)
};

__host__ __device__ inline TcPlan tc_plan(int n, int k)
{
  TcPlan p;
  p.n     = n;
  p.k1    = ((k + 31) / 32) * 32;
  p.kc    = TC_KC;
  p.npad  = ((n + 15) / 16) * 16;
  auto al = [](uint32_t x) { return (x + 1023u) & ~1023u; };
  uint32_t o = 0;
  p.a_hi  = o; o = al(o + TC_M * p.kc * 4);
  p.a_lo  = o; o = al(o + TC_M * p.kc * 4);
  p.b_hi  = o; o = al(o + p.k1 * p.kc * 4);
  p.b_lo  = o; o = al(o + p.k1 * p.kc * 4);
  // the second product reuses the first product's region
  uint32_t o2 = 0;
  p.a2_hi = o2; o2 = al(o2 + TC_M * p.k1 * 4);
  p.a2_lo = o2; o2 = al(o2 + TC_M * p.k1 * 4);
  p.w_hi  = o2; o2 = al(o2 + p.npad * p.k1 * 4);
  p.w_lo  = o2; o2 = al(o2 + p.npad * p.k1 * 4);
  o = o > o2 ? o : o2;
  p.v     = o; o = al(o + k * n * 4);
  p.binv  = o; o = al(o + k * k * 4);
  p.dl    = o; o = al(o + k * 4);
  p.bar   = o; o += 16;
  p.tslot = o; o += 16;
  p.total = al(o);
  return p;
}

template<int TERMS>
__global__ void __launch_bounds__(TC_NT, 2) flush_tc_kernel(FlushArgs<float> f, int* err)
{
  extern __shared__ __align__(1024) unsigned char sm[];
  const TcPlan P = tc_plan(f.n, f.k);
  const int n = f.n, k = f.k, dc = f.dc, lda = f.lda;
  const int iw = blockIdx.x, r0 = blockIdx.y * TC_M;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  float* A             = f.ainv + (size_t)iw * f.sA;
  const float* U       = f.u + (size_t)iw * f.sU;
  const float* V       = f.v + (size_t)iw * f.sU;
  const float* Binv    = f.binv + (size_t)iw * f.sB;
  const int* dlist     = f.delay_list + (size_t)iw * f.sD;
  float* Vs            = reinterpret_cast<float*>(sm + P.v);
  float* Bs            = reinterpret_cast<float*>(sm + P.binv);
  int* dls             = reinterpret_cast<int*>(sm + P.dl);
  const uint32_t bar   = smem_u32(sm + P.bar);
  uint32_t* tslot      = reinterpret_cast<uint32_t*>(sm + P.tslot);
  __shared__ int s_fail;

  if (tid == 0)
  {
    s_fail = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  const int cols = tc_cols(P.npad);
  if (warp == 0)
  {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(tslot)),
                 "r"(cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  for (int e = tid; e < dc * n; e += TC_NT)
    Vs[e] = V[(size_t)(e / n) * lda + (e % n)];
  for (int e = tid; e < dc * dc; e += TC_NT)
    Bs[e] = Binv[(size_t)(e / dc) * k + (e % dc)];
  for (int e = tid; e < dc; e += TC_NT)
    dls[e] = dlist[e];
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = *tslot;
  const uint32_t d1   = tmem;      // columns [0, k1)
  const uint32_t d2   = tmem + 64; // columns [64, 64 + npad)
  uint32_t phase      = 0;
  bool ok             = true;

  // ---------------- T1 = Ainv[rows] U^T, K in chunks of kc.  The next chunk's
  // global loads are issued before waiting for the current chunk's MMAs.
  constexpr int AV = TC_M * (TC_KC / 4) / TC_NT; // float4 of the Ainv chunk per thread (16)
  const int nchunks = (n + P.kc - 1) / P.kc;
  const int ub      = P.k1 * (P.kc / 4);         // float4 of the U chunk (all threads)
  float4 ra[AV];
  float4 ru[(32 * (TC_KC / 4) + TC_NT - 1) / TC_NT * 2];
  // slot e of a (rows x kc) tile: 8 consecutive slots are the 8 rows of one core
  // matrix (conflict-free 16-byte shared stores), 32 consecutive slots cover 64
  // contiguous bytes of 8 rows (full global sectors)
  auto slot_row = [](int e) { return (e / (8 * (TC_KC / 4))) * 8 + (e & 7); };
  auto slot_col = [](int e) { return ((e >> 3) % (TC_KC / 4)) * 4; };
  auto load_chunk = [&](int ch) {
    const int k0 = ch * P.kc;
#pragma unroll
    for (int q = 0; q < AV; q++)
    {
      const int e = tid + q * TC_NT;
      const int r = slot_row(e), c4 = slot_col(e);
      const int gr = r0 + r, gc = k0 + c4;
      ra[q] = (gr < n && gc < n) ? *reinterpret_cast<const float4*>(A + (size_t)gr * lda + gc)
                                 : make_float4(0.f, 0.f, 0.f, 0.f);
    }
#pragma unroll
    for (int q = 0; q < (int)(sizeof(ru) / sizeof(float4)); q++)
    {
      const int e = tid + q * TC_NT;
      const int r = slot_row(e), c4 = slot_col(e);
      const int gc = k0 + c4;
      ru[q] = (e < ub && r < dc && gc < n) ? *reinterpret_cast<const float4*>(U + (size_t)r * lda + gc)
                                           : make_float4(0.f, 0.f, 0.f, 0.f);
    }
  };
  auto split_store = [&](float4 x, uint32_t hi_base, uint32_t lo_base, uint32_t off) {
    float4 h = make_float4(tf32_hi(x.x), tf32_hi(x.y), tf32_hi(x.z), tf32_hi(x.w));
    *reinterpret_cast<float4*>(sm + hi_base + off) = h;
    if (TERMS > 1)
      *reinterpret_cast<float4*>(sm + lo_base + off) = make_float4(x.x - h.x, x.y - h.y, x.z - h.z, x.w - h.w);
  };
  load_chunk(0);
  for (int ch = 0; ch < nchunks && ok; ch++)
  {
#pragma unroll
    for (int q = 0; q < AV; q++)
    {
      const int e = tid + q * TC_NT;
      split_store(ra[q], P.a_hi, P.a_lo, cm_off(slot_row(e), slot_col(e), P.kc));
    }
#pragma unroll
    for (int q = 0; q < (int)(sizeof(ru) / sizeof(float4)); q++)
    {
      const int e = tid + q * TC_NT;
      if (e < ub)
        split_store(ru[q], P.b_hi, P.b_lo, cm_off(slot_row(e), slot_col(e), P.kc));
    }
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (tid == 0)
    {
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      const uint32_t idesc = idesc_tf32(TC_M, P.k1);
      const uint32_t ah = smem_u32(sm + P.a_hi), al = smem_u32(sm + P.a_lo);
      const uint32_t bh = smem_u32(sm + P.b_hi), bl = smem_u32(sm + P.b_lo);
      for (int ks = 0; ks < P.kc / 8; ks++)
      {
        const uint32_t adv = ks * 256; // two core matrices along K per k-step of 8
        const int first    = (ch == 0 && ks == 0);
        mma_tf32(d1, smem_desc(ah + adv, P.kc), smem_desc(bh + adv, P.kc), idesc, first ? 0 : 1);
        if (TERMS > 1)
        {
          mma_tf32(d1, smem_desc(ah + adv, P.kc), smem_desc(bl + adv, P.kc), idesc, 1);
          mma_tf32(d1, smem_desc(al + adv, P.kc), smem_desc(bh + adv, P.kc), idesc, 1);
        }
      }
      mma_commit(bar);
    }
    if (ch + 1 < nchunks)
      load_chunk(ch + 1);
    if (!mbar_wait(bar, phase))
      ok = false;
    phase ^= 1;
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    __syncthreads();
  }

  if (ok)
  {
    // ---------------- W = Binv V, stored transposed (n_pad rows x k1) for the second product
    for (int i = tid; i < P.npad; i += TC_NT)
    {
      float vcol[32];
#pragma unroll
      for (int l = 0; l < 32; l++)
        vcol[l] = (l < dc && i < n) ? Vs[l * n + i] : 0.f;
      for (int c4 = 0; c4 < P.k1; c4 += 4)
      {
        float w[4];
#pragma unroll
        for (int q = 0; q < 4; q++)
        {
          const int c = c4 + q;
          float a     = 0.f;
          if (c < dc)
#pragma unroll
            for (int l = 0; l < 32; l++)
              if (l < dc)
                a += Bs[c * dc + l] * vcol[l];
          w[q] = a;
        }
        float4 h = make_float4(tf32_hi(w[0]), tf32_hi(w[1]), tf32_hi(w[2]), tf32_hi(w[3]));
        float4 lo = make_float4(w[0] - h.x, w[1] - h.y, w[2] - h.z, w[3] - h.w);
        const uint32_t off = cm_off(i, c4, P.k1);
        *reinterpret_cast<float4*>(sm + P.w_hi + off) = h;
        if (TERMS > 1)
          *reinterpret_cast<float4*>(sm + P.w_lo + off) = lo;
      }
    }
    // ---------------- T1 - E from TMEM into the second product's A tile
    {
      const int r = warp * 32 + lane; // this thread's TMEM lane = block row
      for (int c0 = 0; c0 < P.k1; c0 += 32)
      {
        float t[32];
        tmem_ld32(d1 + ((uint32_t)(warp * 32) << 16) + c0, t);
#pragma unroll
        for (int q = 0; q < 32; q++)
        {
          const int c = c0 + q;
          if (c >= dc)
            t[q] = 0.f;
          else if (dls[c] == r0 + r)
            t[q] -= 1.f;
        }
#pragma unroll
        for (int q = 0; q < 32; q += 4)
        {
          float4 h = make_float4(tf32_hi(t[q]), tf32_hi(t[q + 1]), tf32_hi(t[q + 2]), tf32_hi(t[q + 3]));
          float4 lo = make_float4(t[q] - h.x, t[q + 1] - h.y, t[q + 2] - h.z, t[q + 3] - h.w);
          const uint32_t off = cm_off(r, c0 + q, P.k1);
          *reinterpret_cast<float4*>(sm + P.a2_hi + off) = h;
          if (TERMS > 1)
            *reinterpret_cast<float4*>(sm + P.a2_lo + off) = lo;
        }
      }
    }
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    // ---------------- P = (T1 - E) W
    if (tid == 0)
    {
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      const uint32_t idesc = idesc_tf32(TC_M, P.npad);
      const uint32_t ah = smem_u32(sm + P.a2_hi), al = smem_u32(sm + P.a2_lo);
      const uint32_t bh = smem_u32(sm + P.w_hi), bl = smem_u32(sm + P.w_lo);
      for (int ks = 0; ks < P.k1 / 8; ks++)
      {
        const uint32_t adv = ks * 256;
        mma_tf32(d2, smem_desc(ah + adv, P.k1), smem_desc(bh + adv, P.k1), idesc, ks ? 1 : 0);
        if (TERMS > 1)
        {
          mma_tf32(d2, smem_desc(ah + adv, P.k1), smem_desc(bl + adv, P.k1), idesc, 1);
          mma_tf32(d2, smem_desc(al + adv, P.k1), smem_desc(bh + adv, P.k1), idesc, 1);
        }
      }
      mma_commit(bar);
    }
    if (!mbar_wait(bar, phase))
      ok = false;
    phase ^= 1;
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    __syncthreads();
  }

  if (ok)
  {
    // ---------------- epilogue: Ainv[rows] -= P, each thread one row; the next
    // 32-column piece of the row is loaded while the current one is written
    const int r  = warp * 32 + lane;
    const int gr = r0 + r;
    float* row   = A + (size_t)(gr < n ? gr : 0) * lda;
    float4 cur[8], nxt[8];
#pragma unroll
    for (int q = 0; q < 8; q++)
      cur[q] = (gr < n && 4 * q < n) ? *reinterpret_cast<const float4*>(row + 4 * q) : make_float4(0.f, 0.f, 0.f, 0.f);
    for (int c0 = 0; c0 < P.npad; c0 += 32)
    {
#pragma unroll
      for (int q = 0; q < 8; q++)
      {
        const int c = c0 + 32 + 4 * q;
        nxt[q] = (gr < n && c < n) ? *reinterpret_cast<const float4*>(row + c) : make_float4(0.f, 0.f, 0.f, 0.f);
      }
      float p[32];
      tmem_ld32(d2 + ((uint32_t)(warp * 32) << 16) + c0, p);
      if (gr < n)
      {
#pragma unroll
        for (int q = 0; q < 8; q++)
          if (c0 + 4 * q < n)
          {
            float4 a = cur[q];
            a.x -= p[4 * q];
            a.y -= p[4 * q + 1];
            a.z -= p[4 * q + 2];
            a.w -= p[4 * q + 3];
            *reinterpret_cast<float4*>(row + c0 + 4 * q) = a;
          }
      }
#pragma unroll
      for (int q = 0; q < 8; q++)
        cur[q] = nxt[q];
    }
  }
  else if (tid == 0)
    atomicExch(err, 1);

  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(cols) : "memory");
}

// ---------------------------------------------------------------------------
// N-tiled variant for large determinants and delay ranks up to 64: the second
// product runs over column tiles of TN inverse columns, W = Binv V is formed
// per tile from global V, so neither N nor k is bounded by TMEM or by a full V in
// shared memory.  TMEM: T1 in columns [0, KM), the product tile in [KM, KM + TN).
// Two instances: delay ranks up to 64 with 128-column tiles (256 TMEM columns, one CTA
// per SM by shared memory), and delay ranks up to 32 with 96-column tiles (128 TMEM
// columns and 70 KB of shared memory: three CTAs per SM).
// ---------------------------------------------------------------------------
constexpr int TT_KC = 32;  // K chunk of the first product
constexpr int TT_KMAX = 64;

struct TtPlan
{
  int k1;                    // delay rank padded to 16
  uint32_t a_hi, a_lo, u_hi, u_lo; // first product: 128 x KC and k1 x KC
  uint32_t a2_hi, a2_lo, w_hi, w_lo; // second product: 128 x k1 and TN x k1
  uint32_t binv, dl, bar, total;
};

__host__ __device__ inline TtPlan tt_plan(int k, int TN)
{
  TtPlan p;
  p.k1    = ((k + 15) / 16) * 16;
  auto al = [](uint32_t x) { return (x + 1023u) & ~1023u; };
  uint32_t o = 0;
  p.a_hi  = o; o = al(o + TC_M * TT_KC * 4);
  p.a_lo  = o; o = al(o + TC_M * TT_KC * 4);
  p.u_hi  = o; o = al(o + p.k1 * TT_KC * 4);
  p.u_lo  = o; o = al(o + p.k1 * TT_KC * 4);
  uint32_t o2 = 0;
  p.a2_hi = o2; o2 = al(o2 + TC_M * p.k1 * 4);
  p.a2_lo = o2; o2 = al(o2 + TC_M * p.k1 * 4);
  p.w_hi  = o2; o2 = al(o2 + TN * p.k1 * 4);
  p.w_lo  = o2; o2 = al(o2 + TN * p.k1 * 4);
  o = o > o2 ? o : o2;
  p.binv  = o; o = al(o + k * k * 4);
  p.dl    = o; o = al(o + k * 4);
  p.bar   = o; o += 16;
  p.total = al(o);
  return p;
}

template<int TERMS, int TN, int KM, int MINB>
__global__ void __launch_bounds__(TC_NT, MINB) flush_tc_tiled_kernel(FlushArgs<float> f, int* err)
{
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ uint32_t s_tmem;
  __shared__ int s_fail;
  constexpr int TMC = (KM + TN <= 128) ? 128 : 256; // TMEM columns allocated
  const TtPlan P = tt_plan(f.k, TN);
  const int n = f.n, k = f.k, dc = f.dc, lda = f.lda, k1 = P.k1;
  const int iw = blockIdx.x, r0 = blockIdx.y * TC_M;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  float* A         = f.ainv + (size_t)iw * f.sA;
  const float* U   = f.u + (size_t)iw * f.sU;
  const float* V   = f.v + (size_t)iw * f.sU;
  const float* Bi  = f.binv + (size_t)iw * f.sB;
  const int* dlist = f.delay_list + (size_t)iw * f.sD;
  float* Bs        = reinterpret_cast<float*>(sm + P.binv);
  int* dls         = reinterpret_cast<int*>(sm + P.dl);
  const uint32_t bar = smem_u32(sm + P.bar);
  if (tid == 0)
  {
    s_fail = 0;
    mbar_init(bar);
  }
  if (warp == 0)
    tmem_alloc(smem_u32(&s_tmem), TMC);
  for (int e = tid; e < dc * dc; e += TC_NT)
    Bs[e] = Bi[(size_t)(e / dc) * k + (e % dc)];
  for (int e = tid; e < dc; e += TC_NT)
    dls[e] = dlist[e];
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = s_tmem;
  const uint32_t d1 = tmem, d2 = tmem + KM;
  uint32_t phase = 0;
  auto split_store = [&](float4 x, uint32_t hi_base, uint32_t lo_base, uint32_t off) {
    const float4 h = make_float4(tf32_hi(x.x), tf32_hi(x.y), tf32_hi(x.z), tf32_hi(x.w));
    *reinterpret_cast<float4*>(sm + hi_base + off) = h;
    if (TERMS > 1)
      *reinterpret_cast<float4*>(sm + lo_base + off) = make_float4(x.x - h.x, x.y - h.y, x.z - h.z, x.w - h.w);
  };
  auto wait_mma = [&]() {
    if (!mbar_wait(bar, phase))
      atomicExch(&s_fail, 1);
    phase ^= 1;
    tc_fence_after();
    __syncthreads();
    return s_fail == 0;
  };
  // slot e of a (rows x KC) chunk: 8 consecutive slots fill one core matrix
  auto slot_row = [](int e) { return (e / (8 * (TT_KC / 4))) * 8 + (e & 7); };
  auto slot_col = [](int e) { return ((e >> 3) % (TT_KC / 4)) * 4; };
  bool ok = true;

  // ---------------- T1 = Ainv[rows] U^T over K = n in chunks of KC
  constexpr int AV = TC_M * (TT_KC / 4) / TC_NT; // 8 float4 per thread
  const int ub = k1 * (TT_KC / 4);
  for (int k0 = 0; k0 < n && ok; k0 += TT_KC)
  {
#pragma unroll
    for (int q = 0; q < AV; q++)
    {
      const int e = tid + q * TC_NT, r = slot_row(e), c4 = slot_col(e);
      const int gr = r0 + r, gc = k0 + c4;
      const float4 x = (gr < n && gc < n) ? *reinterpret_cast<const float4*>(A + (size_t)gr * lda + gc)
                                          : make_float4(0.f, 0.f, 0.f, 0.f);
      split_store(x, P.a_hi, P.a_lo, cm_off(r, c4, TT_KC));
    }
    for (int e = tid; e < ub; e += TC_NT)
    {
      const int r = slot_row(e), c4 = slot_col(e), gc = k0 + c4;
      const float4 x = (r < dc && gc < n) ? *reinterpret_cast<const float4*>(U + (size_t)r * lda + gc)
                                          : make_float4(0.f, 0.f, 0.f, 0.f);
      split_store(x, P.u_hi, P.u_lo, cm_off(r, c4, TT_KC));
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    if (tid == 0)
    {
      tc_fence_after();
      const uint32_t id = idesc_tf32(TC_M, k1);
      const uint32_t ah = smem_u32(sm + P.a_hi), al = smem_u32(sm + P.a_lo);
      const uint32_t bh = smem_u32(sm + P.u_hi), bl = smem_u32(sm + P.u_lo);
      for (int ks = 0; ks < TT_KC / 8; ks++)
      {
        const uint32_t adv = ks * 256;
        mma_tf32(d1, smem_desc(ah + adv, TT_KC), smem_desc(bh + adv, TT_KC), id, (k0 == 0 && ks == 0) ? 0 : 1);
        if (TERMS > 1)
        {
          mma_tf32(d1, smem_desc(ah + adv, TT_KC), smem_desc(bl + adv, TT_KC), id, 1);
          mma_tf32(d1, smem_desc(al + adv, TT_KC), smem_desc(bh + adv, TT_KC), id, 1);
        }
      }
      mma_commit(bar);
    }
    ok = wait_mma();
  }

  // ---------------- (T1 - E) from TMEM into the second product's A operand
  if (ok)
  {
    const int r = warp * 32 + lane;
    for (int c0 = 0; c0 < k1; c0 += 32)
    {
      float t[32];
      tmem_ld32(d1 + ((uint32_t)(warp * 32) << 16) + c0, t);
#pragma unroll
      for (int q = 0; q < 32; q += 4)
        if (c0 + q < k1)
        {
          float v[4];
#pragma unroll
          for (int u = 0; u < 4; u++)
          {
            const int c = c0 + q + u;
            float x     = t[q + u];
            if (c >= dc)
              x = 0.f;
            else if (dls[c] == r0 + r)
              x -= 1.f;
            v[u] = x;
          }
          split_store(make_float4(v[0], v[1], v[2], v[3]), P.a2_hi, P.a2_lo, cm_off(r, c0 + q, k1));
        }
    }
  }
  // ---------------- column tiles: W_tile = Binv V[:, tile], P_tile = (T1 - E) W_tile^T, Ainv -= P
  for (int t0 = 0; t0 < n && ok; t0 += TN)
  {
    if (tid < TN)
    {
      // thread i owns column t0 + i of the tile
      const int i = tid;
      const int col = t0 + i;
      float vcol[KM];
#pragma unroll
      for (int l = 0; l < KM; l++)
        vcol[l] = (l < dc && col < n) ? V[(size_t)l * lda + col] : 0.f;
      for (int c4 = 0; c4 < k1; c4 += 4)
      {
        float w[4];
#pragma unroll
        for (int q = 0; q < 4; q++)
        {
          const int c = c4 + q;
          float a     = 0.f;
          if (c < dc)
#pragma unroll
            for (int l = 0; l < KM; l++)
              if (l < dc)
                a += Bs[c * dc + l] * vcol[l];
          w[q] = a;
        }
        split_store(make_float4(w[0], w[1], w[2], w[3]), P.w_hi, P.w_lo, cm_off(i, c4, k1));
      }
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    if (tid == 0)
    {
      tc_fence_after();
      const uint32_t id = idesc_tf32(TC_M, TN);
      const uint32_t ah = smem_u32(sm + P.a2_hi), al = smem_u32(sm + P.a2_lo);
      const uint32_t bh = smem_u32(sm + P.w_hi), bl = smem_u32(sm + P.w_lo);
      for (int ks = 0; ks < k1 / 8; ks++)
      {
        const uint32_t adv = ks * 256;
        mma_tf32(d2, smem_desc(ah + adv, k1), smem_desc(bh + adv, k1), id, ks ? 1 : 0);
        if (TERMS > 1)
        {
          mma_tf32(d2, smem_desc(ah + adv, k1), smem_desc(bl + adv, k1), id, 1);
          mma_tf32(d2, smem_desc(al + adv, k1), smem_desc(bh + adv, k1), id, 1);
        }
      }
      mma_commit(bar);
    }
    ok = wait_mma();
    if (!ok)
      break;
    // epilogue: each thread one inverse row, 32 columns at a time
    const int r  = warp * 32 + lane;
    const int gr = r0 + r;
    float* row   = A + (size_t)(gr < n ? gr : 0) * lda + t0;
    for (int c0 = 0; c0 < TN; c0 += 32)
    {
      float p[32];
      tmem_ld32(d2 + ((uint32_t)(warp * 32) << 16) + c0, p);
      if (gr < n)
#pragma unroll
        for (int q = 0; q < 8; q++)
          if (t0 + c0 + 4 * q < n)
          {
            float4 a = *reinterpret_cast<const float4*>(row + c0 + 4 * q);
            a.x -= p[4 * q];
            a.y -= p[4 * q + 1];
            a.z -= p[4 * q + 2];
            a.w -= p[4 * q + 3];
            *reinterpret_cast<float4*>(row + c0 + 4 * q) = a;
          }
    }
    tc_fence_before();
    __syncthreads();
  }
  if (!ok && tid == 0)
    atomicExch(err, 1);
  tc_fence_before();
  __syncthreads();
  if (warp == 0)
    tmem_dealloc(tmem, TMC);
}

// the compact kernel: whole product in TMEM, k <= 32, and the second product is one
// MMA whose N = n_pad must not exceed 256 (the largest N of tcgen05.mma with M = 128)
static bool flush_tc_compact_ok(int n, int k)
{
  const TcPlan p = tc_plan(n, k);
  return k <= 32 && p.npad <= 256 && p.total <= 200 * 1024;
}

bool flush_tc_supported(int n, int k, int lda)
{
  // 16-byte aligned rows; delay rank up to 64 (the tiled kernels cover any N)
  return k >= 1 && k <= TT_KMAX && (lda % 4) == 0 && (n % 4) == 0 && tt_plan(k, 128).total <= 200 * 1024;
}

#define QMCG_TILED_BIG(TERMS) flush_tc_tiled_kernel<TERMS, 128, 64, 1>
#define QMCG_TILED_SMALL(TERMS) flush_tc_tiled_kernel<TERMS, 96, 32, 3>

cudaError_t setup_flush_tc()
{
  cudaError_t e = cudaFuncSetAttribute(flush_tc_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(flush_tc_kernel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(QMCG_TILED_BIG(1), cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(QMCG_TILED_BIG(3), cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(QMCG_TILED_SMALL(1), cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(QMCG_TILED_SMALL(3), cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  return e;
}

// which kernel flushes a shape: 0 one-pass, 1 tiled (k <= 32, 96-column tiles), 2 tiled (k <= 64)
int flush_tc_variant(int n, int k)
{
  if (flush_tc_compact_ok(n, k))
    return 0;
  if (k <= 32)
    return 1;
  return 2;
}

cudaError_t launch_flush_tc(const FlushArgs<float>& f, int terms, int* err, cudaStream_t st)
{
  if (f.dc <= 0 || f.nw <= 0)
    return cudaSuccess;
  dim3 grid(f.nw, (f.n + TC_M - 1) / TC_M);
  const int v = flush_tc_variant(f.n, f.k);
  if (v == 0 && flush_tc_compact_ok(f.n, f.k))
  {
    const TcPlan p = tc_plan(f.n, f.k);
    if (terms == 1)
      flush_tc_kernel<1><<<grid, TC_NT, p.total, st>>>(f, err);
    else
      flush_tc_kernel<3><<<grid, TC_NT, p.total, st>>>(f, err);
  }
  else if (v == 1)
  {
    const TtPlan p = tt_plan(f.k, 96);
    if (terms == 1)
      QMCG_TILED_SMALL(1)<<<grid, TC_NT, p.total, st>>>(f, err);
    else
      QMCG_TILED_SMALL(3)<<<grid, TC_NT, p.total, st>>>(f, err);
  }
  else
  {
    if (f.k > TT_KMAX)
      return cudaErrorInvalidValue;
    const TtPlan p = tt_plan(f.k, 128);
    if (terms == 1)
      QMCG_TILED_BIG(1)<<<grid, TC_NT, p.total, st>>>(f, err);
    else
      QMCG_TILED_BIG(3)<<<grid, TC_NT, p.total, st>>>(f, err);
  }
  return cudaGetLastError();
}

} // namespace qmcg
