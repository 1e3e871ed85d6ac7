// Delayed-update flush on the 5th-generation tensor cores (tcgen05, kind::tf32):
//   T1 = Ainv[rows] U^T            (128 x k,   K = n)   -> TMEM columns [0, k1)
//   X  = (T1 - E) Binv             (128 x k,   K = k)   -> TMEM columns [0, k1)
//   P  = X V                       (128 x n,   K = k)   -> TMEM columns [64, 64+n) (one-pass)
//   Ainv[rows] -= P
// DelayedUpdateBatched::mw_updateInvMat (DelayedUpdateBatched.h:675-738) for one
// walker and a block of 128 inverse rows per CTA.  Operands are staged in shared
// memory in the no-swizzle K-major core-matrix layout (8 rows x 16 bytes per core
// matrix), the MMAs are issued by one thread, accumulate in TMEM and are read
// back with tcgen05.ld for the epilogue.
//
// Split precision (3xTF32): every FP32 operand x is split as hi = rna_tf32(x),
// lo = x - hi, and each product is accumulated as hi*hi + hi*lo + lo*hi, which keeps
// the flush close to FP32 accuracy; the first product's K chunks are summed in FP32
// outside the tensor core.  With one term (TF32) the products carry the 2^-11
// relative error of TF32.
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
// TMEM columns allocated: T1 and X in [0, 32), P in [64, 64 + n_pad); a power of two
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
  uint32_t a_hi, a_lo, b_hi, b_lo;   // first product: 128 x kc and k1 x kc tiles
  uint32_t a2_hi, a2_lo, w_hi, w_lo; // later products: 128 x k1 (T1 - E, then X) and n_pad x k1 (V^T)
  uint32_t v, bt_hi, bt_lo;          // V (k x n) as stored; Binv^T (k1 x k1) over it once V^T is formed
  uint32_t dl, bar, tslot, total;
  int npad;        // n padded to 16 (N of the last product)
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
  // the later products reuse the first product's region
  uint32_t o2 = 0;
  p.a2_hi = o2; o2 = al(o2 + TC_M * p.k1 * 4);
  p.a2_lo = o2; o2 = al(o2 + TC_M * p.k1 * 4);
  p.w_hi  = o2; o2 = al(o2 + p.npad * p.k1 * 4);
  p.w_lo  = o2; o2 = al(o2 + p.npad * p.k1 * 4);
  o = o > o2 ? o : o2;
  p.v     = o;
  p.bt_hi = o;
  p.bt_lo = al(o + p.k1 * p.k1 * 4);
  const uint32_t vend = al(o + k * n * 4), btend = al(p.bt_lo + p.k1 * p.k1 * 4);
  o = vend > btend ? vend : btend;
  p.dl    = o; o = al(o + k * 4);
  p.bar   = o; o += 16;
  p.tslot = o; o += 16;
  p.total = al(o);
  return p;
}

// Binv^T into a (k1 x k1) K-major operand tile: element (l, c) = Binv[c][l], zero
// outside dc x dc; consecutive threads take consecutive rows l
template<int TERMS>
__device__ __forceinline__ void stage_binv_t(unsigned char* sm, uint32_t hi, uint32_t lo, const float* Binv, int k,
                                             int dc, int k1, int tid)
{
  for (int e = tid; e < k1 * (k1 / 4); e += TC_NT)
  {
    const int l = e % k1, c4 = (e / k1) * 4;
    float x[4];
#pragma unroll
    for (int q = 0; q < 4; q++)
      x[q] = (c4 + q < dc && l < dc) ? Binv[(size_t)(c4 + q) * k + l] : 0.f;
    const float4 h = make_float4(tf32_hi(x[0]), tf32_hi(x[1]), tf32_hi(x[2]), tf32_hi(x[3]));
    const uint32_t off = cm_off(l, c4, k1);
    *reinterpret_cast<float4*>(sm + hi + off) = h;
    if (TERMS > 1)
      *reinterpret_cast<float4*>(sm + lo + off) = make_float4(x[0] - h.x, x[1] - h.y, x[2] - h.z, x[3] - h.w);
  }
}

// the three-term (or one-term) product D = A B^T over K = k1 from two K-major tiles
// with row pitch k1, issued by one thread
template<int TERMS>
__device__ __forceinline__ void mma_k1(uint32_t d, unsigned char* sm, uint32_t a_hi, uint32_t a_lo, uint32_t b_hi,
                                       uint32_t b_lo, int k1, uint32_t idesc)
{
  const uint32_t ah = smem_u32(sm + a_hi), al = smem_u32(sm + a_lo);
  const uint32_t bh = smem_u32(sm + b_hi), bl = smem_u32(sm + b_lo);
  for (int ks = 0; ks < k1 / 8; ks++)
  {
    const uint32_t adv = ks * 256; // two core matrices along K per k-step of 8
    mma_tf32(d, smem_desc(ah + adv, k1), smem_desc(bh + adv, k1), idesc, ks ? 1 : 0);
    if (TERMS > 1)
    {
      mma_tf32(d, smem_desc(ah + adv, k1), smem_desc(bl + adv, k1), idesc, 1);
      mma_tf32(d, smem_desc(al + adv, k1), smem_desc(bh + adv, k1), idesc, 1);
    }
  }
}

// Ainv[r0 + (0..127), c_begin + [0, ncol)) -= P with P in TMEM columns [dcol, dcol + ncol),
// ncol a multiple of 32.  P passes through shared memory E (128 rows of pitch EW + 4
// floats: 16-byte stores by row and loads along a row are both conflict-free) in chunks
// of EW columns, so every global load and store of a warp covers whole 128-byte row
// segments; a chunk's loads are all issued before its first store.
template<int EW>
__device__ __forceinline__ void epilogue_rows(float* A, int lda, int n, int r0, int c_begin, int ncol, uint32_t dcol,
                                              float* E, int tid)
{
  static_assert(EW == 32 || EW == 64, "chunk of 32 or 64 columns");
  constexpr int EP = EW + 4;
  constexpr int Q  = EW / 4; // float4 per thread of a full chunk: 128 rows x EW / 4 / 128 threads
  const int warp   = tid >> 5; // this thread's TMEM lane is block row tid
  for (int c0 = 0; c0 < ncol; c0 += EW)
  {
    const int w = ncol - c0 < EW ? ncol - c0 : EW; // 32 or EW
#pragma unroll
    for (int h = 0; h < EW; h += 32)
      if (h < w)
      {
        float p[32];
        tmem_ld32(dcol + ((uint32_t)(warp * 32) << 16) + c0 + h, p);
#pragma unroll
        for (int q = 0; q < 32; q += 4)
          *reinterpret_cast<float4*>(E + tid * EP + h + q) = make_float4(p[q], p[q + 1], p[q + 2], p[q + 3]);
      }
    __syncthreads();
    const int sh = (w == 64) ? 4 : 3; // log2 of the float4 in one row of the chunk
    float4 av[Q];
#pragma unroll
    for (int q = 0; q < Q; q++)
    {
      const int e = tid + q * TC_NT, rr = e >> sh, c4 = (e & ((1 << sh) - 1)) * 4;
      const int gr = r0 + rr, gc = c_begin + c0 + c4;
      av[q] = (rr < TC_M && gr < n && gc < n) ? *reinterpret_cast<const float4*>(A + (size_t)gr * lda + gc)
                                              : make_float4(0.f, 0.f, 0.f, 0.f);
    }
#pragma unroll
    for (int q = 0; q < Q; q++)
    {
      const int e = tid + q * TC_NT, rr = e >> sh, c4 = (e & ((1 << sh) - 1)) * 4;
      const int gr = r0 + rr, gc = c_begin + c0 + c4;
      if (rr < TC_M && gr < n && gc < n)
      {
        const float4 p = *reinterpret_cast<const float4*>(E + rr * EP + c4);
        float4 a       = av[q];
        a.x -= p.x;
        a.y -= p.y;
        a.z -= p.z;
        a.w -= p.w;
        *reinterpret_cast<float4*>(A + (size_t)gr * lda + gc) = a;
      }
    }
    __syncthreads();
  }
}

// The update is evaluated as P = ((T1 - E) Binv) V: the k x k product runs on the
// tensor cores once per row block (128 x k1 x k1) instead of forming W = Binv V
// (k x k x n) on the CUDA cores in every row block; V enters the last product as
// its transpose, staged from shared memory.
template<int TERMS>
__global__ void __launch_bounds__(TC_NT, 2) flush_tc_kernel(FlushArgs<float> f, int* err)
{
  extern __shared__ __align__(1024) unsigned char sm[];
  const TcPlan P = tc_plan(f.n, f.k);
  const int n = f.n, k = f.k, dc = f.dc, lda = f.lda, k1 = P.k1;
  const int iw = blockIdx.x, r0 = blockIdx.y * TC_M;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  float* A             = f.ainv + (size_t)iw * f.sA;
  const float* U       = f.u + (size_t)iw * f.sU;
  const float* V       = f.v + (size_t)iw * f.sU;
  const float* Binv    = f.binv + (size_t)iw * f.sB;
  const int* dlist     = f.delay_list + (size_t)iw * f.sD;
  const float* Vs      = reinterpret_cast<const float*>(sm + P.v);
  int* dls             = reinterpret_cast<int*>(sm + P.dl);
  const uint32_t bar   = smem_u32(sm + P.bar);
  uint32_t* tslot      = reinterpret_cast<uint32_t*>(sm + P.tslot);
  __shared__ int s_fail;

  if (tid == 0)
  {
    s_fail = 0;
    mbar_init(bar);
  }
  const int cols = tc_cols(P.npad);
  if (warp == 0)
    tmem_alloc(smem_u32(tslot), cols);
  // V (dc x n) into shared memory with cp.async: it lands while the first product runs
  {
    const int nv4 = n >> 2;
    for (int e = tid; e < dc * nv4; e += TC_NT)
    {
      const int l = e / nv4, c4 = (e - l * nv4) * 4;
      const uint32_t sa = smem_u32(sm + P.v + (uint32_t)(l * n + c4) * 4);
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(V + (size_t)l * lda + c4) : "memory");
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
  }
  for (int e = tid; e < dc; e += TC_NT)
    dls[e] = dlist[e];
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  const uint32_t d1   = tmem;      // columns [0, k1): T1, then X
  const uint32_t d2   = tmem + 64; // columns [64, 64 + npad): P
  uint32_t phase      = 0;
  // every thread waits on the MMA barrier; a timeout anywhere stops the whole CTA
  auto wait_mma = [&]() {
    if (!mbar_wait(bar, phase))
      atomicExch(&s_fail, 1);
    phase ^= 1;
    tc_fence_after();
    __syncthreads();
    return s_fail == 0;
  };
  bool ok = true;

  // ---------------- T1 = Ainv[rows] U^T, K in chunks of kc.  The next chunk's
  // global loads are issued before waiting for the current chunk's MMAs.
  constexpr int AV = TC_M * (TC_KC / 4) / TC_NT; // float4 of the Ainv chunk per thread (16)
  const int nchunks = (n + P.kc - 1) / P.kc;
  const int ub      = k1 * (P.kc / 4);           // float4 of the U chunk (all threads)
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
  // with split precision the K chunks are summed here in FP32 (round to nearest), each
  // chunk's MMA starting from zero: the tensor core's own FP32 accumulation over all of
  // K = n would add an error growing with n
  float t1[32];
#pragma unroll
  for (int q = 0; q < 32; q++)
    t1[q] = 0.f;
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
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    if (tid == 0)
    {
      tc_fence_after();
      const uint32_t idesc = idesc_tf32(TC_M, k1);
      const uint32_t ah = smem_u32(sm + P.a_hi), al = smem_u32(sm + P.a_lo);
      const uint32_t bh = smem_u32(sm + P.b_hi), bl = smem_u32(sm + P.b_lo);
      for (int ks = 0; ks < P.kc / 8; ks++)
      {
        const uint32_t adv = ks * 256; // two core matrices along K per k-step of 8
        const int first    = TERMS > 1 ? (ks == 0) : (ch == 0 && ks == 0);
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
    ok = wait_mma();
    if (TERMS > 1 && ok)
    {
      float t[32];
      tmem_ld32(d1 + ((uint32_t)(warp * 32) << 16), t);
#pragma unroll
      for (int q = 0; q < 32; q++)
        t1[q] += t[q];
    }
  }
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");

  const int r = warp * 32 + lane; // this thread's TMEM lane = block row
  if (ok)
  {
    // ---------------- T1 - E into the A tile of the second product (k1 = 32)
    for (int c0 = 0; c0 < k1; c0 += 32)
    {
      float t[32];
      if (TERMS > 1)
      {
#pragma unroll
        for (int q = 0; q < 32; q++)
          t[q] = t1[q];
      }
      else
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
        split_store(make_float4(t[q], t[q + 1], t[q + 2], t[q + 3]), P.a2_hi, P.a2_lo, cm_off(r, c0 + q, k1));
    }
    __syncthreads(); // V has landed for every thread's copies
    // ---------------- V^T into the B tile of the last product: element (i, l) = V[l][i]
    for (int e = tid; e < P.npad * (k1 / 4); e += TC_NT)
    {
      const int i = e % P.npad, l4 = (e / P.npad) * 4;
      float x[4];
#pragma unroll
      for (int q = 0; q < 4; q++)
        x[q] = (l4 + q < dc && i < n) ? Vs[(l4 + q) * n + i] : 0.f;
      split_store(make_float4(x[0], x[1], x[2], x[3]), P.w_hi, P.w_lo, cm_off(i, l4, k1));
    }
    __syncthreads(); // V is read; Binv^T takes its place
    stage_binv_t<TERMS>(sm, P.bt_hi, P.bt_lo, Binv, k, dc, k1, tid);
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    // ---------------- X = (T1 - E) Binv into TMEM columns [0, k1)
    if (tid == 0)
    {
      tc_fence_after();
      mma_k1<TERMS>(d1, sm, P.a2_hi, P.a2_lo, P.bt_hi, P.bt_lo, k1, idesc_tf32(TC_M, k1));
      mma_commit(bar);
    }
    ok = wait_mma();
  }
  if (ok)
  {
    // ---------------- X from TMEM into the A tile of the last product
    for (int c0 = 0; c0 < k1; c0 += 32)
    {
      float t[32];
      tmem_ld32(d1 + ((uint32_t)(warp * 32) << 16) + c0, t);
#pragma unroll
      for (int q = 0; q < 32; q += 4)
        split_store(make_float4(t[q], t[q + 1], t[q + 2], t[q + 3]), P.a2_hi, P.a2_lo, cm_off(r, c0 + q, k1));
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    // ---------------- P = X V
    if (tid == 0)
    {
      tc_fence_after();
      mma_k1<TERMS>(d2, sm, P.a2_hi, P.a2_lo, P.w_hi, P.w_lo, k1, idesc_tf32(TC_M, P.npad));
      mma_commit(bar);
    }
    ok = wait_mma();
  }

  if (ok)
  {
    // ---------------- epilogue: Ainv[rows] -= P through shared memory over the
    // first product's region (every MMA has completed)
    epilogue_rows<64>(A, lda, n, r0, 0, (P.npad + 31) & ~31, d2, reinterpret_cast<float*>(sm), tid);
  }
  else if (tid == 0)
    atomicExch(err, 1);

  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(cols) : "memory");
}

// ---------------------------------------------------------------------------
// N-tiled variant for large determinants and delay ranks up to 64: X = (T1 - E) Binv
// is formed once, the last product runs over column tiles of TT_TN inverse columns with
// each V^T tile staged from global V, so neither N nor k is bounded by TMEM or by a full
// V in shared memory.
//   T1  K chunks of 32: the raw Ainv and U chunks arrive by cp.async RAW chunks ahead
//       (each thread copies and later splits the same 16-byte slots, so its own
//       wait_group makes them visible to it), are split in shared memory, and their
//       products alternate between two TMEM buffers; with split precision the previous
//       chunk's product is summed in FP32 while the next chunk's products run
//   X   one product over K = k1, Binv^T staged from a cp.async copy of Binv
//   P   column tiles: while the products of tile t run, its inverse rows and the next
//       tile's V^T values are read into registers; the product then passes through
//       shared memory (over the V^T tile) in 32-column rounds so that every global
//       access of a warp covers whole 128-byte row segments
// TMEM: buffers of 64 columns at 0 and 64 (128 allocated).  Two instances: delay ranks up
// to 64 with two raw chunks in flight (97 KB of shared memory: two CTAs per SM), and delay
// ranks up to 32 with one (61 KB: three CTAs per SM).
// ---------------------------------------------------------------------------
constexpr int TT_KC   = 32; // K chunk of the first product
constexpr int TT_TN   = 64; // columns of a product tile
constexpr int TT_KMAX = 64;
constexpr int TT_TMC  = 128;
constexpr int TT_EP   = 36; // row pitch (floats) of the epilogue staging: 32 columns + 4

struct TtPlan
{
  int k1;                            // delay rank padded to 16
  uint32_t a_hi, a_lo, u_hi, u_lo;   // split chunk tiles: 128 x KC and k1 x KC
  uint32_t raw[2], raw_bytes;        // raw chunk stages: Ainv rows (128 x KC) then U rows (k1 x KC)
  uint32_t a2_hi, a2_lo, w_hi, w_lo; // later products: 128 x k1 (T1 - E, then X) and TN x k1 (V^T tile)
  uint32_t bt_hi, bt_lo;             // Binv^T: k1 x k1, over the V^T tile (read before the first tile)
  int binv_smem;                     // Binv copied into raw stage 0 (clear of Binv^T and big enough)
  uint32_t dl, bar, total;
};

__host__ __device__ inline TtPlan tt_plan(int k, int raw_stages)
{
  TtPlan p;
  p.k1    = ((k + 15) / 16) * 16;
  auto al = [](uint32_t x) { return (x + 1023u) & ~1023u; };
  uint32_t o = 0;
  p.a_hi  = o; o = al(o + TC_M * TT_KC * 4);
  p.a_lo  = o; o = al(o + TC_M * TT_KC * 4);
  p.u_hi  = o; o = al(o + p.k1 * TT_KC * 4);
  p.u_lo  = o; o = al(o + p.k1 * TT_KC * 4);
  p.raw_bytes = (uint32_t)(TC_M + p.k1) * TT_KC * 4;
  p.raw[0] = o;
  o        = al(o + p.raw_bytes);
  p.raw[1] = o;
  if (raw_stages > 1)
    o = al(o + p.raw_bytes);
  uint32_t o2 = 0;
  p.a2_hi = o2; o2 = al(o2 + TC_M * p.k1 * 4);
  p.a2_lo = o2; o2 = al(o2 + TC_M * p.k1 * 4);
  p.w_hi  = o2; o2 = al(o2 + TT_TN * p.k1 * 4);
  p.w_lo  = o2; o2 = al(o2 + TT_TN * p.k1 * 4);
  p.bt_hi = p.w_hi;
  p.bt_lo = al(p.bt_hi + p.k1 * p.k1 * 4);
  const uint32_t btend = al(p.bt_lo + p.k1 * p.k1 * 4);
  o2 = o2 > btend ? o2 : btend;
  // the epilogue's staging of a product tile (128 rows x 36 floats) over the V^T tile
  const uint32_t eend = al(p.w_hi + TC_M * TT_EP * 4);
  o2 = o2 > eend ? o2 : eend;
  o  = o > o2 ? o : o2;
  const uint32_t bbytes = (uint32_t)k * k * 4;
  p.binv_smem = (k % 2 == 0) && bbytes <= p.raw_bytes && (p.raw[0] + bbytes <= p.bt_hi || p.raw[0] >= btend);
  p.dl    = o; o = al(o + k * 4);
  p.bar   = o; o += 16;
  p.total = al(o);
  return p;
}

// 16-byte cp.async from global to shared, zero-filled when `valid` is false
__device__ __forceinline__ void cp16(uint32_t saddr, const void* g, bool valid)
{
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(saddr), "l"(g), "r"(valid ? 16 : 0)
               : "memory");
}

template<int TERMS, int KM, int RAW, int MINB>
__global__ void __launch_bounds__(TC_NT, MINB) flush_tc_tiled_kernel(FlushArgs<float> f, int* err)
{
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ uint32_t s_tmem;
  __shared__ int s_fail;
  const TtPlan P = tt_plan(f.k, RAW);
  const int n = f.n, k = f.k, dc = f.dc, lda = f.lda, k1 = P.k1;
  const int iw = blockIdx.x, r0 = blockIdx.y * TC_M;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  float* A         = f.ainv + (size_t)iw * f.sA;
  const float* U   = f.u + (size_t)iw * f.sU;
  const float* V   = f.v + (size_t)iw * f.sU;
  const float* Bi  = f.binv + (size_t)iw * f.sB;
  const int* dlist = f.delay_list + (size_t)iw * f.sD;
  int* dls         = reinterpret_cast<int*>(sm + P.dl);
  const uint32_t bar = smem_u32(sm + P.bar);
  if (tid == 0)
  {
    s_fail = 0;
    mbar_init(bar);
  }
  if (warp == 0)
    tmem_alloc(smem_u32(&s_tmem), TT_TMC);
  for (int e = tid; e < dc; e += TC_NT)
    dls[e] = dlist[e];
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = s_tmem;
  const uint32_t lrow = (uint32_t)(warp * 32) << 16; // this warp's TMEM lanes
  uint32_t phase      = 0;
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
  constexpr int AV = TC_M * (TT_KC / 4) / TC_NT; // Ainv slots per thread (8)
  constexpr int UV = KM * (TT_KC / 4) / TC_NT;   // U slots per thread (k1 <= KM)
  const int ub     = k1 * (TT_KC / 4);
  const int nch    = (n + TT_KC - 1) / TT_KC;
  // raw stage layout: Ainv chunk rows of KC floats, then the U chunk rows
  auto issue_chunk = [&](int ch, int stage) {
    const int k0    = ch * TT_KC;
    const uint32_t base = smem_u32(sm + (stage ? P.raw[1] : P.raw[0]));
#pragma unroll
    for (int q = 0; q < AV; q++)
    {
      const int e = tid + q * TC_NT, r = slot_row(e), c4 = slot_col(e), gr = r0 + r, gc = k0 + c4;
      const bool v = gr < n && gc < n;
      cp16(base + (uint32_t)(r * TT_KC + c4) * 4, v ? A + (size_t)gr * lda + gc : A, v);
    }
#pragma unroll
    for (int q = 0; q < UV; q++)
    {
      const int e = tid + q * TC_NT;
      if (e < ub)
      {
        const int r = slot_row(e), c4 = slot_col(e), gc = k0 + c4;
        const bool v = r < dc && gc < n;
        cp16(base + (uint32_t)((TC_M + r) * TT_KC + c4) * 4, v ? U + (size_t)r * lda + gc : U, v);
      }
    }
  };
  auto split_chunk = [&](int stage) {
    const unsigned char* raw = sm + (stage ? P.raw[1] : P.raw[0]);
#pragma unroll
    for (int q = 0; q < AV; q++)
    {
      const int e = tid + q * TC_NT, r = slot_row(e), c4 = slot_col(e);
      split_store(*reinterpret_cast<const float4*>(raw + (r * TT_KC + c4) * 4), P.a_hi, P.a_lo,
                  cm_off(r, c4, TT_KC));
    }
#pragma unroll
    for (int q = 0; q < UV; q++)
    {
      const int e = tid + q * TC_NT;
      if (e < ub)
      {
        const int r = slot_row(e), c4 = slot_col(e);
        split_store(*reinterpret_cast<const float4*>(raw + ((TC_M + r) * TT_KC + c4) * 4), P.u_hi, P.u_lo,
                    cm_off(r, c4, TT_KC));
      }
    }
  };
  float t1[KM];
#pragma unroll
  for (int q = 0; q < KM; q++)
    t1[q] = 0.f;
  auto accumulate = [&](uint32_t buf) {
#pragma unroll
    for (int c0 = 0; c0 < KM; c0 += 32)
      if (c0 < k1)
      {
        float t[32];
        tmem_ld32(buf + lrow + c0, t);
#pragma unroll
        for (int q = 0; q < 32; q++)
          t1[c0 + q] += t[q];
      }
  };
#pragma unroll
  for (int st = 0; st < RAW; st++)
  {
    if (st < nch)
      issue_chunk(st, st);
    asm volatile("cp.async.commit_group;\n" ::: "memory");
  }
  for (int c = 0; c < nch && ok; c++)
  {
    // this thread's copies of chunk c have landed: at most RAW - 1 younger groups pending
    if (RAW > 1)
      asm volatile("cp.async.wait_group 1;\n" ::: "memory");
    else
      asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    // every thread waits for chunk c - 1's products itself: the split tiles are then free
    bool mine = true;
    if (c > 0)
    {
      mine = mbar_wait(bar, phase);
      phase ^= 1;
      tc_fence_after();
    }
    split_chunk(c % RAW);
    if (c + RAW < nch)
      issue_chunk(c + RAW, c % RAW);
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    fence_async_smem();
    tc_fence_before();
    if (__syncthreads_or(!mine))
    {
      ok = false;
      break;
    }
    if (c == nch - 1 && P.binv_smem)
    {
      // Binv into raw stage 0, free now: it lands while the last products run
      const uint32_t base = smem_u32(sm + P.raw[0]);
      for (int e = tid; e < k * k / 4; e += TC_NT)
        cp16(base + (uint32_t)e * 16, Bi + 4 * e, true);
      asm volatile("cp.async.commit_group;\n" ::: "memory");
    }
    if (tid == 0)
    {
      tc_fence_after();
      const uint32_t id = idesc_tf32(TC_M, k1);
      const uint32_t ah = smem_u32(sm + P.a_hi), al = smem_u32(sm + P.a_lo);
      const uint32_t bh = smem_u32(sm + P.u_hi), bl = smem_u32(sm + P.u_lo);
      const uint32_t d  = TERMS > 1 ? tmem + 64 * (c & 1) : tmem;
      for (int ks = 0; ks < TT_KC / 8; ks++)
      {
        const uint32_t adv = ks * 256;
        const int first    = TERMS > 1 ? (ks == 0) : (c == 0 && ks == 0);
        mma_tf32(d, smem_desc(ah + adv, TT_KC), smem_desc(bh + adv, TT_KC), id, first ? 0 : 1);
        if (TERMS > 1)
        {
          mma_tf32(d, smem_desc(ah + adv, TT_KC), smem_desc(bl + adv, TT_KC), id, 1);
          mma_tf32(d, smem_desc(al + adv, TT_KC), smem_desc(bh + adv, TT_KC), id, 1);
        }
      }
      mma_commit(bar);
    }
    // with split precision: the previous chunk's product, summed while this one runs
    if (TERMS > 1 && c > 0)
      accumulate(tmem + 64 * ((c - 1) & 1));
    tc_fence_before();
  }
  if (ok)
    ok = wait_mma();
  if (TERMS > 1 && ok)
    accumulate(tmem + 64 * ((nch - 1) & 1));
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
  __syncthreads(); // Binv has landed for every thread's copies

  // ---------------- Binv^T, then (T1 - E) into the A operand of X = (T1 - E) Binv
  const int r = warp * 32 + lane;
  if (ok)
  {
    stage_binv_t<TERMS>(sm, P.bt_hi, P.bt_lo, P.binv_smem ? reinterpret_cast<const float*>(sm + P.raw[0]) : Bi, k,
                        dc, k1, tid);
    __syncthreads(); // the raw Binv (over the operand tiles) has been read
#pragma unroll
    for (int c0 = 0; c0 < KM; c0 += 32)
    {
      if (c0 >= k1)
        break;
      float t[32];
      if (TERMS > 1)
      {
#pragma unroll
        for (int q = 0; q < 32; q++)
          t[q] = t1[c0 + q];
      }
      else
        tmem_ld32(tmem + lrow + c0, t);
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
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    if (tid == 0)
    {
      tc_fence_after();
      mma_k1<TERMS>(tmem, sm, P.a2_hi, P.a2_lo, P.bt_hi, P.bt_lo, k1, idesc_tf32(TC_M, k1));
      mma_commit(bar);
    }
    ok = wait_mma();
  }
  // ---------------- X from TMEM into the A operand of the column-tile products
  if (ok)
  {
    for (int c0 = 0; c0 < k1; c0 += 32)
    {
      float t[32];
      tmem_ld32(tmem + lrow + c0, t);
#pragma unroll
      for (int q = 0; q < 32; q += 4)
        if (c0 + q < k1)
          split_store(make_float4(t[q], t[q + 1], t[q + 2], t[q + 3]), P.a2_hi, P.a2_lo, cm_off(r, c0 + q, k1));
    }
  }
  // ---------------- column tiles: P_tile = X V[:, tile], Ainv -= P.  V^T tile: element
  // (i, l) = V[l][t0 + i], consecutive threads on consecutive columns
  constexpr int VV = TT_TN * (KM / 4) / TC_NT; // slots of a V^T tile per thread (k1 <= KM)
  float vq[VV][4];
  auto load_vt = [&](int t0) {
#pragma unroll
    for (int h = 0; h < VV; h++)
    {
      const int e = tid + h * TC_NT, i = e % TT_TN, l4 = (e / TT_TN) * 4, col = t0 + i;
#pragma unroll
      for (int q = 0; q < 4; q++)
        vq[h][q] = (l4 + q < dc && l4 + q < k1 && col < n) ? V[(size_t)(l4 + q) * lda + col] : 0.f;
    }
  };
  // inverse rows of a tile: round j (32 columns), slot i: row e / 8, float4 e % 8 of the
  // round's 32 columns (e = tid + 128 i), so a warp reads four whole 128-byte row segments
  constexpr int ER = TT_TN / 32;
  float4 ap[ER][8];
  auto load_rows = [&](int t0) {
#pragma unroll
    for (int j = 0; j < ER; j++)
#pragma unroll
      for (int i = 0; i < 8; i++)
      {
        const int e = tid + i * TC_NT, gr = r0 + (e >> 3), gc = t0 + 32 * j + (e & 7) * 4;
        ap[j][i] = (gr < n && gc < n) ? *reinterpret_cast<const float4*>(A + (size_t)gr * lda + gc)
                                      : make_float4(0.f, 0.f, 0.f, 0.f);
      }
  };
  const uint32_t d2 = tmem + 64;
  const int nt      = (n + TT_TN - 1) / TT_TN;
  if (ok)
    load_vt(0);
  for (int t = 0; t < nt && ok; t++)
  {
    const int t0 = t * TT_TN;
    // V^T tile: the previous tile's epilogue staging (over it) is done, and for the first
    // tile the X product (Binv^T over it) has completed
#pragma unroll
    for (int h = 0; h < VV; h++)
    {
      const int e = tid + h * TC_NT, i = e % TT_TN, l4 = (e / TT_TN) * 4;
      if (l4 < k1)
        split_store(make_float4(vq[h][0], vq[h][1], vq[h][2], vq[h][3]), P.w_hi, P.w_lo, cm_off(i, l4, k1));
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    if (tid == 0)
    {
      tc_fence_after();
      mma_k1<TERMS>(d2, sm, P.a2_hi, P.a2_lo, P.w_hi, P.w_lo, k1, idesc_tf32(TC_M, TT_TN));
      mma_commit(bar);
    }
    // while the products run: this tile's inverse rows and the next tile's V^T values
    load_rows(t0);
    if (t + 1 < nt)
      load_vt(t0 + TT_TN);
    ok = wait_mma();
    if (!ok)
      break;
    float* E = reinterpret_cast<float*>(sm + P.w_hi);
#pragma unroll
    for (int j = 0; j < ER; j++)
    {
      float p[32];
      tmem_ld32(d2 + 32 * j + lrow, p);
#pragma unroll
      for (int q = 0; q < 32; q += 4)
        *reinterpret_cast<float4*>(E + r * TT_EP + q) = make_float4(p[q], p[q + 1], p[q + 2], p[q + 3]);
      __syncthreads();
#pragma unroll
      for (int i = 0; i < 8; i++)
      {
        const int e = tid + i * TC_NT, rr = e >> 3, c4 = (e & 7) * 4, gr = r0 + rr, gc = t0 + 32 * j + c4;
        if (gr < n && gc < n)
        {
          const float4 pv = *reinterpret_cast<const float4*>(E + rr * TT_EP + c4);
          const float4 a  = ap[j][i];
          *reinterpret_cast<float4*>(A + (size_t)gr * lda + gc) =
              make_float4(a.x - pv.x, a.y - pv.y, a.z - pv.z, a.w - pv.w);
        }
      }
      tc_fence_before();
      __syncthreads();
    }
  }
  if (!ok && tid == 0)
    atomicExch(err, 1);
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
  tc_fence_before();
  __syncthreads();
  if (warp == 0)
    tmem_dealloc(tmem, TT_TMC);
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
  return k >= 1 && k <= TT_KMAX && (lda % 4) == 0 && (n % 4) == 0 && tt_plan(k, 2).total <= 200 * 1024;
}

#define QMCG_TILED_BIG(TERMS) flush_tc_tiled_kernel<TERMS, 64, 2, 2>
#define QMCG_TILED_SMALL(TERMS) flush_tc_tiled_kernel<TERMS, 32, 1, 3>

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

// which kernel flushes a shape: 0 one-pass, 1 tiled (k <= 32, one raw chunk in flight), 2 tiled (k <= 64)
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
    const TtPlan p = tt_plan(f.k, 1);
    if (terms == 1)
      QMCG_TILED_SMALL(1)<<<grid, TC_NT, p.total, st>>>(f, err);
    else
      QMCG_TILED_SMALL(3)<<<grid, TC_NT, p.total, st>>>(f, err);
  }
  else
  {
    if (f.k > TT_KMAX)
      return cudaErrorInvalidValue;
    const TtPlan p = tt_plan(f.k, 2);
    if (terms == 1)
      QMCG_TILED_BIG(1)<<<grid, TC_NT, p.total, st>>>(f, err);
    else
      QMCG_TILED_BIG(3)<<<grid, TC_NT, p.total, st>>>(f, err);
  }
  return cudaGetLastError();
}

} // namespace qmcg
