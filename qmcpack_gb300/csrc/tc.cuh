// tcgen05 / mbarrier helpers shared by the tensor-core kernels (inline PTX, sm_103a).
//
// Operand tiles live in shared memory in the no-swizzle K-major core-matrix layout:
// a core matrix is 8 rows x 16 bytes; core matrices adjacent along K are 128 bytes
// apart (leading byte offset), 8-row groups are (K bytes / 16) * 128 bytes apart
// (stride byte offset).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace qmcg
{

constexpr long long TC_WAIT_LIMIT = 1ll << 26;

__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// byte offset of element (r, k) of an R x kc tile of esize-byte elements
__device__ __forceinline__ uint32_t cm_off_b(int r, int k, int kc, int esize)
{
  const int per = 16 / esize; // elements per 16-byte core-matrix row
  return (uint32_t)(((r >> 3) * (kc / per) + (k / per)) * 128 + (r & 7) * 16 + (k % per) * esize);
}

// shared-memory matrix descriptor: no swizzle, K-major, LBO = 128 B, SBO = row_bytes/16*128 B, version 1
__device__ __forceinline__ uint64_t smem_desc_b(uint32_t saddr, int row_bytes)
{
  const uint64_t lbo = 128 >> 4;
  const uint64_t sbo = (uint64_t)((row_bytes >> 4) * 128) >> 4;
  return (uint64_t)((saddr >> 4) & 0x3FFF) | (lbo << 16) | (sbo << 32) | (1ull << 46);
}

__device__ __forceinline__ void mma_commit(uint32_t mbar)
{
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mbar)
               : "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t mbar)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(mbar) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}

// bounded wait on an mbarrier phase; returns false on timeout
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity)
{
  for (long long it = 0; it < TC_WAIT_LIMIT; it++)
  {
    uint32_t done;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}\n"
                 : "=r"(done)
                 : "r"(mbar), "r"(parity)
                 : "memory");
    if (done)
      return true;
  }
  return false;
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32])
{
  uint32_t r[32];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
               "%14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                 "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                 "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
                 "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
                 "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
               : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; i++)
    v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_alloc(uint32_t slot_saddr, int cols)
{
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(slot_saddr), "r"(cols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, int cols)
{
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(cols) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

} // namespace qmcg
