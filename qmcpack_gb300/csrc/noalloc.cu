// Allocation-free variant of the delayed-update flush (qmcg_mw_update_inv_mat_noalloc).
//
// Who needs it: a caller whose device memory is owned entirely by another
// allocator (a framework's caching allocator or an offload runtime that
// reserves the device), a caller that cannot afford the device-wide
// synchronisation cudaFree implies because other streams are running latency-
// sensitive work, and a caller running where allocation is forbidden (driver
// callbacks, real-time threads).  Such callers pass their own inputs and
// outputs; where the flush needs scratch (W = Binv V, one delay_rank x lda block
// per walker, for shapes whose tiles do not fit in shared memory) it lives in the
// fixed device array below instead of coming from cudaMalloc or a stream-ordered
// pool.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/qmcg.h"
#include "common.cuh"
#include "launch.h"

namespace
{
// The scratch of every call on this device.  A GPU on which this code is
// loaded holds it until the process exits.
static __device__ __align__(256) unsigned char g_flush_scratch[QMCG_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
void* g_scratch_addr[kMaxDevices] = {};
void* g_scratch_ctx[kMaxDevices]  = {}; // the context the address was looked up in

// the current context, through the driver's cuCtxGetCurrent (found once through the runtime)
void* current_context()
{
  using GetCtx          = int (*)(void**);
  static GetCtx get_ctx = [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      fn = nullptr;
    return reinterpret_cast<GetCtx>(fn);
  }();
  void* ctx = nullptr;
  if (!get_ctx || get_ctx(&ctx) != 0)
    return nullptr;
  return ctx;
}

// Once per device, with that device current: the device address of the array (again
// if the device's context was re-created since, e.g. after cudaDeviceReset, which
// reloads the module).  The array's name is only a host-side stand-in in host code,
// so it is never passed to a kernel directly.
int scratch_address(void** out)
{
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess)
    return qmcg::set_error(QMCG_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices)
    return qmcg::set_error(QMCG_ERR_ARG, "device index beyond the supported range");
  const void* ctx = current_context(); // null before the device's context exists
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_addr[dev] || !ctx || g_scratch_ctx[dev] != ctx)
  {
    void* p = nullptr;
    e       = cudaGetSymbolAddress(&p, g_flush_scratch); // creates the context if needed
    if (e != cudaSuccess || !p)
      return qmcg::set_error(QMCG_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_scratch_addr[dev] = p;
    g_scratch_ctx[dev]  = current_context();
  }
  *out = g_scratch_addr[dev];
  return QMCG_OK;
}

template<typename T>
qmcg::FlushArgs<T> flush_args(int nw, int n, int lda, int k, int dc, void* ainv, const void* u, const void* v,
                              const void* binv, const int* dl, void* w)
{
  qmcg::FlushArgs<T> f;
  f.nw         = nw;
  f.n          = n;
  f.lda        = lda;
  f.k          = k;
  f.dc         = dc;
  f.sA         = (long long)n * lda;
  f.sU         = (long long)k * lda;
  f.sB         = (long long)k * k;
  f.sD         = k;
  f.ainv       = static_cast<T*>(ainv);
  f.u          = static_cast<const T*>(u);
  f.v          = static_cast<const T*>(v);
  f.binv       = static_cast<const T*>(binv);
  f.delay_list = dl;
  f.w          = static_cast<T*>(w);
  return f;
}

// The same kernel choice as qmcg_mw_update_inv_mat: the shared-memory kernel, which
// needs no scratch, where its tiles fit; otherwise the two-kernel flush with W = Binv V
// in the fixed array (the size limit applies to this case only).
template<typename T>
int flush_noalloc(int nw, int n, int lda, int k, int dc, void* ainv, const void* u, const void* v, const void* binv,
                  const int* dl, cudaStream_t st)
{
  cudaError_t e = qmcg::setup_move_kernels<T>();
  if (e != cudaSuccess)
    return qmcg::set_error(QMCG_ERR_CUDA, std::string("kernel set-up: ") + cudaGetErrorString(e));
  if (qmcg::flush_fused_fits<T>(n, k))
  {
    e = qmcg::setup_flush_fused<T>();
    if (e == cudaSuccess)
      e = qmcg::launch_flush_fused(flush_args<T>(nw, n, lda, k, dc, ainv, u, v, binv, dl, nullptr), st);
    if (e != cudaSuccess)
      return qmcg::set_error(QMCG_ERR_CUDA, std::string("flush launch: ") + cudaGetErrorString(e));
    return QMCG_OK;
  }
  void* scratch = nullptr;
  const int rc  = scratch_address(&scratch);
  if (rc != QMCG_OK)
    return rc;
  e = qmcg::launch_flush_args(flush_args<T>(nw, n, lda, k, dc, ainv, u, v, binv, dl, scratch), st);
  if (e != cudaSuccess)
    return qmcg::set_error(QMCG_ERR_CUDA, std::string("flush launch: ") + cudaGetErrorString(e));
  return QMCG_OK;
}
} // namespace

extern "C" int qmcg_mw_update_inv_mat_noalloc(int precision, int nw, int n, int lda, int k, int dc, void* ainv,
                                              const void* u, const void* v, const void* binv, const int* delay_list,
                                              void* stream)
{
  if (precision != 4 && precision != 8)
    return qmcg::set_error(QMCG_ERR_ARG, "precision must be 4 or 8");
  if (nw < 0 || n <= 0 || lda < n || k <= 0 || dc < 0 || dc > k)
    return qmcg::set_error(QMCG_ERR_ARG, "need n > 0, lda >= n, 0 <= delay_count <= delay_rank");
  // only shapes whose tiles do not fit in shared memory use the fixed scratch array
  const bool fused = precision == 8 ? qmcg::flush_fused_fits<double>(n, k) : qmcg::flush_fused_fits<float>(n, k);
  const unsigned long long need = (unsigned long long)nw * k * lda * (unsigned long long)precision;
  if (!fused && need > (unsigned long long)QMCG_NOALLOC_SCRATCH_BYTES)
    return qmcg::set_error(QMCG_ERR_ARG, "num_walkers * delay_rank * lda * element size = " + std::to_string(need) +
                                             " bytes exceeds the " + std::to_string(QMCG_NOALLOC_SCRATCH_BYTES) +
                                             "-byte scratch of the allocation-free flush; split the walkers "
                                             "into smaller batches");
  if (nw == 0 || dc == 0)
    return QMCG_OK;
  if (!ainv || !u || !v || !binv || !delay_list)
    return qmcg::set_error(QMCG_ERR_ARG, "null device buffer");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  return precision == 8 ? flush_noalloc<double>(nw, n, lda, k, dc, ainv, u, v, binv, delay_list, st)
                        : flush_noalloc<float>(nw, n, lda, k, dc, ainv, u, v, binv, delay_list, st);
}
