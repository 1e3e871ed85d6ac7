// C ABI of the library (include/qmcg.h): system and crowd handles, device
// memory, the mw_ call sequence and the captured sweep graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <deque>
#include <limits>
#include <memory>
#include <random>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/qmcg.h"
#include "common.cuh"
#include "launch.h"

using namespace qmcg;

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------
static thread_local std::string g_last_error;

static int fail(int code, const std::string& msg)
{
  g_last_error = msg;
  return code;
}

#define CUDA_TRY(expr)                                                                                                 \
  do                                                                                                                   \
  {                                                                                                                    \
    cudaError_t e_ = (expr);                                                                                           \
    if (e_ != cudaSuccess)                                                                                             \
      return fail(QMCG_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_));                                \
  } while (0)

extern "C" const char* qmcg_last_error(void) { return g_last_error.c_str(); }

namespace qmcg
{
int set_error(int code, const std::string& msg) { return fail(code, msg); }
} // namespace qmcg

extern "C" int qmcg_device_count(int* count)
{
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess)
    n = 0;
  if (count)
    *count = n;
  return n > 0 ? QMCG_OK : fail(QMCG_ERR_NO_DEVICE, "no CUDA device");
}

// ---------------------------------------------------------------------------
// device memory owned by a handle
// ---------------------------------------------------------------------------
struct DeviceArena
{
  std::vector<void*> ptrs;
  ~DeviceArena()
  {
    for (void* p : ptrs)
      cudaFree(p);
  }
  template<typename X>
  cudaError_t alloc(X** p, size_t count)
  {
    void* q       = nullptr;
    cudaError_t e = cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(X));
    if (e != cudaSuccess)
      return e;
    ptrs.push_back(q);
    e = cudaMemset(q, 0, std::max<size_t>(count, 1) * sizeof(X));
    *p = static_cast<X*>(q);
    return e;
  }
};

// BF16 <-> FP32 on the host: round to nearest even (NaN kept quiet)
static uint16_t f2bf(float f)
{
  uint32_t u;
  std::memcpy(&u, &f, 4);
  if ((u & 0x7fffffffu) > 0x7f800000u)
    return static_cast<uint16_t>((u >> 16) | 0x40u);
  u += 0x7fffu + ((u >> 16) & 1u);
  return static_cast<uint16_t>(u >> 16);
}

static float bf2f(uint16_t h)
{
  const uint32_t u = static_cast<uint32_t>(h) << 16;
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}

// ---------------------------------------------------------------------------
// system
// ---------------------------------------------------------------------------
struct qmcg_system_s
{
  int prec;
  int nup, ndn, ne, norb, lda, nions, nions_pad, nion_species;
  int grid[3];
  double L[3];
  DeviceArena mem;
  void* coefs = nullptr;
  void* ions  = nullptr;
  int* ion_species = nullptr;
  void* j1c = nullptr;
  void* j2c = nullptr;
  int j1_ncoef = 0, j2_ncoef = 0;
  double j1_rcut = 0, j2_rcut = 0;
  double j1_dri = 0, j2_dri = 0;
  int has_j1 = 0, has_j2 = 0;
  // Ewald tables for the local energy (precision of the move loop)
  EwaldHost ewh;
  int ew_ng = 0;
  void* ew_gn = nullptr;
  void* ew_fg = nullptr;
  void* ew_rho = nullptr;
  void* ew_q = nullptr;
};

// BsplineFunctor::reset (BsplineFunctor.h:117-133) in the functor precision T
template<typename T>
static void functor_coefs(int nparams, double cutoff, const double* params, double cusp, std::vector<T>& out,
                          double& dri)
{
  const int numCoefs = nparams + 4;
  const int numKnots = numCoefs - 2;
  const T DeltaR     = static_cast<T>(cutoff) / static_cast<T>(numKnots - 1);
  const T DeltaRInv  = T(1.0) / DeltaR;
  std::vector<T> c(numCoefs, T(0));
  c[1] = static_cast<T>(params[0]);
  c[2] = static_cast<T>(params[1]);
  c[0] = static_cast<T>(params[1]) - T(2.0) * DeltaR * static_cast<T>(cusp);
  for (int i = 2; i < nparams; i++)
    c[i + 1] = static_cast<T>(params[i]);
  out.insert(out.end(), c.begin(), c.end());
  dri = static_cast<double>(DeltaRInv);
}

template<typename T>
static int build_system(const qmcg_system_desc* d, qmcg_system_s* s)
{
  const size_t ncoef = (size_t)(d->grid[0] + 3) * (d->grid[1] + 3) * (d->grid[2] + 3) * d->num_orbitals_padded;
  T* coefs;
  CUDA_TRY(s->mem.alloc(&coefs, ncoef));
  CUDA_TRY(cudaMemcpy(coefs, d->spline_coefs, ncoef * sizeof(T), cudaMemcpyHostToDevice));
  s->coefs = coefs;
  std::vector<T> ions((size_t)3 * s->nions_pad, T(0));
  for (int i = 0; i < d->num_ions; i++)
    for (int k = 0; k < 3; k++)
      ions[(size_t)k * s->nions_pad + i] = static_cast<T>(d->ion_pos[i * 3 + k]);
  T* dions;
  CUDA_TRY(s->mem.alloc(&dions, ions.size()));
  CUDA_TRY(cudaMemcpy(dions, ions.data(), ions.size() * sizeof(T), cudaMemcpyHostToDevice));
  s->ions = dions;
  std::vector<int> spc(std::max(d->num_ions, 1), 0);
  for (int i = 0; i < d->num_ions; i++)
    spc[i] = d->ion_species ? d->ion_species[i] : 0;
  CUDA_TRY(s->mem.alloc(&s->ion_species, spc.size()));
  CUDA_TRY(cudaMemcpy(s->ion_species, spc.data(), spc.size() * sizeof(int), cudaMemcpyHostToDevice));
  if (s->has_j1)
  {
    std::vector<T> c;
    for (int sp = 0; sp < d->num_ion_species; sp++)
      functor_coefs<T>(d->j1_num_params, d->j1_rcut, d->j1_params + (size_t)sp * d->j1_num_params,
                       d->j1_cusp ? d->j1_cusp[sp] : 0.0, c, s->j1_dri);
    T* dc;
    CUDA_TRY(s->mem.alloc(&dc, c.size()));
    CUDA_TRY(cudaMemcpy(dc, c.data(), c.size() * sizeof(T), cudaMemcpyHostToDevice));
    s->j1c      = dc;
    s->j1_ncoef = d->j1_num_params + 4;
  }
  if (s->has_j2)
  {
    std::vector<T> c;
    for (int p = 0; p < 2; p++)
      functor_coefs<T>(d->j2_num_params, d->j2_rcut, d->j2_params + (size_t)p * d->j2_num_params,
                       d->j2_cusp ? d->j2_cusp[p] : 0.0, c, s->j2_dri);
    T* dc;
    CUDA_TRY(s->mem.alloc(&dc, c.size()));
    CUDA_TRY(cudaMemcpy(dc, c.data(), c.size() * sizeof(T), cudaMemcpyHostToDevice));
    s->j2c      = dc;
    s->j2_ncoef = d->j2_num_params + 4;
  }
  // Coulomb: ion charges per species (default: a neutral cell), Ewald tables with
  // tolerance 1e-7 (FP32) or 1e-12 (FP64)
  {
    std::vector<double> q(std::max(d->num_ions, 1), 0.0), pos((size_t)3 * std::max(d->num_ions, 1), 0.0);
    for (int i = 0; i < d->num_ions; i++)
    {
      const int sp = d->ion_species ? d->ion_species[i] : 0;
      q[i]         = d->ion_charges ? d->ion_charges[sp] : static_cast<double>(s->ne) / d->num_ions;
      for (int k = 0; k < 3; k++)
        pos[3 * i + k] = d->ion_pos[3 * i + k];
    }
    const double eps = std::is_same<T, float>::value ? 1e-7 : 1e-12;
    if (ewald_build(s->L, s->ne, d->num_ions, pos.data(), q.data(), eps, s->ewh) != 0)
      return fail(QMCG_ERR_ARG, "Ewald tables: the cell is too anisotropic for the reciprocal cutoff");
    const auto& e = s->ewh;
    s->ew_ng      = static_cast<int>(e.fg.size());
    const size_t ng = std::max<size_t>(e.fg.size(), 1);
    std::vector<T> fg(ng, T(0)), rho(2 * ng, T(0)), qt(q.size());
    for (size_t g = 0; g < e.fg.size(); g++)
    {
      fg[g]          = static_cast<T>(e.fg[g]);
      rho[2 * g]     = static_cast<T>(e.rho_ion[2 * g]);
      rho[2 * g + 1] = static_cast<T>(e.rho_ion[2 * g + 1]);
    }
    for (size_t i = 0; i < q.size(); i++)
      qt[i] = static_cast<T>(q[i]);
    char4* dgn;
    T *dfg, *drho, *dq;
    CUDA_TRY(s->mem.alloc(&dgn, ng));
    CUDA_TRY(s->mem.alloc(&dfg, ng));
    CUDA_TRY(s->mem.alloc(&drho, 2 * ng));
    CUDA_TRY(s->mem.alloc(&dq, qt.size()));
    if (!e.gn.empty())
      CUDA_TRY(cudaMemcpy(dgn, e.gn.data(), e.gn.size() * sizeof(char4), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(dfg, fg.data(), ng * sizeof(T), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(drho, rho.data(), 2 * ng * sizeof(T), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(dq, qt.data(), qt.size() * sizeof(T), cudaMemcpyHostToDevice));
    s->ew_gn  = dgn;
    s->ew_fg  = dfg;
    s->ew_rho = drho;
    s->ew_q   = dq;
  }
  return QMCG_OK;
}

extern "C" int qmcg_system_create(const qmcg_system_desc* d, qmcg_system* out)
{
  if (!d || !out)
    return fail(QMCG_ERR_ARG, "null argument");
  *out = nullptr;
  if (d->precision != 4 && d->precision != 8)
    return fail(QMCG_ERR_ARG, "precision must be 4 or 8");
  if (d->n_up <= 0 || d->n_up != d->n_dn || d->num_orbitals != d->n_up)
    return fail(QMCG_ERR_ARG, "need n_up == n_dn == num_orbitals > 0");
  if (d->num_orbitals_padded < d->num_orbitals || d->num_orbitals_padded % 16 != 0)
    return fail(QMCG_ERR_ARG, "num_orbitals_padded must be a multiple of 16 and >= num_orbitals");
  for (int k = 0; k < 3; k++)
  {
    if (!(d->lattice[k] > 0))
      return fail(QMCG_ERR_ARG, "lattice lengths must be positive (periodic orthorhombic cell)");
    if (d->grid[k] < 1)
      return fail(QMCG_ERR_ARG, "grid must be >= 1");
  }
  if (!d->spline_coefs || (d->num_ions > 0 && !d->ion_pos))
    return fail(QMCG_ERR_ARG, "missing spline coefficients or ion positions");
  if (d->num_ions < 0 || (d->num_ions > 0 && d->num_ion_species < 1))
    return fail(QMCG_ERR_ARG, "bad ion count or species count");
  if (d->ion_species)
    for (int i = 0; i < d->num_ions; i++)
      if (d->ion_species[i] < 0 || d->ion_species[i] >= d->num_ion_species)
        return fail(QMCG_ERR_ARG, "ion species index out of range");
  if (d->ion_charges)
    for (int sp = 0; sp < d->num_ion_species; sp++)
      if (!std::isfinite(d->ion_charges[sp]))
        return fail(QMCG_ERR_ARG, "ion charges must be finite");
  if ((d->j1_num_params > 0 && (!d->j1_params || !(d->j1_rcut > 0))) ||
      (d->j2_num_params > 0 && (!d->j2_params || !(d->j2_rcut > 0))))
    return fail(QMCG_ERR_ARG, "Jastrow parameters or cutoff missing");
  if (d->j1_num_params < 0 || d->j2_num_params < 0 || (d->j1_num_params > 0 && d->j1_num_params < 2) ||
      (d->j2_num_params > 0 && d->j2_num_params < 2))
    return fail(QMCG_ERR_ARG, "Jastrow functors need at least 2 parameters");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    return fail(QMCG_ERR_NO_DEVICE, "no CUDA device");
  auto s          = std::make_unique<qmcg_system_s>();
  s->prec         = d->precision;
  s->nup          = d->n_up;
  s->ndn          = d->n_dn;
  s->ne           = d->n_up + d->n_dn;
  s->norb         = d->num_orbitals;
  s->lda          = d->num_orbitals_padded;
  s->nions        = d->num_ions;
  s->nions_pad    = std::max(32, ((d->num_ions + 31) / 32) * 32);
  s->nion_species = std::max(1, d->num_ion_species);
  for (int k = 0; k < 3; k++)
  {
    s->grid[k] = d->grid[k];
    s->L[k]    = d->lattice[k];
  }
  s->has_j1  = (d->j1_num_params > 0 && d->num_ions > 0) ? 1 : 0;
  s->has_j2  = d->j2_num_params > 0 ? 1 : 0;
  s->j1_rcut = d->j1_rcut;
  s->j2_rcut = d->j2_rcut;
  int rc = d->precision == 8 ? build_system<double>(d, s.get()) : build_system<float>(d, s.get());
  if (rc != QMCG_OK)
    return rc;
  *out = s.release();
  return QMCG_OK;
}

extern "C" int qmcg_system_destroy(qmcg_system sys)
{
  delete sys;
  return QMCG_OK;
}

// ---------------------------------------------------------------------------
// host side of the bit-compatible random stream (StdRandom<double> + Box-Muller)
// ---------------------------------------------------------------------------
struct HostStream
{
  std::mt19937 eng;
  std::deque<uint32_t> ahead;
  void seed(uint64_t s)
  {
    eng.seed(static_cast<std::mt19937::result_type>(s));
    ahead.clear();
  }
  uint32_t next()
  {
    if (!ahead.empty())
    {
      const uint32_t x = ahead.front();
      ahead.pop_front();
      return x;
    }
    return eng();
  }
  static double to_uniform(uint32_t x)
  {
    return static_cast<double>(x - std::mt19937::min()) /
        (static_cast<double>(std::mt19937::max() - std::mt19937::min()) + 1.0);
  }
  double uniform() { return to_uniform(next()); }
  void peek_uniforms(double* out, size_t n)
  {
    while (ahead.size() < n)
      ahead.push_back(eng());
    for (size_t i = 0; i < n; i++)
      out[i] = to_uniform(ahead[i]);
  }
  void consume(size_t n)
  {
    for (size_t i = 0; i < n; i++)
      next();
  }
  void gauss(double* a, size_t n)
  {
    const double slightly_less_than_one = 1.0 - std::numeric_limits<double>::epsilon();
    const long nm1 = static_cast<long>(n) - 1;
    for (long i = 0; i < nm1; i += 2)
    {
      const double t1 = std::sqrt(-2.0 * std::log(1.0 - slightly_less_than_one * uniform()));
      const double t2 = 2.0 * M_PI * uniform();
      a[i]            = t1 * std::cos(t2);
      a[i + 1]        = t1 * std::sin(t2);
    }
    if (n % 2 == 1)
    {
      const double t1 = std::sqrt(-2.0 * std::log(1.0 - slightly_less_than_one * uniform()));
      const double t2 = 2.0 * M_PI * uniform();
      a[nm1]          = t1 * std::cos(t2);
    }
  }
};

__global__ void bump_counter_kernel(unsigned long long* c) { c[0] += 1ull; }

// walker positions between the caller's layout [nw][ne][3] and the device's [nw][3][ne_pad]
// (FP64 and the move-precision copy; padding electrons at zero)
template<typename T>
__global__ void positions_from_caller_kernel(const double* __restrict__ aos, double* __restrict__ R,
                                             T* __restrict__ Rt, int nw, int ne, int ne_pad)
{
  const size_t total = (size_t)nw * 3 * ne_pad;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x)
  {
    const int e       = (int)(t % ne_pad);
    const size_t wq   = t / ne_pad; // iw * 3 + q
    const int q       = (int)(wq % 3);
    const size_t iw   = wq / 3;
    const double x    = e < ne ? aos[(iw * ne + e) * 3 + q] : 0.0;
    R[t]              = x;
    Rt[t]             = static_cast<T>(x);
  }
}
// per walker the sums of the J2 and J1 values over its electrons (log J2 = -sum/2,
// log J1 = -sum), a warp per walker: out[iw] (J2), out[nw + iw] (J1)
template<typename T>
__global__ void jastrow_log_sums_kernel(const T* __restrict__ J2, const T* __restrict__ J1, int nw, int ne,
                                        int ne_pad, double* __restrict__ out)
{
  const int iw = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (iw >= nw)
    return;
  double u2 = 0, u1 = 0;
  for (int e = lane; e < ne; e += 32)
  {
    u2 += static_cast<double>(J2[(size_t)iw * 5 * ne_pad + e]);
    u1 += static_cast<double>(J1[(size_t)iw * 5 * ne_pad + e]);
  }
  u2 = warp_sum(u2);
  u1 = warp_sum(u1);
  if (lane == 0)
  {
    out[iw]      = u2;
    out[nw + iw] = u1;
  }
}

__global__ void positions_to_caller_kernel(const double* __restrict__ R, double* __restrict__ aos, int nw, int ne,
                                           int ne_pad)
{
  const size_t total = (size_t)nw * ne * 3;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x)
  {
    const int q     = (int)(t % 3);
    const size_t we = t / 3; // iw * ne + e
    const int e     = (int)(we % ne);
    const size_t iw = we / ne;
    aos[t]          = R[(iw * 3 + q) * ne_pad + e];
  }
}
__global__ void reset_cursor_kernel(int* c) { c[0] = 0; c[1] = 0; }

// ---------------------------------------------------------------------------
// crowd
// ---------------------------------------------------------------------------
struct qmcg_crowd_s
{
  virtual ~qmcg_crowd_s() = default;
  qmcg_system sys        = nullptr;
  cudaStream_t stream    = nullptr;
  // the completing pass of the up spin's block-lazy updates runs here, at a lower priority,
  // beside the down spin's segments (it touches only the up spin's inverse and sets)
  cudaStream_t side      = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  int nw = 0, k = 1;
  int dc[2]              = {0, 0};
  int invrow_iat         = -1;
  virtual int load(const double* R)                      = 0;
  virtual int positions(double* R)                       = 0;
  virtual int evaluate_log(double* lp, int* sg)          = 0;
  virtual int eval_grad(int iat, double* g)              = 0;
  virtual int make_move(int iat, const double* d)        = 0;
  virtual int ratio_grad(int iat, double* r, double* g)  = 0;
  virtual int accept_reject(int iat, const int* acc)     = 0;
  virtual int complete()                                 = 0;
  virtual int get_log(double* lp, int* sg, double* parts) = 0;
  virtual int get_inverse(int spin, double* a)           = 0;
  virtual int get_jastrow(double* j2, double* j1)        = 0;
  virtual int get_phi(double* phi)                       = 0;
  virtual int sweeps(const qmcg_sweep_params* p, int n, qmcg_sweep_stats* st, int* acc_log) = 0;
  virtual int sweeps_host(const qmcg_sweep_params* p, int n, const double* r_in, double* r_out, double* lp,
                          qmcg_sweep_stats* st) = 0;
  virtual int sweeps_async(int n)                        = 0;
  virtual int profile_ratio(int niat, double* ms)        = 0;
  virtual int profile_sweep(int n, double* out)          = 0;
  virtual int sweep_info(int flush, int* out)            = 0;
  virtual int sync(qmcg_sweep_stats* st)                 = 0;
  virtual int local_energy(double* el, double* ke, double* vp) = 0;
  virtual int set_threads(int nt)                        = 0;
  virtual int recompute_walkers(const int* flags)        = 0;
  virtual int proposal_init(uint64_t seed, double scale)  = 0;
  virtual int proposal_params(float* get, const float* set) = 0;
  virtual int proposal_forward(int rows, const float* x, float* out, float* hidden) = 0;
  virtual int proposal_backward(int rows, const float* x, const float* dout, float* grad) = 0;
  virtual int proposal_features(int iat, int at_proposed, float* x) = 0;
  virtual int sweeps_learned(const qmcg_sweep_params* p, int n, int train, double lr, double* el,
                             qmcg_sweep_stats* st, double* tstats) = 0;
  virtual int sweeps_measure(const qmcg_sweep_params* p, int n, double* el, double* ke, qmcg_sweep_stats* st) = 0;
  virtual int sweeps_trace(const qmcg_sweep_params* p, int n, qmcg_sweep_stats* st, double* trace) = 0;
  virtual int evaluate_gl(double* lp, double* grads, double* laps) = 0;
  virtual int profile_recompute(double* ms) = 0;
  virtual int dmc_init(double* el) = 0;
  virtual int dmc_step(const qmcg_sweep_params* p, const qmcg_branch_params* b, double* w, double* el, int* age,
                       double* sums, qmcg_sweep_stats* st, double* trace) = 0;
  virtual int dmc_copy(const int* src) = 0;
  virtual int dmc_reconfigure(double u, int* src) = 0;
  virtual int evaluate_ratios(int nvp, const int* walker, const int* elec, const double* pos, double* ratios) = 0;
  virtual int profile_ratios(int nvp, const int* walker, const int* elec, const double* pos, int reps,
                             double* ms) = 0;
};

// The comb of population control with a fixed walker count
// (WalkerReconfiguration::getIndexPermutation, WalkerReconfiguration.cpp:30-107): nw
// teeth at W (u + i) / nw, W = sum |w|, u in [0, 1); walker iw gets one copy per tooth in
// [sum_{j<iw} |w_j|, sum_{j<=iw} |w_j|).  Slots of walkers with no copy take the extra
// copies of the others in order; every other slot keeps its walker.  Returns the number
// of walkers with at least one copy.
static int comb_sources(int nw, const double* weights, double u, int* src)
{
  double wtot = 0;
  for (int iw = 0; iw < nw; iw++)
    wtot += std::fabs(weights[iw]);
  std::vector<double> zeta(nw + 1);
  const double nw_inv = 1.0 / static_cast<double>(nw), dstep = u * nw_inv;
  for (int iw = 0; iw < nw; iw++)
    zeta[iw] = wtot * (dstep + static_cast<double>(iw) * nw_inv);
  zeta[nw] = wtot + 1.0;
  std::vector<int> plus, minus;
  int ind = 0, kept = 0;
  double wcur = 0;
  for (int iw = 0; iw < nw; iw++)
  {
    const double tryp = wcur + std::fabs(weights[iw]);
    int ni            = 0;
    while (zeta[ind] < tryp && zeta[ind] >= wcur)
    {
      ind++;
      ni++;
    }
    wcur += std::fabs(weights[iw]);
    kept += ni ? 1 : 0;
    if (ni > 1)
      plus.insert(plus.end(), ni - 1, iw);
    else if (ni == 0)
      minus.push_back(iw);
    src[iw] = iw;
  }
  // a tooth lost to rounding at the end of the comb leaves a walker without a copy in its slot
  const size_t ncopy = std::min(plus.size(), minus.size());
  for (size_t i = 0; i < ncopy; i++)
    src[minus[i]] = plus[i];
  return kept;
}

extern "C" int qmcg_dmc_comb(int nw, const double* weights, double u, int* src, int* num_kept)
{
  if (nw <= 0 || !weights || !src || !(u >= 0.0 && u < 1.0))
    return fail(QMCG_ERR_ARG, "need num_walkers > 0, weights, src and 0 <= u < 1");
  for (int i = 0; i < nw; i++)
    if (!std::isfinite(weights[i]))
      return fail(QMCG_ERR_ARG, "non-finite walker weight");
  const int kept = comb_sources(nw, weights, u, src);
  if (num_kept)
    *num_kept = kept;
  return QMCG_OK;
}

template<typename T>
struct Crowd final : qmcg_crowd_s
{
  DevState<T> s{};
  DeviceArena mem;
  double* Mt = nullptr; // FP64 Slater matrices for the recompute, [2][nw][N][N]
  double* aos = nullptr; // positions in the caller's layout [nw][ne][3], staged for the copies
  double* jsum = nullptr; // [2][nw] J2 and J1 value sums of every walker (get_log)
  T* W       = nullptr; // flush scratch, [nw][k][lda]
  double* gauss_d = nullptr;
  double* unif_d  = nullptr;
  // pinned staging of the per-sweep results read back: counters, flush error flag, status words,
  // and the log|psi| parts (log|det| and sign per spin, Jastrow sums)
  struct IoStage
  {
    unsigned long long* cnt = nullptr; // [3]
    int* tce    = nullptr;             // [1]
    int* status = nullptr;             // [nw]
    double* la  = nullptr;             // [2 nw]
    double* js  = nullptr;             // [2 nw]
    int* sg     = nullptr;             // [2 nw]
    void* block = nullptr;
  } io;
  double* gauss_h = nullptr; // pinned
  double* unif_h  = nullptr; // pinned
  HostStream hs;
  bool stream_seeded = false;
  uint64_t hs_seed    = 0;
  cudaGraphExec_t graph = nullptr;
  int graph_rng_mode = -1, graph_use_drift = -1, graph_path = -1;
  int sweep_grid_size = 0;
  int sweep_grid_learned = 0;
  int sweep_nt           = 128; // threads per walker of the drift-diffusion resident kernel
  int graph_nt           = -1;
  int flush_kind      = 0;
  int graph_flush     = -1;
  int* tc_err         = nullptr;
  double graph_tau = 0;
  uint64_t graph_seed = 0;
  int sweeps_since_recompute = 0;
  int recompute_every        = 0;
  // learned MH proposal
  struct Learned
  {
    bool ready = false;
    MlpTrain t{};
    float* out    = nullptr;
    float* aux    = nullptr;
    int* err      = nullptr;
    double* stats = nullptr;
    cudaGraphExec_t graph = nullptr;
    int g_train = -1, g_drift = -1, g_flush = -1, g_path = -1;
    double g_tau = 0;
    uint64_t g_seed = 0;
    float g_lr = 0;
  } ln;
  EwaldDev<T> ew{};
  double* trace_d = nullptr; // [ne][nw][TRACE_FIELDS] move records of a traced resident sweep
  // diffusion Monte Carlo: weights, previous local energies, ages, branch parameters,
  // ensemble sums, the branch kernel's copy of the weights, population-control sources
  struct Dmc
  {
    bool ready     = false;
    double* weight = nullptr;
    double* e_old  = nullptr;
    int* age       = nullptr;
    double* par    = nullptr; // [5]
    double* sums   = nullptr; // [5]
    double* w_out  = nullptr;
    int* src       = nullptr;
    cudaGraphExec_t graph = nullptr;
    int g_drift = -1, g_flush = -1, g_nt = -1;
    double g_tau   = 0;
    uint64_t g_seed = 0;
  } dm;
  // virtual moves (non-local pseudopotential quadrature points): inputs and ratios on the device
  struct VirtualMoves
  {
    size_t cap     = 0;
    int* walker    = nullptr;
    int* elec      = nullptr;
    double* pos    = nullptr;
    double* ratios = nullptr;
    int* bad       = nullptr; // the first invalid move (INT_MAX: none)
    int* bad_h     = nullptr; // pinned copy
    void release()
    {
      cudaFree(walker);
      cudaFree(elec);
      cudaFree(pos);
      cudaFree(ratios);
      cudaFree(bad);
      if (bad_h)
        cudaFreeHost(bad_h);
      walker = elec = bad = bad_h = nullptr;
      pos = ratios = nullptr;
      cap          = 0;
    }
  } vp;
  double* gl_d    = nullptr; // per-electron gradient [nw][ne][3], then Laplacian [nw][ne], of log psi
  double* e_out  = nullptr; // [3][nw] local energy, kinetic, potential
  double* e_hist = nullptr; // [e_hist_cap][2][nw] per-sweep local and kinetic energies
  size_t e_hist_cap = 0;

  ~Crowd() override
  {
    if (graph)
      cudaGraphExecDestroy(graph);
    if (gauss_h)
      cudaFreeHost(gauss_h);
    if (io.block)
      cudaFreeHost(io.block);
    if (unif_h)
      cudaFreeHost(unif_h);
    if (e_hist)
      cudaFree(e_hist);
    if (ln.graph)
      cudaGraphExecDestroy(ln.graph);
    if (dm.graph)
      cudaGraphExecDestroy(dm.graph);
    vp.release();
    if (ev_fork)
      cudaEventDestroy(ev_fork);
    if (ev_join)
      cudaEventDestroy(ev_join);
    if (side)
      cudaStreamDestroy(side);
    if (stream)
      cudaStreamDestroy(stream);
  }

  int init(qmcg_system sys_, int nw_, int k_)
  {
    sys = sys_;
    nw  = nw_;
    k   = k_;
    CUDA_TRY(setup_move_kernels<T>());
    CUDA_TRY(setup_recompute_kernels<T>());
    CUDA_TRY(setup_sweep_kernel<T>());
    CUDA_TRY(setup_flush_fused<T>());
    int prio_low = 0, prio_high = 0;
    CUDA_TRY(cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high));
    CUDA_TRY(cudaStreamCreateWithPriority(&stream, cudaStreamNonBlocking, prio_high));
    CUDA_TRY(cudaStreamCreateWithPriority(&side, cudaStreamNonBlocking, prio_low));
    CUDA_TRY(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
    CUDA_TRY(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming));
    DevState<T>& d = s;
    d.nw        = nw;
    d.ne        = sys->ne;
    d.ne_pad    = ((sys->ne + 31) / 32) * 32;
    d.nup       = sys->nup;
    d.norb      = sys->norb;
    d.lda       = sys->lda;
    d.nions     = sys->nions;
    d.nions_pad = sys->nions_pad;
    d.k         = k;
    d.coefs     = static_cast<const T*>(sys->coefs);
    d.gx        = sys->grid[0];
    d.gy        = sys->grid[1];
    d.gz        = sys->grid[2];
    d.zs        = sys->lda;
    d.ys        = (long long)(sys->grid[2] + 3) * d.zs;
    d.xs        = (long long)(sys->grid[1] + 3) * d.ys;
    for (int q = 0; q < 3; q++)
    {
      d.L[q] = sys->L[q];
      d.G[q] = 1.0 / sys->L[q];
    }
    d.grid_scale[0] = static_cast<T>(sys->grid[0] / sys->L[0]);
    d.grid_scale[1] = static_cast<T>(sys->grid[1] / sys->L[1]);
    d.grid_scale[2] = static_cast<T>(sys->grid[2] / sys->L[2]);
    d.ions        = static_cast<const T*>(sys->ions);
    d.ion_species = sys->ion_species;
    d.j1_nspecies = sys->nion_species;
    d.j1c         = static_cast<const T*>(sys->j1c);
    d.j1_ncoef    = sys->j1_ncoef;
    d.j1_maxidx   = sys->j1_ncoef - 4;
    d.j1_dri      = static_cast<T>(sys->j1_dri);
    d.j1_rcut     = static_cast<T>(sys->j1_rcut);
    d.j2c         = static_cast<const T*>(sys->j2c);
    d.j2_ncoef    = sys->j2_ncoef;
    d.j2_maxidx   = sys->j2_ncoef - 4;
    d.j2_dri      = static_cast<T>(sys->j2_dri);
    d.j2_rcut     = static_cast<T>(sys->j2_rcut);
    d.has_j1      = sys->has_j1;
    d.has_j2      = sys->has_j2;
    const size_t N = sys->norb, lda = sys->lda, ne_pad = d.ne_pad;
    CUDA_TRY(mem.alloc(&d.R, (size_t)nw * 3 * ne_pad));
    CUDA_TRY(mem.alloc(&d.Rt, (size_t)nw * 3 * ne_pad));
    CUDA_TRY(mem.alloc(&d.Ainv, 2 * (size_t)nw * N * lda));
    CUDA_TRY(mem.alloc(&d.dgrad, 2 * (size_t)nw * N * 3 * lda));
    CUDA_TRY(mem.alloc(&d.dlap, 2 * (size_t)nw * N * lda));
    CUDA_TRY(mem.alloc(&d.psiv, 2 * (size_t)nw * N * lda));
    // a set of delayed-update factors per segment where the segment rows are staged (the
    // block-lazy updates read the sets of a whole spin group), one set otherwise
    d.seg_smem = sweep_seg_smem<T>(d) ? 1 : 0;
    d.nsets    = d.seg_smem ? (std::max(sys->nup, sys->ne - sys->nup) + k - 1) / k : 1;
    const size_t ns = d.nsets;
    CUDA_TRY(mem.alloc(&d.U, 2 * (size_t)nw * ns * k * lda));
    CUDA_TRY(mem.alloc(&d.V, 2 * (size_t)nw * ns * k * lda));
    CUDA_TRY(mem.alloc(&d.Binv, 2 * (size_t)nw * ns * k * k));
    CUDA_TRY(mem.alloc(&d.delay_list, 2 * (size_t)nw * ns * k));
    CUDA_TRY(mem.alloc(&d.J2, (size_t)nw * 5 * ne_pad));
    CUDA_TRY(mem.alloc(&d.J1, (size_t)nw * 5 * ne_pad));
    CUDA_TRY(mem.alloc(&d.log_abs, 2 * (size_t)nw));
    CUDA_TRY(mem.alloc(&d.sign, 2 * (size_t)nw));
    CUDA_TRY(mem.alloc(&d.active_pos, (size_t)nw * 3));
    CUDA_TRY(mem.alloc(&d.disp, (size_t)nw * 3));
    CUDA_TRY(mem.alloc(&d.invRow, (size_t)nw * lda));
    CUDA_TRY(mem.alloc(&d.rcopy, (size_t)nw * lda));
    CUDA_TRY(mem.alloc(&d.phi, (size_t)nw * 5 * lda));
    CUDA_TRY(mem.alloc(&d.cur_det, (size_t)nw));
    CUDA_TRY(mem.alloc(&d.cur_j, (size_t)nw * 10));
    CUDA_TRY(mem.alloc(&d.grads_now, (size_t)nw * 3));
    CUDA_TRY(mem.alloc(&d.grads_new, (size_t)nw * 3));
    CUDA_TRY(mem.alloc(&d.ratios, (size_t)nw));
    CUDA_TRY(mem.alloc(&d.log_gf, (size_t)nw));
    CUDA_TRY(mem.alloc(&d.prob, (size_t)nw));
    CUDA_TRY(mem.alloc(&d.flag, (size_t)nw));
    CUDA_TRY(mem.alloc(&d.accepted, (size_t)nw));
    CUDA_TRY(mem.alloc(&d.status, (size_t)nw));
    CUDA_TRY(mem.alloc(&d.counters, 3));
    CUDA_TRY(mem.alloc(&tc_err, 1));
    if (std::is_same<T, float>::value)
      CUDA_TRY(setup_flush_tc());
    CUDA_TRY(setup_block_update<T>());
    CUDA_TRY(mem.alloc(&d.ucursor, 2));
    CUDA_TRY(mem.alloc(&d.sweep_counter, 1));
    CUDA_TRY(mem.alloc(&Mt, 2 * (size_t)nw * N * N));
    CUDA_TRY(mem.alloc(&d.gj_scratch, 2 * (size_t)nw * gj_scratch_doubles((int)N)));
    CUDA_TRY(mem.alloc(&d.repair_list, (size_t)nw + 1));
    CUDA_TRY(mem.alloc(&aos, std::max<size_t>(1, (size_t)nw * sys->ne * 3)));
    CUDA_TRY(mem.alloc(&jsum, 2 * (size_t)nw));
    CUDA_TRY(mem.alloc(&W, (size_t)nw * k * lda));
    const size_t ng = (size_t)sys->ne * nw * 3, nu = (size_t)sys->ne * nw;
    CUDA_TRY(mem.alloc(&gauss_d, ng));
    CUDA_TRY(mem.alloc(&unif_d, nu));
    CUDA_TRY(cudaMallocHost(&gauss_h, ng * sizeof(double)));
    {
      const size_t nwz = (size_t)nw;
      const size_t bytes = 4 * sizeof(unsigned long long) + 4 * nwz * sizeof(double) + (1 + 3 * nwz) * sizeof(int);
      CUDA_TRY(cudaMallocHost(&io.block, bytes));
      char* b   = static_cast<char*>(io.block);
      io.cnt    = reinterpret_cast<unsigned long long*>(b);
      io.la     = reinterpret_cast<double*>(b + 4 * sizeof(unsigned long long));
      io.js     = io.la + 2 * nwz;
      io.tce    = reinterpret_cast<int*>(io.js + 2 * nwz);
      io.status = io.tce + 1;
      io.sg     = io.status + nwz;
    }
    CUDA_TRY(cudaMallocHost(&unif_h, nu * sizeof(double)));
    sweep_nt   = sweep_default_threads<T>(d);
    CUDA_TRY(sweep_grid<T>(d, &sweep_grid_size, false, sweep_nt));
    CUDA_TRY(setup_local_energy<T>());
    CUDA_TRY(mem.alloc(&e_out, 3 * (size_t)nw));
    ew.ng      = sys->ew_ng;
    ew.nmax    = sys->ewh.nmax;
    ew.gn      = static_cast<const char4*>(sys->ew_gn);
    ew.fg      = static_cast<const T*>(sys->ew_fg);
    ew.rho_ion = static_cast<const T*>(sys->ew_rho);
    ew.ion_q   = static_cast<const T*>(sys->ew_q);
    ew.alpha   = static_cast<T>(sys->ewh.alpha);
    ew.rcut    = static_cast<T>(0.5 * std::min(sys->L[0], std::min(sys->L[1], sys->L[2])));
    ew.e_const = sys->ewh.e_const;
    if (local_energy_smem(sys->ne, ew.nmax, sizeof(T)) > 200 * 1024 || sys->ne > 46340)
      return fail(QMCG_ERR_ARG, "local energy: too many electrons for the shared-memory tables");
    d.gauss     = gauss_d;
    d.uniform   = unif_d;
    d.rng_mode  = 1;
    d.tau       = 0.3;
    d.use_drift = 1;
    CUDA_TRY(cudaDeviceSynchronize());
    return QMCG_OK;
  }

  int check_iat(int iat) const { return (iat >= 0 && iat < sys->ne) ? QMCG_OK : fail(QMCG_ERR_ARG, "iat out of range"); }
  int spin_of(int iat) const { return iat >= sys->nup ? 1 : 0; }

  int load(const double* R) override
  {
    if (!R)
      return fail(QMCG_ERR_ARG, "null positions");
    // one copy of the caller's array as it is (a DMA when the caller's memory is pinned),
    // the layout change on the device
    const int ne = sys->ne, ne_pad = s.ne_pad;
    CUDA_TRY(cudaMemcpyAsync(aos, R, (size_t)nw * ne * 3 * sizeof(double), cudaMemcpyHostToDevice, stream));
    positions_from_caller_kernel<T><<<304, 256, 0, stream>>>(aos, s.R, s.Rt, nw, ne, ne_pad);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaStreamSynchronize(stream));
    return QMCG_OK;
  }

  int positions(double* R) override
  {
    const int ne = sys->ne, ne_pad = s.ne_pad;
    positions_to_caller_kernel<<<304, 256, 0, stream>>>(s.R, aos, nw, ne, ne_pad);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemcpyAsync(R, aos, (size_t)nw * ne * 3 * sizeof(double), cudaMemcpyDeviceToHost, stream));
    CUDA_TRY(cudaStreamSynchronize(stream));
    return QMCG_OK;
  }

  int status_check()
  {
    std::vector<int> st(nw);
    CUDA_TRY(cudaMemcpyAsync(st.data(), s.status, nw * sizeof(int), cudaMemcpyDeviceToHost, stream));
    CUDA_TRY(cudaStreamSynchronize(stream));
    int any = 0;
    for (int v : st)
      any |= v;
    if (any)
    {
      CUDA_TRY(cudaMemsetAsync(s.status, 0, nw * sizeof(int), stream));
      if (any & ST_TIMEOUT)
        return fail(QMCG_ERR_CUDA, "walker-resident sweep: a bounded wait on an asynchronous copy timed out");
      if (any & ST_SINGULAR)
        return fail(QMCG_ERR_SINGULAR, "singular Slater matrix");
      if (any & ST_NONFINITE)
        return fail(QMCG_ERR_NONFINITE, "non-finite ratio or gradient");
      if (any & ST_ZERO_RATIO)
        return fail(QMCG_ERR_ZERO_RATIO, "accepted move with zero determinant ratio");
    }
    return QMCG_OK;
  }

  int recompute_device()
  {
    CUDA_TRY(launch_recompute<T>(s, Mt, 0, stream));
    dc[0] = dc[1] = 0;
    invrow_iat    = -1;
    return QMCG_OK;
  }

  int evaluate_log(double* lp, int* sg) override
  {
    int rc = recompute_device();
    if (rc != QMCG_OK)
      return rc;
    rc = status_check();
    if (rc != QMCG_OK)
      return rc;
    return get_log(lp, sg, nullptr);
  }

  int eval_grad(int iat, double* g) override
  {
    int rc = check_iat(iat);
    if (rc)
      return rc;
    CUDA_TRY(launch_propose<T>(s, iat, dc[spin_of(iat)], 0, stream));
    invrow_iat = iat;
    if (g)
      CUDA_TRY(cudaMemcpyAsync(g, s.grads_now, nw * 3 * sizeof(double), cudaMemcpyDeviceToHost, stream));
    CUDA_TRY(cudaStreamSynchronize(stream));
    return QMCG_OK;
  }

  int make_move(int iat, const double* d) override
  {
    int rc = check_iat(iat);
    if (rc)
      return rc;
    if (!d)
      return fail(QMCG_ERR_ARG, "null displacement");
    CUDA_TRY(cudaMemcpyAsync(s.disp, d, nw * 3 * sizeof(double), cudaMemcpyHostToDevice, stream));
    CUDA_TRY(launch_make_move<T>(s, iat, stream));
    CUDA_TRY(cudaStreamSynchronize(stream));
    return QMCG_OK;
  }

  int ratio_grad(int iat, double* r, double* g) override
  {
    int rc = check_iat(iat);
    if (rc)
      return rc;
    if (invrow_iat != iat)
    {
      // the up-to-date inverse row of iat is prepared on demand (DelayedUpdateBatched::mw_getInvRow)
      CUDA_TRY(launch_propose<T>(s, iat, dc[spin_of(iat)], 0, stream));
      invrow_iat = iat;
    }
    CUDA_TRY(launch_ratio<T>(s, iat, 0, stream));
    if (r)
      CUDA_TRY(cudaMemcpyAsync(r, s.ratios, nw * sizeof(double), cudaMemcpyDeviceToHost, stream));
    if (g)
      CUDA_TRY(cudaMemcpyAsync(g, s.grads_new, nw * 3 * sizeof(double), cudaMemcpyDeviceToHost, stream));
    CUDA_TRY(cudaStreamSynchronize(stream));
    return status_check();
  }

  int flush_spin(int sp)
  {
    if (k > 1 && dc[sp] > 0)
    {
      CUDA_TRY(launch_flush_simt<T>(s, sp, dc[sp], W, stream));
      dc[sp] = 0;
    }
    return QMCG_OK;
  }

  int accept_reject(int iat, const int* acc) override
  {
    int rc = check_iat(iat);
    if (rc)
      return rc;
    if (!acc)
      return fail(QMCG_ERR_ARG, "null accept list");
    if (invrow_iat != iat)
      return fail(QMCG_ERR_STATE, "accept_reject without ratio_grad for this electron");
    std::vector<int> a(nw);
    for (int i = 0; i < nw; i++)
      a[i] = acc[i] ? 1 : 0;
    CUDA_TRY(cudaMemcpyAsync(s.accepted, a.data(), nw * sizeof(int), cudaMemcpyHostToDevice, stream));
    const int sp = spin_of(iat);
    CUDA_TRY(launch_accept<T>(s, iat, dc[sp], 0, stream));
    invrow_iat = -1;
    if (k > 1)
    {
      dc[sp]++;
      if (dc[sp] == k)
      {
        rc = flush_spin(sp);
        if (rc)
          return rc;
      }
    }
    CUDA_TRY(cudaStreamSynchronize(stream));
    return status_check();
  }

  int complete() override
  {
    int rc = flush_spin(0);
    if (rc)
      return rc;
    rc = flush_spin(1);
    if (rc)
      return rc;
    invrow_iat = -1;
    CUDA_TRY(cudaStreamSynchronize(stream));
    return QMCG_OK;
  }

  template<typename X>
  int d2h(std::vector<X>& h, const X* d, size_t n)
  {
    h.resize(n);
    CUDA_TRY(cudaMemcpyAsync(h.data(), d, n * sizeof(X), cudaMemcpyDeviceToHost, stream));
    CUDA_TRY(cudaStreamSynchronize(stream));
    return QMCG_OK;
  }

  // the log|psi| parts of every walker to the pinned staging buffer (asynchronous)
  int enqueue_log()
  {
    jastrow_log_sums_kernel<T><<<(nw + 7) / 8, 256, 0, stream>>>(s.J2, s.J1, nw, sys->ne, s.ne_pad, jsum);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemcpyAsync(io.la, s.log_abs, 2 * (size_t)nw * sizeof(double), cudaMemcpyDeviceToHost, stream));
    CUDA_TRY(cudaMemcpyAsync(io.sg, s.sign, 2 * (size_t)nw * sizeof(int), cudaMemcpyDeviceToHost, stream));
    CUDA_TRY(cudaMemcpyAsync(io.js, jsum, 2 * (size_t)nw * sizeof(double), cudaMemcpyDeviceToHost, stream));
    return QMCG_OK;
  }

  int get_log(double* lp, int* sg, double* parts) override
  {
    int rc = enqueue_log();
    if (rc)
      return rc;
    CUDA_TRY(cudaStreamSynchronize(stream));
    log_from_stage(lp, sg, parts);
    return QMCG_OK;
  }

  // log|psi| = log|det up| + log|det down| + J1 + J2 and the sign, from the staged parts
  void log_from_stage(double* lp, int* sg, double* parts) const
  {
    const double* la = io.la;
    const double* js = io.js;
    const int* sgn   = io.sg;
    for (int iw = 0; iw < nw; iw++)
    {
      const double u2 = js[iw], u1 = js[nw + iw];
      const double lj2 = s.has_j2 ? -0.5 * u2 : 0.0, lj1 = s.has_j1 ? -u1 : 0.0;
      if (lp)
        lp[iw] = la[iw] + la[nw + iw] + lj1 + lj2;
      if (sg)
        sg[iw] = sgn[iw] * sgn[nw + iw];
      if (parts)
      {
        parts[iw * 4 + 0] = la[iw];
        parts[iw * 4 + 1] = la[nw + iw];
        parts[iw * 4 + 2] = lj1;
        parts[iw * 4 + 3] = lj2;
      }
    }
  }

  int get_inverse(int spin, double* a) override
  {
    if (spin < 0 || spin > 1 || !a)
      return fail(QMCG_ERR_ARG, "bad spin or null output");
    const size_t N = sys->norb, lda = sys->lda;
    std::vector<T> h;
    int rc = d2h(h, s.Ainv + (size_t)spin * nw * N * lda, (size_t)nw * N * lda);
    if (rc)
      return rc;
    for (int iw = 0; iw < nw; iw++)
      for (size_t i = 0; i < N; i++)
        for (size_t j = 0; j < N; j++)
          a[((size_t)iw * N + i) * N + j] = static_cast<double>(h[((size_t)iw * N + i) * lda + j]);
    return QMCG_OK;
  }

  int get_jastrow(double* j2o, double* j1o) override
  {
    std::vector<T> j1, j2;
    int rc = d2h(j2, s.J2, (size_t)nw * 5 * s.ne_pad);
    if (!rc)
      rc = d2h(j1, s.J1, (size_t)nw * 5 * s.ne_pad);
    if (rc)
      return rc;
    const int ne = sys->ne;
    for (int iw = 0; iw < nw; iw++)
      for (int q = 0; q < 5; q++)
        for (int e = 0; e < ne; e++)
        {
          if (j2o)
            j2o[((size_t)iw * 5 + q) * ne + e] = static_cast<double>(j2[((size_t)iw * 5 + q) * s.ne_pad + e]);
          if (j1o)
            j1o[((size_t)iw * 5 + q) * ne + e] = static_cast<double>(j1[((size_t)iw * 5 + q) * s.ne_pad + e]);
        }
    return QMCG_OK;
  }

  int get_phi(double* phi) override
  {
    std::vector<T> h;
    int rc = d2h(h, s.phi, (size_t)nw * 5 * s.lda);
    if (rc)
      return rc;
    const int N = sys->norb;
    for (int iw = 0; iw < nw; iw++)
      for (int q = 0; q < 5; q++)
        for (int o = 0; o < N; o++)
          phi[((size_t)iw * 5 + q) * N + o] = static_cast<double>(h[((size_t)iw * 5 + q) * s.lda + o]);
    return QMCG_OK;
  }

  // ---- the sweep as one graph: per electron propose -> ratio -> accept, flush every k
  int enqueue_sweep()
  {
    int d[2] = {0, 0};
    if (s.rng_mode == 0)
      reset_cursor_kernel<<<1, 1, 0, stream>>>(s.ucursor);
    for (int iat = 0; iat < sys->ne; iat++)
    {
      const int sp = spin_of(iat);
      CUDA_TRY(launch_propose<T>(s, iat, d[sp], 1, stream));
      CUDA_TRY(launch_ratio<T>(s, iat, 1, stream));
      CUDA_TRY(launch_accept<T>(s, iat, d[sp], 1, stream));
      if (k > 1)
      {
        d[sp]++;
        if (d[sp] == k)
        {
          CUDA_TRY(launch_flush_simt<T>(s, sp, k, W, stream));
          d[sp] = 0;
        }
      }
    }
    for (int sp = 0; sp < 2; sp++)
      if (k > 1 && d[sp] > 0)
        CUDA_TRY(launch_flush_simt<T>(s, sp, d[sp], W, stream));
    CUDA_TRY(launch_recompute<T>(s, Mt, 1, stream));
    bump_counter_kernel<<<1, 1, 0, stream>>>(s.sweep_counter);
    CUDA_TRY(cudaGetLastError());
    return QMCG_OK;
  }

  bool resident(const qmcg_sweep_params* p) const { return p->rng_mode == 1 && p->path == 0; }

  // the flush of one spin after a resident segment (delayed-update set `set`): tensor cores
  // when asked for and possible (the block-lazy kind flushes with 3xTF32 where it does not apply)
  cudaError_t launch_flush_choice(int spin, int dc, int set = 0, cudaStream_t st = nullptr)
  {
    if (!st)
      st = stream;
    if constexpr (std::is_same<T, float>::value)
      if ((flush_kind == 1 || flush_kind == 3 || flush_kind == 4) && flush_tc_supported(sys->norb, k, sys->lda))
        return launch_flush_tc(crowd_flush_args<float>(s, spin, dc, W, set), flush_kind == 1 ? 1 : 3, tc_err, st);
    return launch_flush_fused<T>(crowd_flush_args<T>(s, spin, dc, W, set), st);
  }

  // block-lazy delayed updates on this sweep (flush kind 4, segment rows staged)
  bool lazy_updates() const { return flush_kind == 4 && k > 1 && block_update_supported<T>(s); }

  // the launches of one spin group of the walker-resident sweep with delayed updates: each
  // segment followed by its flush, or (block-lazy) each segment preceded by the update of
  // its row block and the spin group followed by the completing pass; `seg(i0, i1)` and
  // `upd(launch)` enqueue a segment and an update launch
  template<typename Seg, typename Upd>
  int enqueue_spin_group(int g, Seg&& seg, Upd&& upd, bool defer_complete = false)
  {
    const int first = g ? sys->nup : 0, last = g ? sys->ne : sys->nup;
    const bool lazy = lazy_updates();
    const int nseg  = (last - first + k - 1) / k;
    for (int b = 0; b < nseg; b++)
    {
      const int i0 = first + b * k, i1 = std::min(i0 + k, last);
      if (lazy && b > 0)
      {
        const int rc = upd([=] { return launch_block_update<T>(s, g, b, 1, b, false, stream); });
        if (rc)
          return rc;
      }
      int rc = seg(i0, i1);
      if (rc)
        return rc;
      if (!lazy)
        rc = upd([=] { return launch_flush_choice(g, i1 - i0, s.nsets > 1 ? b : 0); });
      if (rc)
        return rc;
    }
    if (lazy && !defer_complete)
      return upd([=] { return launch_block_update<T>(s, g, 0, nseg, nseg, true, stream); });
    return QMCG_OK;
  }

  // the completing pass of spin g on the side stream, after everything enqueued so far
  cudaError_t fork_complete(int g)
  {
    const int nspin = g ? sys->ne - sys->nup : sys->nup;
    const int nseg  = (nspin + k - 1) / k;
    cudaError_t e   = cudaEventRecord(ev_fork, stream);
    if (e == cudaSuccess)
      e = cudaStreamWaitEvent(side, ev_fork, 0);
    if (e == cudaSuccess)
      e = launch_block_update<T>(s, g, 0, nseg, nseg, true, side);
    if (e == cudaSuccess)
      e = cudaEventRecord(ev_join, side);
    return e;
  }

  // the segments [i0, i1) of one sweep on the walker-resident path, in launch order
  std::vector<std::pair<int, int>> segments() const
  {
    std::vector<std::pair<int, int>> out;
    for (int g = 0; g < 2; g++)
    {
      const int first = g ? sys->nup : 0, last = g ? sys->ne : sys->nup;
      if (k > 1)
        for (int i0 = first; i0 < last; i0 += k)
          out.push_back({i0, std::min(i0 + k, last)});
      else
        out.push_back({first, last});
    }
    return out;
  }

  // one sweep on the walker-resident path: with delayed updates, one resident
  // launch per segment of up to k electrons of one spin group followed by the
  // batched flush of that spin; with rank-1 updates one launch for the sweep
  int enqueue_sweep_resident(bool learned = false)
  {
    const int grid = learned ? sweep_grid_learned : sweep_grid_size;
    if (k > 1)
    {
      // block-lazy: the up spin's completing pass overlaps the down spin's segments
      const bool fork = lazy_updates();
      for (int g = 0; g < 2; g++)
      {
        const int rc = enqueue_spin_group(
            g,
            [&](int i0, int i1) -> int {
              CUDA_TRY(launch_sweep_segment<T>(s, grid, i0, i1, stream, learned, sweep_nt));
              return QMCG_OK;
            },
            [&](auto launch) -> int {
              CUDA_TRY(launch());
              return QMCG_OK;
            },
            fork && g == 0);
        if (rc)
          return rc;
        if (fork && g == 0)
          CUDA_TRY(fork_complete(0));
      }
      if (fork)
        CUDA_TRY(cudaStreamWaitEvent(stream, ev_join, 0));
    }
    else
    {
      CUDA_TRY(launch_sweep_segment<T>(s, grid, 0, sys->nup, stream, learned, sweep_nt));
      CUDA_TRY(launch_sweep_segment<T>(s, grid, sys->nup, sys->ne, stream, learned, sweep_nt));
    }
    CUDA_TRY(launch_recompute<T>(s, Mt, 1, stream));
    bump_counter_kernel<<<1, 1, 0, stream>>>(s.sweep_counter);
    CUDA_TRY(cudaGetLastError());
    return QMCG_OK;
  }

  int build_graph(const qmcg_sweep_params* p)
  {
    if (graph && graph_rng_mode == p->rng_mode && graph_use_drift == p->use_drift && graph_tau == p->tau &&
        graph_seed == p->seed && graph_path == (resident(p) ? 0 : 1) && graph_flush == p->flush &&
        graph_nt == sweep_nt)
      return QMCG_OK;
    if (graph)
    {
      cudaGraphExecDestroy(graph);
      graph = nullptr;
    }
    s.rng_mode  = p->rng_mode;
    s.use_drift = p->use_drift;
    s.tau       = p->tau;
    s.seed      = p->seed;
    flush_kind  = p->flush;
    cudaGraph_t g;
    CUDA_TRY(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    int rc = resident(p) ? enqueue_sweep_resident() : enqueue_sweep();
    cudaError_t e = cudaStreamEndCapture(stream, &g);
    if (rc)
      return rc;
    if (e != cudaSuccess)
      return fail(QMCG_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&graph, g, cudaGraphInstantiateFlagUseNodePriority);
    cudaGraphDestroy(g);
    if (e != cudaSuccess)
      return fail(QMCG_ERR_CUDA, std::string("instantiate: ") + cudaGetErrorString(e));
    graph_rng_mode  = p->rng_mode;
    graph_use_drift = p->use_drift;
    graph_tau       = p->tau;
    graph_seed      = p->seed;
    graph_path      = resident(p) ? 0 : 1;
    graph_flush     = p->flush;
    graph_nt        = sweep_nt;
    return QMCG_OK;
  }

  int sweeps(const qmcg_sweep_params* p, int n, qmcg_sweep_stats* st, int* acc_log) override
  {
    return run_sweeps(p, n, st, acc_log, false);
  }

  // one sweep of the walker-resident path launched outside the graph with the move
  // record switched on; trace_h [ne][nw][TRACE_FIELDS] and acc_log [ne][nw] may be null
  int resident_traced_sweep(double* trace_h, int* acc_log)
  {
    const size_t nrec = (size_t)sys->ne * nw;
    if (!trace_d)
      CUDA_TRY(mem.alloc(&trace_d, nrec * TRACE_FIELDS));
    s.trace = trace_d;
    const int rc = enqueue_sweep_resident();
    s.trace = nullptr;
    if (rc)
      return rc;
    std::vector<double> h;
    double* dst = trace_h;
    if (!dst)
    {
      h.resize(nrec * TRACE_FIELDS);
      dst = h.data();
    }
    CUDA_TRY(cudaMemcpyAsync(dst, trace_d, nrec * TRACE_FIELDS * sizeof(double), cudaMemcpyDeviceToHost, stream));
    CUDA_TRY(cudaStreamSynchronize(stream));
    if (acc_log)
      for (size_t r = 0; r < nrec; r++)
        acc_log[r] = dst[r * TRACE_FIELDS + TR_ACCEPT] != 0.0 ? 1 : 0;
    return QMCG_OK;
  }

  int sweeps_trace(const qmcg_sweep_params* p, int n, qmcg_sweep_stats* st, double* trace) override
  {
    if (!p || !trace)
      return fail(QMCG_ERR_ARG, "null arguments");
    if (!resident(p))
      return fail(QMCG_ERR_ARG, "move records come from the walker-resident path: rng_mode 1 and path 0");
    return run_sweeps(p, n, st, nullptr, false, trace);
  }

  // ------------------------------------------------------------------ diffusion Monte Carlo
  int dmc_init(double* el) override
  {
    if (dc[0] || dc[1])
      return fail(QMCG_ERR_STATE, "DMC needs mw_completeUpdates first");
    if (!dm.ready)
    {
      CUDA_TRY(mem.alloc(&dm.weight, (size_t)nw));
      CUDA_TRY(mem.alloc(&dm.e_old, (size_t)nw));
      CUDA_TRY(mem.alloc(&dm.age, (size_t)nw));
      CUDA_TRY(mem.alloc(&dm.par, 5));
      CUDA_TRY(mem.alloc(&dm.sums, 5));
      CUDA_TRY(mem.alloc(&dm.w_out, (size_t)nw));
      CUDA_TRY(mem.alloc(&dm.src, (size_t)nw));
      CUDA_TRY(mem.alloc(&s.rr, 2 * (size_t)nw));
      dm.ready = true;
    }
    std::vector<double> ones(nw, 1.0);
    CUDA_TRY(cudaMemcpyAsync(dm.weight, ones.data(), nw * sizeof(double), cudaMemcpyHostToDevice, stream));
    CUDA_TRY(cudaMemsetAsync(dm.age, 0, nw * sizeof(int), stream));
    CUDA_TRY(cudaMemsetAsync(s.rr, 0, 2 * nw * sizeof(double), stream));
    CUDA_TRY(launch_local_energy<T>(s, ew, e_out, stream));
    CUDA_TRY(cudaMemcpyAsync(dm.e_old, e_out, nw * sizeof(double), cudaMemcpyDeviceToDevice, stream));
    if (el)
      CUDA_TRY(cudaMemcpyAsync(el, e_out, nw * sizeof(double), cudaMemcpyDeviceToHost, stream));
    CUDA_TRY(cudaStreamSynchronize(stream));
    return status_check();
  }

  // one DMC step: fixed-node sweep, local energy, branch weights (DMCBatched::advanceWalkers)
  int enqueue_dmc_step()
  {
    s.dmc      = 1;
    int rc     = enqueue_sweep_resident();
    s.dmc      = 0;
    if (rc)
      return rc;
    CUDA_TRY(launch_local_energy<T>(s, ew, e_out, stream));
    CUDA_TRY(launch_dmc_branch(nw, e_out, dm.e_old, dm.weight, dm.age, s.rr, dm.par, dm.sums, dm.w_out, stream));
    return QMCG_OK;
  }

  int dmc_step(const qmcg_sweep_params* p, const qmcg_branch_params* b, double* w, double* el, int* age,
               double* sums, qmcg_sweep_stats* st, double* trace) override
  {
    if (!p || !b || !(p->tau > 0))
      return fail(QMCG_ERR_ARG, "bad DMC parameters");
    if (!dm.ready)
      return fail(QMCG_ERR_STATE, "call qmcg_dmc_init first");
    if (!resident(p))
      return fail(QMCG_ERR_ARG, "DMC runs on the walker-resident path: rng_mode 1 and path 0");
    if (!(b->branch_max > b->branch_cutoff))
      return fail(QMCG_ERR_ARG, "branch_max must exceed branch_cutoff");
    if (dc[0] || dc[1])
    {
      const int rc = complete();
      if (rc)
        return rc;
    }
    s.rng_mode  = 1;
    s.use_drift = p->use_drift;
    s.tau       = p->tau;
    s.seed      = p->seed;
    flush_kind  = p->flush;
    const double par[5] = {b->e_trial, b->e_ref, b->tau_eff, b->branch_cutoff, b->branch_max};
    CUDA_TRY(cudaMemcpyAsync(dm.par, par, sizeof(par), cudaMemcpyHostToDevice, stream));
    CUDA_TRY(cudaMemsetAsync(s.counters, 0, 3 * sizeof(unsigned long long), stream));
    if (trace)
    {
      const size_t nrec = (size_t)sys->ne * nw;
      if (!trace_d)
        CUDA_TRY(mem.alloc(&trace_d, nrec * TRACE_FIELDS));
      s.trace = trace_d;
      const int rc = enqueue_dmc_step();
      s.trace      = nullptr;
      if (rc)
        return rc;
      CUDA_TRY(cudaMemcpyAsync(trace, trace_d, nrec * TRACE_FIELDS * sizeof(double), cudaMemcpyDeviceToHost,
                               stream));
    }
    else
    {
      if (!dm.graph || dm.g_drift != p->use_drift || dm.g_tau != p->tau || dm.g_seed != p->seed ||
          dm.g_flush != p->flush || dm.g_nt != sweep_nt)
      {
        if (dm.graph)
          cudaGraphExecDestroy(dm.graph);
        dm.graph = nullptr;
        cudaGraph_t g;
        CUDA_TRY(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        const int rc        = enqueue_dmc_step();
        const cudaError_t e = cudaStreamEndCapture(stream, &g);
        if (rc)
          return rc;
        if (e != cudaSuccess)
          return fail(QMCG_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(e));
        const cudaError_t ei = cudaGraphInstantiate(&dm.graph, g, cudaGraphInstantiateFlagUseNodePriority);
        cudaGraphDestroy(g);
        if (ei != cudaSuccess)
          return fail(QMCG_ERR_CUDA, std::string("instantiate: ") + cudaGetErrorString(ei));
        dm.g_drift = p->use_drift;
        dm.g_tau   = p->tau;
        dm.g_seed  = p->seed;
        dm.g_flush = p->flush;
        dm.g_nt    = sweep_nt;
      }
      CUDA_TRY(cudaGraphLaunch(dm.graph, stream));
    }
    if (w)
      CUDA_TRY(cudaMemcpyAsync(w, dm.w_out, nw * sizeof(double), cudaMemcpyDeviceToHost, stream));
    if (el)
      CUDA_TRY(cudaMemcpyAsync(el, e_out, nw * sizeof(double), cudaMemcpyDeviceToHost, stream));
    if (age)
      CUDA_TRY(cudaMemcpyAsync(age, dm.age, nw * sizeof(int), cudaMemcpyDeviceToHost, stream));
    if (sums)
      CUDA_TRY(cudaMemcpyAsync(sums, dm.sums, 5 * sizeof(double), cudaMemcpyDeviceToHost, stream));
    sweeps_since_recompute++;
    if (p->recompute_every > 0 && sweeps_since_recompute >= p->recompute_every)
    {
      const int rc = recompute_device();
      if (rc)
        return rc;
      sweeps_since_recompute = 0;
    }
    return sync(st);
  }

  // population control on the device: slot i takes walker src[i]
  int dmc_copy(const int* src) override
  {
    if (!src)
      return fail(QMCG_ERR_ARG, "null source list");
    if (!dm.ready)
      return fail(QMCG_ERR_STATE, "call qmcg_dmc_init first");
    if (dc[0] || dc[1])
      return fail(QMCG_ERR_STATE, "delayed updates pending: call qmcg_mw_complete_updates first");
    for (int i = 0; i < nw; i++)
    {
      if (src[i] < 0 || src[i] >= nw)
        return fail(QMCG_ERR_ARG, "source walker out of range");
      if (src[src[i]] != src[i])
        return fail(QMCG_ERR_ARG, "a walker copied elsewhere must keep its own slot (src[src[i]] == src[i])");
    }
    CUDA_TRY(cudaMemcpyAsync(dm.src, src, nw * sizeof(int), cudaMemcpyHostToDevice, stream));
    CUDA_TRY(launch_copy_walkers<T>(s, dm.src, dm.weight, dm.e_old, dm.age, stream));
    CUDA_TRY(cudaStreamSynchronize(stream));
    invrow_iat = -1;
    return QMCG_OK;
  }

  // fixed-count population control: comb of the current weights, then the device copies
  int dmc_reconfigure(double u, int* src_out) override
  {
    if (!dm.ready)
      return fail(QMCG_ERR_STATE, "call qmcg_dmc_init first");
    std::vector<double> w;
    int rc = d2h(w, static_cast<const double*>(dm.weight), (size_t)nw);
    if (rc)
      return rc;
    std::vector<int> src(nw);
    rc = qmcg_dmc_comb(nw, w.data(), u, src.data(), nullptr);
    if (rc)
      return rc;
    rc = dmc_copy(src.data());
    if (rc)
      return rc;
    if (src_out)
      std::copy(src.begin(), src.end(), src_out);
    return QMCG_OK;
  }

  // TrialWaveFunction::mw_evaluateRatios over virtual moves (flat list across walkers)
  int evaluate_ratios(int nvp, const int* walker, const int* elec, const double* pos, double* ratios) override
  {
    if (nvp < 0 || (nvp > 0 && (!walker || !elec || !pos || !ratios)))
      return fail(QMCG_ERR_ARG, "bad virtual-move arguments");
    if (dc[0] || dc[1])
      return fail(QMCG_ERR_STATE, "virtual-move ratios need mw_completeUpdates first");
    if (nvp == 0)
      return QMCG_OK;
    if ((size_t)nvp > vp.cap)
    {
      CUDA_TRY(cudaStreamSynchronize(stream));
      vp.release();
      CUDA_TRY(cudaMalloc(&vp.walker, nvp * sizeof(int)));
      CUDA_TRY(cudaMalloc(&vp.elec, nvp * sizeof(int)));
      CUDA_TRY(cudaMalloc(&vp.pos, 3 * (size_t)nvp * sizeof(double)));
      CUDA_TRY(cudaMalloc(&vp.ratios, nvp * sizeof(double)));
      CUDA_TRY(cudaMalloc(&vp.bad, sizeof(int)));
      CUDA_TRY(cudaMallocHost(&vp.bad_h, sizeof(int)));
      vp.cap = nvp;
    }
    // the moves' walker and electron indices and positions are checked by the kernel
    CUDA_TRY(cudaMemsetAsync(vp.bad, 0x7f, sizeof(int), stream));
    CUDA_TRY(cudaMemcpyAsync(vp.walker, walker, nvp * sizeof(int), cudaMemcpyHostToDevice, stream));
    CUDA_TRY(cudaMemcpyAsync(vp.elec, elec, nvp * sizeof(int), cudaMemcpyHostToDevice, stream));
    CUDA_TRY(cudaMemcpyAsync(vp.pos, pos, 3 * (size_t)nvp * sizeof(double), cudaMemcpyHostToDevice, stream));
    CUDA_TRY(launch_vp_ratios<T>(s, nvp, vp.walker, vp.elec, vp.pos, vp.ratios, vp.bad, stream));
    CUDA_TRY(cudaMemcpyAsync(ratios, vp.ratios, nvp * sizeof(double), cudaMemcpyDeviceToHost, stream));
    CUDA_TRY(cudaMemcpyAsync(vp.bad_h, vp.bad, sizeof(int), cudaMemcpyDeviceToHost, stream));
    CUDA_TRY(cudaStreamSynchronize(stream));
    if (*vp.bad_h != 0x7f7f7f7f)
      return fail(QMCG_ERR_ARG, "virtual move " + std::to_string(*vp.bad_h) +
                                    ": walker or electron out of range, or non-finite position");
    return QMCG_OK;
  }

  // device time of the virtual-move ratio kernel alone: inputs uploaded once, reps launches
  // timed with CUDA events on the crowd's stream
  int profile_ratios(int nvp, const int* walker, const int* elec, const double* pos, int reps, double* ms) override
  {
    if (nvp <= 0 || reps <= 0 || !ms)
      return fail(QMCG_ERR_ARG, "bad profile arguments");
    std::vector<double> r(nvp);
    int rc = evaluate_ratios(nvp, walker, elec, pos, r.data()); // validates, uploads, warms up
    if (rc)
      return rc;
    cudaEvent_t a, b;
    CUDA_TRY(cudaEventCreate(&a));
    CUDA_TRY(cudaEventCreate(&b));
    CUDA_TRY(cudaEventRecord(a, stream));
    for (int i = 0; i < reps; i++)
      CUDA_TRY(launch_vp_ratios<T>(s, nvp, vp.walker, vp.elec, vp.pos, vp.ratios, vp.bad, stream));
    CUDA_TRY(cudaEventRecord(b, stream));
    CUDA_TRY(cudaEventSynchronize(b));
    float t = 0;
    CUDA_TRY(cudaEventElapsedTime(&t, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    *ms = t / reps;
    return QMCG_OK;
  }

  // device time of one periodic FP64 recompute of every walker (CUDA events on the stream)
  int profile_recompute(double* ms) override
  {
    if (!ms)
      return fail(QMCG_ERR_ARG, "null output");
    if (dc[0] || dc[1])
      return fail(QMCG_ERR_STATE, "delayed updates pending: call qmcg_mw_complete_updates first");
    cudaEvent_t a, b;
    CUDA_TRY(cudaEventCreate(&a));
    CUDA_TRY(cudaEventCreate(&b));
    CUDA_TRY(cudaEventRecord(a, stream));
    int rc = recompute_device();
    CUDA_TRY(cudaEventRecord(b, stream));
    CUDA_TRY(cudaEventSynchronize(b));
    float t = 0;
    CUDA_TRY(cudaEventElapsedTime(&t, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (rc)
      return rc;
    *ms = t;
    return status_check();
  }

  // TrialWaveFunction::mw_evaluateGL on the tracked state
  int evaluate_gl(double* lp, double* grads, double* laps) override
  {
    if (dc[0] || dc[1])
      return fail(QMCG_ERR_STATE, "mw_evaluateGL needs mw_completeUpdates first");
    const size_t n = (size_t)nw * sys->ne;
    if (!gl_d)
      CUDA_TRY(mem.alloc(&gl_d, n * 4));
    CUDA_TRY(launch_evaluate_gl<T>(s, gl_d, stream));
    // the kernel writes the caller's layouts: straight copies, no host pass
    if (grads)
      CUDA_TRY(cudaMemcpyAsync(grads, gl_d, 3 * n * sizeof(double), cudaMemcpyDeviceToHost, stream));
    if (laps)
      CUDA_TRY(cudaMemcpyAsync(laps, gl_d + 3 * n, n * sizeof(double), cudaMemcpyDeviceToHost, stream));
    if (lp)
      return get_log(lp, nullptr, nullptr);
    CUDA_TRY(cudaStreamSynchronize(stream));
    return QMCG_OK;
  }

  // QMCHamiltonian::mw_evaluate for kinetic + Coulomb after all delayed updates
  int local_energy(double* el, double* ke, double* vp) override
  {
    if (dc[0] || dc[1])
      return fail(QMCG_ERR_STATE, "local energy needs mw_completeUpdates first");
    CUDA_TRY(launch_local_energy<T>(s, ew, e_out, stream));
    std::vector<double> h(3 * (size_t)nw);
    CUDA_TRY(cudaMemcpyAsync(h.data(), e_out, h.size() * sizeof(double), cudaMemcpyDeviceToHost, stream));
    CUDA_TRY(cudaStreamSynchronize(stream));
    if (el)
      std::copy_n(h.data(), nw, el);
    if (ke)
      std::copy_n(h.data() + nw, nw, ke);
    if (vp)
      std::copy_n(h.data() + 2 * nw, nw, vp);
    return QMCG_OK;
  }

  // sweeps with the local energy measured after each one (into a device history,
  // read back once at the end)
  int sweeps_measure(const qmcg_sweep_params* p, int n, double* el, double* ke, qmcg_sweep_stats* st) override
  {
    if (n < 0 || !el)
      return fail(QMCG_ERR_ARG, "bad arguments");
    const size_t need = (size_t)std::max(n, 1) * 3 * nw;
    if (need > e_hist_cap)
    {
      if (e_hist)
        CUDA_TRY(cudaFree(e_hist));
      e_hist = nullptr;
      CUDA_TRY(cudaMalloc(&e_hist, need * sizeof(double)));
      e_hist_cap = need;
    }
    int rc = run_sweeps(p, n, nullptr, nullptr, true);
    if (rc)
      return rc;
    std::vector<double> h((size_t)n * 3 * nw);
    CUDA_TRY(cudaMemcpyAsync(h.data(), e_hist, h.size() * sizeof(double), cudaMemcpyDeviceToHost, stream));
    rc = sync(st);
    if (rc)
      return rc;
    for (int it = 0; it < n; it++)
    {
      std::copy_n(h.data() + (size_t)it * 3 * nw, nw, el + (size_t)it * nw);
      if (ke)
        std::copy_n(h.data() + ((size_t)it * 3 + 1) * nw, nw, ke + (size_t)it * nw);
    }
    return QMCG_OK;
  }

  // the masked (repair) recompute of the flagged walkers
  int recompute_walkers(const int* flags) override
  {
    if (!flags)
      return fail(QMCG_ERR_ARG, "null flags");
    if (dc[0] || dc[1])
      return fail(QMCG_ERR_STATE, "delayed updates pending: call qmcg_mw_complete_updates first");
    std::vector<int> st(nw);
    for (int i = 0; i < nw; i++)
      st[i] = flags[i] ? ST_ILLCOND : 0;
    CUDA_TRY(cudaMemcpyAsync(s.status, st.data(), nw * sizeof(int), cudaMemcpyHostToDevice, stream));
    CUDA_TRY(launch_recompute<T>(s, Mt, 1, stream));
    CUDA_TRY(cudaStreamSynchronize(stream));
    invrow_iat = -1;
    return status_check();
  }

  int set_threads(int nt) override
  {
    if (nt == 0)
      nt = sweep_default_threads<T>(s);
    if (!sweep_threads_ok(nt, sizeof(T)))
      return fail(QMCG_ERR_ARG, "threads per walker must be 128, 256 or 512 (FP32 only)");
    int grid = 0;
    CUDA_TRY(sweep_grid<T>(s, &grid, false, nt));
    sweep_nt        = nt;
    sweep_grid_size = grid;
    return QMCG_OK;
  }

  // ------------------------------------------------------------------ learned proposal
  int proposal_init(uint64_t seed, double scale) override
  {
    const size_t rows = 2 * (size_t)nw;
    if (!ln.ready)
    {
      CUDA_TRY(setup_learned<T>());
      CUDA_TRY(mem.alloc(&ln.t.params, MP_N));
      CUDA_TRY(mem.alloc(&ln.t.m, MP_N));
      CUDA_TRY(mem.alloc(&ln.t.v, MP_N));
      CUDA_TRY(mem.alloc(&ln.t.grad, MP_N));
      CUDA_TRY(mem.alloc(&ln.t.wimg, (size_t)ML_WIMG_BYTES));
      CUDA_TRY(mem.alloc(&ln.t.wsimt, (size_t)ML_WSIMT_BYTES));
      s.mlp_simt   = ln.t.wsimt;
      s.mlp_params = ln.t.params;
      CUDA_TRY(sweep_grid<T>(s, &sweep_grid_learned, true));
      CUDA_TRY(mem.alloc(&ln.t.x, rows * ML_IN));
      CUDA_TRY(mem.alloc(&ln.t.hid, 3 * rows * ML_H));
      CUDA_TRY(mem.alloc(&ln.t.g4, rows * 8));
      CUDA_TRY(mem.alloc(&ln.t.delta, 3 * rows * ML_H));
      CUDA_TRY(mem.alloc(&ln.t.step, 1));
      CUDA_TRY(mem.alloc(&ln.out, rows * 8));
      CUDA_TRY(mem.alloc(&ln.aux, (size_t)nw * ML_AUX));
      CUDA_TRY(mem.alloc(&ln.err, 1));
      CUDA_TRY(mem.alloc(&ln.stats, 3));
    }
    // uniform(-a, a) with a = scale / sqrt(fan_in) for the hidden layers; the output
    // layer starts at zero, so the initial proposal is drift-diffusion
    std::vector<float> h(MP_N, 0.f);
    std::mt19937_64 g(seed);
    std::uniform_real_distribution<double> u(-1.0, 1.0);
    for (int n = 0; n < ML_H; n++)
      for (int k = 0; k < ML_NIN; k++)
        h[MP_W1 + n * ML_IN + k] = static_cast<float>(scale / std::sqrt((double)ML_NIN) * u(g));
    for (int l = 0; l < 2; l++)
      for (int i = 0; i < ML_H * ML_H; i++)
        h[(l ? MP_W3 : MP_W2) + i] = static_cast<float>(scale / std::sqrt((double)ML_H) * u(g));
    ln.ready = true;
    return proposal_params(nullptr, h.data());
  }

  int proposal_params(float* get, const float* set) override
  {
    if (!ln.ready)
      return fail(QMCG_ERR_STATE, "proposal not initialised (qmcg_proposal_init)");
    if (set)
    {
      CUDA_TRY(cudaMemcpyAsync(ln.t.params, set, MP_N * sizeof(float), cudaMemcpyHostToDevice, stream));
      CUDA_TRY(cudaMemsetAsync(ln.t.m, 0, MP_N * sizeof(float), stream));
      CUDA_TRY(cudaMemsetAsync(ln.t.v, 0, MP_N * sizeof(float), stream));
      CUDA_TRY(cudaMemsetAsync(ln.t.step, 0, sizeof(int), stream));
      CUDA_TRY(launch_mlp_pack(ln.t.params, ln.t.wimg, ln.t.wsimt, stream));
    }
    if (get)
      CUDA_TRY(cudaMemcpyAsync(get, ln.t.params, MP_N * sizeof(float), cudaMemcpyDeviceToHost, stream));
    CUDA_TRY(cudaStreamSynchronize(stream));
    return QMCG_OK;
  }

  MlpArgs mlp_args(int rows, const __nv_bfloat16* x, __nv_bfloat16* hid, int hid_rows, int hid_row0, float* out)
  {
    MlpArgs a;
    a.rows     = rows;
    a.x        = x;
    a.wimg     = ln.t.wimg;
    a.params   = ln.t.params;
    a.hid      = hid;
    a.hid_rows = hid_rows;
    a.hid_row0 = hid_row0;
    a.out      = out;
    a.aux      = ln.aux;
    a.err      = ln.err;
    return a;
  }

  // the network on caller inputs x [rows][64] (rounded to BF16): out [rows][6] and
  // optionally the hidden activations [3][rows][128]
  int proposal_forward(int rows, const float* x, float* out, float* hidden) override
  {
    if (!ln.ready)
      return fail(QMCG_ERR_STATE, "proposal not initialised (qmcg_proposal_init)");
    if (rows <= 0 || !x || !out)
      return fail(QMCG_ERR_ARG, "bad arguments");
    return mlp_host_pass(rows, x, out, hidden, nullptr, nullptr);
  }

  int proposal_backward(int rows, const float* x, const float* dout, float* grad) override
  {
    if (!ln.ready)
      return fail(QMCG_ERR_STATE, "proposal not initialised (qmcg_proposal_init)");
    if (rows <= 0 || !x || !dout || !grad)
      return fail(QMCG_ERR_ARG, "bad arguments");
    return mlp_host_pass(rows, x, nullptr, nullptr, dout, grad);
  }

  int mlp_host_pass(int rows, const float* x, float* out, float* hidden, const float* dout, float* grad)
  {
    DeviceArena tmp;
    __nv_bfloat16 *dx, *dh;
    float *dout_d, *g4, *delta, *dgrad;
    CUDA_TRY(tmp.alloc(&dx, (size_t)rows * ML_IN));
    CUDA_TRY(tmp.alloc(&dh, (size_t)3 * rows * ML_H));
    CUDA_TRY(tmp.alloc(&dout_d, (size_t)rows * 8));
    std::vector<uint16_t> xb((size_t)rows * ML_IN);
    for (size_t i = 0; i < xb.size(); i++)
      xb[i] = f2bf(x[i]);
    CUDA_TRY(cudaMemcpy(dx, xb.data(), xb.size() * 2, cudaMemcpyHostToDevice));
    MlpArgs a = mlp_args(rows, dx, dh, rows, 0, dout_d);
    CUDA_TRY(launch_mlp_forward<T>(a, s, 0, 0, stream));
    int err = 0;
    CUDA_TRY(cudaMemcpyAsync(&err, ln.err, sizeof(int), cudaMemcpyDeviceToHost, stream));
    CUDA_TRY(cudaStreamSynchronize(stream));
    if (err)
    {
      CUDA_TRY(cudaMemset(ln.err, 0, sizeof(int)));
      return fail(QMCG_ERR_CUDA, "proposal network: a tensor-core wait timed out");
    }
    if (out)
    {
      std::vector<float> o((size_t)rows * 8);
      CUDA_TRY(cudaMemcpy(o.data(), dout_d, o.size() * 4, cudaMemcpyDeviceToHost));
      for (int r = 0; r < rows; r++)
        for (int q = 0; q < ML_NOUT; q++)
          out[(size_t)r * ML_NOUT + q] = o[(size_t)r * 8 + q];
    }
    if (hidden)
    {
      std::vector<uint16_t> hb((size_t)3 * rows * ML_H);
      CUDA_TRY(cudaMemcpy(hb.data(), dh, hb.size() * 2, cudaMemcpyDeviceToHost));
      for (size_t i = 0; i < hb.size(); i++)
        hidden[i] = bf2f(hb[i]);
    }
    if (dout)
    {
      CUDA_TRY(tmp.alloc(&g4, (size_t)rows * 8));
      CUDA_TRY(tmp.alloc(&delta, (size_t)3 * rows * ML_H));
      CUDA_TRY(tmp.alloc(&dgrad, (size_t)MP_N));
      std::vector<float> gh((size_t)rows * 8, 0.f);
      for (int r = 0; r < rows; r++)
        for (int q = 0; q < ML_NOUT; q++)
          gh[(size_t)r * 8 + q] = dout[(size_t)r * ML_NOUT + q];
      CUDA_TRY(cudaMemcpy(g4, gh.data(), gh.size() * 4, cudaMemcpyHostToDevice));
      MlpTrain t = ln.t;
      t.x        = dx;
      t.hid      = dh;
      t.g4       = g4;
      t.delta    = delta;
      t.grad     = dgrad;
      CUDA_TRY(launch_mlp_backward(t, rows, stream));
      CUDA_TRY(cudaStreamSynchronize(stream));
      CUDA_TRY(cudaMemcpy(grad, dgrad, MP_N * sizeof(float), cudaMemcpyDeviceToHost));
    }
    return QMCG_OK;
  }

  // features of electron iat for every walker at its current position (after
  // mw_evalGrad) or at the proposed one (after mw_calcRatioGrad): x [nw][64]
  int proposal_features(int iat, int at_proposed, float* x) override
  {
    if (!ln.ready)
      return fail(QMCG_ERR_STATE, "proposal not initialised (qmcg_proposal_init)");
    int rc = check_iat(iat);
    if (rc)
      return rc;
    CUDA_TRY(launch_features<T>(s, iat, at_proposed ? 1 : 0, ln.t.x, stream));
    std::vector<uint16_t> xb((size_t)nw * ML_IN);
    CUDA_TRY(cudaMemcpyAsync(xb.data(), ln.t.x, xb.size() * 2, cudaMemcpyDeviceToHost, stream));
    CUDA_TRY(cudaStreamSynchronize(stream));
    for (size_t i = 0; i < xb.size(); i++)
      x[i] = bf2f(xb[i]);
    return QMCG_OK;
  }

  // one sweep with the learned proposal (staged per-electron kernels), optionally
  // with one training step per electron
  int enqueue_sweep_learned(bool train, float lr)
  {
    int d[2] = {0, 0};
    const int rows = 2 * nw;
    __nv_bfloat16* xf = ln.t.x;
    __nv_bfloat16* xr = ln.t.x + (size_t)nw * ML_IN;
    const MlpArgs af  = mlp_args(nw, xf, train ? ln.t.hid : nullptr, rows, 0, nullptr);
    const MlpArgs ar  = mlp_args(nw, xr, train ? ln.t.hid : nullptr, rows, nw, nullptr);
    for (int iat = 0; iat < sys->ne; iat++)
    {
      const int sp = spin_of(iat);
      CUDA_TRY(launch_propose<T>(s, iat, d[sp], 0, stream));
      CUDA_TRY(launch_features<T>(s, iat, 0, xf, stream));
      CUDA_TRY(launch_mlp_forward<T>(af, s, iat, 1, stream));
      CUDA_TRY(launch_ratio<T>(s, iat, 0, stream));
      CUDA_TRY(launch_features<T>(s, iat, 1, xr, stream));
      CUDA_TRY(launch_mlp_forward<T>(ar, s, iat, 2, stream));
      if (train)
      {
        CUDA_TRY(launch_mlp_loss_grad<T>(s, ln.aux, ln.t.g4, ln.stats, stream));
        CUDA_TRY(launch_mlp_backward(ln.t, rows, stream));
        CUDA_TRY(launch_mlp_adam(ln.t, lr, stream));
      }
      CUDA_TRY(launch_accept<T>(s, iat, d[sp], 1, stream));
      if (k > 1)
      {
        d[sp]++;
        if (d[sp] == k)
        {
          CUDA_TRY(launch_flush_choice(sp, k));
          d[sp] = 0;
        }
      }
    }
    for (int sp = 0; sp < 2; sp++)
      if (k > 1 && d[sp] > 0)
        CUDA_TRY(launch_flush_choice(sp, d[sp]));
    CUDA_TRY(launch_recompute<T>(s, Mt, 1, stream));
    bump_counter_kernel<<<1, 1, 0, stream>>>(s.sweep_counter);
    CUDA_TRY(cudaGetLastError());
    return QMCG_OK;
  }

  int sweeps_learned(const qmcg_sweep_params* p, int n, int train, double lr, double* el, qmcg_sweep_stats* st,
                     double* tstats) override
  {
    if (!ln.ready)
      return fail(QMCG_ERR_STATE, "proposal not initialised (qmcg_proposal_init)");
    if (!p || n < 0 || !(p->tau > 0) || p->rng_mode != 1)
      return fail(QMCG_ERR_ARG, "learned sweeps need tau > 0 and the device random numbers (rng_mode 1)");
    if (dc[0] || dc[1])
    {
      int rc = complete();
      if (rc)
        return rc;
    }
    const float flr = static_cast<float>(lr);
    const int gpath = (!train && p->path == 0) ? 0 : 1; // inference on the walker-resident kernel
    if (!ln.graph || ln.g_train != (train ? 1 : 0) || ln.g_tau != p->tau || ln.g_seed != p->seed ||
        ln.g_lr != flr || ln.g_flush != p->flush || ln.g_drift != p->use_drift || ln.g_path != gpath)
    {
      if (ln.graph)
      {
        cudaGraphExecDestroy(ln.graph);
        ln.graph = nullptr;
      }
      // the sweep graph of the plain path must be rebuilt after this
      if (graph)
      {
        cudaGraphExecDestroy(graph);
        graph = nullptr;
      }
      s.rng_mode  = 1;
      s.use_drift = p->use_drift;
      s.tau       = p->tau;
      s.seed      = p->seed;
      flush_kind  = p->flush;
      cudaGraph_t g;
      CUDA_TRY(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
      int rc        = gpath == 0 ? enqueue_sweep_resident(true) : enqueue_sweep_learned(train != 0, flr);
      cudaError_t e = cudaStreamEndCapture(stream, &g);
      if (rc)
        return rc;
      if (e != cudaSuccess)
        return fail(QMCG_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(e));
      e = cudaGraphInstantiate(&ln.graph, g, cudaGraphInstantiateFlagUseNodePriority);
      cudaGraphDestroy(g);
      if (e != cudaSuccess)
        return fail(QMCG_ERR_CUDA, std::string("instantiate: ") + cudaGetErrorString(e));
      ln.g_train = train ? 1 : 0;
      ln.g_tau   = p->tau;
      ln.g_seed  = p->seed;
      ln.g_lr    = flr;
      ln.g_flush = p->flush;
      ln.g_drift = p->use_drift;
      ln.g_path  = gpath;
    }
    if (el)
    {
      const size_t need = (size_t)std::max(n, 1) * 3 * nw;
      if (need > e_hist_cap)
      {
        if (e_hist)
          CUDA_TRY(cudaFree(e_hist));
        e_hist = nullptr;
        CUDA_TRY(cudaMalloc(&e_hist, need * sizeof(double)));
        e_hist_cap = need;
      }
    }
    recompute_every = p->recompute_every;
    CUDA_TRY(cudaMemsetAsync(s.counters, 0, 3 * sizeof(unsigned long long), stream));
    CUDA_TRY(cudaMemsetAsync(ln.stats, 0, 3 * sizeof(double), stream));
    for (int it = 0; it < n; it++)
    {
      CUDA_TRY(cudaGraphLaunch(ln.graph, stream));
      if (el)
        CUDA_TRY(launch_local_energy<T>(s, ew, e_hist + (size_t)it * 3 * nw, stream));
      sweeps_since_recompute++;
      if (p->recompute_every > 0 && sweeps_since_recompute >= p->recompute_every)
      {
        int rc = recompute_device();
        if (rc)
          return rc;
        sweeps_since_recompute = 0;
      }
    }
    double hs2[3];
    int err = 0;
    CUDA_TRY(cudaMemcpyAsync(hs2, ln.stats, sizeof(hs2), cudaMemcpyDeviceToHost, stream));
    CUDA_TRY(cudaMemcpyAsync(&err, ln.err, sizeof(int), cudaMemcpyDeviceToHost, stream));
    std::vector<double> h;
    if (el)
    {
      h.resize((size_t)n * 3 * nw);
      CUDA_TRY(cudaMemcpyAsync(h.data(), e_hist, h.size() * sizeof(double), cudaMemcpyDeviceToHost, stream));
    }
    int rc = sync(st);
    if (rc)
      return rc;
    if (err)
    {
      CUDA_TRY(cudaMemset(ln.err, 0, sizeof(int)));
      return fail(QMCG_ERR_CUDA, "proposal network: a tensor-core wait timed out");
    }
    if (el)
      for (int it = 0; it < n; it++)
        std::copy_n(h.data() + (size_t)it * 3 * nw, nw, el + (size_t)it * nw);
    if (tstats)
    {
      const double moves = (double)n * sys->ne * nw;
      tstats[0]          = train ? hs2[0] / moves : 0.0; // mean alpha |r' - r|^2 over training moves
      tstats[1]          = train ? hs2[1] / moves : 0.0; // mean alpha
      tstats[2]          = train ? hs2[2] / moves : 0.0; // mean training objective (lower is better)
    }
    return QMCG_OK;
  }

  int run_sweeps(const qmcg_sweep_params* p, int n, qmcg_sweep_stats* st, int* acc_log, bool measure,
                 double* trace = nullptr, bool defer_sync = false)
  {
    if (!p || n < 0 || !(p->tau > 0) || (p->rng_mode != 0 && p->rng_mode != 1))
      return fail(QMCG_ERR_ARG, "bad sweep parameters");
    if (dc[0] || dc[1])
    {
      int rc = complete();
      if (rc)
        return rc;
    }
    if (p->rng_mode == 0 && (!stream_seeded || hs_seed != p->seed))
    {
      hs.seed(p->seed);
      hs_seed       = p->seed;
      stream_seeded = true;
    }
    int rc = build_graph(p);
    if (rc)
      return rc;
    recompute_every = p->recompute_every;
    CUDA_TRY(cudaMemsetAsync(s.counters, 0, 3 * sizeof(unsigned long long), stream));
    const size_t ng = (size_t)sys->ne * nw * 3, nu = (size_t)sys->ne * nw;
    std::vector<int> accbuf;
    for (int it = 0; it < n; it++)
    {
      if (p->rng_mode == 0)
      {
        hs.gauss(gauss_h, ng);
        hs.peek_uniforms(unif_h, nu);
        CUDA_TRY(cudaMemcpyAsync(gauss_d, gauss_h, ng * sizeof(double), cudaMemcpyHostToDevice, stream));
        CUDA_TRY(cudaMemcpyAsync(unif_d, unif_h, nu * sizeof(double), cudaMemcpyHostToDevice, stream));
      }
      if (resident(p) && (acc_log || trace))
      {
        // the walker-resident kernel records its own moves
        const size_t nrec = (size_t)sys->ne * nw;
        rc = resident_traced_sweep(trace ? trace + (size_t)it * nrec * TRACE_FIELDS : nullptr,
                                   acc_log ? acc_log + (size_t)it * nrec : nullptr);
        if (rc)
          return rc;
      }
      else if (acc_log)
      {
        // electron-by-electron launches so the decisions can be logged
        rc = sweep_logged(acc_log + (size_t)it * sys->ne * nw);
        if (rc)
          return rc;
      }
      else
        CUDA_TRY(cudaGraphLaunch(graph, stream));
      if (measure)
        CUDA_TRY(launch_local_energy<T>(s, ew, e_hist + (size_t)it * 3 * nw, stream));
      if (p->rng_mode == 0)
      {
        int used[2];
        CUDA_TRY(cudaMemcpyAsync(used, s.ucursor, 2 * sizeof(int), cudaMemcpyDeviceToHost, stream));
        CUDA_TRY(cudaStreamSynchronize(stream));
        hs.consume(static_cast<size_t>(used[sys->ne & 1]));
      }
      sweeps_since_recompute++;
      if (p->recompute_every > 0 && sweeps_since_recompute >= p->recompute_every)
      {
        rc = recompute_device();
        if (rc)
          return rc;
        sweeps_since_recompute = 0;
      }
    }
    return measure || defer_sync ? QMCG_OK : sync(st);
  }

  // positions from the caller's host buffer, n sweeps, positions and log|psi| back to host
  // buffers, with one synchronisation at the end (every copy is stream-ordered; pinned
  // buffers make them DMA transfers)
  int sweeps_host(const qmcg_sweep_params* p, int n, const double* r_in, double* r_out, double* lp,
                  qmcg_sweep_stats* st) override
  {
    const int ne = sys->ne, ne_pad = s.ne_pad;
    const size_t bytes = (size_t)nw * ne * 3 * sizeof(double);
    if (r_in)
    {
      CUDA_TRY(cudaMemcpyAsync(aos, r_in, bytes, cudaMemcpyHostToDevice, stream));
      positions_from_caller_kernel<T><<<304, 256, 0, stream>>>(aos, s.R, s.Rt, nw, ne, ne_pad);
      CUDA_TRY(cudaGetLastError());
    }
    int rc = run_sweeps(p, n, nullptr, nullptr, false, nullptr, true);
    if (rc)
      return rc;
    if (r_out)
    {
      positions_to_caller_kernel<<<304, 256, 0, stream>>>(s.R, aos, nw, ne, ne_pad);
      CUDA_TRY(cudaGetLastError());
      CUDA_TRY(cudaMemcpyAsync(r_out, aos, bytes, cudaMemcpyDeviceToHost, stream));
    }
    if (lp && (rc = enqueue_log()))
      return rc;
    if ((rc = enqueue_stats()))
      return rc;
    CUDA_TRY(cudaStreamSynchronize(stream));
    if (lp)
      log_from_stage(lp, nullptr, nullptr);
    return finish_stats(st);
  }

  int sweep_logged(int* acc_log)
  {
    int d[2] = {0, 0};
    if (s.rng_mode == 0)
      reset_cursor_kernel<<<1, 1, 0, stream>>>(s.ucursor);
    for (int iat = 0; iat < sys->ne; iat++)
    {
      const int sp = spin_of(iat);
      CUDA_TRY(launch_propose<T>(s, iat, d[sp], 1, stream));
      CUDA_TRY(launch_ratio<T>(s, iat, 1, stream));
      CUDA_TRY(launch_accept<T>(s, iat, d[sp], 1, stream));
      CUDA_TRY(cudaMemcpyAsync(acc_log + (size_t)iat * nw, s.accepted, nw * sizeof(int), cudaMemcpyDeviceToHost,
                               stream));
      if (k > 1)
      {
        d[sp]++;
        if (d[sp] == k)
        {
          CUDA_TRY(launch_flush_simt<T>(s, sp, k, W, stream));
          d[sp] = 0;
        }
      }
    }
    for (int sp = 0; sp < 2; sp++)
      if (k > 1 && d[sp] > 0)
        CUDA_TRY(launch_flush_simt<T>(s, sp, d[sp], W, stream));
    CUDA_TRY(launch_recompute<T>(s, Mt, 1, stream));
    bump_counter_kernel<<<1, 1, 0, stream>>>(s.sweep_counter);
    CUDA_TRY(cudaStreamSynchronize(stream));
    return QMCG_OK;
  }

  int sweeps_async(int n) override
  {
    if (!graph || graph_rng_mode != 1)
      return fail(QMCG_ERR_STATE, "no device-RNG sweep graph built yet");
    for (int it = 0; it < n; it++)
    {
      CUDA_TRY(cudaGraphLaunch(graph, stream));
      sweeps_since_recompute++;
      if (recompute_every > 0 && sweeps_since_recompute >= recompute_every)
      {
        int rc = recompute_device();
        if (rc)
          return rc;
        sweeps_since_recompute = 0;
      }
    }
    return QMCG_OK;
  }

  // Device time of the walker-resident path over n real sweeps, split by kernel:
  // out[0] = ms per sweep-kernel launch, out[1] = ms per flush launch,
  // out[2] = sweep-kernel launches per sweep, out[3] = flush launches per sweep.
  // CUDA events on the crowd's stream around every launch; the repair and counter
  // kernels run between sweeps untimed.
  int sweep_info(int flush, int* out) override
  {
    if (!out)
      return fail(QMCG_ERR_ARG, "null output");
    out[0] = sweep_nt;
    out[1] = s.seg_smem;
    out[2] = s.nsets;
    out[3] = flush == 4 && k > 1 && block_update_supported<T>(s) ? 1 : 0;
    return QMCG_OK;
  }

  int profile_sweep(int n, double* out) override
  {
    if (n <= 0 || !out)
      return fail(QMCG_ERR_ARG, "bad profile arguments");
    if (!graph || graph_path != 0)
      return fail(QMCG_ERR_STATE, "no walker-resident sweep graph built yet");
    struct Rec
    {
      cudaEvent_t a, b;
      int flush;
    };
    std::vector<Rec> recs;
    auto timed = [&](int is_flush, auto&& launch) -> int {
      Rec r{nullptr, nullptr, is_flush};
      CUDA_TRY(cudaEventCreate(&r.a));
      CUDA_TRY(cudaEventCreate(&r.b));
      CUDA_TRY(cudaEventRecord(r.a, stream));
      CUDA_TRY(launch());
      CUDA_TRY(cudaEventRecord(r.b, stream));
      recs.push_back(r);
      return QMCG_OK;
    };
    int nsk = 0, nfl = 0;
    for (int it = 0; it < n; it++)
    {
      if (k > 1)
      {
        for (int g = 0; g < 2; g++)
        {
          const int rc = enqueue_spin_group(
              g,
              [&](int i0, int i1) {
                nsk += it == 0;
                return timed(0, [&] {
                  return launch_sweep_segment<T>(s, sweep_grid_size, i0, i1, stream, false, sweep_nt);
                });
              },
              [&](auto launch) {
                nfl += it == 0;
                return timed(1, launch);
              });
          if (rc)
            return rc;
        }
      }
      else
      {
        for (int g = 0; g < 2; g++)
        {
          const int first = g ? sys->nup : 0, last = g ? sys->ne : sys->nup;
          int rc = timed(0, [&] { return launch_sweep_segment<T>(s, sweep_grid_size, first, last, stream, false,
                                                                sweep_nt); });
          if (rc)
            return rc;
          if (it == 0)
            nsk++;
        }
      }
      CUDA_TRY(launch_recompute<T>(s, Mt, 1, stream));
      bump_counter_kernel<<<1, 1, 0, stream>>>(s.sweep_counter);
    }
    CUDA_TRY(cudaStreamSynchronize(stream));
    double ts = 0, tf = 0;
    int cs = 0, cf = 0;
    for (auto& r : recs)
    {
      float t = 0;
      CUDA_TRY(cudaEventElapsedTime(&t, r.a, r.b));
      if (r.flush)
      {
        tf += t;
        cf++;
      }
      else
      {
        ts += t;
        cs++;
      }
      cudaEventDestroy(r.a);
      cudaEventDestroy(r.b);
    }
    out[0] = cs ? ts / cs : 0.0;
    out[1] = cf ? tf / cf : 0.0;
    out[2] = nsk;
    out[3] = nfl;
    return QMCG_OK;
  }

  // Per-launch device time of ratio_kernel over niat consecutive electrons, each
  // preceded by its (untimed) proposal; CUDA events on the crowd's stream.  Only
  // move scratch is written, the walker state is left unchanged.
  int profile_ratio(int niat, double* ms) override
  {
    if (niat <= 0 || !ms)
      return fail(QMCG_ERR_ARG, "bad profile arguments");
    if (dc[0] || dc[1])
      return fail(QMCG_ERR_STATE, "pending delayed updates; call complete_updates first");
    std::vector<cudaEvent_t> ev(2 * (size_t)niat);
    for (auto& e : ev)
      CUDA_TRY(cudaEventCreate(&e));
    for (int i = 0; i < niat; i++)
    {
      const int iat = i % sys->ne;
      CUDA_TRY(launch_propose<T>(s, iat, 0, 1, stream));
      CUDA_TRY(cudaEventRecord(ev[2 * i], stream));
      CUDA_TRY(launch_ratio<T>(s, iat, 1, stream));
      CUDA_TRY(cudaEventRecord(ev[2 * i + 1], stream));
    }
    CUDA_TRY(cudaStreamSynchronize(stream));
    double tot = 0;
    for (int i = 0; i < niat; i++)
    {
      float t = 0;
      CUDA_TRY(cudaEventElapsedTime(&t, ev[2 * i], ev[2 * i + 1]));
      tot += t;
    }
    for (auto& e : ev)
      cudaEventDestroy(e);
    invrow_iat = -1;
    *ms        = tot / niat;
    return QMCG_OK;
  }

  // the sweep counters, the flush error flag and the status words to the pinned staging
  // buffer (asynchronous)
  int enqueue_stats()
  {
    CUDA_TRY(cudaMemcpyAsync(io.tce, tc_err, sizeof(int), cudaMemcpyDeviceToHost, stream));
    CUDA_TRY(cudaMemcpyAsync(io.cnt, s.counters, 3 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, stream));
    CUDA_TRY(cudaMemcpyAsync(io.status, s.status, nw * sizeof(int), cudaMemcpyDeviceToHost, stream));
    return QMCG_OK;
  }

  int sync(qmcg_sweep_stats* st) override
  {
    int rc = enqueue_stats();
    if (rc)
      return rc;
    CUDA_TRY(cudaStreamSynchronize(stream));
    return finish_stats(st);
  }

  // after the stream synchronised: the staged counters into st, the status words cleared,
  // the flags turned into a status code
  int finish_stats(qmcg_sweep_stats* st)
  {
    const unsigned long long* c = io.cnt;
    const int tce = *io.tce;
    int any = 0;
    for (int iw = 0; iw < nw; iw++)
      any |= io.status[iw];
    CUDA_TRY(cudaMemsetAsync(s.status, 0, nw * sizeof(int), stream));
    if (st)
    {
      st->accepted = c[0];
      st->rejected = c[1];
      st->repaired = c[2];
      st->status   = any;
    }
    if (tce)
    {
      CUDA_TRY(cudaMemsetAsync(tc_err, 0, sizeof(int), stream));
      return fail(QMCG_ERR_CUDA, "tensor-core flush: an mbarrier wait timed out");
    }
    if (any & ST_TIMEOUT)
      return fail(QMCG_ERR_CUDA, "walker-resident sweep: a bounded wait on an asynchronous copy timed out");
    if (any & ST_SINGULAR)
      return fail(QMCG_ERR_SINGULAR, "singular Slater matrix");
    if (any & ST_NONFINITE)
      return fail(QMCG_ERR_NONFINITE, "non-finite ratio or gradient");
    if (any & ST_ZERO_RATIO)
      return fail(QMCG_ERR_ZERO_RATIO, "accepted move with zero determinant ratio");
    return QMCG_OK;
  }
};

// ---------------------------------------------------------------------------
// crowds of different systems swept together: one persistent launch per stage
// ---------------------------------------------------------------------------
struct qmcg_group_s
{
  virtual ~qmcg_group_s() = default;
  virtual int sweeps(const qmcg_sweep_params* p, int n, qmcg_sweep_stats* st) = 0;
  virtual int info(int* out) = 0;
};

template<typename T>
struct Group final : qmcg_group_s
{
  std::vector<Crowd<T>*> cs;
  cudaStream_t stream = nullptr; // the first crowd's stream
  DeviceArena mem;
  DevState<T>* table = nullptr;
  int* work          = nullptr; // one dynamic work counter per stage
  std::vector<MultiStage> stages;
  size_t smem = 0;
  int grid    = 0;
  int nt      = 128; // threads per walker of the group launch
  cudaGraphExec_t graph = nullptr;
  double g_tau = 0;
  uint64_t g_seed = 0;
  int g_drift = -1, g_flush = -1;
  std::vector<int> since_recompute;

  cudaEvent_t ev_stage = nullptr; // end of a stage's launch: the crowds' updates fork from it

  ~Group() override
  {
    if (graph)
      cudaGraphExecDestroy(graph);
    if (ev_stage)
      cudaEventDestroy(ev_stage);
  }

  int init(const std::vector<Crowd<T>*>& crowds)
  {
    cs     = crowds;
    stream = cs[0]->stream;
    CUDA_TRY(cudaEventCreateWithFlags(&ev_stage, cudaEventDisableTiming));
    since_recompute.assign(cs.size(), 0);
    for (auto* c : cs)
      smem = std::max(smem, sweep_smem_bytes<T>(c->s));
    if (smem > 220 * 1024)
      return fail(QMCG_ERR_ARG, "group: a crowd's walker state does not fit in shared memory");
    // one CTA size for the launch: 256 threads per walker when any crowd runs more than 128 alone
    nt = 128;
    for (auto* c : cs)
      if (c->sweep_nt > 128)
        nt = 256;
    CUDA_TRY(sweep_multi_grid<T>(smem, &grid, nt));
    CUDA_TRY(mem.alloc(&table, cs.size()));
    // stages: the j-th segment of every crowd; crowds ordered by cost per walker (largest first)
    std::vector<int> order(cs.size());
    for (size_t c = 0; c < cs.size(); c++)
      order[c] = (int)c;
    std::sort(order.begin(), order.end(), [&](int a, int b) {
      const double ca = (double)cs[a]->sys->ne * cs[a]->sys->lda, cb = (double)cs[b]->sys->ne * cs[b]->sys->lda;
      return ca > cb;
    });
    // a crowd with m segments places segment j in stage floor(j * S / m), S the largest m,
    // so every crowd progresses through its sweep at the same pace
    size_t nst = 0;
    for (auto* c : cs)
      nst = std::max(nst, c->segments().size());
    for (size_t j = 0; j < nst; j++)
    {
      MultiStage st{};
      st.nactive = 0;
      st.begin[0] = 0;
      for (int c : order)
      {
        const auto seg = cs[c]->segments();
        const size_t m = seg.size();
        int hit        = -1;
        for (size_t q = 0; q < m; q++)
          if ((q * nst) / m == j)
            hit = (int)q;
        if (hit < 0)
          continue;
        const int a = st.nactive++;
        st.crowd[a]     = c;
        st.i0[a]        = seg[hit].first;
        st.i1[a]        = seg[hit].second;
        st.begin[a + 1] = st.begin[a] + cs[c]->nw;
      }
      if (st.nactive > 0)
        stages.push_back(st);
    }
    CUDA_TRY(mem.alloc(&work, stages.size()));
    return QMCG_OK;
  }

  int build(const qmcg_sweep_params* p)
  {
    if (graph && g_tau == p->tau && g_seed == p->seed && g_drift == p->use_drift && g_flush == p->flush)
      return QMCG_OK;
    if (graph)
    {
      cudaGraphExecDestroy(graph);
      graph = nullptr;
    }
    std::vector<DevState<T>> h(cs.size());
    for (size_t c = 0; c < cs.size(); c++)
    {
      Crowd<T>* x = cs[c];
      if (x->graph)
      {
        cudaGraphExecDestroy(x->graph);
        x->graph = nullptr;
      }
      x->s.rng_mode  = 1;
      x->s.use_drift = p->use_drift;
      x->s.tau       = p->tau;
      // independent counter-based streams per crowd
      x->s.seed   = p->seed ^ (0x9E3779B97F4A7C15ull * (uint64_t)(c + 1));
      x->flush_kind = p->flush;
      h[c]        = x->s;
    }
    CUDA_TRY(cudaMemcpy(table, h.data(), h.size() * sizeof(DevState<T>), cudaMemcpyHostToDevice));
    cudaGraph_t g;
    CUDA_TRY(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    int rc = enqueue();
    cudaError_t e = cudaStreamEndCapture(stream, &g);
    if (rc)
      return rc;
    if (e != cudaSuccess)
      return fail(QMCG_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&graph, g, cudaGraphInstantiateFlagUseNodePriority);
    cudaGraphDestroy(g);
    if (e != cudaSuccess)
      return fail(QMCG_ERR_CUDA, std::string("instantiate: ") + cudaGetErrorString(e));
    g_tau   = p->tau;
    g_seed  = p->seed;
    g_drift = p->use_drift;
    g_flush = p->flush;
    return QMCG_OK;
  }

  int enqueue()
  {
    CUDA_TRY(cudaMemsetAsync(work, 0, stages.size() * sizeof(int), stream));
    for (size_t j = 0; j < stages.size(); j++)
    {
      const MultiStage& st = stages[j];
      CUDA_TRY(launch_sweep_multi<T>(table, st, smem, grid, work + j, stream, nt));
      // the crowds' updates after the stage run side by side, each on its crowd's side
      // stream, and the next stage waits for all of them
      CUDA_TRY(cudaEventRecord(ev_stage, stream));
      for (int a = 0; a < st.nactive; a++)
      {
        Crowd<T>* x = cs[st.crowd[a]];
        if (x->k > 1)
        {
          CUDA_TRY(cudaStreamWaitEvent(x->side, ev_stage, 0));
          const int sp = st.i0[a] >= x->sys->nup ? 1 : 0, first = sp ? x->sys->nup : 0;
          const int blk = (st.i0[a] - first) / x->k;
          if (x->lazy_updates())
          {
            // block-lazy: the crowd's next row block of this spin group receives the sets so
            // far before its segment (a later stage), or the spin group is completed
            const int nspin = sp ? x->sys->ne - x->sys->nup : x->sys->nup;
            const int nseg  = (nspin + x->k - 1) / x->k;
            if (blk + 1 < nseg)
              CUDA_TRY(launch_block_update<T>(x->s, sp, blk + 1, 1, blk + 1, false, x->side));
            else
              CUDA_TRY(launch_block_update<T>(x->s, sp, 0, nseg, nseg, true, x->side));
          }
          else
            CUDA_TRY(x->launch_flush_choice(sp, st.i1[a] - st.i0[a], x->s.nsets > 1 ? blk : 0, x->side));
          CUDA_TRY(cudaEventRecord(x->ev_join, x->side));
          CUDA_TRY(cudaStreamWaitEvent(stream, x->ev_join, 0));
        }
      }
    }
    // the crowds' masked repairs, side by side
    CUDA_TRY(cudaEventRecord(ev_stage, stream));
    for (auto* x : cs)
    {
      CUDA_TRY(cudaStreamWaitEvent(x->side, ev_stage, 0));
      CUDA_TRY(launch_recompute<T>(x->s, x->Mt, 1, x->side));
      bump_counter_kernel<<<1, 1, 0, x->side>>>(x->s.sweep_counter);
      CUDA_TRY(cudaGetLastError());
      CUDA_TRY(cudaEventRecord(x->ev_join, x->side));
      CUDA_TRY(cudaStreamWaitEvent(stream, x->ev_join, 0));
    }
    return QMCG_OK;
  }

  int sweeps(const qmcg_sweep_params* p, int n, qmcg_sweep_stats* st) override
  {
    if (!p || n < 0 || !(p->tau > 0) || p->rng_mode != 1)
      return fail(QMCG_ERR_ARG, "group sweeps need tau > 0 and the device random numbers (rng_mode 1)");
    for (auto* x : cs)
      if (x->dc[0] || x->dc[1])
      {
        int rc = x->complete();
        if (rc)
          return rc;
      }
    // every crowd's pending work is ordered before the group's stream
    for (auto* x : cs)
      CUDA_TRY(cudaStreamSynchronize(x->stream));
    int rc = build(p);
    if (rc)
      return rc;
    for (auto* x : cs)
      CUDA_TRY(cudaMemsetAsync(x->s.counters, 0, 3 * sizeof(unsigned long long), stream));
    for (int it = 0; it < n; it++)
    {
      CUDA_TRY(cudaGraphLaunch(graph, stream));
      for (size_t c = 0; c < cs.size(); c++)
        if (p->recompute_every > 0 && ++since_recompute[c] >= p->recompute_every)
        {
          CUDA_TRY(launch_recompute<T>(cs[c]->s, cs[c]->Mt, 0, stream));
          since_recompute[c] = 0;
        }
    }
    CUDA_TRY(cudaStreamSynchronize(stream));
    for (size_t c = 0; c < cs.size(); c++)
    {
      rc = cs[c]->sync(st ? st + c : nullptr);
      if (rc)
        return rc;
    }
    return QMCG_OK;
  }

  // out: [0] stages per sweep, [1] CTAs of the persistent launch, [2] shared memory bytes per CTA,
  // [3] threads per CTA
  int info(int* out) override
  {
    out[0] = (int)stages.size();
    out[1] = grid;
    out[2] = (int)smem;
    out[3] = nt;
    return QMCG_OK;
  }
};

extern "C" int qmcg_group_create(const qmcg_crowd* crowds, int n, qmcg_group* out)
{
  if (!crowds || !out || n < 1 || n > MULTI_MAX)
    return fail(QMCG_ERR_ARG, "need 1..8 crowds");
  *out = nullptr;
  for (int c = 0; c < n; c++)
    if (!crowds[c] || crowds[c]->sys->prec != crowds[0]->sys->prec)
      return fail(QMCG_ERR_ARG, "group crowds must exist and share one precision");
  auto make = [&](auto tag) -> int {
    using TT = decltype(tag);
    std::vector<Crowd<TT>*> v;
    for (int c = 0; c < n; c++)
      v.push_back(static_cast<Crowd<TT>*>(crowds[c]));
    auto g = std::make_unique<Group<TT>>();
    int rc = g->init(v);
    if (rc)
      return rc;
    *out = g.release();
    return QMCG_OK;
  };
  return crowds[0]->sys->prec == 8 ? make(double{}) : make(float{});
}

extern "C" int qmcg_group_destroy(qmcg_group g)
{
  delete g;
  return QMCG_OK;
}

extern "C" int qmcg_group_sweeps(qmcg_group g, const qmcg_sweep_params* p, int n, qmcg_sweep_stats* stats)
{
  if (!g)
    return fail(QMCG_ERR_ARG, "null group");
  return g->sweeps(p, n, stats);
}

extern "C" int qmcg_group_info(qmcg_group g, int* out)
{
  if (!g || !out)
    return fail(QMCG_ERR_ARG, "null argument");
  return g->info(out);
}

extern "C" int qmcg_crowd_create(qmcg_system sys, int nw, int k, qmcg_crowd* out)
{
  if (!sys || !out || nw <= 0 || k <= 0 || k > sys->norb)
    return fail(QMCG_ERR_ARG, "bad crowd arguments (need 1 <= delay_rank <= num_orbitals)");
  *out = nullptr;
  std::unique_ptr<qmcg_crowd_s> c;
  int rc;
  if (sys->prec == 8)
  {
    auto* p = new Crowd<double>();
    c.reset(p);
    rc = p->init(sys, nw, k);
  }
  else
  {
    auto* p = new Crowd<float>();
    c.reset(p);
    rc = p->init(sys, nw, k);
  }
  if (rc != QMCG_OK)
    return rc;
  *out = c.release();
  return QMCG_OK;
}

extern "C" int qmcg_crowd_destroy(qmcg_crowd c)
{
  delete c;
  return QMCG_OK;
}

extern "C" int qmcg_crowd_stream(qmcg_crowd c, void** stream)
{
  if (!c || !stream)
    return fail(QMCG_ERR_ARG, "null argument");
  *stream = c->stream;
  return QMCG_OK;
}

#define CROWD_CALL(c, call)                                                                                            \
  do                                                                                                                   \
  {                                                                                                                    \
    if (!(c))                                                                                                          \
      return fail(QMCG_ERR_ARG, "null crowd");                                                                         \
    return (c)->call;                                                                                                  \
  } while (0)

extern "C" int qmcg_load_walkers(qmcg_crowd c, const double* R) { CROWD_CALL(c, load(R)); }
extern "C" int qmcg_get_positions(qmcg_crowd c, double* R) { CROWD_CALL(c, positions(R)); }
extern "C" int qmcg_mw_evaluate_log(qmcg_crowd c, double* lp, int* sg) { CROWD_CALL(c, evaluate_log(lp, sg)); }
extern "C" int qmcg_mw_recompute_walkers(qmcg_crowd c, const int* flags) { CROWD_CALL(c, recompute_walkers(flags)); }
extern "C" int qmcg_mw_prepare_group(qmcg_crowd c, int group)
{
  if (!c || group < 0 || group > 1)
    return fail(QMCG_ERR_ARG, "bad group");
  return QMCG_OK;
}
extern "C" int qmcg_mw_eval_grad(qmcg_crowd c, int iat, double* g) { CROWD_CALL(c, eval_grad(iat, g)); }
extern "C" int qmcg_mw_make_move(qmcg_crowd c, int iat, const double* d, int* valid)
{
  if (!c)
    return fail(QMCG_ERR_ARG, "null crowd");
  if (valid)
    for (int i = 0; i < c->nw; i++)
      valid[i] = 1;
  return c->make_move(iat, d);
}
extern "C" int qmcg_mw_calc_ratio_grad(qmcg_crowd c, int iat, double* r, double* g)
{
  CROWD_CALL(c, ratio_grad(iat, r, g));
}
extern "C" int qmcg_mw_accept_reject_move(qmcg_crowd c, int iat, const int* acc)
{
  CROWD_CALL(c, accept_reject(iat, acc));
}
extern "C" int qmcg_mw_complete_updates(qmcg_crowd c) { CROWD_CALL(c, complete()); }
extern "C" int qmcg_get_log(qmcg_crowd c, double* lp, int* sg, double* parts) { CROWD_CALL(c, get_log(lp, sg, parts)); }
extern "C" int qmcg_get_inverse(qmcg_crowd c, int spin, double* a) { CROWD_CALL(c, get_inverse(spin, a)); }
extern "C" int qmcg_get_jastrow_state(qmcg_crowd c, double* j2, double* j1) { CROWD_CALL(c, get_jastrow(j2, j1)); }
extern "C" int qmcg_get_phi_vgl(qmcg_crowd c, double* phi)
{
  if (!phi)
    return fail(QMCG_ERR_ARG, "null output");
  CROWD_CALL(c, get_phi(phi));
}
extern "C" int qmcg_vmc_sweeps(qmcg_crowd c, const qmcg_sweep_params* p, int n, qmcg_sweep_stats* st, int* acc)
{
  CROWD_CALL(c, sweeps(p, n, st, acc));
}
extern "C" int qmcg_vmc_sweeps_async(qmcg_crowd c, int n) { CROWD_CALL(c, sweeps_async(n)); }
extern "C" int qmcg_vmc_sweeps_host(qmcg_crowd c, const qmcg_sweep_params* p, int n, const double* r_in,
                                    double* r_out, double* log_psi, qmcg_sweep_stats* st)
{
  CROWD_CALL(c, sweeps_host(p, n, r_in, r_out, log_psi, st));
}
extern "C" int qmcg_proposal_init(qmcg_crowd c, uint64_t seed, double init_scale)
{
  CROWD_CALL(c, proposal_init(seed, init_scale));
}
extern "C" int qmcg_proposal_get_params(qmcg_crowd c, float* params)
{
  if (!params)
    return fail(QMCG_ERR_ARG, "null output");
  CROWD_CALL(c, proposal_params(params, nullptr));
}
extern "C" int qmcg_proposal_set_params(qmcg_crowd c, const float* params)
{
  if (!params)
    return fail(QMCG_ERR_ARG, "null input");
  CROWD_CALL(c, proposal_params(nullptr, params));
}
extern "C" int qmcg_proposal_forward(qmcg_crowd c, int rows, const float* x, float* out, float* hidden)
{
  CROWD_CALL(c, proposal_forward(rows, x, out, hidden));
}
extern "C" int qmcg_proposal_backward(qmcg_crowd c, int rows, const float* x, const float* dout, float* grad)
{
  CROWD_CALL(c, proposal_backward(rows, x, dout, grad));
}
extern "C" int qmcg_proposal_features(qmcg_crowd c, int iat, int at_proposed, float* x)
{
  if (!x)
    return fail(QMCG_ERR_ARG, "null output");
  CROWD_CALL(c, proposal_features(iat, at_proposed, x));
}
extern "C" int qmcg_vmc_sweeps_learned(qmcg_crowd c, const qmcg_sweep_params* p, int n, int train, double lr,
                                       double* e_local, qmcg_sweep_stats* st, double* train_stats)
{
  CROWD_CALL(c, sweeps_learned(p, n, train, lr, e_local, st, train_stats));
}
extern "C" int qmcg_crowd_set_threads(qmcg_crowd c, int threads) { CROWD_CALL(c, set_threads(threads)); }
extern "C" int qmcg_mw_evaluate_local_energy(qmcg_crowd c, double* el, double* ke, double* vp)
{
  CROWD_CALL(c, local_energy(el, ke, vp));
}
extern "C" int qmcg_vmc_sweeps_measure(qmcg_crowd c, const qmcg_sweep_params* p, int n, double* el, double* ke,
                                       qmcg_sweep_stats* st)
{
  CROWD_CALL(c, sweeps_measure(p, n, el, ke, st));
}
extern "C" int qmcg_crowd_sync(qmcg_crowd c, qmcg_sweep_stats* st) { CROWD_CALL(c, sync(st)); }
extern "C" int qmcg_vmc_sweeps_trace(qmcg_crowd c, const qmcg_sweep_params* p, int n, qmcg_sweep_stats* st,
                                     double* trace)
{
  static_assert(QMCG_TRACE_FIELDS == TRACE_FIELDS, "trace record layout");
  CROWD_CALL(c, sweeps_trace(p, n, st, trace));
}
extern "C" int qmcg_profile_recompute(qmcg_crowd c, double* ms) { CROWD_CALL(c, profile_recompute(ms)); }
extern "C" int qmcg_dmc_init(qmcg_crowd c, double* el) { CROWD_CALL(c, dmc_init(el)); }
extern "C" int qmcg_dmc_step(qmcg_crowd c, const qmcg_sweep_params* p, const qmcg_branch_params* b, double* w,
                             double* el, int* age, double* sums, qmcg_sweep_stats* st, double* trace)
{
  CROWD_CALL(c, dmc_step(p, b, w, el, age, sums, st, trace));
}
extern "C" int qmcg_dmc_copy_walkers(qmcg_crowd c, const int* src) { CROWD_CALL(c, dmc_copy(src)); }
extern "C" int qmcg_dmc_reconfigure(qmcg_crowd c, double u, int* src) { CROWD_CALL(c, dmc_reconfigure(u, src)); }
extern "C" int qmcg_profile_ratios(qmcg_crowd c, int nvp, const int* walker, const int* elec, const double* pos,
                                   int reps, double* ms)
{
  CROWD_CALL(c, profile_ratios(nvp, walker, elec, pos, reps, ms));
}
extern "C" int qmcg_mw_evaluate_ratios(qmcg_crowd c, int nvp, const int* walker, const int* elec, const double* pos,
                                       double* ratios)
{
  CROWD_CALL(c, evaluate_ratios(nvp, walker, elec, pos, ratios));
}
extern "C" int qmcg_mw_evaluate_gl(qmcg_crowd c, double* lp, double* grads, double* laps)
{
  CROWD_CALL(c, evaluate_gl(lp, grads, laps));
}
extern "C" int qmcg_profile_ratio(qmcg_crowd c, int niat, double* ms) { CROWD_CALL(c, profile_ratio(niat, ms)); }
extern "C" int qmcg_profile_sweep(qmcg_crowd c, int n, double* ms) { CROWD_CALL(c, profile_sweep(n, ms)); }
extern "C" int qmcg_sweep_info(qmcg_crowd c, int flush, int* out) { CROWD_CALL(c, sweep_info(flush, out)); }

// ---------------------------------------------------------------------------
// determinant-engine flush on caller device buffers
// (DelayedUpdateBatched::mw_updateInvMat, DelayedUpdateBatched.h:675-738)
// ---------------------------------------------------------------------------
extern "C" int qmcg_mw_update_inv_mat(int precision, int nw, int n, int lda, int k, int dc, void* ainv, const void* u,
                                      const void* v, const void* binv, const int* delay_list, void* stream);

static int check_flush_args(int prec, int nw, int n, int lda, int k, int dc, void* ainv, const void* u,
                            const void* v, const void* binv, const int* dl)
{
  if (prec != 4 && prec != 8)
    return fail(QMCG_ERR_ARG, "precision must be 4 or 8");
  if (nw < 0 || n <= 0 || lda < n || k <= 0 || dc < 0 || dc > k)
    return fail(QMCG_ERR_ARG, "need n > 0, lda >= n, 0 <= delay_count <= delay_rank");
  if (nw > 0 && dc > 0 && (!ainv || !u || !v || !binv || !dl))
    return fail(QMCG_ERR_ARG, "null device buffer");
  return QMCG_OK;
}

template<typename T>
static FlushArgs<T> make_flush_args(int nw, int n, int lda, int k, int dc, void* ainv, const void* u, const void* v,
                                    const void* binv, const int* dl, T* w)
{
  FlushArgs<T> f;
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
  f.w          = w;
  return f;
}

template<typename T>
static int flush_with_malloc(int nw, int n, int lda, int k, int dc, void* ainv, const void* u, const void* v,
                             const void* binv, const int* dl, cudaStream_t st)
{
  CUDA_TRY(setup_move_kernels<T>());
  if (flush_fused_fits<T>(n, k))
  {
    // shared-memory tiles, no scratch
    CUDA_TRY(setup_flush_fused<T>());
    CUDA_TRY(launch_flush_fused(make_flush_args<T>(nw, n, lda, k, dc, ainv, u, v, binv, dl, nullptr), st));
    return QMCG_OK;
  }
  T* w = nullptr;
  CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&w), std::max<size_t>(1, (size_t)nw * k * lda) * sizeof(T), st));
  const cudaError_t e = launch_flush_args(make_flush_args<T>(nw, n, lda, k, dc, ainv, u, v, binv, dl, w), st);
  CUDA_TRY(cudaFreeAsync(w, st));
  CUDA_TRY(e);
  return QMCG_OK;
}

extern "C" int qmcg_mw_update_inv_mat_ex(int precision, int nw, int n, int lda, int k, int dc, void* ainv,
                                         const void* u, const void* v, const void* binv, const int* delay_list,
                                         int method, void* stream)
{
  if (method == 0)
    return qmcg_mw_update_inv_mat(precision, nw, n, lda, k, dc, ainv, u, v, binv, delay_list, stream);
  if (method != 1 && method != 3)
    return fail(QMCG_ERR_ARG, "method must be 0, 1 or 3");
  int rc = check_flush_args(precision, nw, n, lda, k, dc, ainv, u, v, binv, delay_list);
  if (rc)
    return rc;
  if (precision != 4 || !flush_tc_supported(n, k, lda))
    return fail(QMCG_ERR_ARG, "tensor-core flush needs precision 4, delay_rank <= 64, n and lda multiples of 4");
  if (((uintptr_t)ainv | (uintptr_t)u | (uintptr_t)v) & 15)
    return fail(QMCG_ERR_ARG, "tensor-core flush needs ainv, u and v on 16-byte boundaries");
  if (nw == 0 || dc == 0)
    return QMCG_OK;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  CUDA_TRY(setup_flush_tc());
  int* err = nullptr;
  CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&err), sizeof(int), st));
  CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), st));
  const cudaError_t e =
      launch_flush_tc(make_flush_args<float>(nw, n, lda, k, dc, ainv, u, v, binv, delay_list, nullptr), method, err, st);
  int herr = 0;
  CUDA_TRY(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaFreeAsync(err, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  CUDA_TRY(e);
  if (herr)
    return fail(QMCG_ERR_CUDA, "tensor-core flush: an mbarrier wait timed out");
  return QMCG_OK;
}

extern "C" int qmcg_mw_update_inv_mat(int precision, int nw, int n, int lda, int k, int dc, void* ainv, const void* u,
                                      const void* v, const void* binv, const int* delay_list, void* stream)
{
  int rc = check_flush_args(precision, nw, n, lda, k, dc, ainv, u, v, binv, delay_list);
  if (rc)
    return rc;
  if (nw == 0 || dc == 0)
    return QMCG_OK;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  return precision == 8 ? flush_with_malloc<double>(nw, n, lda, k, dc, ainv, u, v, binv, delay_list, st)
                        : flush_with_malloc<float>(nw, n, lda, k, dc, ainv, u, v, binv, delay_list, st);
}
