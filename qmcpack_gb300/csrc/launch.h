// Host-side launch interface between the translation units of the library.
#pragma once
#include <cuda_runtime.h>
#include <string>
#include <vector>
#include "common.cuh"

namespace qmcg
{
// records the message returned by qmcg_last_error() and returns code
int set_error(int code, const std::string& msg);

template<typename T>
cudaError_t launch_propose(const DevState<T>& s, int iat, int dc, int driver, cudaStream_t st);
template<typename T>
cudaError_t launch_make_move(const DevState<T>& s, int iat, cudaStream_t st);
template<typename T>
cudaError_t launch_ratio(const DevState<T>& s, int iat, int driver, cudaStream_t st);
template<typename T>
cudaError_t launch_accept(const DevState<T>& s, int iat, int dc, int driver, cudaStream_t st);
template<typename T>
cudaError_t launch_flush_simt(const DevState<T>& s, int spin, int dc, T* W, cudaStream_t st);
template<typename T>
cudaError_t launch_flush_args(const FlushArgs<T>& f, cudaStream_t st);

template<typename T>
cudaError_t setup_move_kernels();
template<typename T>
cudaError_t setup_recompute_kernels();

// walker-resident sweep (sweep_kernel.cu)
template<typename T>
cudaError_t setup_sweep_kernel();
template<typename T>
size_t sweep_smem_bytes(const DevState<T>& s);
template<typename T>
cudaError_t sweep_grid(const DevState<T>& s, int* grid);
template<typename T>
cudaError_t launch_sweep_segment(const DevState<T>& s, int grid, int i0, int i1, cudaStream_t st);
// batched, shared-memory-staged flush of one spin for all walkers (flush_kernels.cu);
// falls back to the two-kernel SIMT flush when the tiles do not fit
template<typename T>
cudaError_t launch_flush_fused(const FlushArgs<T>& f, cudaStream_t st);
template<typename T>
cudaError_t setup_flush_fused();
// the fused flush needs no global scratch when its tiles fit in shared memory
template<typename T>
bool flush_fused_fits(int n, int k);

// tensor-core flush (flush_tc.cu), FP32 only: terms 1 = TF32, 3 = 3xTF32
bool flush_tc_supported(int n, int k, int lda);
cudaError_t setup_flush_tc();
cudaError_t launch_flush_tc(const FlushArgs<float>& f, int terms, int* err, cudaStream_t st);

// flush arguments of one spin of a crowd
template<typename T>
inline FlushArgs<T> crowd_flush_args(const DevState<T>& s, int spin, int dc, T* W)
{
  FlushArgs<T> f;
  f.nw         = s.nw;
  f.n          = s.norb;
  f.lda        = s.lda;
  f.k          = s.k;
  f.dc         = dc;
  f.sA         = (long long)s.norb * s.lda;
  f.sU         = (long long)s.k * s.lda;
  f.sB         = (long long)s.k * s.k;
  f.sD         = s.k;
  f.ainv       = s.Ainv + (size_t)spin * s.nw * f.sA;
  f.u          = s.U + (size_t)spin * s.nw * f.sU;
  f.v          = s.V + (size_t)spin * s.nw * f.sU;
  f.binv       = s.Binv + (size_t)spin * s.nw * f.sB;
  f.delay_list = s.delay_list + (size_t)spin * s.nw * f.sD;
  f.w          = W;
  return f;
}

// local energy (energy.cu)
struct EwaldHost
{
  double alpha = 0, e_const = 0;
  int nmax     = 0;
  std::vector<char4> gn;
  std::vector<double> fg, rho_ion;
};
int ewald_build(const double L[3], int ne, int nions, const double* ion_pos, const double* ion_q, double eps,
                EwaldHost& t);
size_t local_energy_smem(int ne, int nmax, int tsize);
template<typename T>
cudaError_t setup_local_energy();
// out: [3][nw] doubles = local energy, kinetic, potential
template<typename T>
cudaError_t launch_local_energy(const DevState<T>& s, const EwaldDev<T>& ew, double* out, cudaStream_t st);

// recompute path (recompute_kernels.cu)
template<typename T>
cudaError_t launch_recompute(const DevState<T>& s, double* mscratch, int masked, cudaStream_t st);
} // namespace qmcg
