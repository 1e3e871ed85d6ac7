// Host-side launch interface between the translation units of the library.
#pragma once
#include <cuda_runtime.h>
#include <string>
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
cudaError_t launch_sweep(const DevState<T>& s, T* W, int grid, cudaStream_t st);

// recompute path (recompute_kernels.cu)
template<typename T>
cudaError_t launch_recompute(const DevState<T>& s, double* mscratch, cudaStream_t st);
} // namespace qmcg
