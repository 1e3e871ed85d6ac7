// Host-side launch interface between the translation units of the library.
#pragma once
#include <cuda_bf16.h>
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
size_t sweep_smem_bytes(const DevState<T>& s, bool learned = false);
// whether a segment's inverse rows can be staged in shared memory without enlarging the footprint
template<typename T>
bool sweep_seg_smem(const DevState<T>& s);
template<typename T>
cudaError_t sweep_grid(const DevState<T>& s, int* grid, bool learned = false, int threads = 128);
template<typename T>
int sweep_default_threads(const DevState<T>& s);
bool sweep_threads_ok(int threads, int tsize);
template<typename T>
cudaError_t launch_sweep_segment(const DevState<T>& s, int grid, int i0, int i1, cudaStream_t st,
                                 bool learned = false, int threads = 128);
// uneven crowds: one launch per stage over (crowd, walker) work items
constexpr int MULTI_MAX = 8;
struct MultiStage
{
  int nactive;                 // crowds with a segment in this stage
  int crowd[MULTI_MAX];        // their indices in the state table, most expensive first
  int i0[MULTI_MAX], i1[MULTI_MAX];
  int begin[MULTI_MAX + 1];    // prefix of walker counts: items [begin[a], begin[a+1]) belong to crowd[a]
};
template<typename T>
cudaError_t launch_sweep_multi(const DevState<T>* table, const MultiStage& st, size_t smem, int grid, int* work,
                               cudaStream_t stm, int threads);
template<typename T>
cudaError_t sweep_multi_grid(size_t smem, int* grid, int threads);
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

// flush arguments of one spin of a crowd, delayed-update set `set`
template<typename T>
inline FlushArgs<T> crowd_flush_args(const DevState<T>& s, int spin, int dc, T* W, int set = 0)
{
  FlushArgs<T> f;
  f.nw         = s.nw;
  f.n          = s.norb;
  f.lda        = s.lda;
  f.k          = s.k;
  f.dc         = dc;
  f.sA         = (long long)s.norb * s.lda;
  f.sU         = (long long)s.nsets * s.k * s.lda;
  f.sB         = (long long)s.nsets * s.k * s.k;
  f.sD         = s.nsets * s.k;
  f.ainv       = s.Ainv + (size_t)spin * s.nw * f.sA;
  f.u          = s.U + (size_t)spin * s.nw * f.sU + (size_t)set * s.k * s.lda;
  f.v          = s.V + (size_t)spin * s.nw * f.sU + (size_t)set * s.k * s.lda;
  f.binv       = s.Binv + (size_t)spin * s.nw * f.sB + (size_t)set * s.k * s.k;
  f.delay_list = s.delay_list + (size_t)spin * s.nw * f.sD + (size_t)set * s.k;
  f.w          = W;
  return f;
}

// block-lazy delayed updates of the walker-resident sweep (block_update.cu): the row block
// `block` (and, with complete, every block from it on: grid y = nblocks) of one spin
// receives the sets it has not seen: [0, set_hi) before the segment that reads it, or
// [block, set_hi) at the end of the spin group
template<typename T>
bool block_update_supported(const DevState<T>& s);
template<typename T>
cudaError_t setup_block_update();
template<typename T>
cudaError_t launch_block_update(const DevState<T>& s, int spin, int block, int nblocks, int set_hi, bool complete,
                                cudaStream_t st);

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
// ratios of virtual moves (nlpp.cu): out[v] = psi(R, electron elec[v] at pos[v]) / psi(R) of walker walker[v];
// a move whose walker or electron is out of range or whose position is not finite gets a NaN ratio
// and its index lowers *bad (atomicMin; the caller sets it to INT_MAX)
template<typename T>
cudaError_t launch_vp_ratios(const DevState<T>& s, int nvp, const int* walker, const int* elec, const double* pos,
                             double* out, int* bad, cudaStream_t st);
// diffusion Monte Carlo (dmc.cu)
cudaError_t launch_dmc_branch(int nw, const double* e_new, double* e_old, double* weight, int* age, double* rr,
                              const double* par, double* sums, double* w_out, cudaStream_t st);
template<typename T>
cudaError_t launch_copy_walkers(const DevState<T>& s, const int* src, double* weight, double* e_old, int* age,
                                cudaStream_t st);
// per-electron gradient and Laplacian of log psi, gl: [nw][ne][4] (G xyz, L)
template<typename T>
cudaError_t launch_evaluate_gl(const DevState<T>& s, double* gl, cudaStream_t st);

// learned MH proposal (learned.cu): MLP 51 -> 128 -> 128 -> 128 -> 6, inputs padded
// to 64 and outputs to 16 for the tensor cores
constexpr int ML_IN = 64, ML_NIN = 51, ML_H = 128, ML_OUT = 16, ML_NOUT = 6, ML_M = 128, ML_AUX = 24;
// FP32 master parameters, flat: W1 [128][64], b1 [128], W2 [128][128], b2, W3, b3, W4 [16][128], b4 [16]
constexpr int MP_W1 = 0;
constexpr int MP_B1 = MP_W1 + ML_H * ML_IN;
constexpr int MP_W2 = MP_B1 + ML_H;
constexpr int MP_B2 = MP_W2 + ML_H * ML_H;
constexpr int MP_W3 = MP_B2 + ML_H;
constexpr int MP_B3 = MP_W3 + ML_H * ML_H;
constexpr int MP_W4 = MP_B3 + ML_H;
constexpr int MP_B4 = MP_W4 + ML_OUT * ML_H;
constexpr int MP_N  = MP_B4 + ML_OUT;
constexpr int ML_WIMG_BYTES = (ML_H * ML_IN + 2 * ML_H * ML_H + ML_OUT * ML_H) * 2;
constexpr int ML_WSIMT_BYTES = (ML_IN / 2 + ML_H) * ML_H * 4 + 6 * ML_H * 2;

struct MlpArgs
{
  int rows;
  const __nv_bfloat16* x;    // [rows][64]
  const unsigned char* wimg; // packed BF16 weights
  const float* params;       // FP32 master parameters (biases are read from here)
  __nv_bfloat16* hid;        // [3][hid_rows][128] post-activations, or null
  int hid_rows, hid_row0;
  float* out;                // [rows][8] raw outputs, or null
  float* aux;                // [nw][ML_AUX] proposal terms kept for training
  int* err;                  // set when a tensor-core wait times out
};

struct MlpTrain
{
  float *params, *m, *v, *grad;
  unsigned char* wimg;  // tensor-core image
  unsigned char* wsimt; // SIMT image for the walker-resident sweep
  __nv_bfloat16* x;   // [rows][64]
  __nv_bfloat16* hid; // [3][rows][128]
  float* g4;          // [rows][8]
  float* delta;       // [3][rows][128]
  int* step;
};

template<typename T>
cudaError_t setup_learned();
cudaError_t launch_mlp_pack(const float* params, unsigned char* img, unsigned char* simt, cudaStream_t st);
template<typename T>
cudaError_t launch_features(const DevState<T>& s, int iat, int at_proposed, __nv_bfloat16* X, cudaStream_t st);
template<typename T>
cudaError_t launch_mlp_forward(const MlpArgs& a, const DevState<T>& s, int iat, int mode, cudaStream_t st);
template<typename T>
cudaError_t launch_mlp_loss_grad(const DevState<T>& s, const float* aux, float* g4, double* stats, cudaStream_t st);
cudaError_t launch_mlp_backward(const MlpTrain& t, int rows, cudaStream_t st);
cudaError_t launch_mlp_adam(const MlpTrain& t, float lr, cudaStream_t st);

// recompute path (recompute_kernels.cu)
__host__ __device__ size_t gj_scratch_doubles(int n);
template<typename T>
cudaError_t launch_recompute(const DevState<T>& s, double* mscratch, int masked, cudaStream_t st);
} // namespace qmcg
