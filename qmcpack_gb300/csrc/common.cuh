// Device-side state and helpers shared by the move-loop kernels.
//
// One crowd = nw walkers of one system, resident in HBM for a whole run:
//   positions      R    double [nw][3][ne_pad]   (SoA, FP64 always)
//                  Rt   T      [nw][3][ne_pad]   (copy in the move-loop precision)
//   determinants   Ainv T      [2][nw][N][lda]   (Ainv = (M^-1)^T, row e = electron)
//                  dgrad T     [2][nw][N][3][lda], dlap T [2][nw][N][lda]
//   delayed update U, V T [2][nw][k][lda], Binv T [2][nw][k][k], delay_list int [2][nw][k]
//   Jastrow state  J2 T [nw][5][ne_pad] (Uat, dUat xyz, d2Uat), J1 likewise (Vat, Grad xyz, Lap)
// lda = orbitals padded to 16 elements, so every row starts on a 64-byte boundary.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace qmcg
{

enum : int
{
  ST_OK          = 0,
  ST_ZERO_RATIO  = 1,  // accepted move with a zero determinant ratio
  ST_NONFINITE   = 2,  // NaN/Inf ratio or gradient
  ST_SINGULAR    = 4,  // exact zero pivot in the FP64 inverse
  ST_ILLCOND     = 8,  // the tracked inverse lost accuracy: |Ainv[row] . phi(r_row) - 1| above tolerance
  ST_ILLCOND_UP  = 16, // the same, found in the spin-up determinant only
  ST_ILLCOND_DN  = 32, // the same, found in the spin-down determinant only
  ST_TIMEOUT     = 64, // a bounded wait on an asynchronous copy ran out (the walker was skipped)
  ST_REPAIR_MASK = ST_NONFINITE | ST_ILLCOND | ST_ILLCOND_UP | ST_ILLCOND_DN,
};

// repair bits that call for a new inverse of spin `spin`
__host__ __device__ constexpr int st_repair_spin(int spin)
{
  return ST_NONFINITE | ST_ILLCOND | (spin ? ST_ILLCOND_DN : ST_ILLCOND_UP);
}

// tolerance of the self-ratio health check |Ainv[row] . phi(r_row) - 1|
template<typename T>
struct HealthTol;
template<>
struct HealthTol<float>
{
  static constexpr float v = 1e-2f;
};
template<>
struct HealthTol<double>
{
  static constexpr double v = 1e-7;
};

template<typename T>
struct DevState
{
  // ---------------- sizes
  int nw, ne, ne_pad, nup, norb, lda, nions, nions_pad, k;
  // ---------------- system (read-only)
  const T* coefs;
  int gx, gy, gz;
  long long xs, ys, zs; // element strides of the coefficient table
  double L[3];          // orthorhombic cell lengths
  double G[3];          // 1 / L: the diagonal of the reciprocal lattice G = R^-1 (CrystalLattice::G)
  T grid_scale[3];      // g_d / L_d in the move precision: the Cartesian factor of spline derivatives
  const T* ions;        // [3][nions_pad]
  const int* ion_species;
  const T* j1c;         // [n_ion_species][j1_ncoef]
  int j1_ncoef, j1_maxidx;
  T j1_dri, j1_rcut;
  const T* j2c;         // [2][j2_ncoef]: same spin, opposite spin
  int j2_ncoef, j2_maxidx;
  T j2_dri, j2_rcut;
  int has_j1, has_j2;
  // ---------------- walker state
  double* R;
  T* Rt;
  T* Ainv;
  T* dgrad;
  T* dlap;
  T* psiv;   // [2][nw][N][lda] orbital values of the current electron positions
  T* U;
  T* V;
  T* Binv;
  int* delay_list;
  T* J2;
  T* J1;
  double* log_abs; // [2][nw]
  int* sign;       // [2][nw]
  // ---------------- move scratch
  double* active_pos; // [nw][3]
  double* disp;       // [nw][3]  proposed displacement (drift + diffusion)
  T* invRow;          // [nw][lda]
  T* rcopy;           // [nw][lda]   (SM-1 row copy)
  T* phi;             // [nw][5][lda]  proposed orbital VGL (v, gx, gy, gz, lap)
  T* cur_det;         // [nw]          determinant ratio of the proposed move
  T* cur_j;           // [nw][10]      J1 (U,gx,gy,gz,lap), J2 (U,gx,gy,gz,lap) at the proposed position
  double* grads_now;  // [nw][3]
  double* grads_new;  // [nw][3]
  double* ratios;     // [nw]
  double* log_gf;     // [nw]
  double* prob;       // [nw]  acceptance probability argument p*exp(log_gb-log_gf)
  int* flag;          // [nw]  valid && p >= eps (a uniform is consumed)
  int* accepted;      // [nw]
  int* status;        // [nw]
  unsigned long long* counters; // [0] accepted, [1] rejected, [2] walkers repaired by an FP64 recompute
  // ---------------- random numbers
  const double* gauss;   // stream mode: [ne][nw][3] unit Gaussians of the current sweep
  const double* uniform; // stream mode: uniforms, consumed in walker order
  int* ucursor;          // [2] ping-pong consumption cursor
  unsigned long long seed;
  unsigned long long* sweep_counter; // device RNG: sweeps done
  int rng_mode;          // 0: stream from the host, 1: counter-based on the device
  double tau;
  int use_drift;
  double* gj_scratch;  // [2 nw][3 N + 8] pivot broadcast of the cluster Gauss-Jordan repair
  int* repair_list;     // [1 + nw]: count, then the walkers with a repair bit (masked recompute)
  // learned proposal (walker-resident path): SIMT weight image and FP32 master parameters
  const void* mlp_simt;
  const float* mlp_params;
  // optional per-move record of the walker-resident drift-diffusion sweep, [ne][nw][TRACE_FIELDS]
  // (null: nothing recorded)
  double* trace;
  // fixed-node DMC moves (walker-resident path): a move that changes the sign of psi is
  // rejected, and rr [nw][2] accumulates tau |xi|^2 over the proposed and the accepted moves
  int dmc;
  double* rr;
  // the walker-resident sweep keeps a segment's inverse rows in shared memory (set by the host
  // when that does not enlarge the kernel's shared-memory footprint)
  int seg_smem;
  int j1_nspecies; // ion species of the one-body functors (rows of j1c)
  // delayed-update sets per spin slot: U, V, Binv and delay_list hold nsets sets of k slots
  // per (spin, walker) ([2][nw][nsets][k][...]); a segment of the walker-resident sweep writes
  // set (i0 - first) / k when nsets > 1, and every other user works on set 0
  int nsets;
};

// fields of one move record of the walker-resident sweep (qmcg_vmc_sweeps_trace)
enum : int
{
  TR_POS      = 0,  // proposed position x, y, z
  TR_RATIO    = 3,  // psi(R') / psi(R)
  TR_GRAD_NEW = 4,  // grad log psi at the proposed position, x, y, z
  TR_GRAD_NOW = 7,  // grad log psi at the current position, x, y, z
  TR_ACCEPT   = 10, // 1 accepted, 0 rejected
  TR_SELF     = 11, // Ainv[row] . phi(r_row): 1 for an exact inverse (the health check's value)
  TRACE_FIELDS = 12,
};

// Ewald tables of a system for the local-energy kernel (energy.cu)
template<typename T>
struct EwaldDev
{
  int ng, nmax;       // half-space G vectors; largest |n| along any axis
  const char4* gn;    // [ng] (n1, n2, n3): G = 2 pi (n1/Lx, n2/Ly, n3/Lz), sorted
  const T* fg;        // [ng] 4 pi/V exp(-G^2/4a^2)/G^2
  const T* rho_ion;   // [ng][2] ion structure factor sum_I Z_I exp(i G.R_I)
  const T* ion_q;     // [nions] ion charges
  T alpha;
  T rcut;             // pairs beyond rcut (half the shortest cell side) contribute below the tolerance
  double e_const;     // ion-ion, self-energy and background terms
};

// Arguments of the delayed-update flush Ainv -= (Ainv U^T - E)(Binv V) over a
// batch of walkers: row-major per walker, per-walker strides in elements.
template<typename T>
struct FlushArgs
{
  int nw, n, lda, k, dc;
  long long sA, sU, sB, sD; // walker strides of Ainv, U/V, Binv, delay_list
  T* ainv;
  const T* u;
  const T* v;
  const T* binv;
  const int* delay_list;
  T* w;                     // scratch [nw][k][lda]
};

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), counter-based.
// ---------------------------------------------------------------------------
struct u4
{
  uint32_t x, y, z, w;
};

__device__ __forceinline__ u4 philox4x32_10(u4 c, uint32_t k0, uint32_t k1)
{
#pragma unroll
  for (int r = 0; r < 10; r++)
  {
    const uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
    const uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
    c  = u4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return c;
}

// 53-bit uniform in [0,1) from two 32-bit words
__device__ __forceinline__ double u01(uint32_t a, uint32_t b)
{
  const uint64_t v = (static_cast<uint64_t>(a) << 21) ^ static_cast<uint64_t>(b >> 11);
  return static_cast<double>(v & ((1ull << 53) - 1)) * (1.0 / 9007199254740992.0);
}

// ---------------------------------------------------------------------------
// cubic B-spline weights of one axis: value, first and second derivative
// (MultiBsplineData::compute_prefactors).
// ---------------------------------------------------------------------------
template<typename T>
__device__ __forceinline__ void bspline_weights(T t, T a[4], T da[4], T d2a[4])
{
  a[0]   = ((T(-1.0 / 6.0) * t + T(3.0 / 6.0)) * t + T(-3.0 / 6.0)) * t + T(1.0 / 6.0);
  a[1]   = ((T(3.0 / 6.0) * t + T(-1.0)) * t + T(0.0)) * t + T(4.0 / 6.0);
  a[2]   = ((T(-3.0 / 6.0) * t + T(3.0 / 6.0)) * t + T(3.0 / 6.0)) * t + T(1.0 / 6.0);
  a[3]   = ((T(1.0 / 6.0) * t + T(0.0)) * t + T(0.0)) * t + T(0.0);
  da[0]  = (T(-0.5) * t + T(1.0)) * t + T(-0.5);
  da[1]  = (T(1.5) * t + T(-2.0)) * t + T(0.0);
  da[2]  = (T(-1.5) * t + T(1.0)) * t + T(0.5);
  da[3]  = (T(0.5) * t + T(0.0)) * t + T(0.0);
  d2a[0] = T(-1.0) * t + T(1.0);
  d2a[1] = T(3.0) * t + T(-2.0);
  d2a[2] = T(-3.0) * t + T(1.0);
  d2a[3] = T(1.0) * t + T(0.0);
}

template<typename T>
struct Eps;
template<>
struct Eps<float>
{
  static constexpr float v = 1.19209290e-07f;
};
template<>
struct Eps<double>
{
  static constexpr double v = 2.2204460492503131e-16;
};

// getSplineBound: integer cell and fraction, clamped to [0, nmax] (SplineBound.hpp:36-61);
// a NaN argument takes the x < 0 branch so no index can leave the table
template<typename T>
__device__ __forceinline__ void spline_bound(T x, int nmax, int& ind, T& dx)
{
  if (!(x >= T(0)))
  {
    ind = 0;
    dx  = T(0);
  }
  else
  {
    const T ip = floor(x);
    dx         = x - ip;
    ind        = static_cast<int>(ip);
    if (ind > nmax)
    {
      ind = nmax;
      dx  = T(1) - Eps<T>::v;
    }
  }
}

// radial B-spline functor: u, du/dr, d2u/dr2 (BsplineFunctor::evaluate_impl)
template<typename T>
__device__ __forceinline__ T functor_eval(const T* __restrict__ c, T dri, int maxidx, T r, T& du, T& d2u)
{
  r *= dri;
  int i;
  T t;
  spline_bound(r, maxidx, i, t);
  const T c0 = c[i], c1 = c[i + 1], c2 = c[i + 2], c3 = c[i + 3];
  d2u = dri * dri *
      (c0 * (T(-1.0) * t + T(1.0)) + c1 * (T(3.0) * t + T(-2.0)) + c2 * (T(-3.0) * t + T(1.0)) +
       c3 * (T(1.0) * t + T(0.0)));
  du = dri *
      (c0 * ((T(-0.5) * t + T(1.0)) * t + T(-0.5)) + c1 * ((T(1.5) * t + T(-2.0)) * t + T(0.0)) +
       c2 * ((T(-1.5) * t + T(1.0)) * t + T(0.5)) + c3 * ((T(0.5) * t + T(0.0)) * t + T(0.0)));
  return c0 * (((T(-1.0 / 6.0) * t + T(3.0 / 6.0)) * t + T(-3.0 / 6.0)) * t + T(1.0 / 6.0)) +
      c1 * (((T(3.0 / 6.0) * t + T(-1.0)) * t + T(0.0)) * t + T(4.0 / 6.0)) +
      c2 * (((T(-3.0 / 6.0) * t + T(3.0 / 6.0)) * t + T(3.0 / 6.0)) * t + T(1.0 / 6.0)) +
      c3 * (((T(1.0 / 6.0) * t + T(0.0)) * t + T(0.0)) * t + T(0.0));
}

// 1/sqrt(x): one special-function instruction in FP32 (rsqrtf, at most 2 ulp), the
// library rsqrt in FP64
__device__ __forceinline__ float inv_sqrt(float x) { return rsqrtf(x); }
__device__ __forceinline__ double inv_sqrt(double x) { return rsqrt(x); }

// orthorhombic minimum image of d = R_j - r (DTD_BConds<T,3,PPPO>)
template<typename T>
__device__ __forceinline__ T min_image(T d, T L, T Linv)
{
  const T s = d * Linv;
  return L * (s - round(s));
}

// ---------------------------------------------------------------------------
// block reductions
// ---------------------------------------------------------------------------
template<typename T>
__device__ __forceinline__ T warp_sum(T v)
{
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
    v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// sum NV values over the block; result valid in every thread. scratch: NV * 32 elements
template<typename T, int NV>
__device__ __forceinline__ void block_sum(T (&v)[NV], T* scratch)
{
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nwarp = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int q = 0; q < NV; q++)
    v[q] = warp_sum(v[q]);
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < NV; q++)
      scratch[q * 32 + wid] = v[q];
  __syncthreads();
#pragma unroll
  for (int q = 0; q < NV; q++)
  {
    T x = lane < nwarp ? scratch[q * 32 + lane] : T(0);
    v[q] = warp_sum(x);
  }
  __syncthreads();
}

// sum NV <= 16 values over the block; the totals are valid in warp 0 (thread 0 included).
// Inside a warp a reduce-scatter halves the values a lane keeps at every step (16
// shuffles for 16 values instead of 5 per value; NV padded to the next power of two P,
// then plain butterfly sums) until lane l holds the warp's total of value l / (32 / P);
// warp 0 then adds the warps' totals and broadcasts them to its lanes.
// scratch: 16 * stride elements, stride >= the number of warps.  No trailing barrier: the
// caller synchronises before scratch is written again.
template<typename T, int NV>
__device__ __forceinline__ void block_sum_to0(T (&v)[NV], T* scratch, int stride = 32)
{
  static_assert(NV <= 16, "up to 16 values");
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nwarp = (blockDim.x + 31) >> 5;
  // NV padded to P = 2^S: S transposing stages at distances 16, 8, ... keep half the values
  // each, plain butterfly sums cover the smaller distances; value q ends in lanes q * (32 / P)
  constexpr int S = NV <= 1 ? 0 : (NV <= 2 ? 1 : (NV <= 4 ? 2 : (NV <= 8 ? 3 : 4)));
  constexpr int P = 1 << S, G = 32 / P;
  T x[P];
#pragma unroll
  for (int q = 0; q < P; q++)
    x[q] = q < NV ? v[q] : T(0);
#pragma unroll
  for (int h = P / 2; h >= 1; h >>= 1)
  {
    const int d   = G * h; // exchange distance, keep h values
    const bool up = (lane & d) != 0;
#pragma unroll
    for (int q = 0; q < h; q++)
    {
      const T send = up ? x[q] : x[q + h];
      const T recv = __shfl_xor_sync(0xffffffffu, send, d);
      x[q]         = (up ? x[q + h] : x[q]) + recv;
    }
  }
#pragma unroll
  for (int d = G / 2; d >= 1; d >>= 1)
    x[0] += __shfl_xor_sync(0xffffffffu, x[0], d);
  if ((lane & (G - 1)) == 0 && lane / G < NV)
    scratch[(lane / G) * stride + wid] = x[0];
  __syncthreads();
  if (wid == 0)
  {
    T t = T(0);
    if (lane < NV)
      for (int w = 0; w < nwarp; w++)
        t += scratch[lane * stride + w];
#pragma unroll
    for (int q = 0; q < NV; q++)
      v[q] = __shfl_sync(0xffffffffu, t, q);
  }
}

// Umrigar drift scaling (DriftModifierUNR::getDrift, a = 1)
__device__ __forceinline__ void unr_drift(double tau, const double g[3], double d[3])
{
  const double vsq = g[0] * g[0] + g[1] * g[1] + g[2] * g[2];
  const double sc  = vsq < 2.2204460492503131e-16 ? tau : ((-1.0 + sqrt(1.0 + 2.0 * tau * vsq)) / vsq);
  d[0]             = g[0] * sc;
  d[1]             = g[1] * sc;
  d[2]             = g[2] * sc;
}

// Box-Muller (RandomSeqGenerator.h:33-51) on counter-based uniforms
template<typename T>
__device__ __forceinline__ void gaussians(uint32_t w, uint32_t iat, uint32_t sweep, uint32_t k0, uint32_t k1, T out[3])
{
  const u4 r0 = philox4x32_10(u4{w, iat, sweep, 0u}, k0, k1);
  const u4 r1 = philox4x32_10(u4{w, iat, sweep, 1u}, k0, k1);
  const T one_m = T(1) - Eps<T>::v;
  const T twopi = T(6.283185307179586476925286766559);
  const T t1    = sqrt(T(-2) * log(T(1) - one_m * T(u01(r0.x, r0.y))));
  const T t2    = twopi * T(u01(r0.z, r0.w));
  const T t3    = sqrt(T(-2) * log(T(1) - one_m * T(u01(r1.x, r1.y))));
  const T t4    = twopi * T(u01(r1.z, r1.w));
  out[0]        = t1 * cos(t2);
  out[1]        = t1 * sin(t2);
  out[2]        = t3 * cos(t4);
}

// Umrigar drift (DriftModifierUNR::getDrift, a = 1) in precision T
template<typename T>
__device__ __forceinline__ void unr_drift_t(T tau, const T g[3], T d[3])
{
  const T vsq = g[0] * g[0] + g[1] * g[1] + g[2] * g[2];
  const T sc  = vsq < Eps<T>::v ? tau : ((T(-1) + sqrt(T(1) + T(2) * tau * vsq)) / vsq);
  d[0]        = g[0] * sc;
  d[1]        = g[1] * sc;
  d[2]        = g[2] * sc;
}

} // namespace qmcg
