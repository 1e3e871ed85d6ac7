// Orbitals from plane-wave coefficients: the numeric part of QMCPACK's ESHDF orbital
// input (EinsplineSetBuilderESHDF.fft.cpp, SplineSetReader.cpp:30-240 and
// OneSplineOrbData::fft_spline, OneSplineOrbData.cpp:62-95) for real Gamma-point
// orbitals, on the GPU.  The caller has read the plane-wave coefficients c_G and the
// Miller indices G of every band (from the ESHDF file); per band:
//   1. unpack4fftw (einspline_helper.hpp:34-59): c_G placed at ((G + n) mod n) of an
//      n_x x n_y x n_z complex box, for G inside [lower, upper] = [(n-1)/2 - n + 1, (n-1)/2];
//   2. the backward 3-D transform psi(r) = sum_G c_G exp(+2 pi i G.r/n), unnormalized (the
//      FFTW plan of OneSplineOrbData.cpp:30-31): here three passes of 1-D transforms, one
//      warp per line, each output a direct sum over the line with exact twiddles (the
//      grids are ~50-100 points per axis, so O(n) per output point costs milliseconds for
//      a few hundred orbitals, once per run);
//   3. fix_phase_rotate_c2r (einspline_helper.hpp:70-127) at twist 0: the sums Re^2, Im^2
//      and Re Im over the box give one phase (phase_r, phase_i) per band, and the real
//      orbital is phase_r Re - phase_i Im;
//   4. einspline's periodic interpolation (set_multi_UBspline_3d_d,
//      multi_bspline_create.c:1186-1240, find_coefs_1d_d and solve_periodic_interp_1d_d,
//      bspline_create.c:991-1043, 1095-1118): the cyclic tridiagonal system
//      (1/6, 2/3, 1/6) c = data along x, then y, then z, with the ghost coefficients
//      c[0] = c[M], c[M+1] = c[1], c[M+2] = c[2].  The elimination of the band matrix does
//      not depend on the data, so its factors are formed once per axis on the host (the
//      same operations as the reference's band loop) and every line only carries its
//      right-hand side through them, one thread per line;
//   5. the coefficients into the move loop's table [n_x+3][n_y+3][n_z+3][lda], orbital
//      fastest, in the crowd's precision (the reference solves in FP64 and stores the
//      multi-spline in its precision).
#include <cuda_runtime.h>

#include <cmath>
#include <string>
#include <vector>

#include "../../include/qmcg.h"
#include "launch.h"

namespace qmcg
{
namespace
{

constexpr int OB_MAXN = 256; // grid points per axis

// 1: unpack the bands' coefficients into their boxes (zeroed before)
__global__ void pw_unpack_kernel(int norb, int ng, const int* __restrict__ gv, const double* __restrict__ cg, int nx,
                                 int ny, int nz, double2* __restrict__ box)
{
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)norb * ng)
    return;
  const int o = (int)(t / ng), g = (int)(t % ng);
  const int n[3] = {nx, ny, nz};
  int idx[3];
#pragma unroll
  for (int d = 0; d < 3; d++)
  {
    const int up = (n[d] - 1) / 2, lo = up - n[d] + 1, v = gv[3 * g + d];
    if (v > up || v < lo)
      return;
    idx[d] = (v + n[d]) % n[d];
  }
  const size_t at = (size_t)o * nx * ny * nz + ((size_t)idx[0] * ny + idx[1]) * nz + idx[2];
  box[at] = make_double2(cg[2 * ((size_t)o * ng + g)], cg[2 * ((size_t)o * ng + g) + 1]);
}

// 2: in-place 1-D backward transforms of length n along one axis (element stride `stride`);
// line L = (o, a, b) starts at o * vol + a * sa + b * sb.  One warp per line.
__global__ void dft_lines_kernel(double2* __restrict__ box, int n, long stride, long vol, int na, long sa, int nb,
                                 long sb, long nlines)
{
  __shared__ double2 tw[OB_MAXN];
  __shared__ double2 line[8][OB_MAXN];
  for (int m = threadIdx.x; m < n; m += blockDim.x)
  {
    double s, c;
    sincospi(2.0 * m / n, &s, &c); // exp(+2 pi i m / n)
    tw[m] = make_double2(c, s);
  }
  __syncthreads();
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long L = (long)blockIdx.x * 8 + wid;
  if (L >= nlines)
    return;
  const long o = L / ((long)na * nb), r = L % ((long)na * nb);
  const long base = o * vol + (r / nb) * sa + (r % nb) * sb;
  double2* ln = line[wid];
  for (int j = lane; j < n; j += 32)
    ln[j] = box[base + j * stride];
  __syncwarp();
  for (int k = lane; k < n; k += 32)
  {
    double re = 0, im = 0;
    int m = 0; // j k mod n
    for (int j = 0; j < n; j++)
    {
      const double2 x = ln[j], w = tw[m];
      re += x.x * w.x - x.y * w.y;
      im += x.x * w.y + x.y * w.x;
      m += k;
      if (m >= n)
        m -= n;
    }
    box[base + k * stride] = make_double2(re, im);
  }
}

// 3: per band the sums Re^2, Im^2, Re Im, the phase, and the rotated real orbital
__global__ void phase_rotate_kernel(const double2* __restrict__ box, long vol, double* __restrict__ data,
                                    double* __restrict__ phases)
{
  __shared__ double red[3][32];
  __shared__ double ph[2];
  const int o = blockIdx.x;
  const double2* b = box + (size_t)o * vol;
  double rn = 0, in = 0, ri = 0;
  for (long e = threadIdx.x; e < vol; e += blockDim.x)
  {
    const double2 v = b[e];
    rn += v.x * v.x;
    in += v.y * v.y;
    ri += v.x * v.y;
  }
  double v3[3] = {rn, in, ri};
#pragma unroll
  for (int q = 0; q < 3; q++)
  {
    double v = v3[q];
    for (int s = 16; s > 0; s >>= 1)
      v += __shfl_xor_sync(0xffffffffu, v, s);
    if ((threadIdx.x & 31) == 0)
      red[q][threadIdx.x >> 5] = v;
  }
  __syncthreads();
  if (threadIdx.x == 0)
  {
    double t[3] = {0, 0, 0};
    for (int w = 0; w < (int)(blockDim.x >> 5); w++)
      for (int q = 0; q < 3; q++)
        t[q] += red[q][w];
    // fix_phase_rotate_c2r at twist 0
    const double x   = (t[0] - t[1]) / t[2];
    const double y   = 1.0 / sqrt(x * x + 4.0);
    const double phs = sqrt(0.5 - y);
    ph[0]            = phs;
    ph[1]            = x < 0 ? sqrt(1.0 - phs * phs) : -sqrt(1.0 - phs * phs);
    if (phases)
    {
      phases[2 * o]     = ph[0];
      phases[2 * o + 1] = ph[1];
    }
  }
  __syncthreads();
  const double pr = ph[0], pi = ph[1];
  double* out = data + (size_t)o * vol;
  for (long e = threadIdx.x; e < vol; e += blockDim.x)
  {
    const double2 v = b[e];
    out[e]          = pr * v.x - pi * v.y;
  }
}

// the data-independent factors of solve_periodic_interp_1d_d for one axis of M points
struct BandFactors
{
  double b1_0, b2last_0; // row 0's divisor, the last row's coupling to row 0
  double b0;             // basis[0] of every row
  double b0last, b1last; // the last row's final factors
  // per row: b1 after its update (rows 1..M-2), the last row's coupling while row is
  // eliminated (rows 1..M-3), b2 after its division and lastCol (rows 0..M-2)
  double b1[OB_MAXN], b2last[OB_MAXN], b2[OB_MAXN], lc[OB_MAXN];
};

// the band loop of solve_periodic_interp_1d_d (bspline_create.c:991-1031) on the basis
// rows of find_coefs_1d_d, recording the factors the right-hand side meets
static void band_factors(int M, BandFactors& f)
{
  std::vector<double> b0(M, 1.0 / 6.0), b1(M, 2.0 / 3.0), b2(M, 1.0 / 6.0), lc(M, 0.0);
  f.b0       = 1.0 / 6.0;
  f.b1_0     = b1[0];
  b2[0]     /= b1[0];
  b0[0]     /= b1[0];
  b1[0]      = 1.0;
  b1[M - 1] -= b2[M - 1] * b0[0];
  f.b2last_0 = b2[M - 1];
  b2[M - 1]  = -b2[M - 1] * b2[0];
  lc[0]      = b0[0];
  for (int row = 1; row < M - 1; row++)
  {
    b1[row] -= b0[row] * b2[row - 1];
    lc[row]  = -b0[row] * lc[row - 1];
    b0[row]  = 0.0;
    b2[row] /= b1[row];
    lc[row] /= b1[row];
    f.b1[row] = b1[row];
    b1[row]   = 1.0;
    if (row < M - 2)
    {
      f.b2last[row] = b2[M - 1];
      b1[M - 1] -= b2[M - 1] * lc[row];
      b2[M - 1]  = -b2[M - 1] * b2[row];
    }
  }
  b0[M - 1] += b2[M - 1];
  b1[M - 1] -= b0[M - 1] * (b2[M - 2] + lc[M - 2]);
  f.b0last = b0[M - 1];
  f.b1last = b1[M - 1];
  for (int row = 0; row < M - 1; row++)
  {
    f.b2[row] = b2[row];
    f.lc[row] = lc[row];
  }
}

// 4: one periodic interpolation per thread along one axis: the right-hand side (M values at
// `in`, stride is) through the band factors, the M + 3 coefficients to `out` (stride os).
// Line L = (o, a, b): in at o * ivol + a * ia + b * ib, out at o * ovol + a * oa + b * ob.
__global__ void periodic_coefs_kernel(const double* in, long is, long ivol, long ia, long ib, double* out, long os,
                                      long ovol, long oa, long ob, int na, int nb, long nlines, int M,
                                      const BandFactors* __restrict__ fp)
{
  const long L = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (L >= nlines)
    return;
  const BandFactors& f = *fp;
  const long o = L / ((long)na * nb), r = L % ((long)na * nb), a = r / nb, b = r % nb;
  const double* x = in + o * ivol + a * ia + b * ib;
  double* c       = out + o * ovol + a * oa + b * ob;
  double b3[OB_MAXN];
  for (int i = 0; i < M; i++)
    b3[i] = x[i * is];
  // forward elimination, the right-hand side column of solve_periodic_interp_1d_d
  b3[0] /= f.b1_0;
  b3[M - 1] -= f.b2last_0 * b3[0];
  for (int row = 1; row < M - 1; row++)
  {
    b3[row] -= f.b0 * b3[row - 1];
    b3[row] /= f.b1[row];
    if (row < M - 2)
      b3[M - 1] -= f.b2last[row] * b3[row];
  }
  b3[M - 1] -= f.b0last * b3[M - 2];
  b3[M - 1] /= f.b1last;
  // back substitution and the periodic ghosts
  const double cM = b3[M - 1];
  c[M * os]       = cM;
  double next     = cM; // c[row + 2]
  for (int row = M - 2; row >= 0; row--)
  {
    const double v = b3[row] - f.b2[row] * next - f.lc[row] * cM;
    c[(row + 1) * os] = v;
    next              = v;
  }
  c[0]            = cM;
  c[(M + 1) * os] = c[1 * os];
  c[(M + 2) * os] = c[2 * os];
}

// 5: [norb][Nx][Ny][Nz] FP64 -> [Nx][Ny][Nz][lda] in the crowd's precision, zero beyond norb
template<typename T>
__global__ void coef_layout_kernel(const double* __restrict__ c, int norb, long nvol, int lda, T* __restrict__ out)
{
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nvol * lda)
    return;
  const long p = t / lda;
  const int o  = (int)(t % lda);
  out[t]       = o < norb ? static_cast<T>(c[(size_t)o * nvol + p]) : T(0);
}

struct DevBuf
{
  std::vector<void*> ptrs;
  ~DevBuf()
  {
    for (void* p : ptrs)
      cudaFree(p);
  }
  template<typename X>
  cudaError_t get(X** p, size_t n)
  {
    void* q       = nullptr;
    cudaError_t e = cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(X));
    if (e == cudaSuccess)
      ptrs.push_back(q);
    *p = static_cast<X*>(q);
    return e;
  }
};

} // namespace
} // namespace qmcg

#define OB_TRY(x)                                                                                       \
  do                                                                                                    \
  {                                                                                                     \
    cudaError_t e_ = (x);                                                                               \
    if (e_ != cudaSuccess)                                                                              \
      return qmcg::set_error(QMCG_ERR_CUDA, std::string("orbital splines: ") + cudaGetErrorString(e_)); \
  } while (0)

extern "C" int qmcg_spline_from_planewaves(int precision, int num_orbitals, int num_g, const int* gvecs,
                                           const double* coefs_g, const int mesh[3], int num_orbitals_padded,
                                           void* spline_coefs, double* phases)
{
  using namespace qmcg;
  if (precision != 4 && precision != 8)
    return set_error(QMCG_ERR_ARG, "precision must be 4 or 8");
  if (num_orbitals <= 0 || num_g <= 0 || !gvecs || !coefs_g || !mesh || !spline_coefs ||
      num_orbitals_padded < num_orbitals)
    return set_error(QMCG_ERR_ARG, "bad orbital arguments");
  const int nx = mesh[0], ny = mesh[1], nz = mesh[2];
  if (nx < 4 || ny < 4 || nz < 4 || nx > OB_MAXN || ny > OB_MAXN || nz > OB_MAXN)
    return set_error(QMCG_ERR_ARG, "mesh points per axis must be in [4, 256]");
  const int norb = num_orbitals, lda = num_orbitals_padded;
  const long vol = (long)nx * ny * nz;
  const int Nx = nx + 3, Ny = ny + 3, Nz = nz + 3;
  const long nvol = (long)Nx * Ny * Nz;
  DevBuf db;
  int* d_g       = nullptr;
  double* d_cg   = nullptr;
  double2* d_box = nullptr;
  double* d_data = nullptr;
  double* d_c    = nullptr;
  double* d_ph   = nullptr;
  BandFactors* d_f = nullptr;
  OB_TRY(db.get(&d_g, 3 * (size_t)num_g));
  OB_TRY(db.get(&d_cg, 2 * (size_t)norb * num_g));
  OB_TRY(db.get(&d_box, (size_t)norb * vol));
  OB_TRY(db.get(&d_data, (size_t)norb * vol));
  OB_TRY(db.get(&d_c, (size_t)norb * nvol));
  OB_TRY(db.get(&d_ph, 2 * (size_t)norb));
  OB_TRY(db.get(&d_f, 3));
  std::vector<BandFactors> f(3);
  band_factors(nx, f[0]);
  band_factors(ny, f[1]);
  band_factors(nz, f[2]);
  OB_TRY(cudaMemcpy(d_f, f.data(), 3 * sizeof(BandFactors), cudaMemcpyHostToDevice));
  OB_TRY(cudaMemcpy(d_g, gvecs, 3 * (size_t)num_g * sizeof(int), cudaMemcpyHostToDevice));
  OB_TRY(cudaMemcpy(d_cg, coefs_g, 2 * (size_t)norb * num_g * sizeof(double), cudaMemcpyHostToDevice));
  OB_TRY(cudaMemset(d_box, 0, (size_t)norb * vol * sizeof(double2)));
  const long npw = (long)norb * num_g;
  pw_unpack_kernel<<<(unsigned)((npw + 255) / 256), 256>>>(norb, num_g, d_g, d_cg, nx, ny, nz, d_box);
  OB_TRY(cudaGetLastError());
  // the 3-D transform as 1-D transforms along z, y, x
  auto lines = [&](int n, long stride, int na, long sa, int nb, long sb) {
    const long nl = (long)norb * na * nb;
    dft_lines_kernel<<<(unsigned)((nl + 7) / 8), 256>>>(d_box, n, stride, vol, na, sa, nb, sb, nl);
    return cudaGetLastError();
  };
  OB_TRY(lines(nz, 1, nx, (long)ny * nz, ny, nz));
  OB_TRY(lines(ny, nz, nx, (long)ny * nz, nz, 1));
  OB_TRY(lines(nx, (long)ny * nz, ny, nz, nz, 1));
  phase_rotate_kernel<<<norb, 256>>>(d_box, vol, d_data, d_ph);
  OB_TRY(cudaGetLastError());
  // periodic interpolation along x (data -> coefficients), then y and z in place
  auto solve = [&](const double* in, long is, long ivol, long ia, long ib, long os, long oa, long ob, int na, int nb,
                   int M, int axis) {
    const long nl = (long)norb * na * nb;
    periodic_coefs_kernel<<<(unsigned)((nl + 127) / 128), 128>>>(in, is, ivol, ia, ib, d_c, os, nvol, oa, ob, na, nb,
                                                                  nl, M, d_f + axis);
    return cudaGetLastError();
  };
  // x: lines (iy < ny, iz < nz)
  OB_TRY(solve(d_data, (long)ny * nz, vol, nz, 1, (long)Ny * Nz, Nz, 1, ny, nz, nx, 0));
  // y: lines (ix < Nx, iz < nz), in place
  OB_TRY(solve(d_c, Nz, nvol, (long)Ny * Nz, 1, Nz, (long)Ny * Nz, 1, Nx, nz, ny, 1));
  // z: lines (ix < Nx, iy < Ny), in place
  OB_TRY(solve(d_c, 1, nvol, (long)Ny * Nz, Nz, 1, (long)Ny * Nz, Nz, Nx, Ny, nz, 2));
  const long nout = nvol * lda;
  const size_t esz = precision == 8 ? sizeof(double) : sizeof(float);
  void* d_out = nullptr;
  OB_TRY(db.get(reinterpret_cast<unsigned char**>(&d_out), (size_t)nout * esz));
  if (precision == 8)
    coef_layout_kernel<double><<<(unsigned)((nout + 255) / 256), 256>>>(d_c, norb, nvol, lda,
                                                                          static_cast<double*>(d_out));
  else
    coef_layout_kernel<float><<<(unsigned)((nout + 255) / 256), 256>>>(d_c, norb, nvol, lda,
                                                                         static_cast<float*>(d_out));
  OB_TRY(cudaGetLastError());
  OB_TRY(cudaMemcpy(spline_coefs, d_out, (size_t)nout * esz, cudaMemcpyDeviceToHost));
  if (phases)
    OB_TRY(cudaMemcpy(phases, d_ph, 2 * (size_t)norb * sizeof(double), cudaMemcpyDeviceToHost));
  return QMCG_OK;
}
