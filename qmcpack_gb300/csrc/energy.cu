// Local energy of every walker, E_L = T + V, one CTA per walker:
//
//   kinetic  T = -1/2 sum_i (|G_i|^2 + L_i) with G_i, L_i the gradient and Laplacian
//            of log psi from the tracked state (TrialWaveFunction::mw_evaluateGL:
//            DiracDeterminantBatched.cpp:594-603, TwoBodyJastrow.cpp:774-775,
//            J1OrbitalSoA.h:119-120; BareKineticEnergy.cpp:110-117)
//   Coulomb  V = Ewald energy of the electrons (charge -1) and the ions in the
//            periodic cell (the total of CoulombPBCAA for e-e and i-i and CoulombPBCAB
//            for e-i; the reference's standalone sum is EwaldRef.cpp:337-398):
//              V = sum_{i<j} q_i q_j erfc(a r_ij)/r_ij   (minimum image, r_ij < L_min/2)
//                + sum_{G in half space, |G| <= G_c} f(G) (|rho_e + rho_I|^2 - |rho_I|^2)
//                + constant (ion-ion terms, self energy, background)
//            with f(G) = 4 pi/V exp(-G^2/4a^2)/G^2 and rho_e(G) = -sum_i exp(i G.r_i).
//
// The cutoffs follow from a tolerance eps: a L_min/2 = G_c/(2a) = sqrt(-ln eps)
// (eps = 1e-7 for the FP32 move loop, 1e-12 for FP64).  Sums are FP64; the terms are
// evaluated in the move-loop precision T.  The structure factor uses per-electron
// phase tables exp(i n 2 pi x_d / L_d), n = 0..n_max, built in shared memory for a
// chunk of electrons, and from them the products exp(i 2 pi (n1 x/Lx + n2 y/Ly)) for
// every (n1 >= 0, n2) of the half space, so a (G, electron) term is two table reads and
// one complex multiply-add; each thread owns a set of G vectors (sorted by (n1, n2, n3)
// so a warp's table reads are mostly broadcasts) and accumulates rho_e(G) in registers.
#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "launch.h"

namespace qmcg
{

constexpr int LE_NT  = 256; // threads per walker
constexpr int LE_CH  = 32;  // electrons per phase-table chunk at most
constexpr int LE_GPT = 12;  // G vectors per thread per pass
constexpr size_t LE_SMEM_MAX = 200 * 1024;

// a complex value from two consecutive elements of shared memory (8- or 16-byte aligned)
template<typename T>
struct Cplx
{
  T x, y;
};
__device__ __forceinline__ Cplx<float> ld_cplx(const float* p)
{
  const float2 v = *reinterpret_cast<const float2*>(p);
  return {v.x, v.y};
}
__device__ __forceinline__ Cplx<double> ld_cplx(const double* p)
{
  const double2 v = *reinterpret_cast<const double2*>(p);
  return {v.x, v.y};
}

__device__ __forceinline__ float t_erfc(float x) { return erfcf(x); }
__device__ __forceinline__ double t_erfc(double x) { return erfc(x); }
__device__ __forceinline__ void t_sincospi(float x, float* s, float* c) { sincospif(x, s, c); }
__device__ __forceinline__ void t_sincospi(double x, double* s, double* c) { sincospi(x, s, c); }

// shared memory of the local-energy kernel for `ch` electrons per table chunk: positions
// (padded to 4 elements), the 1-D phase tables and the (n1, n2) products of the chunk
static size_t le_smem_ch(int ne, int nmax, int tsize, int ch)
{
  const size_t nm1 = (size_t)nmax + 1, nb = 2 * (size_t)nmax + 1;
  return (size_t)tsize * ((3 * (size_t)ne + 3) / 4 * 4 + (size_t)ch * (3 * nm1 * 2 + nm1 * nb * 2));
}

// electrons per table chunk: as many as fit (LE_CH at most)
static int le_chunk(int ne, int nmax, int tsize)
{
  int ch = LE_CH;
  while (ch > 1 && le_smem_ch(ne, nmax, tsize, ch) > LE_SMEM_MAX)
    ch--;
  return ch;
}

size_t local_energy_smem(int ne, int nmax, int tsize)
{
  return le_smem_ch(ne, nmax, tsize, le_chunk(ne, nmax, tsize));
}

// a thread's sum of many terms: compensated (Kahan) in FP32, which keeps the sum to
// about one rounding of its value without FP64 additions; plain FP64 otherwise
template<typename T>
struct CompSum
{
  double s = 0;
  __device__ void add(T x) { s += static_cast<double>(x); }
  __device__ double get() const { return s; }
};
template<>
struct CompSum<float>
{
  float s = 0.f, c = 0.f;
  __device__ void add(float x)
  {
    const float y = x - c;
    const float t = s + y;
    c             = (t - s) - y;
    s             = t;
  }
  __device__ double get() const { return static_cast<double>(s) - static_cast<double>(c); }
};

template<typename T>
__global__ void __launch_bounds__(LE_NT) local_energy_kernel(DevState<T> s, EwaldDev<T> ew, double* out, int ch)
{
  extern __shared__ __align__(16) unsigned char le_smem[];
  __shared__ double red[3 * 32];
  const int iw = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int ne = s.ne, N = s.norb, lda = s.lda, nm1 = ew.nmax + 1, nb = 2 * ew.nmax + 1;
  T* pos = reinterpret_cast<T*>(le_smem);   // [3][ne], wrapped into the cell
  T* tab = pos + (3 * ne + 3) / 4 * 4;      // [ch][3][nm1] complex
  T* t12 = tab + (size_t)ch * 3 * nm1 * 2;  // [ch][nm1][nb] complex: e1(n1) e2(n2), n2 = -nmax..nmax
  const T Lc[3]   = {T(s.L[0]), T(s.L[1]), T(s.L[2])};
  const T Li[3]   = {T(s.G[0]), T(s.G[1]), T(s.G[2])};

  for (int i = tid; i < ne; i += LE_NT)
#pragma unroll
    for (int d = 0; d < 3; d++)
    {
      double x = s.R[((size_t)iw * 3 + d) * s.ne_pad + i];
      x -= s.L[d] * floor(x * s.G[d]);
      pos[d * ne + i] = static_cast<T>(x);
    }
  __syncthreads();

  double ke = 0, vk = 0;
  CompSum<T> vr; // the ~300 pair terms of a thread
  // ---------------- kinetic energy: a warp per electron, lanes over orbital pairs (lda is
  // even), the four sums of a row in flight together.  The per-electron combination runs in
  // FP64 for 32 electrons at once: lane q keeps the sums of the warp's q-th electron of a
  // batch (the FP64 pipe's time goes by warp instruction, whatever the active lanes)
  T kg[4]  = {T(0), T(0), T(0), T(0)};
  int kel  = -1; // the electron whose sums this lane keeps
  int slot = 0;
  for (int i = warp; i < ne; i += LE_NT / 32, slot = (slot + 1) & 31)
  {
    const int sp     = i < s.nup ? 0 : 1;
    const size_t rb  = ((size_t)sp * s.nw + iw) * N + (i - sp * s.nup);
    const T* a       = s.Ainv + rb * lda;
    const T* g       = s.dgrad + rb * 3 * lda;
    const T* l       = s.dlap + rb * lda;
    T gx = 0, gy = 0, gz = 0, lp = 0;
#pragma unroll 4
    for (int o = 2 * lane; o < N; o += 64)
    {
      const bool h1 = o + 1 < N;
      const T a0 = a[o], a1 = h1 ? a[o + 1] : T(0);
      gx += a0 * g[o] + (h1 ? a1 * g[o + 1] : T(0));
      gy += a0 * g[lda + o] + (h1 ? a1 * g[lda + o + 1] : T(0));
      gz += a0 * g[2 * lda + o] + (h1 ? a1 * g[2 * lda + o + 1] : T(0));
      lp += a0 * l[o] + (h1 ? a1 * l[o + 1] : T(0));
    }
    // butterfly sums: every lane holds the same totals
    gx = warp_sum(gx);
    gy = warp_sum(gy);
    gz = warp_sum(gz);
    lp = warp_sum(lp);
    if (lane == slot)
    {
      kg[0] = gx;
      kg[1] = gy;
      kg[2] = gz;
      kg[3] = lp;
      kel   = i;
    }
    if (slot == 31 || i + LE_NT / 32 >= ne)
    {
      if (kel >= 0)
      {
        // the Jastrow terms of the electron (gradient xyz, Laplacian)
        T j2v[4] = {T(0), T(0), T(0), T(0)}, j1v[4] = {T(0), T(0), T(0), T(0)};
        if (s.has_j2)
        {
          const T* j2 = s.J2 + (size_t)iw * 5 * s.ne_pad + kel;
#pragma unroll
          for (int d = 0; d < 4; d++)
            j2v[d] = j2[(1 + d) * s.ne_pad];
        }
        if (s.has_j1)
        {
          const T* j1 = s.J1 + (size_t)iw * 5 * s.ne_pad + kel;
#pragma unroll
          for (int d = 0; d < 4; d++)
            j1v[d] = j1[(1 + d) * s.ne_pad];
        }
        double G[3] = {static_cast<double>(kg[0]), static_cast<double>(kg[1]), static_cast<double>(kg[2])};
        double L    = static_cast<double>(kg[3]) - (G[0] * G[0] + G[1] * G[1] + G[2] * G[2]);
#pragma unroll
        for (int d = 0; d < 3; d++)
          G[d] += static_cast<double>(j2v[d]) + static_cast<double>(j1v[d]);
        L += static_cast<double>(j2v[3]) - static_cast<double>(j1v[3]);
        ke += -0.5 * (G[0] * G[0] + G[1] * G[1] + G[2] * G[2] + L);
      }
      kel = -1;
    }
  }

  // ---------------- real space: electron pairs enumerated by cyclic separation
  // m = 1..nsep for every i (j = i + m mod ne), plus m = ne/2 for i < ne/2 when ne is even
  const T al          = ew.alpha;
  const int nsep      = (ne - 1) / 2;
  const int nfull = ne * nsep; // ne <= 46340 keeps the pair count in 32 bits
  const int npair = nfull + ((ne & 1) ? 0 : ne / 2);
  for (int p = tid; p < npair; p += LE_NT)
  {
    int i, j;
    if (p < nfull)
    {
      const int m = p / ne;
      i = p - m * ne;
      j = i + 1 + m;
      if (j >= ne)
        j -= ne;
    }
    else
    {
      i = p - nfull;
      j = i + ne / 2;
    }
    T r2 = 0;
#pragma unroll
    for (int d = 0; d < 3; d++)
    {
      T dx = pos[d * ne + j] - pos[d * ne + i];
      dx -= Lc[d] * rint(dx * Li[d]);
      r2 += dx * dx;
    }
    const T r = sqrt(r2);
    if (r > T(0) && r < ew.rcut)
      vr.add(t_erfc(al * r) / r);
  }
  // electron-ion pairs
  for (int p = tid; p < ne * s.nions; p += LE_NT)
  {
    const int i = p / s.nions, I = p - i * s.nions;
    T r2 = 0;
#pragma unroll
    for (int d = 0; d < 3; d++)
    {
      T dx = s.ions[d * s.nions_pad + I] - pos[d * ne + i];
      dx -= Lc[d] * rint(dx * Li[d]);
      r2 += dx * dx;
    }
    const T r = sqrt(r2);
    if (r > T(0) && r < ew.rcut)
      vr.add(-(ew.ion_q[I] * t_erfc(al * r) / r));
  }

  // ---------------- reciprocal space
  for (int g0 = 0; g0 < ew.ng; g0 += LE_NT * LE_GPT)
  {
    T re[LE_GPT], im[LE_GPT], sg3[LE_GPT];
    int i12[LE_GPT], a3[LE_GPT];
#pragma unroll
    for (int q = 0; q < LE_GPT; q++)
    {
      const int g = g0 + tid + q * LE_NT;
      const char4 c = g < ew.ng ? ew.gn[g] : make_char4(0, 0, 0, 0);
      i12[q] = c.x * nb + c.y + ew.nmax;
      a3[q]  = c.z < 0 ? -c.z : c.z;
      sg3[q] = c.z < 0 ? T(-1) : T(1);
      re[q] = im[q] = T(0);
    }
    for (int c0 = 0; c0 < ne; c0 += ch)
    {
      const int cn = min(ch, ne - c0);
      __syncthreads();
      for (int e = tid; e < cn * 3 * nm1; e += LE_NT)
      {
        const int ci = e / (3 * nm1), rem = e - ci * 3 * nm1, d = rem / nm1, n = rem - d * nm1;
        const T u    = pos[d * ne + c0 + ci] * Li[d];
        T sv, cv;
        t_sincospi(T(2) * T(n) * u, &sv, &cv);
        tab[2 * e]     = cv;
        tab[2 * e + 1] = sv;
      }
      __syncthreads();
      // e1(n1) e2(n2) of every electron of the chunk; e2(-n) = conj(e2(n))
      for (int e = tid; e < cn * nm1 * nb; e += LE_NT)
      {
        const int ci = e / (nm1 * nb), rem = e - ci * nm1 * nb, a = rem / nb, b = rem - a * nb - ew.nmax;
        const T* t   = tab + (size_t)ci * 3 * nm1 * 2;
        const T c1 = t[2 * a], s1 = t[2 * a + 1];
        const int ab = b < 0 ? -b : b;
        const T c2 = t[2 * (nm1 + ab)], s2 = b < 0 ? -t[2 * (nm1 + ab) + 1] : t[2 * (nm1 + ab) + 1];
        t12[2 * e]     = c1 * c2 - s1 * s2;
        t12[2 * e + 1] = s1 * c2 + c1 * s2;
      }
      __syncthreads();
      for (int ci = 0; ci < cn; ci++)
      {
        const T* t3 = tab + (size_t)ci * 3 * nm1 * 2 + 2 * (2 * nm1);
        const T* u  = t12 + (size_t)ci * nm1 * nb * 2;
#pragma unroll
        for (int q = 0; q < LE_GPT; q++)
          if (g0 + q * LE_NT < ew.ng) // uniform: the G slots past the last vector are skipped
          {
            const Cplx<T> p = ld_cplx(u + 2 * i12[q]), z = ld_cplx(t3 + 2 * a3[q]);
            const T s3      = sg3[q] * z.y;
            re[q] += p.x * z.x - p.y * s3;
            im[q] += p.y * z.x + p.x * s3;
          }
      }
    }
#pragma unroll
    for (int q = 0; q < LE_GPT; q++)
    {
      const int g = g0 + tid + q * LE_NT;
      if (g < ew.ng)
      {
        // rho_e = -(re, im); |rho_e|^2 + 2 Re(conj(rho_I) rho_e)
        const double er = -static_cast<double>(re[q]), ei = -static_cast<double>(im[q]);
        const double ir = static_cast<double>(ew.rho_ion[2 * g]), ii = static_cast<double>(ew.rho_ion[2 * g + 1]);
        vk += static_cast<double>(ew.fg[g]) * (er * er + ei * ei + 2.0 * (ir * er + ii * ei));
      }
    }
  }

  double v[3] = {ke, vr.get(), vk};
  block_sum<double, 3>(v, red);
  if (tid == 0)
  {
    const double pot     = v[1] + v[2] + ew.e_const;
    out[iw]              = v[0] + pot;
    out[s.nw + iw]       = v[0];
    out[2 * s.nw + iw]   = pot;
  }
}

template<typename T>
cudaError_t setup_local_energy()
{
  return cudaFuncSetAttribute(local_energy_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
}

template<typename T>
cudaError_t launch_local_energy(const DevState<T>& s, const EwaldDev<T>& ew, double* out, cudaStream_t st)
{
  const int ch    = le_chunk(s.ne, ew.nmax, sizeof(T));
  const size_t sm = le_smem_ch(s.ne, ew.nmax, sizeof(T), ch);
  if (sm > LE_SMEM_MAX)
    return cudaErrorInvalidValue;
  local_energy_kernel<T><<<s.nw, LE_NT, sm, st>>>(s, ew, out, ch);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Per-electron gradient and Laplacian of log psi from the tracked state
// (TrialWaveFunction::mw_evaluateGL, TrialWaveFunction.cpp:869-919, over the
// components' mw_evaluateGL: DiracDeterminantBatched.cpp:594-603,
// TwoBodyJastrow.cpp:774-775, J1OrbitalSoA.h:119-120):
//   G_i = Ainv[r].dphi_i + dUat_i + Grad1_i
//   L_i = Ainv[r].d2phi_i - |Ainv[r].dphi_i|^2 + d2Uat_i - Lap1_i
// The same sums as the kinetic term of local_energy_kernel.  One CTA of 256
// threads covers 8 electrons (a warp each) of one walker: grid (ceil(ne / 8), nw).
// gl: [nw][ne][4] FP64 = G xyz, L.
// ---------------------------------------------------------------------------
template<typename T>
__global__ void __launch_bounds__(256) evaluate_gl_kernel(DevState<T> s, double* __restrict__ gl)
{
  // a warp per 32 consecutive electrons: the row sums of one electron at a time over the
  // lanes, then the FP64 combination for all 32 at once, lane q holding electron i0 + q (the
  // FP64 pipe's time goes by warp instruction, whatever the active lanes)
  const int iw = blockIdx.y, lane = threadIdx.x & 31;
  const int i0 = (blockIdx.x * 8 + (threadIdx.x >> 5)) * 32;
  if (i0 >= s.ne)
    return;
  const int N = s.norb, lda = s.lda;
  const int cnt = min(32, s.ne - i0);
  T kg[4] = {T(0), T(0), T(0), T(0)};
  for (int q = 0; q < cnt; q++)
  {
    const int i     = i0 + q;
    const int sp    = i < s.nup ? 0 : 1;
    const size_t rb = ((size_t)sp * s.nw + iw) * N + (i - sp * s.nup);
    const T* a      = s.Ainv + rb * lda;
    const T* g      = s.dgrad + rb * 3 * lda;
    const T* l      = s.dlap + rb * lda;
    T gx = 0, gy = 0, gz = 0, lp = 0;
    for (int o = lane; o < N; o += 32)
    {
      const T av = a[o];
      gx += av * g[o];
      gy += av * g[lda + o];
      gz += av * g[2 * lda + o];
      lp += av * l[o];
    }
    gx = warp_sum(gx);
    gy = warp_sum(gy);
    gz = warp_sum(gz);
    lp = warp_sum(lp);
    if (lane == q)
    {
      kg[0] = gx;
      kg[1] = gy;
      kg[2] = gz;
      kg[3] = lp;
    }
  }
  if (lane >= cnt)
    return;
  const int i = i0 + lane;
  double G[3] = {static_cast<double>(kg[0]), static_cast<double>(kg[1]), static_cast<double>(kg[2])};
  double L    = static_cast<double>(kg[3]) - (G[0] * G[0] + G[1] * G[1] + G[2] * G[2]);
  if (s.has_j2)
  {
    const T* j2 = s.J2 + (size_t)iw * 5 * s.ne_pad + i;
#pragma unroll
    for (int d = 0; d < 3; d++)
      G[d] += static_cast<double>(j2[(1 + d) * s.ne_pad]);
    L += static_cast<double>(j2[4 * s.ne_pad]);
  }
  if (s.has_j1)
  {
    const T* j1 = s.J1 + (size_t)iw * 5 * s.ne_pad + i;
#pragma unroll
    for (int d = 0; d < 3; d++)
      G[d] += static_cast<double>(j1[(1 + d) * s.ne_pad]);
    L -= static_cast<double>(j1[4 * s.ne_pad]);
  }
  // G [nw][ne][3] then L [nw][ne], the caller's layouts
  const size_t e = (size_t)iw * s.ne + i;
  gl[3 * e]     = G[0];
  gl[3 * e + 1] = G[1];
  gl[3 * e + 2] = G[2];
  gl[3 * (size_t)s.nw * s.ne + e] = L;
}

template<typename T>
cudaError_t launch_evaluate_gl(const DevState<T>& s, double* gl, cudaStream_t st)
{
  const dim3 grid((s.ne + 255) / 256, s.nw);
  evaluate_gl_kernel<T><<<grid, 256, 0, st>>>(s, gl);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// host: G vectors, ion structure factor and constants
// ---------------------------------------------------------------------------
int ewald_build(const double L[3], int ne, int nions, const double* ion_pos, const double* ion_q, double eps,
                EwaldHost& t)
{
  const double vol  = L[0] * L[1] * L[2];
  const double sq   = std::sqrt(-std::log(eps));
  const double rcut = 0.5 * std::min(L[0], std::min(L[1], L[2]));
  const double al   = sq / rcut;
  const double gc   = 2 * al * sq;
  int nm[3];
  for (int d = 0; d < 3; d++)
    nm[d] = (int)std::floor(gc * L[d] / (2 * M_PI));
  const int nmax = std::max(nm[0], std::max(nm[1], nm[2]));
  if (nmax > 127)
    return -1;
  t.alpha = al;
  t.nmax  = nmax;
  t.gn.clear();
  t.fg.clear();
  t.rho_ion.clear();
  double e_ion_k = 0;
  for (int a = 0; a <= nm[0]; a++)
    for (int b = -nm[1]; b <= nm[1]; b++)
      for (int c = -nm[2]; c <= nm[2]; c++)
      {
        if (a == 0 && (b < 0 || (b == 0 && c <= 0)))
          continue;
        const double g[3] = {2 * M_PI * a / L[0], 2 * M_PI * b / L[1], 2 * M_PI * c / L[2]};
        const double g2   = g[0] * g[0] + g[1] * g[1] + g[2] * g[2];
        if (g2 > gc * gc)
          continue;
        const double f = 4 * M_PI / vol * std::exp(-g2 / (4 * al * al)) / g2;
        double rr = 0, ri = 0;
        for (int I = 0; I < nions; I++)
        {
          const double ph = g[0] * ion_pos[3 * I] + g[1] * ion_pos[3 * I + 1] + g[2] * ion_pos[3 * I + 2];
          rr += ion_q[I] * std::cos(ph);
          ri += ion_q[I] * std::sin(ph);
        }
        t.gn.push_back({(signed char)a, (signed char)b, (signed char)c, 0});
        t.fg.push_back(f);
        t.rho_ion.push_back(rr);
        t.rho_ion.push_back(ri);
        e_ion_k += f * (rr * rr + ri * ri);
      }
  // ion-ion real-space part over the neighbouring images
  double e_ion_r = 0;
  for (int I = 0; I < nions; I++)
    for (int J = 0; J < I; J++)
      for (int x = -1; x <= 1; x++)
        for (int y = -1; y <= 1; y++)
          for (int z = -1; z <= 1; z++)
          {
            double d[3] = {ion_pos[3 * I] - ion_pos[3 * J], ion_pos[3 * I + 1] - ion_pos[3 * J + 1],
                           ion_pos[3 * I + 2] - ion_pos[3 * J + 2]};
            for (int k = 0; k < 3; k++)
              d[k] -= L[k] * std::round(d[k] / L[k]);
            d[0] += x * L[0];
            d[1] += y * L[1];
            d[2] += z * L[2];
            const double r = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            e_ion_r += ion_q[I] * ion_q[J] * std::erfc(al * r) / r;
          }
  double q2 = ne, qt = -ne;
  for (int I = 0; I < nions; I++)
  {
    q2 += ion_q[I] * ion_q[I];
    qt += ion_q[I];
  }
  // self energy -a/sqrt(pi) sum q^2, background -pi Q^2/(2 a^2 V)
  t.e_const = e_ion_r + e_ion_k - al / std::sqrt(M_PI) * q2 - M_PI * qt * qt / (2 * al * al * vol);
  return 0;
}

template cudaError_t setup_local_energy<float>();
template cudaError_t setup_local_energy<double>();
template cudaError_t launch_local_energy<float>(const DevState<float>&, const EwaldDev<float>&, double*, cudaStream_t);
template cudaError_t launch_local_energy<double>(const DevState<double>&, const EwaldDev<double>&, double*,
                                                 cudaStream_t);
template cudaError_t launch_evaluate_gl<float>(const DevState<float>&, double*, cudaStream_t);
template cudaError_t launch_evaluate_gl<double>(const DevState<double>&, double*, cudaStream_t);

} // namespace qmcg
