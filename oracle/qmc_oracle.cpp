// CPU oracle for the batched particle-by-particle Slater-Jastrow move loop.
//
// TEST INFRASTRUCTURE ONLY.  This file is a plain, scalar CPU restatement of the
// reference (QMCPACK 4.3.0) algorithms for the hot path.  It is compiled into
// liboracle.so and used by tests/, by __graft_entry__.smoke() and by the
// cpu_baseline / --impl reference legs of bench.py, always as the checker,
// never as the product path.  Every function cites the reference file:line it
// restates.  Parity is pinned by the reference's own golden vectors (see
// tests/test_oracle_golden.py) and cross-checked against the reference headers
// compiled as-is (oracle/build_ref.sh -> oracle/_ref/).
//
// Conventions (same as the reference):
//   * M[e][o] = phi_o(r_e) is the Slater matrix of one spin group;
//     Ainv = (M^-1)^T is stored row-major, so a determinant ratio for electron
//     e is dot(Ainv[e], phi(r_new))  (DiracDeterminantBatched.cpp:300).
//   * displacement rows are dr_j = R_j - r (minimum image), see
//     ParticleBConds3DSoa.h:120-130.
//   * two-body Jastrow J2 = exp(-sum_{i<j} u(r_ij)); Uat[i] = sum_j u(r_ij),
//     dUat = grad log J2 contribution, d2Uat = lap log J2 contribution
//     (BsplineFunctor.cpp:26-133, TwoBodyJastrow.cpp:581-629).
//   * the delayed-update engine follows the batched variant, including the
//     crowd-wide delay count and the "pseudo accept" of rejected walkers
//     (DelayedUpdateBatched.h:542-670, matrix_update_helper.cu:298-386).

#include <cmath>
#include <cstdint>
#include <cstring>
#include <cfloat>
#include <limits>
#include <random>
#include <vector>
#include <algorithm>
#include <complex>
#include <stdexcept>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc
{

// ---------------------------------------------------------------------------
// Random numbers: StdRandom<double> (src/Utilities/StdRandom.h:34-59):
// std::mt19937, uniform = (eng()-min)/(max-min+1).  Box-Muller pairs as in
// assignGaussRand (src/Particle/ParticleBase/RandomSeqGenerator.h:33-51).
// ---------------------------------------------------------------------------
struct Rng
{
  std::mt19937 eng;
  explicit Rng(uint32_t seed) : eng(seed) {}
  double uniform()
  {
    const uint32_t x = eng();
    return static_cast<double>(x - std::mt19937::min()) /
        (static_cast<double>(std::mt19937::max() - std::mt19937::min()) + 1.0);
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

// ---------------------------------------------------------------------------
// The counter-based stream of the device sweeps (no reference counterpart: the
// reference draws from mt19937 on the host).  Philox4x32-10 as published by
// Salmon, Moraes, Dror and Shaw (SC'11, "Parallel random numbers: as easy as
// 1, 2, 3"): ten rounds of two 32x32->64 multiplies with the Weyl key schedule.
// Counter (walker, electron, sweep, j) under the key (seed low, seed high):
// j = 0, 1 give four uniforms for the Box-Muller Gaussians of the proposal
// (pairs as in assignGaussRand, RandomSeqGenerator.h:33-51), j = 2 the uniform of
// the acceptance test.  A uniform is 53 bits of two words, in [0, 1).
// ---------------------------------------------------------------------------
struct P4
{
  uint32_t x, y, z, w;
};

inline P4 philox4x32_10(P4 c, uint32_t k0, uint32_t k1)
{
  for (int r = 0; r < 10; r++)
  {
    const uint64_t p0 = static_cast<uint64_t>(0xD2511F53u) * c.x;
    const uint64_t p1 = static_cast<uint64_t>(0xCD9E8D57u) * c.z;
    const uint32_t hi0 = static_cast<uint32_t>(p0 >> 32), lo0 = static_cast<uint32_t>(p0);
    const uint32_t hi1 = static_cast<uint32_t>(p1 >> 32), lo1 = static_cast<uint32_t>(p1);
    c = P4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return c;
}

inline double philox_u01(uint32_t a, uint32_t b)
{
  const uint64_t v = (static_cast<uint64_t>(a) << 21) ^ static_cast<uint64_t>(b >> 11);
  return static_cast<double>(v & ((1ull << 53) - 1)) * (1.0 / 9007199254740992.0);
}

struct PhiloxStream
{
  uint32_t k0, k1;
  explicit PhiloxStream(uint64_t seed) : k0(static_cast<uint32_t>(seed)), k1(static_cast<uint32_t>(seed >> 32)) {}
  // three unit Gaussians of the proposal of electron iat of walker w in sweep `sweep`
  void gauss3(uint32_t w, uint32_t iat, uint32_t sweep, double out[3]) const
  {
    const P4 r0 = philox4x32_10(P4{w, iat, sweep, 0u}, k0, k1);
    const P4 r1 = philox4x32_10(P4{w, iat, sweep, 1u}, k0, k1);
    const double one_m = 1.0 - std::numeric_limits<double>::epsilon();
    const double t1    = std::sqrt(-2.0 * std::log(1.0 - one_m * philox_u01(r0.x, r0.y)));
    const double t2    = 2.0 * M_PI * philox_u01(r0.z, r0.w);
    const double t3    = std::sqrt(-2.0 * std::log(1.0 - one_m * philox_u01(r1.x, r1.y)));
    const double t4    = 2.0 * M_PI * philox_u01(r1.z, r1.w);
    out[0]             = t1 * std::cos(t2);
    out[1]             = t1 * std::sin(t2);
    out[2]             = t3 * std::cos(t4);
  }
  double uniform(uint32_t w, uint32_t iat, uint32_t sweep) const
  {
    const P4 r2 = philox4x32_10(P4{w, iat, sweep, 2u}, k0, k1);
    return philox_u01(r2.x, r2.y);
  }
};

// fields of one move record (the layout of the library's move trace)
enum : int
{
  TR_POS = 0, TR_RATIO = 3, TR_GRAD_NEW = 4, TR_GRAD_NOW = 7, TR_ACCEPT = 10, TR_SELF = 11, TRACE_FIELDS = 12
};

// ---------------------------------------------------------------------------
// getSplineBound (src/Numerics/SplineBound.hpp:36-61)
// ---------------------------------------------------------------------------
template<typename T>
inline void spline_bound(T x, int nmax, int& ind, T& dx)
{
  if (x < 0)
  {
    ind = 0;
    dx  = T(0);
  }
  else
  {
    T ipart;
    dx  = std::modf(x, &ipart);
    ind = static_cast<int>(ipart);
    if (ind > nmax)
    {
      ind = nmax;
      dx  = T(1) - std::numeric_limits<T>::epsilon();
    }
  }
}

// ---------------------------------------------------------------------------
// cubic B-spline prefactors (src/spline2/MultiBsplineData.hpp:52-80)
// ---------------------------------------------------------------------------
template<typename T>
inline void prefactors(T a[4], T da[4], T d2a[4], T t)
{
  const T A00 = T(-1.0 / 6.0), A01 = T(3.0 / 6.0), A02 = T(-3.0 / 6.0), A03 = T(1.0 / 6.0);
  const T A10 = T(3.0 / 6.0), A11 = T(-6.0 / 6.0), A12 = T(0.0), A13 = T(4.0 / 6.0);
  const T A20 = T(-3.0 / 6.0), A21 = T(3.0 / 6.0), A22 = T(3.0 / 6.0), A23 = T(1.0 / 6.0);
  const T A30 = T(1.0 / 6.0), A31 = T(0.0), A32 = T(0.0), A33 = T(0.0);
  a[0]   = ((A00 * t + A01) * t + A02) * t + A03;
  a[1]   = ((A10 * t + A11) * t + A12) * t + A13;
  a[2]   = ((A20 * t + A21) * t + A22) * t + A23;
  a[3]   = ((A30 * t + A31) * t + A32) * t + A33;
  da[0]  = (T(-0.5) * t + T(1.0)) * t + T(-0.5);
  da[1]  = (T(1.5) * t + T(-2.0)) * t + T(0.0);
  da[2]  = (T(-1.5) * t + T(1.0)) * t + T(0.5);
  da[3]  = (T(0.5) * t + T(0.0)) * t + T(0.0);
  d2a[0] = T(-1.0) * t + T(1.0);
  d2a[1] = T(3.0) * t + T(-2.0);
  d2a[2] = T(-3.0) * t + T(1.0);
  d2a[3] = T(1.0) * t + T(0.0);
}

// ---------------------------------------------------------------------------
// Multi-orbital tricubic spline on a periodic unit cube, ghost layout
// N = M + 3 per axis (src/spline2/MultiBsplineBase.hpp:75-130), orbital index
// fastest (z_stride = npad).
// ---------------------------------------------------------------------------
template<typename ST>
struct Spline
{
  int M[3];
  int npad;
  size_t xs, ys, zs;
  std::vector<ST> coefs;
  void init(const int grid[3], int npad_, const double* c)
  {
    for (int d = 0; d < 3; d++)
      M[d] = grid[d];
    npad = npad_;
    zs   = npad;
    ys   = (size_t)(M[2] + 3) * zs;
    xs   = (size_t)(M[1] + 3) * ys;
    const size_t n = (size_t)(M[0] + 3) * xs;
    coefs.resize(n);
    for (size_t i = 0; i < n; i++)
      coefs[i] = static_cast<ST>(c[i]);
  }

  // evaluate_vgh_impl (src/spline2/MultiBsplineVGLH.hpp:120-230): value,
  // gradient and hessian (xx,xy,xz,yy,yz,zz) in unit-cube coordinates.
  void vgh(ST x, ST y, ST z, int norb, ST* v, ST* g /*[3][norb]*/, ST* h /*[6][norb]*/) const
  {
    int ix, iy, iz;
    ST tx, ty, tz;
    // grid start 0, delta_inv = M (MultiBsplineEval_helper.hpp:65-95)
    spline_bound<ST>(x * ST(M[0]), M[0] - 1, ix, tx);
    spline_bound<ST>(y * ST(M[1]), M[1] - 1, iy, ty);
    spline_bound<ST>(z * ST(M[2]), M[2] - 1, iz, tz);
    ST a[4], b[4], c[4], da[4], db[4], dc[4], d2a[4], d2b[4], d2c[4];
    prefactors<ST>(a, da, d2a, tx);
    prefactors<ST>(b, db, d2b, ty);
    prefactors<ST>(c, dc, d2c, tz);
    for (int n = 0; n < norb; n++)
    {
      v[n] = 0;
      for (int d = 0; d < 3; d++)
        g[d * norb + n] = 0;
      for (int d = 0; d < 6; d++)
        h[d * norb + n] = 0;
    }
    for (int i = 0; i < 4; i++)
      for (int j = 0; j < 4; j++)
      {
        const ST* cf   = coefs.data() + (ix + i) * xs + (iy + j) * ys + iz * zs;
        const ST pre20 = d2a[i] * b[j];
        const ST pre10 = da[i] * b[j];
        const ST pre00 = a[i] * b[j];
        const ST pre11 = da[i] * db[j];
        const ST pre01 = a[i] * db[j];
        const ST pre02 = a[i] * d2b[j];
        for (int n = 0; n < norb; n++)
        {
          const ST c0   = cf[n];
          const ST c1   = cf[n + zs];
          const ST c2   = cf[n + 2 * zs];
          const ST c3   = cf[n + 3 * zs];
          const ST sum0 = c[0] * c0 + c[1] * c1 + c[2] * c2 + c[3] * c3;
          const ST sum1 = dc[0] * c0 + dc[1] * c1 + dc[2] * c2 + dc[3] * c3;
          const ST sum2 = d2c[0] * c0 + d2c[1] * c1 + d2c[2] * c2 + d2c[3] * c3;
          h[0 * norb + n] += pre20 * sum0;
          h[1 * norb + n] += pre11 * sum0;
          h[2 * norb + n] += pre10 * sum1;
          h[3 * norb + n] += pre02 * sum0;
          h[4 * norb + n] += pre01 * sum1;
          h[5 * norb + n] += pre00 * sum2;
          g[0 * norb + n] += pre10 * sum0;
          g[1 * norb + n] += pre01 * sum0;
          g[2 * norb + n] += pre00 * sum1;
          v[n] += pre00 * sum0;
        }
      }
    const ST dxi = ST(M[0]), dyi = ST(M[1]), dzi = ST(M[2]);
    for (int n = 0; n < norb; n++)
    {
      g[0 * norb + n] *= dxi;
      g[1 * norb + n] *= dyi;
      g[2 * norb + n] *= dzi;
      h[0 * norb + n] *= dxi * dxi;
      h[3 * norb + n] *= dyi * dyi;
      h[5 * norb + n] *= dzi * dzi;
      h[1 * norb + n] *= dxi * dyi;
      h[2 * norb + n] *= dxi * dzi;
      h[4 * norb + n] *= dyi * dzi;
    }
  }
};

// ---------------------------------------------------------------------------
// Radial B-spline functor (src/QMCWaveFunctions/Jastrow/BsplineFunctor.h:100-133
// for reset(), :254-280 for evaluate_impl with derivatives).
// ---------------------------------------------------------------------------
template<typename T>
struct Functor
{
  std::vector<T> coefs;
  T DeltaRInv = 0;
  T rcut      = 0;
  int max_index = 0;
  void reset(int nparams, double cutoff, const double* params, double cusp)
  {
    const int numCoefs = nparams + 4;
    const int numKnots = numCoefs - 2;
    const T DeltaR     = static_cast<T>(cutoff) / static_cast<T>(numKnots - 1);
    DeltaRInv          = T(1.0) / DeltaR;
    rcut               = static_cast<T>(cutoff);
    coefs.assign(numCoefs, T(0));
    coefs[1] = static_cast<T>(params[0]);
    coefs[2] = static_cast<T>(params[1]);
    coefs[0] = static_cast<T>(params[1]) - T(2.0) * DeltaR * static_cast<T>(cusp);
    for (int i = 2; i < nparams; i++)
      coefs[i + 1] = static_cast<T>(params[i]);
    max_index = numCoefs - 4;
  }
  // u, du/dr, d2u/dr2 (r < rcut assumed by the caller)
  T eval(T r, T& dudr, T& d2udr2) const
  {
    r *= DeltaRInv;
    int i;
    T t;
    spline_bound<T>(r, max_index, i, t);
    const T c0 = coefs[i], c1 = coefs[i + 1], c2 = coefs[i + 2], c3 = coefs[i + 3];
    d2udr2 = DeltaRInv * DeltaRInv *
        (c0 * (T(-1.0) * t + T(1.0)) + c1 * (T(3.0) * t + T(-2.0)) + c2 * (T(-3.0) * t + T(1.0)) +
         c3 * (T(1.0) * t + T(0.0)));
    dudr = DeltaRInv *
        (c0 * ((T(-0.5) * t + T(1.0)) * t + T(-0.5)) + c1 * ((T(1.5) * t + T(-2.0)) * t + T(0.0)) +
         c2 * ((T(-1.5) * t + T(1.0)) * t + T(0.5)) + c3 * ((T(0.5) * t + T(0.0)) * t + T(0.0)));
    return c0 * (((T(-1.0 / 6.0) * t + T(3.0 / 6.0)) * t + T(-3.0 / 6.0)) * t + T(1.0 / 6.0)) +
        c1 * (((T(3.0 / 6.0) * t + T(-6.0 / 6.0)) * t + T(0.0)) * t + T(4.0 / 6.0)) +
        c2 * (((T(-3.0 / 6.0) * t + T(3.0 / 6.0)) * t + T(3.0 / 6.0)) * t + T(1.0 / 6.0)) +
        c3 * (((T(1.0 / 6.0) * t + T(0.0)) * t + T(0.0)) * t + T(0.0));
  }
};

// ---------------------------------------------------------------------------
// Orthorhombic minimum image, DTD_BConds<T,3,PPPO>::computeDistances
// (src/Particle/Lattice/ParticleBConds3DSoa.h:94-140).  A zero length means
// an open (non-periodic) axis.
// ---------------------------------------------------------------------------
template<typename T>
struct Cell
{
  T L[3], Linv[3];
  bool periodic[3];
  void init(const double lat[3])
  {
    for (int d = 0; d < 3; d++)
    {
      periodic[d] = lat[d] > 0;
      L[d]        = static_cast<T>(lat[d]);
      Linv[d]     = periodic[d] ? static_cast<T>(1.0 / lat[d]) : T(0);
    }
  }
  // dr = R_j - r, minimum image
  inline void disp(T xj, T yj, T zj, T x0, T y0, T z0, T& dx, T& dy, T& dz) const
  {
    T d[3] = {xj - x0, yj - y0, zj - z0};
    for (int k = 0; k < 3; k++)
      if (periodic[k])
      {
        const T s = d[k] * Linv[k];
        d[k]      = L[k] * (s - std::round(s));
      }
    dx = d[0];
    dy = d[1];
    dz = d[2];
  }
};

// ---------------------------------------------------------------------------
// FP64 LU with partial pivoting (getrf semantics: first maximal |a| in the
// column) followed by the inverse, and the log determinant as in
// computeLogDet (src/QMCWaveFunctions/Fermion/DiracMatrix.h:100-110).
// Input a is n x n row-major; on return a holds its inverse.
// ---------------------------------------------------------------------------
inline void invert_lu(double* a, int n, double& log_abs, int& sign)
{
  std::vector<int> piv(n);
  log_abs = 0;
  sign    = 1;
  // LU, row-major, A = P L U
  for (int k = 0; k < n; k++)
  {
    int p      = k;
    double amx = std::fabs(a[k * n + k]);
    for (int i = k + 1; i < n; i++)
      if (std::fabs(a[i * n + k]) > amx)
      {
        amx = std::fabs(a[i * n + k]);
        p   = i;
      }
    piv[k] = p;
    if (p != k)
    {
      for (int j = 0; j < n; j++)
        std::swap(a[k * n + j], a[p * n + j]);
      sign = -sign;
    }
    const double d = a[k * n + k];
    if (d == 0.0)
      throw std::runtime_error("singular matrix");
    if (d < 0)
      sign = -sign;
    log_abs += std::log(std::fabs(d));
    const double dinv = 1.0 / d;
    for (int i = k + 1; i < n; i++)
      a[i * n + k] *= dinv;
    for (int i = k + 1; i < n; i++)
    {
      const double l = a[i * n + k];
      if (l != 0.0)
        for (int j = k + 1; j < n; j++)
          a[i * n + j] -= l * a[k * n + j];
    }
  }
  // inv(U)
  std::vector<double> inv((size_t)n * n, 0.0);
  for (int j = 0; j < n; j++)
  {
    inv[j * n + j] = 1.0 / a[j * n + j];
    for (int i = j - 1; i >= 0; i--)
    {
      double s = 0;
      for (int k = i + 1; k <= j; k++)
        s += a[i * n + k] * inv[k * n + j];
      inv[i * n + j] = -s / a[i * n + i];
    }
  }
  // inv(A) = inv(U) inv(L) P : solve X L = inv(U) column by column from the right
  for (int j = n - 2; j >= 0; j--)
    for (int i = 0; i < n; i++)
    {
      double s = inv[i * n + j];
      for (int k = j + 1; k < n; k++)
        s -= inv[i * n + k] * a[k * n + j];
      inv[i * n + j] = s;
    }
  // apply column interchanges in reverse
  for (int k = n - 1; k >= 0; k--)
    if (piv[k] != k)
      for (int i = 0; i < n; i++)
        std::swap(inv[i * n + k], inv[i * n + piv[k]]);
  std::copy(inv.begin(), inv.end(), a);
}

// ---------------------------------------------------------------------------
// Delayed rank-k Sherman-Morrison engine of one determinant of one walker
// (src/QMCWaveFunctions/Fermion/DelayedUpdate.h:85-215 for the algebra,
// DelayedUpdateBatched.h:174-738 for the batched semantics).  All matrices are
// row-major: U,V are k x n, Binv is k x k, tempMat is n x k.
// ---------------------------------------------------------------------------
template<typename T>
struct DelayEngine
{
  int n = 0, k = 1;
  std::vector<T> U, V, Binv, tempMat, p, invRow;
  std::vector<int> delay_list;
  void resize(int n_, int k_)
  {
    n = n_;
    k = k_;
    U.assign((size_t)k * n, T(0));
    V.assign((size_t)k * n, T(0));
    Binv.assign((size_t)k * k, T(0));
    tempMat.assign((size_t)n * k, T(0));
    p.assign(k, T(0));
    invRow.assign(n, T(0));
    delay_list.assign(k, 0);
  }
  // mw_prepareInvRow / getInvRow: invRow = Ainv[row] + V^T * (-Binv^T * (U * Ainv[row]))
  // The intermediate -Binv^T p is left in Binv row dc (DelayedUpdate.h:100-106).
  void prepare_inv_row(const T* Ainv, int row, int dc)
  {
    std::copy_n(Ainv + (size_t)row * n, n, invRow.data());
    if (dc == 0)
      return;
    for (int c = 0; c < dc; c++)
      p[c] = dot(U.data() + (size_t)c * n, invRow.data(), n);
    T* brow = Binv.data() + (size_t)dc * k;
    for (int i = 0; i < dc; i++)
    {
      T s = 0;
      for (int c = 0; c < dc; c++)
        s += Binv[(size_t)c * k + i] * p[c];
      brow[i] = -s;
    }
    for (int c = 0; c < dc; c++)
    {
      const T b     = brow[c];
      const T* vrow = V.data() + (size_t)c * n;
      for (int j = 0; j < n; j++)
        invRow[j] += vrow[j] * b;
    }
  }
  // mw_accept_rejectRow for one walker (DelayedUpdateBatched.h:542-670 and
  // add_delay_list_save_sigma_VGL_kernel, matrix_update_helper.cu:298-386).
  void accept_reject(const T* Ainv, int row, int dc, bool accepted, const T* phi, T ratio)
  {
    std::copy_n(Ainv + (size_t)row * n, n, V.data() + (size_t)dc * n);
    if (accepted)
    {
      for (int c = 0; c < dc; c++)
        p[c] = -dot(V.data() + (size_t)c * n, phi, n);
      const T sigma = T(1) / ratio;
      // y = sigma * Binv * p  -> column dc
      for (int i = 0; i < dc; i++)
      {
        T s = 0;
        for (int c = 0; c < dc; c++)
          s += Binv[(size_t)i * k + c] * p[c];
        Binv[(size_t)i * k + dc] = sigma * s;
      }
      // X += y * zrow  (zrow = Binv row dc left by prepare_inv_row)
      for (int i = 0; i < dc; i++)
        for (int j = 0; j < dc; j++)
          Binv[(size_t)i * k + j] += Binv[(size_t)dc * k + j] * Binv[(size_t)i * k + dc];
      delay_list[dc]            = row;
      Binv[(size_t)dc * k + dc] = sigma;
      for (int j = 0; j < dc; j++)
        Binv[(size_t)dc * k + j] *= sigma;
      std::copy_n(phi, n, U.data() + (size_t)dc * n);
    }
    else
    {
      std::fill_n(U.data() + (size_t)dc * n, n, T(0));
      for (int i = 0; i < dc; i++)
        Binv[(size_t)i * k + dc] = T(0);
      Binv[(size_t)dc * k + dc] = T(1);
      delay_list[dc]            = -1;
    }
  }
  // mw_updateInvMat (DelayedUpdateBatched.h:675-738; the CPU engine's three GEMMs,
  // DelayedUpdate.h:145-215): Ainv -= (Ainv U^T - E) (Binv V).  Loop orders keep every
  // inner loop contiguous (dot products with eight partial sums, row updates as axpy)
  // so the compiler vectorises them as a BLAS would.
  void update_inv(T* Ainv, int dc)
  {
    if (dc == 0)
      return;
    // tempMat[j][c] = sum_i Ainv[j][i] U[c][i]
    for (int j = 0; j < n; j++)
      for (int c = 0; c < dc; c++)
        tempMat[(size_t)j * k + c] = dot(Ainv + (size_t)j * n, U.data() + (size_t)c * n, n);
    for (int c = 0; c < dc; c++)
      if (delay_list[c] >= 0)
        tempMat[(size_t)delay_list[c] * k + c] -= T(1);
    // W = Binv V  (stored in U, k x n)
    std::vector<T> W((size_t)dc * n, T(0));
    for (int l = 0; l < dc; l++)
      for (int c = 0; c < dc; c++)
      {
        const T b     = Binv[(size_t)l * k + c];
        const T* vrow = V.data() + (size_t)c * n;
        T* wrow       = W.data() + (size_t)l * n;
        for (int i = 0; i < n; i++)
          wrow[i] += b * vrow[i];
      }
    std::copy(W.begin(), W.end(), U.begin());
    for (int j = 0; j < n; j++)
    {
      T* arow = Ainv + (size_t)j * n;
      for (int l = 0; l < dc; l++)
      {
        const T t     = tempMat[(size_t)j * k + l];
        const T* wrow = U.data() + (size_t)l * n;
        for (int i = 0; i < n; i++)
          arow[i] -= t * wrow[i];
      }
    }
  }
  // sum_i a[i] b[i] with eight independent partial sums
  static T dot(const T* a, const T* b, int n)
  {
    T acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    int i = 0;
    for (; i + 8 <= n; i += 8)
      for (int q = 0; q < 8; q++)
        acc[q] += a[i + q] * b[i + q];
    T s = ((acc[0] + acc[1]) + (acc[2] + acc[3])) + ((acc[4] + acc[5]) + (acc[6] + acc[7]));
    for (; i < n; i++)
      s += a[i] * b[i];
    return s;
  }
};

// ---------------------------------------------------------------------------
// Fahy's Sherman-Morrison rank-1 update (DelayedUpdateBatched.h:252-340 with
// copyAinvRow_saveGL_kernel, matrix_update_helper.cu:35-74):
//   temp = Ainv phi; temp[row] -= 1; Ainv -= (1/ratio) temp (x) Ainv[row]
// ---------------------------------------------------------------------------
template<typename T>
void sm1(T* Ainv, int n, int row, const T* phi, T ratio)
{
  std::vector<T> temp(n), rcopy(n);
  for (int j = 0; j < n; j++)
  {
    T sacc = 0;
    for (int i = 0; i < n; i++)
      sacc += Ainv[(size_t)j * n + i] * phi[i];
    temp[j] = sacc;
  }
  temp[row] -= T(1);
  std::copy_n(Ainv + (size_t)row * n, n, rcopy.data());
  const T c = T(-1) / ratio;
  for (int j = 0; j < n; j++)
    for (int i = 0; i < n; i++)
      Ainv[(size_t)j * n + i] += c * rcopy[i] * temp[j];
}

// ---------------------------------------------------------------------------
// The system and the crowd.
// ---------------------------------------------------------------------------
template<typename T>
struct Crowd
{
  // system
  int nup, ndn, ne, norb, npad, nions, nion_species;
  Cell<T> cell;
  double lattice[3];
  std::vector<double> ions;   // [nions][3]
  std::vector<int> ion_species;
  Spline<T> spline;
  std::vector<Functor<T>> j1f; // per ion species
  Functor<T> j2f[2];           // 0: same spin, 1: opposite spin
  bool has_j1 = false, has_j2 = false;
  int nw, delay;
  // walker state
  struct Det
  {
    std::vector<T> Ainv;   // n x n
    DelayEngine<T> eng;
    double log_abs = 0;
    int sign       = 1;
    T cur_ratio    = 1;
    std::vector<T> phi_v, phi_g, phi_l; // proposed move: n, 3n (SoA), n
  };
  struct Walker
  {
    std::vector<double> R; // ne x 3
    Det det[2];
    // J2
    std::vector<T> Uat, dUat, d2Uat; // ne, 3*ne (SoA), ne
    T cur_Uat;
    T cur_vgl[5];
    // J1
    std::vector<T> Vat, Grad, Lap; // ne, 3*ne (SoA), ne
    T curAt, curGrad[3], curLap;
    // proposed move
    double active_pos[3];
    // temp rows
    std::vector<T> new_r, new_dr, old_r, old_dr, ei_r, ei_dr;
  };
  std::vector<Walker> w;
  int delay_count[2] = {0, 0};

  int group_of(int iat) const { return iat < nup ? 0 : 1; }
  int first_of(int g) const { return g == 0 ? 0 : nup; }

  void init_walkers()
  {
    w.resize(nw);
    for (auto& wk : w)
    {
      wk.R.assign((size_t)ne * 3, 0.0);
      for (int s = 0; s < 2; s++)
      {
        Det& d = wk.det[s];
        d.Ainv.assign((size_t)norb * norb, T(0));
        d.eng.resize(norb, delay);
        d.phi_v.assign(norb, T(0));
        d.phi_g.assign((size_t)norb * 3, T(0));
        d.phi_l.assign(norb, T(0));
      }
      wk.Uat.assign(ne, T(0));
      wk.dUat.assign((size_t)ne * 3, T(0));
      wk.d2Uat.assign(ne, T(0));
      wk.Vat.assign(ne, T(0));
      wk.Grad.assign((size_t)ne * 3, T(0));
      wk.Lap.assign(ne, T(0));
      wk.new_r.assign(ne, T(0));
      wk.new_dr.assign((size_t)ne * 3, T(0));
      wk.old_r.assign(ne, T(0));
      wk.old_dr.assign((size_t)ne * 3, T(0));
      wk.ei_r.assign(std::max(nions, 1), T(0));
      wk.ei_dr.assign((size_t)std::max(nions, 1) * 3, T(0));
    }
  }

  // SplineR2R::convertPos (SplineR2R.h:156-169) for an orthorhombic cell:
  // PrimLattice.toUnit is r . G (CrystalLattice.h:182-185) with G = R^-1, a per-axis
  // product with 1/L here; the Gamma-point sign is +1.
  void convert_pos(const double r[3], T ru[3]) const
  {
    for (int d = 0; d < 3; d++)
    {
      T u = static_cast<T>(r[d] * (1.0 / lattice[d]));
      if (-std::numeric_limits<T>::epsilon() < u && u < 0)
        u = T(0);
      else
        u -= std::floor(u);
      ru[d] = u;
    }
  }

  // SplineR2R::evaluateVGL = evaluate_vgh + assign_vgl (SplineR2R.cpp:338-374, 392-404):
  // Cartesian gradient G*g and laplacian SymTrace(H, G G^T), orthorhombic G.
  void spo_vgl(const double r[3], T* v, T* g /*[3][norb]*/, T* l) const
  {
    T ru[3];
    convert_pos(r, ru);
    std::vector<T> gg((size_t)3 * norb), hh((size_t)6 * norb);
    spline.vgh(ru[0], ru[1], ru[2], norb, v, gg.data(), hh.data());
    const T G0 = T(1.0 / lattice[0]), G1 = T(1.0 / lattice[1]), G2 = T(1.0 / lattice[2]);
    const T GG0 = G0 * G0, GG1 = G1 * G1, GG2 = G2 * G2;
    for (int n = 0; n < norb; n++)
    {
      g[0 * norb + n] = G0 * gg[0 * norb + n];
      g[1 * norb + n] = G1 * gg[1 * norb + n];
      g[2 * norb + n] = G2 * gg[2 * norb + n];
      l[n]            = hh[0 * norb + n] * GG0 + hh[3 * norb + n] * GG1 + hh[5 * norb + n] * GG2;
    }
  }

  // distance row from position r to all electrons, dr_j = R_j - r
  void ee_row(const Walker& wk, const double r[3], T* dist, T* dr /*[3][ne]*/) const
  {
    const T x0 = static_cast<T>(r[0]), y0 = static_cast<T>(r[1]), z0 = static_cast<T>(r[2]);
    for (int j = 0; j < ne; j++)
    {
      T dx, dy, dz;
      cell.disp(static_cast<T>(wk.R[j * 3 + 0]), static_cast<T>(wk.R[j * 3 + 1]), static_cast<T>(wk.R[j * 3 + 2]), x0,
                y0, z0, dx, dy, dz);
      dr[0 * ne + j] = dx;
      dr[1 * ne + j] = dy;
      dr[2 * ne + j] = dz;
      dist[j]        = std::sqrt(dx * dx + dy * dy + dz * dz);
    }
  }
  void ei_row(const double r[3], T* dist, T* dr /*[3][nions]*/) const
  {
    const T x0 = static_cast<T>(r[0]), y0 = static_cast<T>(r[1]), z0 = static_cast<T>(r[2]);
    for (int j = 0; j < nions; j++)
    {
      T dx, dy, dz;
      cell.disp(static_cast<T>(ions[j * 3 + 0]), static_cast<T>(ions[j * 3 + 1]), static_cast<T>(ions[j * 3 + 2]), x0,
                y0, z0, dx, dy, dz);
      dr[0 * nions + j] = dx;
      dr[1 * nions + j] = dy;
      dr[2 * nions + j] = dz;
      dist[j]           = std::sqrt(dx * dx + dy * dy + dz * dz);
    }
  }

  const Functor<T>& j2_functor(int i, int j) const { return j2f[group_of(i) == group_of(j) ? 0 : 1]; }

  // J2 value/grad/lap sum over j != iat at distances dist (BsplineFunctor.cpp:93-131)
  void j2_vgl(int iat, const T* dist, const T* dr, T vgl[5], T* cu, T* cdu, T* cd2u) const
  {
    T val = 0, gx = 0, gy = 0, gz = 0, lap = 0;
    for (int j = 0; j < ne; j++)
    {
      T u = 0, du = 0, d2u = 0;
      if (j != iat)
      {
        const Functor<T>& f = j2_functor(iat, j);
        const T r           = dist[j];
        if (r < f.rcut)
        {
          u = f.eval(r, du, d2u);
          du *= T(1) / r;
        }
        val += u;
        lap += d2u + T(2) * du;
        gx += du * dr[0 * ne + j];
        gy += du * dr[1 * ne + j];
        gz += du * dr[2 * ne + j];
      }
      if (cu)
      {
        cu[j]   = u;
        cdu[j]  = du;
        cd2u[j] = d2u;
      }
    }
    vgl[0] = val;
    vgl[1] = gx;
    vgl[2] = gy;
    vgl[3] = gz;
    vgl[4] = -lap;
  }

  // J1 U, grad, lap at distances to ions (J1OrbitalSoA.h:136-188)
  void j1_vgl(const T* dist, const T* dr, T& U, T g[3], T& lap) const
  {
    U = 0;
    g[0] = g[1] = g[2] = 0;
    lap                = 0;
    std::vector<T> du(nions, T(0)), d2u(nions, T(0)), u(nions, T(0));
    for (int j = 0; j < nions; j++)
    {
      const Functor<T>& f = j1f[ion_species[j]];
      const T r           = dist[j];
      if (r < f.rcut)
      {
        T d1, d2;
        u[j]   = f.eval(r, d1, d2);
        du[j]  = d1 * (T(1) / r);
        d2u[j] = d2;
      }
    }
    for (int j = 0; j < nions; j++)
      lap += d2u[j] + T(2) * du[j];
    for (int d = 0; d < 3; d++)
    {
      T s = 0;
      for (int j = 0; j < nions; j++)
        s += du[j] * dr[d * nions + j];
      g[d] = s;
    }
    for (int j = 0; j < nions; j++)
      U += u[j];
  }

  // ---------------- mw_evaluateLog / mw_recompute -------------------------
  // DiracDeterminantBatched::mw_recompute (DiracDeterminantBatched.cpp:1122-1199):
  // all-electron VGL, FP64 inverse of the transpose and log det; J2 recompute
  // (TwoBodyJastrow.cpp:662-714); J1 recompute (J1OrbitalSoA.h:240-250).
  void recompute(int iw)
  {
    Walker& wk = w[iw];
    std::vector<T> v(norb), g((size_t)3 * norb), l(norb);
    for (int s = 0; s < 2; s++)
    {
      Det& d    = wk.det[s];
      const int first = first_of(s);
      std::vector<double> Mt((size_t)norb * norb);
      for (int e = 0; e < norb; e++)
      {
        spo_vgl(&wk.R[(size_t)(first + e) * 3], v.data(), g.data(), l.data());
        for (int o = 0; o < norb; o++)
          Mt[(size_t)o * norb + e] = static_cast<double>(v[o]); // transpose
        // orbital gradients / laplacians of electron e, stored [3][norb] and [norb]
        std::copy(g.begin(), g.end(), dgrad_row(iw, s, e));
        std::copy(l.begin(), l.end(), dlap_row(iw, s, e));
      }
      invert_lu(Mt.data(), norb, d.log_abs, d.sign);
      for (size_t i = 0; i < (size_t)norb * norb; i++)
        d.Ainv[i] = static_cast<T>(Mt[i]);
    }
    // J2
    std::fill(wk.Uat.begin(), wk.Uat.end(), T(0));
    std::fill(wk.dUat.begin(), wk.dUat.end(), T(0));
    std::fill(wk.d2Uat.begin(), wk.d2Uat.end(), T(0));
    if (has_j2)
    {
      std::vector<T> dist(ne), dr((size_t)3 * ne);
      for (int i = 0; i < ne; i++)
      {
        ee_row(wk, &wk.R[(size_t)i * 3], dist.data(), dr.data());
        T u_sum = 0, lap = 0, gr[3] = {0, 0, 0};
        std::vector<T> u(ne, T(0)), du(ne, T(0)), d2u(ne, T(0));
        for (int j = 0; j < i; j++)
        {
          const Functor<T>& f = j2_functor(i, j);
          const T r           = dist[j];
          if (r < f.rcut)
          {
            T d1, d2;
            u[j]   = f.eval(r, d1, d2);
            du[j]  = d1 * (T(1) / r);
            d2u[j] = d2;
          }
        }
        for (int j = 0; j < i; j++)
          u_sum += u[j];
        wk.Uat[i] += u_sum; // Uat[i] = sum_{j<i} u  (plus upper-triangle contributions later)
        for (int j = 0; j < i; j++)
          lap += d2u[j] + T(2) * du[j];
        for (int dd = 0; dd < 3; dd++)
        {
          T s = 0;
          for (int j = 0; j < i; j++)
            s += du[j] * dr[(size_t)dd * ne + j];
          gr[dd] = s;
        }
        for (int dd = 0; dd < 3; dd++)
          wk.dUat[(size_t)dd * ne + i] = gr[dd];
        wk.d2Uat[i] = -lap;
        for (int j = 0; j < i; j++)
        {
          wk.Uat[j] += u[j];
          wk.d2Uat[j] -= d2u[j] + T(2) * du[j];
        }
        for (int dd = 0; dd < 3; dd++)
          for (int j = 0; j < i; j++)
            wk.dUat[(size_t)dd * ne + j] -= du[j] * dr[(size_t)dd * ne + j];
      }
    }
    // J1
    for (int i = 0; i < ne; i++)
    {
      T U = 0, gr[3] = {0, 0, 0}, lap = 0;
      if (has_j1)
      {
        ei_row(&wk.R[(size_t)i * 3], wk.ei_r.data(), wk.ei_dr.data());
        j1_vgl(wk.ei_r.data(), wk.ei_dr.data(), U, gr, lap);
      }
      wk.Vat[i] = U;
      for (int dd = 0; dd < 3; dd++)
        wk.Grad[(size_t)dd * ne + i] = gr[dd];
      wk.Lap[i] = lap;
    }
  }

  // per-walker storage of orbital gradient / laplacian rows, [spin][e][3][norb] and [spin][e][norb]
  std::vector<T> dgrad, dlap;
  T* dgrad_row(int iw, int s, int e) { return dgrad.data() + (((size_t)iw * 2 + s) * norb + e) * 3 * norb; }
  T* dlap_row(int iw, int s, int e) { return dlap.data() + (((size_t)iw * 2 + s) * norb + e) * norb; }
  const T* dgrad_row(int iw, int s, int e) const { return dgrad.data() + (((size_t)iw * 2 + s) * norb + e) * 3 * norb; }
  const T* dlap_row(int iw, int s, int e) const { return dlap.data() + (((size_t)iw * 2 + s) * norb + e) * norb; }

  double log_j2(int iw) const
  {
    double s = 0;
    for (int i = 0; i < ne; i++)
      s += static_cast<double>(w[iw].Uat[i]);
    return -0.5 * s;
  }
  double log_j1(int iw) const
  {
    double s = 0;
    for (int i = 0; i < ne; i++)
      s += static_cast<double>(w[iw].Vat[i]);
    return -s;
  }

  // ---------------- TrialWaveFunction::mw_evaluateGL + BareKineticEnergy ----
  // With all delayed updates applied, per electron i of spin s and row r:
  //   G_i = Ainv[r].dphi_i + dUat_i + Grad1_i
  //   L_i = Ainv[r].d2phi_i - |Ainv[r].dphi_i|^2 + d2Uat_i - Lap1_i
  // (DiracDeterminantBatched.cpp:594-603, TwoBodyJastrow.cpp:774-775,
  // J1OrbitalSoA.h:119-120) and KE = -1/2 sum_i (|G_i|^2 + L_i) for unit mass
  // (BareKineticEnergy.cpp:110-117).  gl (optional): [ne][4] = G xyz, L.
  double kinetic(int iw, double* gl) const
  {
    const Walker& wk = w[iw];
    double ke        = 0;
    for (int iat = 0; iat < ne; iat++)
    {
      const int s   = group_of(iat);
      const int row = iat - first_of(s);
      const T* inv  = wk.det[s].Ainv.data() + (size_t)row * norb;
      const T* gr   = dgrad_row(iw, s, row);
      const T* lp   = dlap_row(iw, s, row);
      double g[3], l = 0;
      for (int dd = 0; dd < 3; dd++)
      {
        double acc = 0;
        for (int o = 0; o < norb; o++)
          acc += static_cast<double>(inv[o]) * static_cast<double>(gr[(size_t)dd * norb + o]);
        g[dd] = acc;
      }
      for (int o = 0; o < norb; o++)
        l += static_cast<double>(inv[o]) * static_cast<double>(lp[o]);
      l -= g[0] * g[0] + g[1] * g[1] + g[2] * g[2];
      for (int dd = 0; dd < 3; dd++)
      {
        if (has_j1)
          g[dd] += static_cast<double>(wk.Grad[(size_t)dd * ne + iat]);
        if (has_j2)
          g[dd] += static_cast<double>(wk.dUat[(size_t)dd * ne + iat]);
      }
      if (has_j1)
        l -= static_cast<double>(wk.Lap[iat]);
      if (has_j2)
        l += static_cast<double>(wk.d2Uat[iat]);
      ke += -0.5 * (g[0] * g[0] + g[1] * g[1] + g[2] * g[2] + l);
      if (gl)
      {
        for (int dd = 0; dd < 3; dd++)
          gl[(size_t)iat * 4 + dd] = g[dd];
        gl[(size_t)iat * 4 + 3] = l;
      }
    }
    return ke;
  }

  // ---------------- TrialWaveFunction::mw_evalGrad -------------------------
  void eval_grad(int iat, double* grads)
  {
    const int s   = group_of(iat);
    const int row = iat - first_of(s);
#pragma omp parallel for schedule(static)
    for (int iw = 0; iw < nw; iw++)
    {
      Walker& wk = w[iw];
      Det& d     = wk.det[s];
      const T* inv;
      if (delay > 1)
      {
        d.eng.prepare_inv_row(d.Ainv.data(), row, delay_count[s]);
        inv = d.eng.invRow.data();
      }
      else
        inv = d.Ainv.data() + (size_t)row * norb;
      const T* gr = dgrad_row(iw, s, row);
      T g[3]      = {0, 0, 0};
      for (int dd = 0; dd < 3; dd++)
      {
        T acc = 0;
        for (int o = 0; o < norb; o++)
          acc += inv[o] * gr[(size_t)dd * norb + o];
        g[dd] = acc;
      }
      for (int dd = 0; dd < 3; dd++)
      {
        double gsum = static_cast<double>(g[dd]);
        if (has_j1)
          gsum += static_cast<double>(wk.Grad[(size_t)dd * ne + iat]);
        if (has_j2)
          gsum += static_cast<double>(wk.dUat[(size_t)dd * ne + iat]);
        grads[iw * 3 + dd] = gsum;
      }
    }
  }

  // ---------------- ParticleSet::mw_makeMove -------------------------------
  void make_move(int iat, const double* displ)
  {
#pragma omp parallel for schedule(static)
    for (int iw = 0; iw < nw; iw++)
    {
      Walker& wk = w[iw];
      for (int dd = 0; dd < 3; dd++)
        wk.active_pos[dd] = wk.R[(size_t)iat * 3 + dd] + displ[iw * 3 + dd];
      ee_row(wk, wk.active_pos, wk.new_r.data(), wk.new_dr.data());
      ee_row(wk, &wk.R[(size_t)iat * 3], wk.old_r.data(), wk.old_dr.data());
      wk.old_r[iat] = std::numeric_limits<T>::max();
      if (nions > 0)
        ei_row(wk.active_pos, wk.ei_r.data(), wk.ei_dr.data());
    }
  }

  // ParticleSet::mw_makeMove with the proposed positions given directly
  void make_move_to(int iat, const double* pos /*[nw][3]*/)
  {
#pragma omp parallel for schedule(static)
    for (int iw = 0; iw < nw; iw++)
    {
      Walker& wk = w[iw];
      for (int dd = 0; dd < 3; dd++)
        wk.active_pos[dd] = pos[iw * 3 + dd];
      ee_row(wk, wk.active_pos, wk.new_r.data(), wk.new_dr.data());
      ee_row(wk, &wk.R[(size_t)iat * 3], wk.old_r.data(), wk.old_dr.data());
      wk.old_r[iat] = std::numeric_limits<T>::max();
      if (nions > 0)
        ei_row(wk.active_pos, wk.ei_r.data(), wk.ei_dr.data());
    }
  }

  // ---------------- TrialWaveFunction::mw_calcRatioGrad --------------------
  // component order: determinant, J1, J2; ratios multiplied, grads summed
  // (TrialWaveFunction.cpp:685-772).
  void ratio_grad(int iat, double* ratios, double* grads)
  {
    const int s   = group_of(iat);
    const int row = iat - first_of(s);
#pragma omp parallel for schedule(static)
    for (int iw = 0; iw < nw; iw++)
    {
      Walker& wk = w[iw];
      Det& d     = wk.det[s];
      const T* inv;
      if (delay > 1)
        inv = d.eng.invRow.data();
      else
        inv = d.Ainv.data() + (size_t)row * norb;
      spo_vgl(wk.active_pos, d.phi_v.data(), d.phi_g.data(), d.phi_l.data());
      T ratio = 0, gx = 0, gy = 0, gz = 0;
      for (int o = 0; o < norb; o++)
      {
        ratio += d.phi_v[o] * inv[o];
        gx += d.phi_g[0 * norb + o] * inv[o];
        gy += d.phi_g[1 * norb + o] * inv[o];
        gz += d.phi_g[2 * norb + o] * inv[o];
      }
      d.cur_ratio    = ratio;
      double r_total = static_cast<double>(ratio);
      double g[3]    = {static_cast<double>(gx / ratio), static_cast<double>(gy / ratio),
                        static_cast<double>(gz / ratio)};
      if (has_j1)
      {
        j1_vgl(wk.ei_r.data(), wk.ei_dr.data(), wk.curAt, wk.curGrad, wk.curLap);
        r_total *= std::exp(static_cast<double>(wk.Vat[iat] - wk.curAt));
        for (int dd = 0; dd < 3; dd++)
          g[dd] += static_cast<double>(wk.curGrad[dd]);
      }
      if (has_j2)
      {
        j2_vgl(iat, wk.new_r.data(), wk.new_dr.data(), wk.cur_vgl, nullptr, nullptr, nullptr);
        wk.cur_Uat = wk.cur_vgl[0];
        r_total *= std::exp(static_cast<double>(wk.Uat[iat] - wk.cur_Uat));
        for (int dd = 0; dd < 3; dd++)
          g[dd] += static_cast<double>(wk.cur_vgl[1 + dd]);
      }
      ratios[iw] = r_total;
      for (int dd = 0; dd < 3; dd++)
        grads[iw * 3 + dd] = g[dd];
    }
  }

  // ---------------- TrialWaveFunction::mw_accept_rejectMove ----------------
  void accept_reject(int iat, const int* accepted)
  {
    const int s   = group_of(iat);
    const int row = iat - first_of(s);
#pragma omp parallel for schedule(static)
    for (int iw = 0; iw < nw; iw++)
    {
      Walker& wk = w[iw];
      Det& d     = wk.det[s];
      const bool acc = accepted[iw] != 0;
      // determinant (DiracDeterminantBatched.cpp:464-523)
      if (acc)
      {
        const double rr = static_cast<double>(d.cur_ratio);
        d.log_abs += std::log(std::fabs(rr));
        if (rr < 0)
          d.sign = -d.sign;
      }
      if (delay > 1)
        d.eng.accept_reject(d.Ainv.data(), row, delay_count[s], acc, d.phi_v.data(), d.cur_ratio);
      else if (acc)
        sm1_update(d, row);
      if (acc)
      {
        std::copy(d.phi_g.begin(), d.phi_g.end(), dgrad_row(iw, s, row));
        std::copy(d.phi_l.begin(), d.phi_l.end(), dlap_row(iw, s, row));
      }
      d.cur_ratio = 1;
      if (acc)
      {
        // J1 acceptMove (J1OrbitalSoA.h:456-468)
        if (has_j1)
        {
          wk.Vat[iat] = wk.curAt;
          for (int dd = 0; dd < 3; dd++)
            wk.Grad[(size_t)dd * ne + iat] = wk.curGrad[dd];
          wk.Lap[iat] = wk.curLap;
        }
        // J2 mw_updateVGL (BsplineFunctor.cpp:203-320)
        if (has_j2)
        {
          for (int j = 0; j < ne; j++)
          {
            if (j == iat)
              continue;
            const Functor<T>& f = j2_functor(iat, j);
            T u = 0, du = 0, d2u = 0;
            const T r = wk.old_r[j];
            if (r < f.rcut)
            {
              u = f.eval(r, du, d2u);
              du *= T(1) / r;
            }
            T cu = 0, cdu = 0, cd2u = 0;
            const T rn = wk.new_r[j];
            if (rn < f.rcut)
            {
              cu = f.eval(rn, cdu, cd2u);
              cdu *= T(1) / rn;
            }
            wk.Uat[j] += cu - u;
            for (int dd = 0; dd < 3; dd++)
              wk.dUat[(size_t)dd * ne + j] -= wk.new_dr[(size_t)dd * ne + j] * cdu - wk.old_dr[(size_t)dd * ne + j] * du;
            wk.d2Uat[j] -= cd2u + T(2) * cdu - (d2u + T(2) * du);
          }
          wk.Uat[iat] = wk.cur_vgl[0];
          for (int dd = 0; dd < 3; dd++)
            wk.dUat[(size_t)dd * ne + iat] = wk.cur_vgl[1 + dd];
          wk.d2Uat[iat] = wk.cur_vgl[4];
        }
        for (int dd = 0; dd < 3; dd++)
          wk.R[(size_t)iat * 3 + dd] = wk.active_pos[dd];
      }
    }
    if (delay > 1)
    {
      delay_count[s]++;
      if (delay_count[s] == delay)
        flush(s);
    }
  }

  void sm1_update(Det& d, int row) { sm1(d.Ainv.data(), norb, row, d.phi_v.data(), d.cur_ratio); }

  void flush(int s)
  {
    if (delay_count[s] == 0)
      return;
#pragma omp parallel for schedule(static)
    for (int iw = 0; iw < nw; iw++)
      w[iw].det[s].eng.update_inv(w[iw].det[s].Ainv.data(), delay_count[s]);
    delay_count[s] = 0;
  }
  void complete_updates()
  {
    if (delay > 1)
    {
      flush(0);
      flush(1);
    }
  }

  // ---------------- VMCBatched::advanceWalkers (VMCBatched.cpp:106-177) -----
  // drift-diffusion with the Umrigar drift (DriftModifierUNR.cpp:20-30, a = 1)
  static void unr_drift(double tau, const double g[3], double d[3])
  {
    const double vsq = g[0] * g[0] + g[1] * g[1] + g[2] * g[2];
    const double sc  = vsq < std::numeric_limits<double>::epsilon() ? tau : ((-1.0 + std::sqrt(1.0 + 2.0 * tau * vsq)) / vsq);
    for (int k = 0; k < 3; k++)
      d[k] = g[k] * sc;
  }

  void sweep(Rng& rng, double tau, bool use_drift, long* n_accept, long* n_reject, int* accept_log /*[ne][nw] or null*/)
  {
    std::vector<double> deltas((size_t)nw * ne * 3);
    rng.gauss(deltas.data(), deltas.size());
    const double sqrttau = std::sqrt(tau), oneover2tau = 0.5 / tau;
    std::vector<double> grads_now((size_t)nw * 3), grads_new((size_t)nw * 3), drift((size_t)nw * 3), ratios(nw);
    std::vector<double> log_gf(nw), log_gb(nw), prob(nw);
    std::vector<int> acc(nw);
    const double eps = std::numeric_limits<T>::epsilon();
    for (int g = 0; g < 2; g++)
    {
      const int first = first_of(g), last = g == 0 ? nup : ne;
      for (int iat = first; iat < last; iat++)
      {
        double* dl = &deltas[(size_t)iat * nw * 3];
        for (size_t i = 0; i < (size_t)nw * 3; i++)
          dl[i] *= sqrttau;
        if (use_drift)
        {
          eval_grad(iat, grads_now.data());
          for (int iw = 0; iw < nw; iw++)
          {
            unr_drift(tau, &grads_now[iw * 3], &drift[iw * 3]);
            for (int k = 0; k < 3; k++)
              drift[iw * 3 + k] += dl[iw * 3 + k];
          }
        }
        else
        {
          // the up-to-date inverse row of iat is formed here for the ratio (mw_getInvRow)
          if (delay > 1)
            eval_grad(iat, grads_now.data());
          std::copy_n(dl, (size_t)nw * 3, drift.data());
        }
        make_move(iat, drift.data());
        if (use_drift)
        {
          ratio_grad(iat, ratios.data(), grads_new.data());
          for (int iw = 0; iw < nw; iw++)
          {
            const double* d = dl + iw * 3;
            log_gf[iw]      = -oneover2tau * (d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            double dr[3];
            unr_drift(tau, &grads_new[iw * 3], dr);
            for (int k = 0; k < 3; k++)
              dr[k] += drift[iw * 3 + k];
            log_gb[iw] = -oneover2tau * (dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2]);
          }
        }
        else
        {
          ratio_grad(iat, ratios.data(), grads_new.data());
          std::fill(log_gf.begin(), log_gf.end(), 0.0);
          std::fill(log_gb.begin(), log_gb.end(), 0.0);
        }
        for (int iw = 0; iw < nw; iw++)
          prob[iw] = ratios[iw] * ratios[iw];
        for (int iw = 0; iw < nw; iw++)
        {
          if (prob[iw] >= eps && rng.uniform() < prob[iw] * std::exp(log_gb[iw] - log_gf[iw]))
          {
            acc[iw] = 1;
            (*n_accept)++;
          }
          else
          {
            acc[iw] = 0;
            (*n_reject)++;
          }
          if (accept_log)
            accept_log[(size_t)iat * nw + iw] = acc[iw];
        }
        accept_reject(iat, acc.data());
      }
    }
    complete_updates();
  }
};

// ---------------------------------------------------------------------------
// Sweeps on the counter-based stream, electron by electron as
// VMCBatched::advanceWalkers (VMCBatched.cpp:106-177), one record per move in
// trace [ne][nw][TRACE_FIELDS] (may be null).  Every walker draws its own numbers,
// so the acceptance uniform of walker w does not depend on the other walkers.
// ---------------------------------------------------------------------------
template<typename T>
void sweep_philox(Crowd<T>& c, const PhiloxStream& ps, uint32_t sweep, double tau, bool use_drift, long* n_accept,
                  long* n_reject, double* trace)
{
  const int nw = c.nw, ne = c.ne;
  const double sqrttau = std::sqrt(tau), oneover2tau = 0.5 / tau;
  std::vector<double> grads_now((size_t)nw * 3), grads_new((size_t)nw * 3), drift((size_t)nw * 3), dl((size_t)nw * 3);
  std::vector<double> ratios(nw), log_gf(nw), log_gb(nw);
  std::vector<int> acc(nw);
  const double eps = std::numeric_limits<T>::epsilon();
  for (int iat = 0; iat < ne; iat++)
  {
    for (int iw = 0; iw < nw; iw++)
    {
      double g[3];
      ps.gauss3((uint32_t)iw, (uint32_t)iat, sweep, g);
      for (int k = 0; k < 3; k++)
        dl[iw * 3 + k] = g[k] * sqrttau;
    }
    c.eval_grad(iat, grads_now.data());
    for (int iw = 0; iw < nw; iw++)
    {
      if (use_drift)
      {
        Crowd<T>::unr_drift(tau, &grads_now[iw * 3], &drift[iw * 3]);
        for (int k = 0; k < 3; k++)
          drift[iw * 3 + k] += dl[iw * 3 + k];
      }
      else
        for (int k = 0; k < 3; k++)
          drift[iw * 3 + k] = dl[iw * 3 + k];
    }
    c.make_move(iat, drift.data());
    c.ratio_grad(iat, ratios.data(), grads_new.data());
    for (int iw = 0; iw < nw; iw++)
    {
      log_gf[iw] = log_gb[iw] = 0.0;
      if (use_drift)
      {
        const double* d = &dl[iw * 3];
        log_gf[iw]      = -oneover2tau * (d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        double dr[3];
        Crowd<T>::unr_drift(tau, &grads_new[iw * 3], dr);
        for (int k = 0; k < 3; k++)
          dr[k] += drift[iw * 3 + k];
        log_gb[iw] = -oneover2tau * (dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2]);
      }
      const double prob = ratios[iw] * ratios[iw];
      acc[iw] = (prob >= eps && ps.uniform((uint32_t)iw, (uint32_t)iat, sweep) < prob * std::exp(log_gb[iw] - log_gf[iw]))
          ? 1
          : 0;
      if (acc[iw])
        (*n_accept)++;
      else
        (*n_reject)++;
      if (trace)
      {
        double* tr = trace + ((size_t)iat * nw + iw) * TRACE_FIELDS;
        for (int k = 0; k < 3; k++)
        {
          tr[TR_POS + k]      = c.w[iw].active_pos[k];
          tr[TR_GRAD_NEW + k] = grads_new[iw * 3 + k];
          tr[TR_GRAD_NOW + k] = grads_now[iw * 3 + k];
        }
        tr[TR_RATIO]  = ratios[iw];
        tr[TR_ACCEPT] = acc[iw];
        tr[TR_SELF]   = 1.0;
      }
    }
    c.accept_reject(iat, acc.data());
  }
  c.complete_updates();
}

// ---------------------------------------------------------------------------
// Replay of a recorded trajectory: for every move the proposed positions and the
// decisions of trace_in [ne][nw][TRACE_FIELDS] (from any implementation), this
// crowd's own gradients and ratios on those positions into trace_out (same layout).
// ---------------------------------------------------------------------------
template<typename T>
void replay(Crowd<T>& c, const double* trace_in, double* trace_out)
{
  const int nw = c.nw, ne = c.ne;
  std::vector<double> pos((size_t)nw * 3), gnow((size_t)nw * 3), gnew((size_t)nw * 3), ratios(nw);
  std::vector<int> acc(nw);
  for (int iat = 0; iat < ne; iat++)
  {
    c.eval_grad(iat, gnow.data());
    for (int iw = 0; iw < nw; iw++)
    {
      const double* tr = trace_in + ((size_t)iat * nw + iw) * TRACE_FIELDS;
      for (int k = 0; k < 3; k++)
        pos[iw * 3 + k] = tr[TR_POS + k];
      acc[iw] = tr[TR_ACCEPT] != 0.0 ? 1 : 0;
    }
    c.make_move_to(iat, pos.data());
    c.ratio_grad(iat, ratios.data(), gnew.data());
    for (int iw = 0; iw < nw; iw++)
    {
      double* o = trace_out + ((size_t)iat * nw + iw) * TRACE_FIELDS;
      for (int k = 0; k < 3; k++)
      {
        o[TR_POS + k]      = pos[iw * 3 + k];
        o[TR_GRAD_NEW + k] = gnew[iw * 3 + k];
        o[TR_GRAD_NOW + k] = gnow[iw * 3 + k];
      }
      o[TR_RATIO]  = ratios[iw];
      o[TR_ACCEPT] = acc[iw];
      o[TR_SELF]   = 1.0;
    }
    c.accept_reject(iat, acc.data());
  }
  c.complete_updates();
}

// ---------------------------------------------------------------------------
// Ratio of one virtual move: psi(R with electron e at pos) / psi(R) of walker iw, after
// every delayed update (TrialWaveFunction::mw_evaluateRatios over a VirtualParticleSet,
// TrialWaveFunction.cpp:1079-1110): the determinant Ainv[row] . phi(pos)
// (SplineR2R::evaluateDetRatios, SplineR2R.cpp:184-196), the J2 factor
// exp(Uat[e] - sum_{j != e} u(|r_j - pos|)) (TwoBodyJastrow::evaluateRatios,
// TwoBodyJastrow.cpp:166-171) and the J1 factor exp(Vat[e] - sum_I u1(|R_I - pos|))
// (J1OrbitalSoA::evaluateRatios, J1OrbitalSoA.h:295-299).
// ---------------------------------------------------------------------------
template<typename T>
double vp_ratio(const Crowd<T>& c, int iw, int e, const double pos[3])
{
  const int s   = c.group_of(e);
  const int row = e - c.first_of(s);
  std::vector<T> v(c.norb), g((size_t)3 * c.norb), l(c.norb);
  c.spo_vgl(pos, v.data(), g.data(), l.data());
  const T* inv = c.w[iw].det[s].Ainv.data() + (size_t)row * c.norb;
  T det        = 0;
  for (int o = 0; o < c.norb; o++)
    det += v[o] * inv[o];
  double logj = 0;
  const auto& wk = c.w[iw];
  if (c.has_j2)
  {
    std::vector<T> dist(c.ne), dr((size_t)3 * c.ne);
    c.ee_row(wk, pos, dist.data(), dr.data());
    T vgl[5];
    c.j2_vgl(e, dist.data(), dr.data(), vgl, nullptr, nullptr, nullptr);
    logj += static_cast<double>(wk.Uat[e] - vgl[0]);
  }
  if (c.has_j1)
  {
    std::vector<T> dist(c.nions), dr((size_t)3 * c.nions);
    c.ei_row(pos, dist.data(), dr.data());
    T U, gr[3], lap;
    c.j1_vgl(dist.data(), dr.data(), U, gr, lap);
    logj += static_cast<double>(wk.Vat[e] - U);
  }
  return static_cast<double>(det) * std::exp(logj);
}

// ---------------------------------------------------------------------------
// Step-by-step check of a recorded trajectory on the counter-based stream.  The
// state follows trace_in (its proposed positions and decisions); at every move this
// crowd also forms, independently, what the driver step would do from that state:
// the gradient at R, its own proposal r + drift(R) + sqrt(tau) xi with the stream's
// Gaussians, the ratio and gradient at the recorded R', and its own decision with
// the stream's uniform, u < |ratio|^2 exp(log_gb - log_gf) (VMCBatched.cpp:125-158).
// trace_out gets those (TR_POS = its own proposal, TR_ACCEPT = its own decision);
// margin [ne][nw] = (u - P) / P, the relative distance of the decision from a tie;
// TR_SELF of trace_out carries tau |xi|^2 of the move.  dmc: fixed-node moves.
// ---------------------------------------------------------------------------
template<typename T>
void replay_philox(Crowd<T>& c, const PhiloxStream& ps, uint32_t sweep, double tau, bool use_drift, bool dmc,
                   const double* trace_in, double* trace_out, double* margin)
{
  const int nw = c.nw, ne = c.ne;
  const double sqrttau = std::sqrt(tau), oneover2tau = 0.5 / tau;
  const double eps = std::numeric_limits<T>::epsilon();
  std::vector<double> pos((size_t)nw * 3), gnow((size_t)nw * 3), gnew((size_t)nw * 3), ratios(nw);
  std::vector<int> acc(nw);
  for (int iat = 0; iat < ne; iat++)
  {
    c.eval_grad(iat, gnow.data());
    for (int iw = 0; iw < nw; iw++)
    {
      const double* tr = trace_in + ((size_t)iat * nw + iw) * TRACE_FIELDS;
      double* o        = trace_out + ((size_t)iat * nw + iw) * TRACE_FIELDS;
      double xi[3], drift[3] = {0, 0, 0};
      ps.gauss3((uint32_t)iw, (uint32_t)iat, sweep, xi);
      // tau |xi|^2 of the move (DMCBatched.cpp:165-167): the DMC r^2 of the step
      o[TR_SELF] = tau * (xi[0] * xi[0] + xi[1] * xi[1] + xi[2] * xi[2]);
      if (use_drift)
        Crowd<T>::unr_drift(tau, &gnow[iw * 3], drift);
      for (int k = 0; k < 3; k++)
      {
        o[TR_POS + k]      = c.w[iw].R[(size_t)iat * 3 + k] + (drift[k] + xi[k] * sqrttau);
        o[TR_GRAD_NOW + k] = gnow[iw * 3 + k];
        pos[iw * 3 + k]    = tr[TR_POS + k];
      }
      acc[iw] = tr[TR_ACCEPT] != 0.0 ? 1 : 0;
    }
    c.make_move_to(iat, pos.data());
    c.ratio_grad(iat, ratios.data(), gnew.data());
    for (int iw = 0; iw < nw; iw++)
    {
      double* o = trace_out + ((size_t)iat * nw + iw) * TRACE_FIELDS;
      double log_gf = 0, log_gb = 0;
      if (use_drift)
      {
        // the recorded displacement, split into drift at R and diffusion
        double dnow[3], dnew[3], disp[3], delta[3];
        Crowd<T>::unr_drift(tau, &gnow[iw * 3], dnow);
        Crowd<T>::unr_drift(tau, &gnew[iw * 3], dnew);
        for (int k = 0; k < 3; k++)
        {
          disp[k]  = pos[iw * 3 + k] - c.w[iw].R[(size_t)iat * 3 + k];
          delta[k] = disp[k] - dnow[k];
          dnew[k] += disp[k];
        }
        log_gf = -oneover2tau * (delta[0] * delta[0] + delta[1] * delta[1] + delta[2] * delta[2]);
        log_gb = -oneover2tau * (dnew[0] * dnew[0] + dnew[1] * dnew[1] + dnew[2] * dnew[2]);
      }
      const double P = ratios[iw] * ratios[iw] * std::exp(log_gb - log_gf);
      const double u = ps.uniform((uint32_t)iw, (uint32_t)iat, sweep);
      // DMC: a move that changes the sign of psi is rejected (SFNBranch::phaseChanged
      // for a real ratio, DMCBatched.cpp:203-215)
      const bool phase_ok = !dmc || ratios[iw] > 0;
      const int own       = (phase_ok && ratios[iw] * ratios[iw] >= eps && u < P) ? 1 : 0;
      for (int k = 0; k < 3; k++)
        o[TR_GRAD_NEW + k] = gnew[iw * 3 + k];
      o[TR_RATIO]  = ratios[iw];
      o[TR_ACCEPT] = own;
      if (margin)
        margin[(size_t)iat * nw + iw] = (u - P) / std::max(P, 1e-300);
    }
    c.accept_reject(iat, acc.data());
  }
  c.complete_updates();
}

template<typename T>
Crowd<T>* make_crowd(int n_up, int n_dn, int norb, int npad, const double lattice[3], int n_ions, const double* ion_pos,
                     const int* ion_species, int n_ion_species, const int grid[3], const double* coefs, int j1_nparams,
                     double j1_rcut, const double* j1_params, const double* j1_cusp, int j2_nparams, double j2_rcut,
                     const double* j2_params, const double* j2_cusp, int nw, int delay)
{
  auto* c  = new Crowd<T>();
  c->nup   = n_up;
  c->ndn   = n_dn;
  c->ne    = n_up + n_dn;
  c->norb  = norb;
  c->npad  = npad;
  c->nions = n_ions;
  c->nion_species = n_ion_species;
  for (int d = 0; d < 3; d++)
    c->lattice[d] = lattice[d];
  c->cell.init(lattice);
  c->ions.assign(ion_pos, ion_pos + (size_t)n_ions * 3);
  c->ion_species.assign(ion_species, ion_species + n_ions);
  c->spline.init(grid, npad, coefs);
  c->has_j1 = j1_nparams > 0 && n_ions > 0;
  if (c->has_j1)
  {
    c->j1f.resize(n_ion_species);
    for (int s = 0; s < n_ion_species; s++)
      c->j1f[s].reset(j1_nparams, j1_rcut, j1_params + (size_t)s * j1_nparams, j1_cusp[s]);
  }
  c->has_j2 = j2_nparams > 0;
  if (c->has_j2)
    for (int s = 0; s < 2; s++)
      c->j2f[s].reset(j2_nparams, j2_rcut, j2_params + (size_t)s * j2_nparams, j2_cusp[s]);
  c->nw    = nw;
  c->delay = delay;
  c->init_walkers();
  c->dgrad.assign((size_t)nw * 2 * norb * 3 * norb, T(0));
  c->dlap.assign((size_t)nw * 2 * norb * norb, T(0));
  return c;
}

} // namespace orc

// ===========================================================================
// C interface (ctypes).  Handles carry the precision: 8 = FP64, 4 = FP32.
// ===========================================================================
struct OrcHandle
{
  int prec;
  orc::Crowd<double>* d = nullptr;
  orc::Crowd<float>* f  = nullptr;
};

template<typename F>
inline void dispatch(OrcHandle* h, F&& fn)
{
  if (h->prec == 8)
    fn(h->d);
  else
    fn(h->f);
}

extern "C" {

void* orc_crowd_create(int prec, int n_up, int n_dn, int norb, int npad, const double* lattice, int n_ions,
                       const double* ion_pos, const int* ion_species, int n_ion_species, const int* grid,
                       const double* coefs, int j1_nparams, double j1_rcut, const double* j1_params,
                       const double* j1_cusp, int j2_nparams, double j2_rcut, const double* j2_params,
                       const double* j2_cusp, int nw, int delay)
{
  auto* h = new OrcHandle();
  h->prec = prec;
  if (prec == 8)
    h->d = orc::make_crowd<double>(n_up, n_dn, norb, npad, lattice, n_ions, ion_pos, ion_species, n_ion_species, grid,
                                   coefs, j1_nparams, j1_rcut, j1_params, j1_cusp, j2_nparams, j2_rcut, j2_params,
                                   j2_cusp, nw, delay);
  else
    h->f = orc::make_crowd<float>(n_up, n_dn, norb, npad, lattice, n_ions, ion_pos, ion_species, n_ion_species, grid,
                                  coefs, j1_nparams, j1_rcut, j1_params, j1_cusp, j2_nparams, j2_rcut, j2_params,
                                  j2_cusp, nw, delay);
  return h;
}

void orc_crowd_destroy(void* hv)
{
  auto* h = static_cast<OrcHandle*>(hv);
  delete h->d;
  delete h->f;
  delete h;
}

void orc_load_walkers(void* hv, const double* R)
{
  auto* h = static_cast<OrcHandle*>(hv);
  dispatch(h, [&](auto* c) {
    for (int iw = 0; iw < c->nw; iw++)
      std::copy_n(R + (size_t)iw * c->ne * 3, (size_t)c->ne * 3, c->w[iw].R.data());
  });
}

void orc_get_positions(void* hv, double* R)
{
  auto* h = static_cast<OrcHandle*>(hv);
  dispatch(h, [&](auto* c) {
    for (int iw = 0; iw < c->nw; iw++)
      std::copy_n(c->w[iw].R.data(), (size_t)c->ne * 3, R + (size_t)iw * c->ne * 3);
  });
}

// log|psi| per walker after a full recompute; sign product in signs (may be null)
int orc_evaluate_log(void* hv, double* logpsi, int* signs, int nthreads)
{
  auto* h = static_cast<OrcHandle*>(hv);
  int err = 0;
  dispatch(h, [&](auto* c) {
#pragma omp parallel for num_threads(nthreads > 0 ? nthreads : 1) schedule(dynamic)
    for (int iw = 0; iw < c->nw; iw++)
    {
      try
      {
        c->recompute(iw);
      }
      catch (...)
      {
        err = -1;
      }
    }
    c->delay_count[0] = c->delay_count[1] = 0;
    for (int iw = 0; iw < c->nw; iw++)
    {
      const auto& wk = c->w[iw];
      if (logpsi)
        logpsi[iw] = wk.det[0].log_abs + wk.det[1].log_abs + c->log_j1(iw) + c->log_j2(iw);
      if (signs)
        signs[iw] = wk.det[0].sign * wk.det[1].sign;
    }
  });
  return err;
}

// current log|psi| from the tracked state (det logs accumulated from ratios)
void orc_get_log(void* hv, double* logpsi, int* signs, double* parts /*[nw][4] det_up, det_dn, j1, j2*/)
{
  auto* h = static_cast<OrcHandle*>(hv);
  dispatch(h, [&](auto* c) {
    for (int iw = 0; iw < c->nw; iw++)
    {
      const auto& wk = c->w[iw];
      const double lj1 = c->log_j1(iw), lj2 = c->log_j2(iw);
      if (logpsi)
        logpsi[iw] = wk.det[0].log_abs + wk.det[1].log_abs + lj1 + lj2;
      if (signs)
        signs[iw] = wk.det[0].sign * wk.det[1].sign;
      if (parts)
      {
        parts[iw * 4 + 0] = wk.det[0].log_abs;
        parts[iw * 4 + 1] = wk.det[1].log_abs;
        parts[iw * 4 + 2] = lj1;
        parts[iw * 4 + 3] = lj2;
      }
    }
  });
}

void orc_eval_grad(void* hv, int iat, double* grads)
{
  auto* h = static_cast<OrcHandle*>(hv);
  dispatch(h, [&](auto* c) { c->eval_grad(iat, grads); });
}

void orc_make_move(void* hv, int iat, const double* displ)
{
  auto* h = static_cast<OrcHandle*>(hv);
  dispatch(h, [&](auto* c) { c->make_move(iat, displ); });
}

void orc_ratio_grad(void* hv, int iat, double* ratios, double* grads)
{
  auto* h = static_cast<OrcHandle*>(hv);
  dispatch(h, [&](auto* c) { c->ratio_grad(iat, ratios, grads); });
}

void orc_accept_reject(void* hv, int iat, const int* accepted)
{
  auto* h = static_cast<OrcHandle*>(hv);
  dispatch(h, [&](auto* c) { c->accept_reject(iat, accepted); });
}

void orc_complete_updates(void* hv)
{
  auto* h = static_cast<OrcHandle*>(hv);
  dispatch(h, [&](auto* c) { c->complete_updates(); });
}

// Ainv of spin s for all walkers, [nw][n][n], as double
void orc_get_ainv(void* hv, int s, double* out)
{
  auto* h = static_cast<OrcHandle*>(hv);
  dispatch(h, [&](auto* c) {
    const size_t nn = (size_t)c->norb * c->norb;
    for (int iw = 0; iw < c->nw; iw++)
      for (size_t i = 0; i < nn; i++)
        out[iw * nn + i] = static_cast<double>(c->w[iw].det[s].Ainv[i]);
  });
}

// J2 state [nw][5][ne] (Uat, dUat xyz, d2Uat) and J1 state [nw][5][ne] (Vat, Grad xyz, Lap)
void orc_get_jastrow_state(void* hv, double* j2, double* j1)
{
  auto* h = static_cast<OrcHandle*>(hv);
  dispatch(h, [&](auto* c) {
    const int ne = c->ne;
    for (int iw = 0; iw < c->nw; iw++)
    {
      const auto& wk = c->w[iw];
      for (int i = 0; i < ne; i++)
      {
        if (j2)
        {
          j2[((size_t)iw * 5 + 0) * ne + i] = wk.Uat[i];
          for (int d = 0; d < 3; d++)
            j2[((size_t)iw * 5 + 1 + d) * ne + i] = wk.dUat[(size_t)d * ne + i];
          j2[((size_t)iw * 5 + 4) * ne + i] = wk.d2Uat[i];
        }
        if (j1)
        {
          j1[((size_t)iw * 5 + 0) * ne + i] = wk.Vat[i];
          for (int d = 0; d < 3; d++)
            j1[((size_t)iw * 5 + 1 + d) * ne + i] = wk.Grad[(size_t)d * ne + i];
          j1[((size_t)iw * 5 + 4) * ne + i] = wk.Lap[i];
        }
      }
    }
  });
}

// orbital VGL of the proposed move of spin s, [nw][5][norb]
void orc_get_phi_vgl(void* hv, int s, double* out)
{
  auto* h = static_cast<OrcHandle*>(hv);
  dispatch(h, [&](auto* c) {
    const int n = c->norb;
    for (int iw = 0; iw < c->nw; iw++)
    {
      const auto& d = c->w[iw].det[s];
      for (int o = 0; o < n; o++)
      {
        out[((size_t)iw * 5 + 0) * n + o] = d.phi_v[o];
        for (int k = 0; k < 3; k++)
          out[((size_t)iw * 5 + 1 + k) * n + o] = d.phi_g[(size_t)k * n + o];
        out[((size_t)iw * 5 + 4) * n + o] = d.phi_l[o];
      }
    }
  });
}

// ---- threads used by the per-walker loops (OpenMP over walkers, like crowds) ---
// kinetic energy per walker from the tracked state (after complete_updates);
// gl (optional): [nw][ne][4] gradient and Laplacian of log psi per electron
void orc_kinetic(void* hv, double* ke, double* gl)
{
  auto* h = static_cast<OrcHandle*>(hv);
  dispatch(h, [&](auto* c) {
#pragma omp parallel for schedule(static)
    for (int iw = 0; iw < c->nw; iw++)
      ke[iw] = c->kinetic(iw, gl ? gl + (size_t)iw * c->ne * 4 : nullptr);
  });
}

void orc_set_threads(int n)
{
#ifdef _OPENMP
  omp_set_num_threads(n > 0 ? n : 1);
#else
  (void)n;
#endif
}

// ---- RNG stream -----------------------------------------------------------
void* orc_rng_create(unsigned seed) { return new orc::Rng(seed); }
void orc_rng_destroy(void* r) { delete static_cast<orc::Rng*>(r); }
void orc_rng_uniform(void* r, double* out, long n)
{
  for (long i = 0; i < n; i++)
    out[i] = static_cast<orc::Rng*>(r)->uniform();
}
void orc_rng_gauss(void* r, double* out, long n) { static_cast<orc::Rng*>(r)->gauss(out, (size_t)n); }

// ---- whole sweeps (VMCBatched::advanceWalkers, sub_steps = 1 per step) -----
void orc_vmc_sweeps(void* hv, void* rng, int nsteps, double tau, int use_drift, long* n_accept, long* n_reject,
                    int* accept_log /*[nsteps][ne][nw] or null*/)
{
  auto* h = static_cast<OrcHandle*>(hv);
  auto* r = static_cast<orc::Rng*>(rng);
  dispatch(h, [&](auto* c) {
    for (int s = 0; s < nsteps; s++)
      c->sweep(*r, tau, use_drift != 0, n_accept, n_reject,
               accept_log ? accept_log + (size_t)s * c->ne * c->nw : nullptr);
  });
}

// ---- sweeps on the counter-based stream of the device (Philox4x32-10) --------
// sweeps sweep0, sweep0 + 1, ...; trace [nsteps][ne][nw][TRACE_FIELDS] or null
void orc_vmc_sweeps_philox(void* hv, uint64_t seed, unsigned sweep0, int nsteps, double tau, int use_drift,
                           long* n_accept, long* n_reject, double* trace)
{
  auto* h = static_cast<OrcHandle*>(hv);
  const orc::PhiloxStream ps(seed);
  dispatch(h, [&](auto* c) {
    for (int s = 0; s < nsteps; s++)
      orc::sweep_philox(*c, ps, sweep0 + (unsigned)s, tau, use_drift != 0, n_accept, n_reject,
                        trace ? trace + (size_t)s * c->ne * c->nw * orc::TRACE_FIELDS : nullptr);
  });
}

// replay of nsteps recorded sweeps: trace_in, trace_out [nsteps][ne][nw][TRACE_FIELDS]
void orc_replay_trace(void* hv, int nsteps, const double* trace_in, double* trace_out)
{
  auto* h = static_cast<OrcHandle*>(hv);
  dispatch(h, [&](auto* c) {
    const size_t per = (size_t)c->ne * c->nw * orc::TRACE_FIELDS;
    for (int s = 0; s < nsteps; s++)
      orc::replay(*c, trace_in + s * per, trace_out + s * per);
  });
}

// step-by-step check of nsteps recorded sweeps (sweep indices sweep0, sweep0 + 1, ...):
// trace_in, trace_out [nsteps][ne][nw][TRACE_FIELDS], margin [nsteps][ne][nw] or null
void orc_replay_trace_philox(void* hv, uint64_t seed, unsigned sweep0, int nsteps, double tau, int use_drift, int dmc,
                             const double* trace_in, double* trace_out, double* margin)
{
  auto* h = static_cast<OrcHandle*>(hv);
  const orc::PhiloxStream ps(seed);
  dispatch(h, [&](auto* c) {
    const size_t nrec = (size_t)c->ne * c->nw, per = nrec * orc::TRACE_FIELDS;
    for (int s = 0; s < nsteps; s++)
      orc::replay_philox(*c, ps, sweep0 + (unsigned)s, tau, use_drift != 0, dmc != 0, trace_in + s * per,
                         trace_out + s * per, margin ? margin + s * nrec : nullptr);
  });
}

// ratios of virtual moves (call after complete_updates): ratios[v] for walker[v],
// electron elec[v] at pos[v] (pos [nvp][3])
void orc_evaluate_ratios(void* hv, int nvp, const int* walker, const int* elec, const double* pos, double* ratios)
{
  auto* h = static_cast<OrcHandle*>(hv);
  dispatch(h, [&](auto* c) {
#pragma omp parallel for schedule(dynamic, 16)
    for (int v = 0; v < nvp; v++)
      ratios[v] = orc::vp_ratio(*c, walker[v], elec[v], pos + 3 * (size_t)v);
  });
}

// population control: walker i takes the state of walker src[i] (Walker::makeCopy);
// call after complete_updates
void orc_copy_walkers(void* hv, const int* src)
{
  auto* h = static_cast<OrcHandle*>(hv);
  dispatch(h, [&](auto* c) {
    auto old = c->w;
    auto dg  = c->dgrad;
    auto dl  = c->dlap;
    const size_t gpw = (size_t)2 * c->norb * 3 * c->norb, lpw = (size_t)2 * c->norb * c->norb;
    for (int i = 0; i < c->nw; i++)
    {
      c->w[i] = old[src[i]];
      std::copy_n(dg.begin() + src[i] * gpw, gpw, c->dgrad.begin() + i * gpw);
      std::copy_n(dl.begin() + src[i] * lpw, lpw, c->dlap.begin() + i * lpw);
    }
  });
}

// ---- unit functions used by the golden-vector tests ------------------------
void orc_prefactors(double t, double* a, double* da, double* d2a) { orc::prefactors<double>(a, da, d2a, t); }

// Multi-spline VGH at unit coordinate u on a periodic grid; outputs [norb], [3][norb], [6][norb]
void orc_spline_vgh(const int* grid, int npad, const double* coefs, int norb, const double* u, double* v, double* g,
                    double* hs)
{
  orc::Spline<double> s;
  s.init(grid, npad, coefs);
  s.vgh(u[0], u[1], u[2], norb, v, g, hs);
}

// u, du/dr, d2u/dr2 of a cusp-corrected radial B-spline functor at r (0 beyond rcut)
void orc_functor_eval(int nparams, double rcut, const double* params, double cusp, int nr, const double* r, double* u,
                      double* du, double* d2u)
{
  orc::Functor<double> f;
  f.reset(nparams, rcut, params, cusp);
  for (int i = 0; i < nr; i++)
  {
    u[i] = du[i] = d2u[i] = 0;
    if (r[i] < f.rcut)
      u[i] = f.eval(r[i], du[i], d2u[i]);
  }
}

// FP64 inverse + log|det| + sign of an n x n row-major matrix (in place)
int orc_invert(double* a, int n, double* log_abs, int* sign)
{
  try
  {
    orc::invert_lu(a, n, *log_abs, *sign);
  }
  catch (...)
  {
    return -1;
  }
  return 0;
}

// minimum-image displacement rows dr_j = R_j - r
void orc_distance_row(const double* lattice, int n, const double* R /*[n][3]*/, const double* r, double* dist,
                      double* dr /*[3][n]*/)
{
  orc::Cell<double> cell;
  cell.init(lattice);
  for (int j = 0; j < n; j++)
  {
    double dx, dy, dz;
    cell.disp(R[j * 3], R[j * 3 + 1], R[j * 3 + 2], r[0], r[1], r[2], dx, dy, dz);
    dr[0 * n + j] = dx;
    dr[1 * n + j] = dy;
    dr[2 * n + j] = dz;
    dist[j]       = std::sqrt(dx * dx + dy * dy + dz * dz);
  }
}

} // extern "C"

// ---- one determinant with its update engine (for the FakeSPO golden tests) --
struct OrcDet
{
  int n, k, dc = 0;
  std::vector<double> Ainv;
  orc::DelayEngine<double> eng;
  int row_prepared = -1;
};

extern "C" {
void* orc_det_create(int n, int k)
{
  auto* d = new OrcDet();
  d->n    = n;
  d->k    = k;
  d->Ainv.assign((size_t)n * n, 0.0);
  d->eng.resize(n, k);
  return d;
}
void orc_det_destroy(void* p) { delete static_cast<OrcDet*>(p); }
// psiM[e][o]; Ainv = inverse of the transpose (DiracMatrix::invert_transpose)
int orc_det_recompute(void* p, const double* psiM, double* log_abs, int* sign)
{
  auto* d = static_cast<OrcDet*>(p);
  const int n = d->n;
  for (int e = 0; e < n; e++)
    for (int o = 0; o < n; o++)
      d->Ainv[(size_t)o * n + e] = psiM[(size_t)e * n + o];
  d->dc = 0;
  try
  {
    orc::invert_lu(d->Ainv.data(), n, *log_abs, *sign);
  }
  catch (...)
  {
    return -1;
  }
  return 0;
}
double orc_det_ratio(void* p, int row, const double* phi)
{
  auto* d = static_cast<OrcDet*>(p);
  const double* inv;
  if (d->k > 1)
  {
    d->eng.prepare_inv_row(d->Ainv.data(), row, d->dc);
    inv = d->eng.invRow.data();
  }
  else
    inv = d->Ainv.data() + (size_t)row * d->n;
  double r = 0;
  for (int o = 0; o < d->n; o++)
    r += inv[o] * phi[o];
  return r;
}
void orc_det_accept_reject(void* p, int row, const double* phi, double ratio, int accepted)
{
  auto* d = static_cast<OrcDet*>(p);
  if (d->k > 1)
  {
    d->eng.accept_reject(d->Ainv.data(), row, d->dc, accepted != 0, phi, ratio);
    d->dc++;
    if (d->dc == d->k)
    {
      d->eng.update_inv(d->Ainv.data(), d->dc);
      d->dc = 0;
    }
  }
  else if (accepted)
    orc::sm1(d->Ainv.data(), d->n, row, phi, ratio);
}
void orc_det_complete(void* p)
{
  auto* d = static_cast<OrcDet*>(p);
  if (d->k > 1 && d->dc > 0)
  {
    d->eng.update_inv(d->Ainv.data(), d->dc);
    d->dc = 0;
  }
}
void orc_det_get_ainv(void* p, double* out)
{
  auto* d = static_cast<OrcDet*>(p);
  std::copy(d->Ainv.begin(), d->Ainv.end(), out);
}
}
