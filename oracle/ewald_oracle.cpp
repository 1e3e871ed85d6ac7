// CPU oracle for the Coulomb part of the local energy (test infrastructure only:
// tests/, the smoke check and the bench's CPU legs use it; the product path never does).
//
// 1. ewald_ref_energy: a restatement of the reference's standalone Ewald sum
//    (src/QMCHamiltonians/EwaldRef.cpp:140-398, Drummond et al., Phys. Rev. B 78,
//    125106 (2008), formulas 5-7): total energy of point charges in a periodic cell,
//      E = sum_{i<j} q_i q_j v_E(r_ij) + 1/2 v_M sum_i q_i^2,
//    where the pair potential v_E and the Madelung constant v_M are lattice sums
//    over cubic shells of real- and reciprocal-lattice vectors, each summed until a
//    shell contributes less than a tolerance (EwaldRef.cpp:140-214).  The splitting
//    constants are those of EwaldRef.cpp:217-228, 275-289.  Pinned to the golden
//    values of src/QMCHamiltonians/tests/test_EwaldRef.cpp.
//
// 2. ewald_split_energy: the same total energy evaluated the way the GPU kernel
//    does it for an orthorhombic cell: minimum-image real-space erfc sum, a
//    half-space reciprocal sum over |G| <= G_c through the structure factor, and
//    constants; alpha and G_c follow from a tolerance eps (alpha * L_min/2 and
//    G_c / (2 alpha) both equal sqrt(-ln eps)).
#include <algorithm>
#include <cmath>
#include <complex>
#include <limits>
#include <vector>

namespace orc_ewald
{

struct M3
{
  double m[3][3]; // rows are the cell vectors a_0, a_1, a_2
};

static double det3(const M3& a)
{
  const auto& m = a.m;
  return m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) - m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
      m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
}

static M3 inv3(const M3& a)
{
  const auto& m = a.m;
  const double d = det3(a);
  M3 r;
  r.m[0][0] = (m[1][1] * m[2][2] - m[1][2] * m[2][1]) / d;
  r.m[0][1] = (m[0][2] * m[2][1] - m[0][1] * m[2][2]) / d;
  r.m[0][2] = (m[0][1] * m[1][2] - m[0][2] * m[1][1]) / d;
  r.m[1][0] = (m[1][2] * m[2][0] - m[1][0] * m[2][2]) / d;
  r.m[1][1] = (m[0][0] * m[2][2] - m[0][2] * m[2][0]) / d;
  r.m[1][2] = (m[0][2] * m[1][0] - m[0][0] * m[1][2]) / d;
  r.m[2][0] = (m[1][0] * m[2][1] - m[1][1] * m[2][0]) / d;
  r.m[2][1] = (m[0][1] * m[2][0] - m[0][0] * m[2][1]) / d;
  r.m[2][2] = (m[0][0] * m[1][1] - m[0][1] * m[1][0]) / d;
  return r;
}

// reciprocal vectors as rows: b = 2 pi (a^-1)^T
static M3 recip(const M3& a)
{
  const M3 ai = inv3(a);
  M3 b;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      b.m[i][j] = 2 * M_PI * ai.m[j][i];
  return b;
}

static void comb(const M3& a, int i, int j, int k, double v[3])
{
  for (int d = 0; d < 3; d++)
    v[d] = i * a.m[0][d] + j * a.m[1][d] + k * a.m[2][d];
}

// Sum f over integer triples in growing cubic shells: each round adds the two new
// planes normal to x, then to y, then to z, and stops once a round's summed
// magnitude is at most tol (EwaldRef.cpp:140-214).
template<typename F>
static double shell_sum(const F& f, bool with_origin, double tol)
{
  double v = with_origin ? f(0, 0, 0) : 0.0;
  int nx = 0, ny = 0, nz = 0;
  double mag = std::numeric_limits<double>::max();
  while (std::fabs(mag) > tol)
  {
    mag       = 0;
    double dv = 0;
    auto add  = [&](int i, int j, int k) {
      const double t = f(i, j, k);
      dv += t;
      mag += std::fabs(t);
    };
    nx++;
    for (int i : {-nx, nx})
      for (int j = -ny; j <= ny; j++)
        for (int k = -nz; k <= nz; k++)
          add(i, j, k);
    ny++;
    for (int j : {-ny, ny})
      for (int k = -nz; k <= nz; k++)
        for (int i = -nx; i <= nx; i++)
          add(i, j, k);
    nz++;
    for (int k : {-nz, nz})
      for (int i = -nx; i <= nx; i++)
        for (int j = -ny; j <= ny; j++)
          add(i, j, k);
    v += dv;
  }
  return v;
}

static double ws_radius(double vol) { return std::cbrt(3 * vol / (4 * M_PI)); }

// Madelung constant v_M (Drummond 2008 formula 7; EwaldRef.cpp:217-272)
static double madelung(const M3& a, double tol)
{
  const double vol = std::fabs(det3(a));
  const M3 b       = recip(a);
  const double kap = std::sqrt(M_PI) / ws_radius(vol);
  const double c0  = -M_PI / (kap * kap * vol) - 2 * kap / std::sqrt(M_PI);
  auto fr          = [&](int i, int j, int k) {
    double R[3];
    comb(a, i, j, k, R);
    const double r = std::sqrt(R[0] * R[0] + R[1] * R[1] + R[2] * R[2]);
    return std::erfc(kap * r) / r;
  };
  auto fk = [&](int i, int j, int k) {
    double K[3];
    comb(b, i, j, k, K);
    const double k2 = K[0] * K[0] + K[1] * K[1] + K[2] * K[2];
    return 4 * M_PI / vol * std::exp(-k2 / (4 * kap * kap)) / k2;
  };
  return c0 + shell_sum(fr, false, tol) + shell_sum(fk, false, tol);
}

// Ewald pair potential v_E(r) (Drummond 2008 formula 6; EwaldRef.cpp:275-334)
static double pair(const double r[3], const M3& a, double tol)
{
  const double vol = std::fabs(det3(a));
  const M3 b       = recip(a);
  const double kap = ws_radius(vol) / std::sqrt(2 * M_PI);
  const double rc  = 1 / (std::sqrt(2.0) * kap);
  auto fr          = [&](int i, int j, int k) {
    double R[3];
    comb(a, i, j, k, R);
    const double dx = R[0] - r[0], dy = R[1] - r[1], dz = R[2] - r[2];
    const double d  = std::sqrt(dx * dx + dy * dy + dz * dz);
    return std::erfc(rc * d) / d;
  };
  auto fk = [&](int i, int j, int k) {
    double K[3];
    comb(b, i, j, k, K);
    const double k2 = K[0] * K[0] + K[1] * K[1] + K[2] * K[2];
    return 4 * M_PI / vol * std::exp(-kap * kap * k2 / 2) * std::cos(K[0] * r[0] + K[1] * r[1] + K[2] * r[2]) / k2;
  };
  return -2 * M_PI * kap * kap / vol + shell_sum(fr, true, tol) + shell_sum(fk, false, tol);
}

double ref_energy(const M3& a, int n, const double* R, const double* Q, double tol)
{
  double qq_max = 0;
  for (int i = 0; i < n; i++)
    qq_max = std::max(qq_max, Q[i] * Q[i]);
  const double vm = madelung(a, tol * 2 / qq_max);
  double e        = 0;
  for (int i = 0; i < n; i++)
    e += Q[i] * Q[i] * vm / 2;
  const M3 ai = inv3(a);
  for (int i = 1; i < n; i++)
    for (int j = 0; j < i; j++)
    {
      // wrap the separation into the cell (fractional coordinates in [0, 1))
      double d[3] = {R[3 * i] - R[3 * j], R[3 * i + 1] - R[3 * j + 1], R[3 * i + 2] - R[3 * j + 2]};
      double f[3];
      for (int c = 0; c < 3; c++)
      {
        f[c] = d[0] * ai.m[0][c] + d[1] * ai.m[1][c] + d[2] * ai.m[2][c];
        f[c] -= std::floor(f[c]);
      }
      double r[3];
      for (int c = 0; c < 3; c++)
        r[c] = f[0] * a.m[0][c] + f[1] * a.m[1][c] + f[2] * a.m[2][c];
      const double qq = Q[i] * Q[j];
      if (qq != 0)
        e += qq * pair(r, a, tol / std::fabs(qq));
    }
  return e;
}

// ---------------------------------------------------------------------------
// split evaluation for an orthorhombic cell (the GPU method, in FP64)
// ---------------------------------------------------------------------------
void split_energy(const double L[3], int n, const double* R, const double* Q, double eps, double parts[4])
{
  const double vol  = L[0] * L[1] * L[2];
  const double s    = std::sqrt(-std::log(eps));
  const double rcut = 0.5 * std::min(L[0], std::min(L[1], L[2]));
  const double al   = s / rcut;
  const double gc   = 2 * al * s;
  double q2 = 0, qt = 0;
  for (int i = 0; i < n; i++)
  {
    q2 += Q[i] * Q[i];
    qt += Q[i];
  }
  // real space, minimum image
  double er = 0;
  for (int i = 1; i < n; i++)
    for (int j = 0; j < i; j++)
    {
      double r2 = 0;
      for (int c = 0; c < 3; c++)
      {
        double d = R[3 * i + c] - R[3 * j + c];
        d -= L[c] * std::round(d / L[c]);
        r2 += d * d;
      }
      const double r = std::sqrt(r2);
      er += Q[i] * Q[j] * std::erfc(al * r) / r;
    }
  // reciprocal space over the half space n1 > 0 | (n1 == 0, n2 > 0) | (n1 == n2 == 0, n3 > 0)
  int nm[3];
  for (int c = 0; c < 3; c++)
    nm[c] = (int)std::floor(gc * L[c] / (2 * M_PI));
  double ek = 0;
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
        std::complex<double> rho(0, 0);
        for (int i = 0; i < n; i++)
        {
          const double ph = g[0] * R[3 * i] + g[1] * R[3 * i + 1] + g[2] * R[3 * i + 2];
          rho += Q[i] * std::complex<double>(std::cos(ph), std::sin(ph));
        }
        ek += 4 * M_PI / vol * std::exp(-g2 / (4 * al * al)) / g2 * (std::norm(rho) - q2);
      }
  const M3 a = {{{L[0], 0, 0}, {0, L[1], 0}, {0, 0, L[2]}}};
  const double vm = madelung(a, 1e-14);
  const double ec = -M_PI / (2 * al * al * vol) * (qt * qt - q2) + 0.5 * vm * q2;
  parts[0]        = er;
  parts[1]        = ek;
  parts[2]        = ec;
  parts[3]        = er + ek + ec;
}

} // namespace orc_ewald

extern "C" {

// a9: cell vectors as rows; R: [n][3]; Q: [n]
double orc_ewald_ref_energy(const double* a9, int n, const double* R, const double* Q, double tol)
{
  orc_ewald::M3 a;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      a.m[i][j] = a9[3 * i + j];
  return orc_ewald::ref_energy(a, n, R, Q, tol);
}

double orc_madelung(const double* a9, double tol)
{
  orc_ewald::M3 a;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      a.m[i][j] = a9[3 * i + j];
  return orc_ewald::madelung(a, tol);
}

// parts: real-space, reciprocal, constant, total
void orc_ewald_split_energy(const double* L, int n, const double* R, const double* Q, double eps, double* parts)
{
  orc_ewald::split_energy(L, n, R, Q, eps, parts);
}

} // extern "C"
