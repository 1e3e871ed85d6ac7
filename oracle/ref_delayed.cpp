// C entry point around the reference's CPU delayed-update engine
// (qmcplusplus::DelayedUpdate, src/QMCWaveFunctions/Fermion/DelayedUpdate.h:26-215)
// compiled in place from the reference sources by oracle/build_ref.sh, with the BLAS
// calls it makes forwarded to the OpenBLAS build that ships with scipy.  Test
// infrastructure only: it cross-checks the oracle's delayed-update restatement.
#include <cstring>
#include <vector>

#include "CPU/SIMD/aligned_allocator.hpp"
#include "QMCWaveFunctions/Fermion/DelayedUpdate.h"

// single-threaded stand-ins for the reference's BLAS threading guard (its real
// definition lives in a compiled source this recipe does not build)
namespace qmcplusplus
{
BlasThreadingEnv::BlasThreadingEnv(int) : old_state_(0) {}
BlasThreadingEnv::~BlasThreadingEnv() {}
bool BlasThreadingEnv::NestedThreadingSupported() { return false; }
} // namespace qmcplusplus

extern "C" {
// Fortran BLAS entry points the reference headers call, forwarded to scipy's OpenBLAS
void scipy_dgemm_(const char*, const char*, const int*, const int*, const int*, const double*, const double*,
                  const int*, const double*, const int*, const double*, double*, const int*);
void scipy_dgemv_(const char*, const int*, const int*, const double*, const double*, const int*, const double*,
                  const int*, const double*, double*, const int*);
void scipy_dger_(const int*, const int*, const double*, const double*, const int*, const double*, const int*,
                 double*, const int*);
// the same entry points under the undecorated names and reference-argument signatures
// the headers declare on this platform
void dgemm(const char& ta, const char& tb, const int& m, const int& n, const int& k, const double& al,
           const double* a, const int& lda, const double* b, const int& ldb, const double& be, double* c,
           const int& ldc)
{
  scipy_dgemm_(&ta, &tb, &m, &n, &k, &al, a, &lda, b, &ldb, &be, c, &ldc);
}
void dgemv(const char& t, const int& m, const int& n, const double& al, const double* a, const int& lda,
           const double* x, const int& incx, const double& be, double* y, const int& incy)
{
  scipy_dgemv_(&t, &m, &n, &al, a, &lda, x, &incx, &be, y, &incy);
}
void dger(const int* m, const int* n, const double* al, const double* x, const int* incx, const double* y,
          const int* incy, double* a, const int* lda)
{
  scipy_dger_(m, n, al, x, incx, y, incy, a, lda);
}

// Runs nmoves row changes through the reference engine starting from ainv0 (n x n,
// Ainv = (M^-1)^T, row e = electron e): per move getInvRow, ratio = invRow . phi,
// acceptRow for accepted moves (the engine flushes when its window of k fills),
// and a final updateInvMat.  ratios[m] and the final inverse are returned.
int ref_delayed_run(int n, int k, const double* ainv0, int nmoves, const int* rows, const double* phis,
                    const int* accept, double* ratios, double* ainv_out)
{
  using namespace qmcplusplus;
  Matrix<double> Ainv(n, n);
  std::memcpy(Ainv.data(), ainv0, sizeof(double) * n * n);
  DelayedUpdate<double> eng;
  eng.resize(n, k);
  Vector<double> invRow(n);
  for (int m = 0; m < nmoves; m++)
  {
    const double* phi = phis + (size_t)m * n;
    eng.getInvRow(Ainv, rows[m], invRow);
    double r = 0;
    for (int j = 0; j < n; j++)
      r += invRow[j] * phi[j];
    ratios[m] = r;
    if (accept[m])
    {
      Vector<double> pv(const_cast<double*>(phi), n);
      eng.acceptRow(Ainv, rows[m], pv, r);
    }
  }
  eng.updateInvMat(Ainv);
  std::memcpy(ainv_out, Ainv.data(), sizeof(double) * n * n);
  return 0;
}
}
