// A C++ caller of libqmcg.so through include/qmcg.h: the adapter that forwards
// QMCPACK's batched (mw_) calls of one crowd to a qmcg_crowd handle, exercised on a
// small system, electron by electron, then one device-resident sweep.
//
// usage: adapter_crowd <input.bin> <output.bin>
// input  (little-endian): int32 header [precision, n_up, n_dn, norb, npad, nions, gx, gy, gz,
//        j1_np, j2_np, nw, k, sweeps_by_electron], float64 lattice[3], j1_rcut, j2_rcut, tau,
//        ion_pos[nions*3], j1_params[j1_np], j1_cusp[1], j2_params[2*j2_np], j2_cusp[2],
//        coefs[(gx+3)(gy+3)(gz+3)npad] (float64; converted to float for precision 4),
//        R[nw*ne*3], displacements[sweeps*ne*nw*3], accept[sweeps*ne*nw] (int32)
// output: float64 log_psi_after_recompute[nw], per move: grads_now[nw*3], ratios[nw],
//         grads_new[nw*3]; then log_psi[nw], G[nw*ne*3], L[nw*ne], positions[nw*ne*3]
//         after the electron-by-electron sweeps; accepted/rejected of one resident sweep.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include "qmcg.h"

namespace
{
void check(int rc)
{
  if (rc != QMCG_OK)
    throw std::runtime_error(std::string("qmcg: ") + qmcg_last_error());
}

// The adapter a QMCPACK maintainer adds (one per crowd), with the reference's method names.
struct QMCGCrowdAdapter
{
  qmcg_system sys  = nullptr;
  qmcg_crowd crowd = nullptr;
  int nw = 0, ne = 0;

  void create(const qmcg_system_desc& desc, int walkers, int delay_rank)
  {
    check(qmcg_system_create(&desc, &sys));
    check(qmcg_crowd_create(sys, walkers, delay_rank, &crowd));
    nw = walkers;
    ne = desc.n_up + desc.n_dn;
  }
  ~QMCGCrowdAdapter()
  {
    if (crowd)
      qmcg_crowd_destroy(crowd);
    if (sys)
      qmcg_system_destroy(sys);
  }
  // TrialWaveFunction::mw_evaluateLog
  void mw_evaluateLog(const std::vector<double>& R_aos, std::vector<double>& log_psi)
  {
    check(qmcg_load_walkers(crowd, R_aos.data()));
    check(qmcg_mw_evaluate_log(crowd, log_psi.data(), nullptr));
  }
  // TrialWaveFunction::mw_evalGrad
  void mw_evalGrad(int iat, std::vector<double>& grads) { check(qmcg_mw_eval_grad(crowd, iat, grads.data())); }
  // ParticleSet::mw_makeMove
  void mw_makeMove(int iat, const std::vector<double>& displ, std::vector<bool>& valid)
  {
    std::vector<int> v(nw);
    check(qmcg_mw_make_move(crowd, iat, displ.data(), v.data()));
    for (int i = 0; i < nw; i++)
      valid[i] = v[i] != 0;
  }
  // TrialWaveFunction::mw_calcRatioGrad
  void mw_calcRatioGrad(int iat, std::vector<double>& ratios, std::vector<double>& grads)
  {
    check(qmcg_mw_calc_ratio_grad(crowd, iat, ratios.data(), grads.data()));
  }
  // TrialWaveFunction::mw_accept_rejectMove + ParticleSet::mw_accept_rejectMove
  void mw_accept_rejectMove(int iat, const std::vector<bool>& acc)
  {
    std::vector<int> a(acc.begin(), acc.end());
    check(qmcg_mw_accept_reject_move(crowd, iat, a.data()));
  }
  // TrialWaveFunction::mw_completeUpdates
  void mw_completeUpdates() { check(qmcg_mw_complete_updates(crowd)); }
  // TrialWaveFunction::mw_evaluateGL (fromscratch = false)
  void mw_evaluateGL(std::vector<double>& log_psi, std::vector<double>& G, std::vector<double>& L)
  {
    check(qmcg_mw_evaluate_gl(crowd, log_psi.data(), G.data(), L.data()));
  }
};

template<typename X>
void rd(FILE* f, X* p, size_t n)
{
  if (std::fread(p, sizeof(X), n, f) != n)
    throw std::runtime_error("short input");
}
template<typename X>
void wr(FILE* f, const X* p, size_t n)
{
  if (std::fwrite(p, sizeof(X), n, f) != n)
    throw std::runtime_error("short write");
}
} // namespace

int main(int argc, char** argv)
{
  if (argc != 3)
  {
    std::fprintf(stderr, "usage: %s input.bin output.bin\n", argv[0]);
    return 2;
  }
  try
  {
    FILE* in = std::fopen(argv[1], "rb");
    if (!in)
      throw std::runtime_error("cannot open input");
    int32_t h[14];
    rd(in, h, 14);
    const int prec = h[0], nup = h[1], ndn = h[2], norb = h[3], npad = h[4], nions = h[5];
    const int grid[3] = {h[6], h[7], h[8]};
    const int j1np = h[9], j2np = h[10], nw = h[11], k = h[12], nsw = h[13];
    const int ne = nup + ndn;
    double lat[3], j1rc, j2rc, tau;
    rd(in, lat, 3);
    rd(in, &j1rc, 1);
    rd(in, &j2rc, 1);
    rd(in, &tau, 1);
    std::vector<double> ions((size_t)nions * 3), j1p(j1np), j1c(1), j2p(2 * (size_t)j2np), j2c(2);
    rd(in, ions.data(), ions.size());
    rd(in, j1p.data(), j1p.size());
    rd(in, j1c.data(), 1);
    rd(in, j2p.data(), j2p.size());
    rd(in, j2c.data(), 2);
    const size_t ncoef = (size_t)(grid[0] + 3) * (grid[1] + 3) * (grid[2] + 3) * npad;
    std::vector<double> coefs(ncoef);
    rd(in, coefs.data(), ncoef);
    std::vector<float> coefs32;
    if (prec == 4)
      coefs32.assign(coefs.begin(), coefs.end());
    std::vector<double> R((size_t)nw * ne * 3), displ((size_t)nsw * ne * nw * 3);
    std::vector<int32_t> acc((size_t)nsw * ne * nw);
    rd(in, R.data(), R.size());
    rd(in, displ.data(), displ.size());
    rd(in, acc.data(), acc.size());
    std::fclose(in);

    std::vector<int> species(nions, 0);
    qmcg_system_desc d{};
    d.precision           = prec;
    d.n_up                = nup;
    d.n_dn                = ndn;
    d.num_orbitals        = norb;
    d.num_orbitals_padded = npad;
    for (int q = 0; q < 3; q++)
    {
      d.lattice[q] = lat[q];
      d.grid[q]    = grid[q];
    }
    d.num_ions        = nions;
    d.ion_pos         = ions.data();
    d.ion_species     = species.data();
    d.num_ion_species = 1;
    d.spline_coefs    = prec == 4 ? static_cast<const void*>(coefs32.data()) : coefs.data();
    d.j1_num_params   = j1np;
    d.j1_rcut         = j1rc;
    d.j1_params       = j1p.data();
    d.j1_cusp         = j1c.data();
    d.j2_num_params   = j2np;
    d.j2_rcut         = j2rc;
    d.j2_params       = j2p.data();
    d.j2_cusp         = j2c.data();
    d.ion_charges     = nullptr;

    QMCGCrowdAdapter a;
    a.create(d, nw, k);
    FILE* out = std::fopen(argv[2], "wb");
    if (!out)
      throw std::runtime_error("cannot open output");
    std::vector<double> lp(nw), gnow((size_t)nw * 3), gnew((size_t)nw * 3), ratios(nw), dsp((size_t)nw * 3);
    std::vector<bool> valid(nw), accept(nw);
    a.mw_evaluateLog(R, lp);
    wr(out, lp.data(), lp.size());
    for (int sw = 0; sw < nsw; sw++)
    {
      for (int iat = 0; iat < ne; iat++)
      {
        a.mw_evalGrad(iat, gnow);
        const size_t m = (size_t)sw * ne + iat;
        for (size_t q = 0; q < dsp.size(); q++)
          dsp[q] = displ[m * nw * 3 + q];
        a.mw_makeMove(iat, dsp, valid);
        a.mw_calcRatioGrad(iat, ratios, gnew);
        for (int iw = 0; iw < nw; iw++)
          accept[iw] = acc[m * nw + iw] != 0 && valid[iw];
        a.mw_accept_rejectMove(iat, accept);
        wr(out, gnow.data(), gnow.size());
        wr(out, ratios.data(), ratios.size());
        wr(out, gnew.data(), gnew.size());
      }
      a.mw_completeUpdates();
    }
    std::vector<double> G((size_t)nw * ne * 3), L((size_t)nw * ne), P((size_t)nw * ne * 3);
    a.mw_evaluateGL(lp, G, L);
    check(qmcg_get_positions(a.crowd, P.data()));
    wr(out, lp.data(), lp.size());
    wr(out, G.data(), G.size());
    wr(out, L.data(), L.size());
    wr(out, P.data(), P.size());
    // the whole loop body of VMCBatched::advanceWalkers as one call
    qmcg_sweep_params p{};
    p.tau             = tau;
    p.use_drift       = 1;
    p.rng_mode        = 1;
    p.seed            = 12345;
    p.recompute_every = 0;
    p.path            = 0;
    p.flush           = 0;
    qmcg_sweep_stats st{};
    check(qmcg_vmc_sweeps(a.crowd, &p, 1, &st, nullptr));
    const double counts[2] = {static_cast<double>(st.accepted), static_cast<double>(st.rejected)};
    wr(out, counts, 2);
    // the same with the walkers' positions in host buffers: in, one sweep, positions and
    // log|psi| out in one call; they must equal what the separate getters return after it
    std::vector<double> Pin((size_t)nw * ne * 3), Pout((size_t)nw * ne * 3), lph(nw), Pchk((size_t)nw * ne * 3),
        lchk(nw);
    check(qmcg_get_positions(a.crowd, Pin.data()));
    qmcg_sweep_stats st2{};
    check(qmcg_vmc_sweeps_host(a.crowd, &p, 1, Pin.data(), Pout.data(), lph.data(), &st2));
    check(qmcg_get_positions(a.crowd, Pchk.data()));
    check(qmcg_get_log(a.crowd, lchk.data(), nullptr, nullptr));
    double dpos = 0, dlog = 0;
    for (size_t e = 0; e < Pout.size(); e++)
      dpos = std::max(dpos, std::fabs(Pout[e] - Pchk[e]));
    for (int w = 0; w < nw; w++)
      dlog = std::max(dlog, std::fabs(lph[w] - lchk[w]));
    const double host_sweep[4] = {static_cast<double>(st2.accepted), static_cast<double>(st2.rejected), dpos, dlog};
    wr(out, host_sweep, 4);
    std::fclose(out);
  }
  catch (const std::exception& e)
  {
    std::fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  return 0;
}
