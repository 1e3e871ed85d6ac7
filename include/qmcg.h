/* qmcg — GB300-native batched particle-by-particle Slater-Jastrow move loop.
 *
 * C ABI over opaque handles.  Plain pointers and sizes only; every function
 * returns QMCG_OK (0) or a negative error code and never throws.  One crowd
 * handle belongs to one host thread (like one QMCPACK crowd); all work of a
 * crowd runs on that crowd's own CUDA stream.
 *
 * The entry points mirror the static batched ("mw_") calls the reference's
 * batched VMC/DMC drivers make for one crowd (QMCPACK 4.3.0):
 *   TrialWaveFunction::mw_*  src/QMCWaveFunctions/TrialWaveFunction.cpp
 *   ParticleSet::mw_*        src/Particle/ParticleSet.cpp
 * Positions, gradients and ratios cross the ABI as FP64 host arrays, as the
 * reference's TWFGrads<POS> / std::vector<PsiValue> do.
 */
#ifndef QMCG_H
#define QMCG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- errors */
#define QMCG_OK 0
#define QMCG_ERR_ARG (-1)        /* invalid argument or size                       */
#define QMCG_ERR_CUDA (-2)       /* a CUDA call failed (see qmcg_last_error)       */
#define QMCG_ERR_SINGULAR (-3)   /* zero pivot in the FP64 inverse                 */
#define QMCG_ERR_NONFINITE (-4)  /* NaN/Inf ratio or gradient (NaNguard)           */
#define QMCG_ERR_ZERO_RATIO (-5) /* accepted move with a zero determinant ratio    */
#define QMCG_ERR_STATE (-6)      /* call out of sequence                           */
#define QMCG_ERR_NO_DEVICE (-7)  /* no usable CUDA device                          */

typedef struct qmcg_system_s* qmcg_system;
typedef struct qmcg_crowd_s* qmcg_crowd;
typedef struct qmcg_group_s* qmcg_group;

/* A Slater-Jastrow system: what QMCPACK reads from its XML input for this path.
 *   cell       orthorhombic, periodic in x, y, z (DTD_BConds<T,3,PPPO>,
 *              src/Particle/Lattice/ParticleBConds3DSoa.h:94-185)
 *   orbitals   real Gamma-point orbitals as one periodic tricubic multi-B-spline
 *              (SplineR2R, src/QMCWaveFunctions/BsplineFactory/SplineR2R.h), coefficient
 *              table [gx+3][gy+3][gz+3][num_orbitals_padded] in the einspline ghost
 *              layout (src/spline2/MultiBsplineBase.hpp:75-130), orbital index fastest
 *   J1, J2     cusp-corrected B-spline radial functors (BsplineFunctor::reset,
 *              src/QMCWaveFunctions/Jastrow/BsplineFunctor.h:117-133); J2 functor 0 acts
 *              between equal spins, functor 1 between opposite spins.
 * Both spin determinants use the same orbital set, so n_up == n_dn == num_orbitals. */
typedef struct
{
  int precision;           /* 8: FP64 move loop; 4: FP32 move loop with FP64 recompute */
  int n_up, n_dn;
  int num_orbitals;
  int num_orbitals_padded; /* multiple of 16 */
  double lattice[3];       /* cell lengths, bohr */
  int num_ions;
  const double* ion_pos;   /* [num_ions][3] */
  const int* ion_species;  /* [num_ions], 0 <= species < num_ion_species */
  int num_ion_species;
  int grid[3];             /* unique periodic grid points per axis */
  const void* spline_coefs;/* float (precision 4) or double (precision 8) */
  int j1_num_params;       /* 0 disables J1 */
  double j1_rcut;
  const double* j1_params; /* [num_ion_species][j1_num_params] */
  const double* j1_cusp;   /* [num_ion_species] */
  int j2_num_params;       /* 0 disables J2 */
  double j2_rcut;
  const double* j2_params; /* [2][j2_num_params] */
  const double* j2_cusp;   /* [2] */
  const double* ion_charges; /* [num_ion_species] valence charges for the Coulomb energy; NULL = a
                                neutral cell, (n_up + n_dn) / num_ions on every ion */
} qmcg_system_desc;

/* Driver parameters of one VMC sweep loop (VMCBatched::advanceWalkers,
 * src/QMCDrivers/VMC/VMCBatched.cpp:57-228).
 * rng_mode 0: the bit-compatible stream of the reference — std::mt19937 seeded
 *             with `seed`, Box-Muller Gaussians [iat][iw][xyz] per sweep and one
 *             uniform per walker and electron consumed only when the move is valid
 *             and |ratio|^2 >= epsilon (StdRandom.h:34-59, RandomSeqGenerator.h:33-51,
 *             VMCBatched.cpp:109,156-158); the host generates it between sweeps.
 * rng_mode 1: counter-based Philox4x32-10 on the device, no host round trip. */
typedef struct
{
  double tau;
  int use_drift;
  int rng_mode;
  uint64_t seed;
  int recompute_every; /* FP64 recompute after every this many sweeps; 0 = never */
  int path;            /* 0: walker-resident sweep kernel when rng_mode is 1 (one CTA owns a walker for a whole
                          sweep), else the staged per-electron kernels; 1: always the staged kernels */
  int flush;           /* delayed-update flush of the walker-resident path: 0 = SIMT (FP32 or FP64),
                          1 = tensor cores TF32, 3 = tensor cores 3xTF32 split precision (FP32 move loop,
                          delay rank <= 64; otherwise the SIMT flush is used), 4 = block-lazy updates: a
                          segment's row block receives the pending updates of its spin group right before
                          the segment, and one pass completes the inverse after the spin group (crowds
                          whose segment rows are staged, see qmcg_sweep_info; otherwise as 3) */
} qmcg_sweep_params;

typedef struct
{
  uint64_t accepted;
  uint64_t rejected;
  uint64_t repaired;   /* walkers whose state was rebuilt by an FP64 recompute after a sweep because the
                          tracked inverse failed its health check |Ainv[row] . phi(r_row) - 1| > tol
                          (1e-2 in FP32, 1e-7 in FP64) or produced a non-finite ratio */
  int status;          /* OR of walker status bits since the last call */
} qmcg_sweep_stats;

/* ---------------------------------------------------------------- library */
const char* qmcg_last_error(void);   /* message of the last failed call on this thread */
int qmcg_device_count(int* count);

/* ---------------------------------------------------------------- system */
/* Builds the device-resident system (spline table, ions, Jastrow functors).
 * Replaces the construction done by EinsplineSetBuilder / RadialJastrowBuilder
 * for the SPOSet and Jastrow objects of one TrialWaveFunction. */
int qmcg_system_create(const qmcg_system_desc* desc, qmcg_system* out);
int qmcg_system_destroy(qmcg_system sys);

/* ---------------------------------------------------------------- crowd */
/* nw walkers with delay rank k (k = 1: Sherman-Morrison rank-1).  Replaces the
 * per-crowd resources acquired by TrialWaveFunction::acquireResource /
 * ParticleSet::acquireResource (src/QMCWaveFunctions/WaveFunctionComponent.h:424-436). */
int qmcg_crowd_create(qmcg_system sys, int num_walkers, int delay_rank, qmcg_crowd* out);
int qmcg_crowd_destroy(qmcg_crowd crowd);
/* the crowd's cudaStream_t, for callers that time or order work around it */
int qmcg_crowd_stream(qmcg_crowd crowd, void** stream);

/* R: [nw][n_elec][3] FP64.  Replaces copying walker positions into the ParticleSets
 * (ParticleSet::loadWalker, src/Particle/ParticleSet.cpp). */
int qmcg_load_walkers(qmcg_crowd crowd, const double* R);
int qmcg_get_positions(qmcg_crowd crowd, double* R);

/* Full recompute of every walker: all-electron orbitals, FP64 inverse and log
 * det, J1/J2 state.  TrialWaveFunction::mw_evaluateLog / mw_recompute
 * (src/QMCWaveFunctions/TrialWaveFunction.cpp:161-260).  log_psi, signs may be NULL. */
int qmcg_mw_evaluate_log(qmcg_crowd crowd, double* log_psi, int* signs);

/* TrialWaveFunction::mw_prepareGroup (TrialWaveFunction.cpp:523): no-op kept for the call sequence. */
int qmcg_mw_prepare_group(qmcg_crowd crowd, int group);

/* grads [nw][3]: gradient of log psi w.r.t. electron iat at the current positions.
 * TrialWaveFunction::mw_evalGrad (TrialWaveFunction.cpp:568-595). */
int qmcg_mw_eval_grad(qmcg_crowd crowd, int iat, double* grads);

/* Propose r_iat + displ[iw] for every walker and build the distance rows.
 * ParticleSet::mw_makeMove (src/Particle/ParticleSet.cpp:397-427).  valid[nw] may be
 * NULL; a fully periodic cell makes every move valid. */
int qmcg_mw_make_move(qmcg_crowd crowd, int iat, const double* displ, int* valid);

/* ratios [nw] psi(new)/psi(old), grads [nw][3] gradient of log psi at the proposed
 * position.  TrialWaveFunction::mw_calcRatioGrad (TrialWaveFunction.cpp:685-772). */
int qmcg_mw_calc_ratio_grad(qmcg_crowd crowd, int iat, double* ratios, double* grads);

/* accepted [nw] (0/1).  TrialWaveFunction::mw_accept_rejectMove (TrialWaveFunction.cpp:790-821)
 * together with ParticleSet::mw_accept_rejectMove (ParticleSet.cpp:717-758). */
int qmcg_mw_accept_reject_move(qmcg_crowd crowd, int iat, const int* accepted);

/* Flush pending delayed updates.  TrialWaveFunction::mw_completeUpdates (TrialWaveFunction.cpp:833). */
int qmcg_mw_complete_updates(qmcg_crowd crowd);

/* From-scratch recompute of the walkers with flags[iw] != 0 (host array [nw]) by the
 * repair path the resident sweeps use when a walker's tracked inverse loses accuracy:
 * orbitals, inverse and log|det| of both spins and the Jastrow state.  The inverse is a
 * Gauss-Jordan elimination over a cluster of SMs per matrix, in FP32 for precision-4
 * crowds (FP64 log|det| sums; the reference inverts in full precision, which this GPU
 * runs at a small fraction of its FP32 rate) and in FP64 otherwise.
 * TrialWaveFunction::mw_recompute with its recompute mask (TrialWaveFunction.cpp:225-240;
 * DiracDeterminantBatched::mw_recompute, DiracDeterminantBatched.cpp:1121-1196).
 * Returns QMCG_ERR_STATE while delayed updates are pending. */
int qmcg_mw_recompute_walkers(qmcg_crowd crowd, const int* flags);

/* Tracked log|psi| per walker (determinant logs accumulated from accepted ratios plus
 * the Jastrow state), signs (+1/-1), parts [nw][4] = log|det_up|, log|det_dn|, log J1,
 * log J2.  Any pointer may be NULL. */
int qmcg_get_log(qmcg_crowd crowd, double* log_psi, int* signs, double* parts);

/* Ainv = (M^-1)^T of spin s, [nw][N][N] as FP64 (DiracDeterminantBatched::get_psiMinv). */
int qmcg_get_inverse(qmcg_crowd crowd, int spin, double* ainv);

/* J2 [nw][5][n_elec] = Uat, dUat xyz, d2Uat; J1 [nw][5][n_elec] = Vat, Grad xyz, Lap.  Either may be NULL. */
int qmcg_get_jastrow_state(qmcg_crowd crowd, double* j2, double* j1);

/* Orbital value, gradient xyz and Laplacian at the proposed position, [nw][5][N]
 * (the phi_vgl_v array of SplineR2R::mw_evaluateVGLandDetRatioGrads). */
int qmcg_get_phi_vgl(qmcg_crowd crowd, double* phi);

/* Device-resident VMC sweeps: num_sweeps x (every electron proposed, tested and
 * accepted or rejected for every walker), then mw_completeUpdates, with the FP64
 * recompute every params->recompute_every sweeps.  Replaces the body of
 * VMCBatched::advanceWalkers (VMCBatched.cpp:106-177); runs as one captured CUDA
 * graph per sweep.  accept_log [num_sweeps][n_elec][nw] (0/1) may be NULL; with
 * rng_mode 1 and path 0 the decisions are recorded by the walker-resident kernel
 * itself (its launches then run outside the graph), otherwise by the staged kernels. */
int qmcg_vmc_sweeps(qmcg_crowd crowd, const qmcg_sweep_params* params, int num_sweeps, qmcg_sweep_stats* stats,
                    int* accept_log);

/* Replays the captured sweep graph num_sweeps times with counter-based random
 * numbers and returns without synchronizing (timing helper for benchmarks; the
 * graph must have been built by a previous qmcg_vmc_sweeps with rng_mode 1). */
int qmcg_vmc_sweeps_async(qmcg_crowd crowd, int num_sweeps);

/* The body of VMCBatched::advanceWalkers for walkers whose positions live in host
 * memory (the driver's ParticleSet R): positions_in [nw][n_elec][3] copied in (NULL:
 * keep the device's positions), num_sweeps as qmcg_vmc_sweeps (no accept log), then
 * the positions and log|psi| [nw] copied back to positions_out and log_psi (either may
 * be NULL), with a single synchronisation at the end.  positions_in may equal
 * positions_out.  Pinned (page-locked) buffers make the copies DMA transfers. */
int qmcg_vmc_sweeps_host(qmcg_crowd crowd, const qmcg_sweep_params* params, int num_sweeps,
                         const double* positions_in, double* positions_out, double* log_psi,
                         qmcg_sweep_stats* stats);

/* Local energy E_L = T + V of every walker after all delayed updates
 * (QMCHamiltonian::mw_evaluate over BareKineticEnergy::mw_evaluate,
 * src/QMCHamiltonians/BareKineticEnergy.cpp:102-160, and the Coulomb terms
 * CoulombPBCAA (e-e, i-i) + CoulombPBCAB (e-i)).  T = -1/2 sum_i (|G_i|^2 + L_i) from
 * the tracked gradients and Laplacians of log psi (mw_evaluateGL); V is the Ewald
 * energy of the electrons (charge -1) and the ions, the quantity the reference's
 * standalone sum src/QMCHamiltonians/EwaldRef.cpp:337-398 computes, evaluated with a
 * real/reciprocal split to 1e-7 (FP32 systems) or 1e-12 (FP64) relative tolerance.
 * Outputs are host arrays of num_walkers doubles; any may be NULL.  Returns
 * QMCG_ERR_STATE while delayed updates are pending. */
int qmcg_mw_evaluate_local_energy(qmcg_crowd crowd, double* e_local, double* kinetic, double* potential);

/* qmcg_vmc_sweeps (without an accept log) with the local energy of every walker
 * measured after every sweep, as the VMC driver's estimator step does:
 * e_local and kinetic (may be NULL) are host arrays [num_sweeps][num_walkers]. */
int qmcg_vmc_sweeps_measure(qmcg_crowd crowd, const qmcg_sweep_params* params, int num_sweeps, double* e_local,
                            double* kinetic, qmcg_sweep_stats* stats);

/* Per-electron gradient and Laplacian of log psi from the tracked state, after all
 * delayed updates: grads [nw][n_elec][3], laplacians [nw][n_elec], log_psi [nw] (the
 * tracked log|psi|); any pointer may be NULL.  TrialWaveFunction::mw_evaluateGL with
 * fromscratch = false (TrialWaveFunction.cpp:869-919: P.G and P.L, the inputs of the
 * Hamiltonian's kinetic and other G/L-based terms); fromscratch = true is
 * qmcg_mw_evaluate_log followed by this call.  Returns QMCG_ERR_STATE while delayed
 * updates are pending. */
int qmcg_mw_evaluate_gl(qmcg_crowd crowd, double* log_psi, double* grads, double* laplacians);

/* Ratios of virtual moves: ratios[v] = psi(R with electron electron[v] at pos[v]) / psi(R)
 * for walker walker[v] — the quadrature points of a non-local pseudopotential
 * (TrialWaveFunction::mw_evaluateRatios, TrialWaveFunction.cpp:1079-1110, over the
 * VirtualParticleSets of NonLocalECPotential; per component SplineR2R::mw_evaluateDetRatios,
 * SplineR2R.cpp:204-335, TwoBodyJastrow::mw_evaluateRatios, TwoBodyJastrow.cpp:174-206, and
 * J1OrbitalSoA::evaluateRatios, J1OrbitalSoA.h:295-299).  The virtual moves of every walker
 * form one flat list of num_moves entries: walker [num_moves], electron [num_moves],
 * pos [num_moves][3] (bohr, FP64 host arrays); ratios [num_moves] FP64.  Nothing of the
 * walkers changes.  Returns QMCG_ERR_STATE while delayed updates are pending, and
 * QMCG_ERR_ARG naming the first move whose walker or electron is out of range or whose
 * position is not finite (checked on the GPU; that move's ratio is NaN, the others are
 * computed). */
int qmcg_mw_evaluate_ratios(qmcg_crowd crowd, int num_moves, const int* walker, const int* electron, const double* pos,
                            double* ratios);

/* Verification helper (no reference counterpart; it exposes what the driver loop of
 * VMCBatched::advanceWalkers sees for every move): qmcg_vmc_sweeps on the
 * walker-resident path (rng_mode 1, path 0, drift-diffusion) with one record per move,
 * trace [num_sweeps][n_elec][nw][QMCG_TRACE_FIELDS] FP64:
 *   0-2  proposed position          3  psi(R')/psi(R)
 *   4-6  grad log psi at R'         7-9  grad log psi at R (the drift's input)
 *   10   1 accepted / 0 rejected    11   Ainv[row] . phi(r_row) of the tracked inverse
 *                                        (1 when exact; the repair health check's value)
 * The kernels run outside the sweep graph while recording. */
#define QMCG_TRACE_FIELDS 12
int qmcg_vmc_sweeps_trace(qmcg_crowd crowd, const qmcg_sweep_params* params, int num_sweeps, qmcg_sweep_stats* stats,
                          double* trace);

/* ---------------------------------------------------------------- diffusion Monte Carlo
 * The DMC step of DMCBatched::advanceWalkers (src/QMCDrivers/DMC/DMCBatched.cpp:72-290) on
 * the walker-resident path: a drift-diffusion sweep in which a move that changes the sign
 * of psi is rejected (fixed node; SFNBranch::phaseChanged, SFNBranch.h:161-169), with
 * tau |xi|^2 summed per walker over proposed and accepted moves (R2PROPOSED, R2ACCEPTED),
 * then the local energy (as qmcg_mw_evaluate_local_energy) and the branch weight
 * w *= exp(tau_eff' (2 E_trial - E_new - E_old)) of SFNBranch::branchWeight
 * (SFNBranch.h:199-208), tau_eff' = tau_eff / 2 scaled down linearly between
 * branch_cutoff and branch_max of x = max(E_ref - E_new, E_ref - E_old) and zero beyond.
 * Population control (which walkers die or are copied, SFNBranch's E_trial feedback)
 * stays on the host; qmcg_dmc_copy_walkers moves the walkers' device state. */
typedef struct
{
  double e_trial;       /* SFNBranch ETRIAL */
  double e_ref;         /* EREF, the centre of the branching cutoff window */
  double tau_eff;       /* TAUEFF */
  double branch_cutoff; /* BRANCHCUTOFF */
  double branch_max;    /* BRANCHMAX, > branch_cutoff */
} qmcg_branch_params;

/* Starts DMC on the crowd's current walkers: weights 1, ages 0, and the local energy of
 * every walker (e_local [nw], may be NULL) kept as the E_old of the first branch weight. */
int qmcg_dmc_init(qmcg_crowd crowd, double* e_local);
/* One DMC step (params: rng_mode 1, path 0; recompute_every counts steps).  Outputs (any
 * may be NULL): weights [nw] after the branch factor, e_local [nw], age [nw] (steps since a
 * walker's last proposed move, DMCBatched.cpp:271-274), sums [5] = sum w, sum w E_L,
 * sum w E_L^2, sum R2ACCEPTED, sum R2PROPOSED (WalkerControl::computeCurData,
 * WalkerControl.cpp:243-270), and trace (as qmcg_vmc_sweeps_trace, the step's sweep then
 * runs outside its graph). */
int qmcg_dmc_step(qmcg_crowd crowd, const qmcg_sweep_params* params, const qmcg_branch_params* branch,
                  double* weights, double* e_local, int* age, double* sums, qmcg_sweep_stats* stats, double* trace);
/* Population control on the device (Walker::makeCopy of WalkerControl::branch and
 * WalkerReconfiguration::getIndexPermutation): slot i takes the state of walker src[i]
 * (positions, inverses, orbital rows, Jastrow state, log|psi|, E_old, age); every walker
 * whose state is copied must keep its own slot (src[src[i]] == src[i]); all weights
 * become 1.  Returns QMCG_ERR_STATE while delayed updates are pending. */
int qmcg_dmc_copy_walkers(qmcg_crowd crowd, const int* src);
/* Population control with a fixed walker count, host part (no GPU needed): the comb of
 * WalkerReconfiguration::getIndexPermutation (src/QMCDrivers/DMC/WalkerReconfiguration.cpp:30-107).
 * num_walkers teeth at W (u + i) / num_walkers, W = sum |w|, 0 <= u < 1; walker i gets one copy
 * per tooth inside its stretch of the cumulative weights.  src [num_walkers]: the walker each
 * slot takes (slots of walkers without a copy take the extra copies of the others, in order;
 * the others keep their own), ready for qmcg_dmc_copy_walkers; num_kept (may be NULL): walkers
 * with at least one copy. */
int qmcg_dmc_comb(int num_walkers, const double* weights, double u, int* src, int* num_kept);
/* qmcg_dmc_comb on the crowd's current weights followed by qmcg_dmc_copy_walkers; src (may be
 * NULL) receives the sources. */
int qmcg_dmc_reconfigure(qmcg_crowd crowd, double u, int* src);

/* ---------------------------------------------------------------- learned MH proposal
 * No reference counterpart: a new proposal for the same exact Metropolis-Hastings step
 * (it replaces the drift-diffusion move of VMCBatched::advanceWalkers,
 * src/QMCDrivers/VMC/VMCBatched.cpp:106-177, and the Green's-function ratio of
 * QMCDriverNew::computeLogGreensFunction, src/QMCDrivers/QMCDriverNew.h:282-296).
 * For electron i a per-electron MLP (51 inputs: displacements to the 8 nearest other
 * electrons and the 8 nearest ions, scaled by 1/2 bohr, and the UNR drift / sqrt(tau);
 * three tanh layers of width 128; outputs mu, s in R^3) proposes
 *   r' = r + drift(R) + sqrt(tau) mu + sqrt(tau) exp(s) xi,  xi ~ N(0, 1),
 * with mu clipped to [-4, 4] and s to [-3, 2], and the move is accepted with
 * probability min(1, |psi(R')/psi(R)|^2 q(r|R') / q(r'|R)).  Inference runs on the
 * tensor cores with BF16 weights and FP32 accumulation; training maximises the
 * expected squared jump distance with hand-written backward and Adam kernels on FP32
 * master parameters.  With the last layer zero the proposal is drift-diffusion. */
#define QMCG_PROPOSAL_NUM_PARAMS 43408 /* W1[128][64] b1[128] W2[128][128] b2 W3 b3 W4[16][128] b4[16];
                                          W1 columns >= 51 and W4/b4 rows >= 6 are kept at zero */
#define QMCG_PROPOSAL_NUM_INPUTS 64    /* 51 features + 13 zero columns */

/* Allocates the network on the crowd's device and initialises it from `seed`:
 * hidden layers uniform(-a, a), a = init_scale / sqrt(fan_in); output layer zero. */
int qmcg_proposal_init(qmcg_crowd crowd, uint64_t seed, double init_scale);
/* FP32 master parameters, QMCG_PROPOSAL_NUM_PARAMS floats (set resets the optimiser). */
int qmcg_proposal_get_params(qmcg_crowd crowd, float* params);
int qmcg_proposal_set_params(qmcg_crowd crowd, const float* params);
/* The network on caller inputs x [rows][64] (rounded to BF16): out [rows][6] = (mu, s)
 * before clipping; hidden (may be NULL) [3][rows][128] = the BF16 post-activations. */
int qmcg_proposal_forward(qmcg_crowd crowd, int rows, const float* x, float* out, float* hidden);
/* Gradient of sum_r dout[r] . out[r] with respect to the parameters (the training
 * backward pass on caller inputs): grad [QMCG_PROPOSAL_NUM_PARAMS]. */
int qmcg_proposal_backward(qmcg_crowd crowd, int rows, const float* x, const float* dout, float* grad);
/* Features of electron iat for every walker, x [num_walkers][64]: at the current
 * position (after qmcg_mw_eval_grad) or at the proposed one (at_proposed = 1, after
 * qmcg_mw_calc_ratio_grad). */
int qmcg_proposal_features(qmcg_crowd crowd, int iat, int at_proposed, float* x);
/* Sweeps with the learned proposal (rng_mode must be 1).  Without training and with
 * params->path 0 they run on the walker-resident sweep kernel (the network evaluated
 * by each walker's CTA); otherwise on the staged per-electron kernels (the network on
 * the tensor cores over all walkers), one CUDA graph per sweep.  train != 0 adds one
 * Adam step (learning rate lr) per electron move over the crowd's walkers.  e_local (may be NULL)
 * [num_sweeps][num_walkers] as in qmcg_vmc_sweeps_measure; train_stats (may be NULL)
 * [3] = mean alpha |r' - r|^2, mean acceptance probability and mean training objective
 * over the training moves.  The objective per move is lambda^4 / j - j with
 * j = alpha |r' - r|^2 and lambda^2 = 3 tau (Levy, Hoffman and Sohl-Dickstein, ICLR 2018). */
int qmcg_vmc_sweeps_learned(qmcg_crowd crowd, const qmcg_sweep_params* params, int num_sweeps, int train, double lr,
                            double* e_local, qmcg_sweep_stats* stats, double* train_stats);

/* ---------------------------------------------------------------- uneven crowds
 * No single reference counterpart: QMCPACK runs one crowd per thread, each with its
 * own launches.  A group sweeps crowds of different systems (up to 8, one precision,
 * the crowds keep their state and ownership) together: per stage, ONE persistent
 * launch of the walker-resident kernel covers the stage's segment of every crowd
 * (work items (crowd, walker) handed out through a device counter, most expensive
 * crowd first), followed by each crowd's delayed-update flush; one CUDA graph per
 * sweep on the first crowd's stream.  Every crowd gets its own counter-based stream
 * (params->seed mixed with the crowd's index). */
int qmcg_group_create(const qmcg_crowd* crowds, int num_crowds, qmcg_group* out);
int qmcg_group_destroy(qmcg_group group);
/* rng_mode must be 1; stats (may be NULL) [num_crowds]. */
int qmcg_group_sweeps(qmcg_group group, const qmcg_sweep_params* params, int num_sweeps, qmcg_sweep_stats* stats);
/* out[4]: stages per sweep, CTAs of the persistent launch, shared memory bytes per CTA,
 * threads per CTA (256 when any crowd runs more than 128 threads per walker alone). */
int qmcg_group_info(qmcg_group group, int* out);

/* Threads per walker (CTA size) of the walker-resident drift-diffusion kernel: 128,
 * 256 or 512 (512 for FP32 only); 0 restores the default, which grows with the
 * walker's shared-memory footprint so that an SM keeps enough warps when it holds only
 * one or two walkers.  The learned proposal always runs 128 threads per walker. */
int qmcg_crowd_set_threads(qmcg_crowd crowd, int threads);

/* Waits for the crowd's stream, then reports and clears the walker status bits. */
int qmcg_crowd_sync(qmcg_crowd crowd, qmcg_sweep_stats* stats);

/* ---------------------------------------------------------------- determinant engine */
/* Delayed-update flush on caller device buffers for num_walkers walkers:
 *   Ainv -= (Ainv U^T - E) (Binv V),  E[delay_list[c]][c] = 1 (slots with -1 skipped)
 * DelayedUpdateBatched::mw_updateInvMat (src/QMCWaveFunctions/Fermion/DelayedUpdateBatched.h:675-738).
 * precision 4 (float) or 8 (double); per walker, row-major and contiguous:
 *   ainv [n][lda], u and v [delay_rank][lda], binv [delay_rank][delay_rank], delay_list [delay_rank];
 * walker w's buffers start at w * (n*lda), w * (delay_rank*lda), w * delay_rank^2, w * delay_rank.
 * Only the first delay_count slots are used.  Enqueued on `stream` (a cudaStream_t, NULL =
 * the legacy default stream).  When the per-walker tiles fit in shared memory the flush
 * needs no global scratch; otherwise a scratch buffer of num_walkers*delay_rank*lda
 * elements is taken from the stream-ordered allocator for the duration of the call. */
int qmcg_mw_update_inv_mat(int precision, int num_walkers, int n, int lda, int delay_rank, int delay_count,
                           void* ainv, const void* u, const void* v, const void* binv, const int* delay_list,
                           void* stream);

/* qmcg_mw_update_inv_mat with a choice of method: 0 = SIMT, 1 = tcgen05 tensor cores
 * in TF32, 3 = tcgen05 tensor cores in 3xTF32 split precision.  Methods 1 and 3 need
 * precision 4, delay_rank <= 64, n and lda multiples of 4 and ainv, u, v on 16-byte
 * boundaries; other cases return QMCG_ERR_ARG.  The update is evaluated as
 * ((T1 - E) Binv) V with T1 = Ainv U^T.  Shapes whose last product is one MMA
 * (delay_rank <= 32, n padded to 16 <= 256) run in one pass; others run the last
 * product over tiles of inverse columns.  A tensor-core wait that times out returns
 * QMCG_ERR_CUDA. */
int qmcg_mw_update_inv_mat_ex(int precision, int num_walkers, int n, int lda, int delay_rank, int delay_count,
                              void* ainv, const void* u, const void* v, const void* binv, const int* delay_list,
                              int method, void* stream);

/* Allocation-free variant of qmcg_mw_update_inv_mat.  It has no counterpart in
 * the reference: QMCPACK's engine always allocates its own scratch.  It exists for
 * callers that cannot call cudaMalloc or a stream-ordered allocator: code whose
 * device memory is owned entirely by another allocator (a framework's caching
 * allocator, an offload runtime that reserves the device), code that cannot
 * afford the device-wide synchronisation cudaFree implies while other streams run,
 * and code running where allocation is forbidden (driver callbacks, real-time
 * threads).  Same arguments and layout as qmcg_mw_update_inv_mat, and the same
 * kernel for every shape, hence the same result; the caller still passes every
 * input and output.
 * Limit: shapes whose per-walker tiles fit in shared memory need no scratch; the
 * others use one fixed device array of QMCG_NOALLOC_SCRATCH_BYTES (16 MiB) that
 * every GPU on which this code is loaded holds until the process exits, and calls
 * needing num_walkers*delay_rank*lda*element_size bytes beyond it return
 * QMCG_ERR_ARG: the caller splits its walkers into batches.
 * The first call that uses the array on a device looks up its device address (once
 * per device, with that device current, and again if the device's context was
 * re-created); make that first call before any stream capture.  Every call shares
 * the array and it keeps the last call's contents; nothing in it has to start at
 * zero (every element a call reads is written earlier by the same call), but calls
 * that overlap on the GPU race and must be ordered by the caller, for example by
 * issuing them on one stream. */
#define QMCG_NOALLOC_SCRATCH_BYTES (16u * 1024u * 1024u)
int qmcg_mw_update_inv_mat_noalloc(int precision, int num_walkers, int n, int lda, int delay_rank, int delay_count,
                                   void* ainv, const void* u, const void* v, const void* binv, const int* delay_list,
                                   void* stream);

/* Orbital input (QMCPACK's ESHDF orbitals, EinsplineSetBuilderESHDF.fft.cpp and
 * OneSplineOrbData::fft_spline, OneSplineOrbData.cpp:62-95, for real Gamma-point orbitals):
 * the spline coefficient table of qmcg_system_desc.spline_coefs from the bands' plane-wave
 * coefficients, which the caller has read from the ESHDF file.  Per band: the coefficients
 * placed on the mesh (unpack4fftw), the backward 3-D transform psi(r) = sum_G c_G
 * exp(+2 pi i G.r/mesh), unnormalized, the global phase rotation of fix_phase_rotate_c2r,
 * and einspline's periodic cubic B-spline interpolation (set_multi_UBspline_3d_d), all on the
 * GPU in FP64.
 *   gvecs        [num_g][3] Miller indices (shared by the bands; distinct)
 *   coefs_g      [num_orbitals][num_g][2] real, imaginary parts
 *   mesh         grid points per axis (4..256), the spline grid of qmcg_system_desc.grid
 *   spline_coefs host output [mesh0+3][mesh1+3][mesh2+3][num_orbitals_padded], float
 *                (precision 4) or double (precision 8), zero beyond num_orbitals
 *   phases       [num_orbitals][2] (phase_r, phase_i) of each band, may be NULL
 * The HDF5 reading itself stays with the caller (no HDF5 library here).  Synchronous: it
 * allocates its device scratch (about 40 bytes per band and mesh point), works on the default
 * stream and returns with the table in spline_coefs. */
int qmcg_spline_from_planewaves(int precision, int num_orbitals, int num_g, const int* gvecs, const double* coefs_g,
                                const int mesh[3], int num_orbitals_padded, void* spline_coefs, double* phases);

/* Measurement helper (no reference counterpart): average device time in ms of
 * the proposed-position evaluation kernel (distance rows, J1/J2, spline VGL and
 * determinant ratio) over num_electrons consecutive electrons, timed with CUDA
 * events on the crowd's stream.  Writes only move scratch. */
int qmcg_profile_ratio(qmcg_crowd crowd, int num_electrons, double* ms_per_launch);

/* Measurement helper (no reference counterpart): device time of the
 * walker-resident path over num_sweeps real sweeps, every launch bracketed by
 * CUDA events on the crowd's stream.  out[0] = ms per walker-resident kernel
 * launch (a segment of up to delay_rank electrons of every walker), out[1] = ms
 * per batched flush launch, out[2] and out[3] = launches of each per sweep.
 * Needs a graph built by qmcg_vmc_sweeps with rng_mode 1 and path 0. */
int qmcg_profile_sweep(qmcg_crowd crowd, int num_sweeps, double* out4);

/* Configuration helper (no reference counterpart): how the walker-resident sweep of
 * this crowd runs with delayed-update flush kind `flush` (qmcg_sweep_params.flush).
 * out[0] = threads per walker of the resident kernel, out[1] = 1 if a segment's inverse
 * rows are staged in shared memory, out[2] = delayed-update sets kept per spin and
 * walker, out[3] = 1 if the flush kind runs as block-lazy updates on this crowd. */
int qmcg_sweep_info(qmcg_crowd crowd, int flush, int* out4);

/* Measurement helper (no reference counterpart): device time in ms of one periodic
 * FP64 recompute of every walker (the full recompute qmcg_vmc_sweeps runs every
 * recompute_every sweeps), timed with CUDA events on the crowd's stream.  Leaves the
 * crowd freshly recomputed; returns QMCG_ERR_STATE while delayed updates are pending. */
int qmcg_profile_recompute(qmcg_crowd crowd, double* ms);

/* Measurement helper (no reference counterpart): device time in ms of one launch of the
 * virtual-move ratio kernel of qmcg_mw_evaluate_ratios on these moves (inputs uploaded once,
 * reps launches timed with CUDA events on the crowd's stream). */
int qmcg_profile_ratios(qmcg_crowd crowd, int num_moves, const int* walker, const int* electron, const double* pos,
                        int reps, double* ms);

#ifdef __cplusplus
}
#endif

#endif /* QMCG_H */
