"""Host-side mirror of the reference's batched (mw_) interface for one crowd.

The method names and argument meanings follow QMCPACK's static batched calls
(TrialWaveFunction::mw_* in src/QMCWaveFunctions/TrialWaveFunction.cpp and
ParticleSet::mw_* in src/Particle/ParticleSet.cpp); every call goes through the
C ABI of libqmcg.so to the sm_103a kernels.  Errors raise QmcgError (the
reference throws std::runtime_error for the same conditions).
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import _lib
from ._lib import BranchParams, QmcgError, SweepParams, SweepStats, SystemDesc, check
from .system import System

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_fp = C.POINTER(C.c_float)


def _d(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _p(a, t=_dp):
    return a.ctypes.data_as(t)


class DeviceSystem:
    """Device-resident system: spline table, ions and Jastrow functors."""

    def __init__(self, system: System):
        L = _lib.load()
        s = system
        self.system = s
        prec = s.spec.precision
        coef_dtype = np.float64 if prec == 8 else np.float32
        self._coefs = np.ascontiguousarray(s.coefs, dtype=coef_dtype)
        self._ions = _d(s.ion_pos)
        self._spec = np.ascontiguousarray(s.ion_species, np.int32)
        self._j1p, self._j1c = _d(s.j1_params), _d(s.j1_cusp)
        self._j2p, self._j2c = _d(s.j2_params), _d(s.j2_cusp)
        d = SystemDesc()
        d.precision = prec
        d.n_up, d.n_dn = s.spec.n_up, s.spec.n_dn
        d.num_orbitals, d.num_orbitals_padded = s.norb, s.npad
        d.lattice = (C.c_double * 3)(*[float(x) for x in s.lattice])
        d.num_ions = len(self._ions)
        d.ion_pos = _p(self._ions)
        d.ion_species = _p(self._spec, _ip)
        d.num_ion_species = s.n_ion_species
        d.grid = (C.c_int * 3)(*[int(x) for x in s.grid])
        d.spline_coefs = self._coefs.ctypes.data
        d.j1_num_params, d.j1_rcut = self._j1p.shape[1], s.spec.j1_rcut
        d.j1_params, d.j1_cusp = _p(self._j1p), _p(self._j1c)
        d.j2_num_params, d.j2_rcut = self._j2p.shape[1], s.spec.j2_rcut
        d.j2_params, d.j2_cusp = _p(self._j2p), _p(self._j2c)
        self._q = _d(s.ion_charges) if s.ion_charges is not None else None
        d.ion_charges = _p(self._q) if self._q is not None else None
        self.handle = C.c_void_p()
        check(L.qmcg_system_create(C.byref(d), C.byref(self.handle)))

    def close(self):
        if getattr(self, "handle", None) and self.handle.value:
            _lib.load().qmcg_system_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        self.close()


class Crowd:
    """nw walkers of one system; one CUDA stream; the mw_ call sequence."""

    def __init__(self, dsys: DeviceSystem, nw: int, delay_rank: int):
        self.L = _lib.load()
        self.dsys = dsys
        self.nw, self.k = nw, delay_rank
        s = dsys.system
        self.ne, self.norb, self.nup = s.n_elec, s.norb, s.spec.n_up
        self.handle = C.c_void_p()
        check(self.L.qmcg_crowd_create(dsys.handle, nw, delay_rank, C.byref(self.handle)))

    def close(self):
        if getattr(self, "handle", None) and self.handle.value:
            self.L.qmcg_crowd_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        self.close()

    # ---- ParticleSet side
    def load_walkers(self, R):
        R = _d(R)
        assert R.shape == (self.nw, self.ne, 3)
        check(self.L.qmcg_load_walkers(self.handle, _p(R)))

    def positions(self, out: Optional[np.ndarray] = None):
        """Positions [nw][ne][3] (float64), written into `out` when given (a C-contiguous
        float64 array of that shape, e.g. in pinned memory) instead of a new array."""
        R = np.empty((self.nw, self.ne, 3)) if out is None else out
        assert R.shape == (self.nw, self.ne, 3) and R.dtype == np.float64 and R.flags.c_contiguous
        check(self.L.qmcg_get_positions(self.handle, _p(R)))
        return R

    def mw_makeMove(self, iat: int, displ):
        d = _d(displ)
        valid = np.zeros(self.nw, np.int32)
        check(self.L.qmcg_mw_make_move(self.handle, iat, _p(d), _p(valid, _ip)))
        return valid.astype(bool)

    # ---- TrialWaveFunction side
    def mw_evaluateLog(self):
        lp = np.zeros(self.nw)
        sg = np.zeros(self.nw, np.int32)
        check(self.L.qmcg_mw_evaluate_log(self.handle, _p(lp), _p(sg, _ip)))
        return lp, sg

    def mw_recompute_walkers(self, flags):
        """From-scratch recompute of the flagged walkers by the repair path."""
        f = np.ascontiguousarray(np.asarray(flags, dtype=np.int32).reshape(self.nw))
        check(self.L.qmcg_mw_recompute_walkers(self.handle, _p(f, _ip)))

    def mw_prepareGroup(self, group: int):
        check(self.L.qmcg_mw_prepare_group(self.handle, group))

    def mw_evalGrad(self, iat: int):
        g = np.zeros((self.nw, 3))
        check(self.L.qmcg_mw_eval_grad(self.handle, iat, _p(g)))
        return g

    def mw_calcRatioGrad(self, iat: int):
        r = np.zeros(self.nw)
        g = np.zeros((self.nw, 3))
        check(self.L.qmcg_mw_calc_ratio_grad(self.handle, iat, _p(r), _p(g)))
        return r, g

    def mw_accept_rejectMove(self, iat: int, accepted):
        a = np.ascontiguousarray(np.asarray(accepted).astype(np.int32))
        check(self.L.qmcg_mw_accept_reject_move(self.handle, iat, _p(a, _ip)))

    def mw_completeUpdates(self):
        check(self.L.qmcg_mw_complete_updates(self.handle))

    # ---- state readback
    def get_log(self, out: Optional[tuple] = None):
        """(log|psi| [nw], sign [nw], parts [nw][4]); `out` may supply the three arrays."""
        if out is None:
            lp, sg, parts = np.zeros(self.nw), np.zeros(self.nw, np.int32), np.zeros((self.nw, 4))
        else:
            lp, sg, parts = out
        check(self.L.qmcg_get_log(self.handle, _p(lp), _p(sg, _ip), _p(parts)))
        return lp, sg, parts

    def inverse(self, spin: int):
        a = np.zeros((self.nw, self.norb, self.norb))
        check(self.L.qmcg_get_inverse(self.handle, spin, _p(a)))
        return a

    def jastrow_state(self):
        j2 = np.zeros((self.nw, 5, self.ne))
        j1 = np.zeros((self.nw, 5, self.ne))
        check(self.L.qmcg_get_jastrow_state(self.handle, _p(j2), _p(j1)))
        return j2, j1

    def phi_vgl(self):
        out = np.zeros((self.nw, 5, self.norb))
        check(self.L.qmcg_get_phi_vgl(self.handle, _p(out)))
        return out

    # ---- device-resident sweeps
    def vmc_sweeps(self, nsweeps: int, tau: float, seed: int, rng_mode: int = 1, use_drift: bool = True,
                   recompute_every: int = 0, log_accepts: bool = False, staged: bool = False, flush: int = 0):
        p = SweepParams(tau=tau, use_drift=int(use_drift), rng_mode=rng_mode, seed=seed,
                        recompute_every=recompute_every, path=1 if staged else 0, flush=flush)
        st = SweepStats()
        acc = np.zeros((nsweeps, self.ne, self.nw), np.int32) if log_accepts else None
        check(self.L.qmcg_vmc_sweeps(self.handle, C.byref(p), nsweeps, C.byref(st),
                                     _p(acc, _ip) if acc is not None else None))
        self.last_repaired = st.repaired
        return st.accepted, st.rejected, acc

    def mw_evaluateGL(self):
        """(log|psi| [nw], G [nw][ne][3], L [nw][ne]) from the tracked state (after mw_completeUpdates)."""
        lp = np.zeros(self.nw)
        G = np.zeros((self.nw, self.ne, 3))
        L = np.zeros((self.nw, self.ne))
        check(self.L.qmcg_mw_evaluate_gl(self.handle, _p(lp), _p(G), _p(L)))
        return lp, G, L

    def vmc_sweeps_trace(self, nsweeps: int, tau: float, seed: int, use_drift: bool = True, recompute_every: int = 0,
                         flush: int = 0):
        """Walker-resident sweeps with one record per move: (accepted, rejected,
        trace [nsweeps][ne][nw][TRACE_FIELDS]); fields as QMCG_TRACE_FIELDS in the header."""
        p = SweepParams(tau=tau, use_drift=int(use_drift), rng_mode=1, seed=seed,
                        recompute_every=recompute_every, path=0, flush=flush)
        st = SweepStats()
        tr = np.zeros((nsweeps, self.ne, self.nw, _lib.TRACE_FIELDS))
        check(self.L.qmcg_vmc_sweeps_trace(self.handle, C.byref(p), nsweeps, C.byref(st), _p(tr)))
        self.last_repaired = st.repaired
        return st.accepted, st.rejected, tr

    def mw_evaluateRatios(self, walker, electron, pos):
        """Ratios psi(R, electron at pos) / psi(R) of a flat list of virtual moves
        (non-local pseudopotential quadrature points); needs mw_completeUpdates first."""
        wk = np.ascontiguousarray(walker, np.int32).ravel()
        el = np.ascontiguousarray(electron, np.int32).ravel()
        ps = _d(pos).reshape(-1, 3)
        assert wk.size == el.size == ps.shape[0]
        r = np.zeros(wk.size)
        check(self.L.qmcg_mw_evaluate_ratios(self.handle, wk.size, _p(wk, _ip), _p(el, _ip), _p(ps), _p(r)))
        return r

    def profile_ratios(self, walker, electron, pos, reps: int = 10) -> float:
        """Device ms of one launch of the virtual-move ratio kernel on these moves."""
        wk = np.ascontiguousarray(walker, np.int32).ravel()
        el = np.ascontiguousarray(electron, np.int32).ravel()
        ps = _d(pos).reshape(-1, 3)
        ms = C.c_double()
        check(self.L.qmcg_profile_ratios(self.handle, wk.size, _p(wk, _ip), _p(el, _ip), _p(ps), reps, C.byref(ms)))
        return ms.value

    # ---- diffusion Monte Carlo
    def dmc_init(self):
        """Weights 1, ages 0; returns the local energy of every walker (the first E_old)."""
        el = np.zeros(self.nw)
        check(self.L.qmcg_dmc_init(self.handle, _p(el)))
        return el

    def dmc_step(self, tau: float, seed: int, e_trial: float, e_ref: float, tau_eff: float, branch_cutoff: float,
                 branch_max: float, use_drift: bool = True, recompute_every: int = 0, flush: int = 0,
                 trace: bool = False):
        """One fixed-node DMC step with branch weights: dict of weights [nw], e_local [nw],
        age [nw], sums [5] (sum w, sum w E, sum w E^2, sum r2 accepted, sum r2 proposed),
        accepted, rejected and the move trace (if asked)."""
        p = SweepParams(tau=tau, use_drift=int(use_drift), rng_mode=1, seed=seed,
                        recompute_every=recompute_every, path=0, flush=flush)
        b = BranchParams(e_trial=e_trial, e_ref=e_ref, tau_eff=tau_eff, branch_cutoff=branch_cutoff,
                         branch_max=branch_max)
        w, el, sums = np.zeros(self.nw), np.zeros(self.nw), np.zeros(5)
        age = np.zeros(self.nw, np.int32)
        st = SweepStats()
        tr = np.zeros((1, self.ne, self.nw, _lib.TRACE_FIELDS)) if trace else None
        check(self.L.qmcg_dmc_step(self.handle, C.byref(p), C.byref(b), _p(w), _p(el), _p(age, _ip), _p(sums),
                                   C.byref(st), _p(tr) if tr is not None else None))
        self.last_repaired = st.repaired
        return {"weights": w, "e_local": el, "age": age, "sums": sums, "accepted": st.accepted,
                "rejected": st.rejected, "trace": tr}

    def dmc_copy_walkers(self, src):
        a = np.ascontiguousarray(np.asarray(src, dtype=np.int32).reshape(self.nw))
        check(self.L.qmcg_dmc_copy_walkers(self.handle, _p(a, _ip)))

    def dmc_reconfigure(self, u: float):
        """Comb of the current weights (fixed walker count) and the device copies; returns the sources."""
        src = np.zeros(self.nw, np.int32)
        check(self.L.qmcg_dmc_reconfigure(self.handle, float(u), _p(src, _ip)))
        return src

    def mw_evaluate_local_energy(self):
        """(E_L, kinetic, potential) per walker; needs all delayed updates completed."""
        el, ke, vp = np.zeros(self.nw), np.zeros(self.nw), np.zeros(self.nw)
        check(self.L.qmcg_mw_evaluate_local_energy(self.handle, _p(el), _p(ke), _p(vp)))
        return el, ke, vp

    def vmc_sweeps_measure(self, nsweeps: int, tau: float, seed: int, rng_mode: int = 1, use_drift: bool = True,
                           recompute_every: int = 0, staged: bool = False, flush: int = 0):
        """Sweeps with the local energy of every walker after each: (accepted, rejected, E_L[nsweeps][nw],
        kinetic[nsweeps][nw])."""
        p = SweepParams(tau=tau, use_drift=int(use_drift), rng_mode=rng_mode, seed=seed,
                        recompute_every=recompute_every, path=1 if staged else 0, flush=flush)
        st = SweepStats()
        el = np.zeros((nsweeps, self.nw))
        ke = np.zeros((nsweeps, self.nw))
        check(self.L.qmcg_vmc_sweeps_measure(self.handle, C.byref(p), nsweeps, _p(el), _p(ke), C.byref(st)))
        self.last_repaired = st.repaired
        return st.accepted, st.rejected, el, ke

    def set_threads(self, threads: int = 0):
        """Threads per walker of the resident drift-diffusion kernel (128/256/512; 0 = default)."""
        check(self.L.qmcg_crowd_set_threads(self.handle, threads))

    # ---- learned MH proposal
    def proposal_init(self, seed: int = 1, init_scale: float = 1.0):
        check(self.L.qmcg_proposal_init(self.handle, seed, init_scale))

    def proposal_params(self) -> np.ndarray:
        p = np.zeros(_lib.PROPOSAL_NUM_PARAMS, np.float32)
        check(self.L.qmcg_proposal_get_params(self.handle, _p(p, _fp)))
        return p

    def set_proposal_params(self, params):
        p = np.ascontiguousarray(params, np.float32)
        assert p.size == _lib.PROPOSAL_NUM_PARAMS
        check(self.L.qmcg_proposal_set_params(self.handle, _p(p, _fp)))

    def proposal_forward(self, x, with_hidden: bool = False):
        x = np.ascontiguousarray(x, np.float32)
        rows = x.shape[0]
        out = np.zeros((rows, 6), np.float32)
        hid = np.zeros((3, rows, 128), np.float32) if with_hidden else None
        check(self.L.qmcg_proposal_forward(self.handle, rows, _p(x, _fp), _p(out, _fp),
                                           _p(hid, _fp) if hid is not None else None))
        return (out, hid) if with_hidden else out

    def proposal_backward(self, x, dout):
        x = np.ascontiguousarray(x, np.float32)
        d = np.ascontiguousarray(dout, np.float32)
        g = np.zeros(_lib.PROPOSAL_NUM_PARAMS, np.float32)
        check(self.L.qmcg_proposal_backward(self.handle, x.shape[0], _p(x, _fp), _p(d, _fp), _p(g, _fp)))
        return g

    def proposal_features(self, iat: int, at_proposed: bool = False):
        x = np.zeros((self.nw, 64), np.float32)
        check(self.L.qmcg_proposal_features(self.handle, iat, int(at_proposed), _p(x, _fp)))
        return x

    def vmc_sweeps_learned(self, nsweeps: int, tau: float, seed: int, train: bool = False, lr: float = 1e-3,
                           measure: bool = False, use_drift: bool = True, recompute_every: int = 0, flush: int = 0,
                           staged: bool = False):
        """(accepted, rejected, E_L[nsweeps][nw] or None, (mean alpha|dr|^2, mean alpha, mean objective));
        inference runs on the walker-resident kernel unless staged (training always uses the staged kernels)."""
        p = SweepParams(tau=tau, use_drift=int(use_drift), rng_mode=1, seed=seed,
                        recompute_every=recompute_every, path=1 if staged else 0, flush=flush)
        st = SweepStats()
        el = np.zeros((nsweeps, self.nw)) if measure else None
        ts = np.zeros(3)
        check(self.L.qmcg_vmc_sweeps_learned(self.handle, C.byref(p), nsweeps, int(train), lr,
                                             _p(el) if el is not None else None, C.byref(st), _p(ts)))
        self.last_repaired = st.repaired
        return st.accepted, st.rejected, el, (float(ts[0]), float(ts[1]), float(ts[2]))

    def vmc_sweeps_async(self, nsweeps: int):
        check(self.L.qmcg_vmc_sweeps_async(self.handle, nsweeps))

    def vmc_sweeps_host(self, nsweeps: int, tau: float, seed: int, R_in: Optional[np.ndarray] = None,
                        R_out: Optional[np.ndarray] = None, log_out: Optional[np.ndarray] = None,
                        use_drift: bool = True, recompute_every: int = 0, flush: int = 0):
        """Positions in from R_in, nsweeps device-RNG sweeps, positions and log|psi| out to R_out and
        log_out (C-contiguous float64 arrays, e.g. pinned; any may be None) with one synchronisation."""
        for a, shape in ((R_in, (self.nw, self.ne, 3)), (R_out, (self.nw, self.ne, 3)), (log_out, (self.nw,))):
            assert a is None or (a.shape == shape and a.dtype == np.float64 and a.flags.c_contiguous)
        p = SweepParams(tau=tau, use_drift=int(use_drift), rng_mode=1, seed=seed,
                        recompute_every=recompute_every, path=0, flush=flush)
        st = SweepStats()
        check(self.L.qmcg_vmc_sweeps_host(self.handle, C.byref(p), nsweeps,
                                          _p(R_in) if R_in is not None else None,
                                          _p(R_out) if R_out is not None else None,
                                          _p(log_out) if log_out is not None else None, C.byref(st)))
        self.last_repaired = st.repaired
        return st.accepted, st.rejected

    def sync(self):
        st = SweepStats()
        check(self.L.qmcg_crowd_sync(self.handle, C.byref(st)))
        self.last_repaired = st.repaired
        return st.accepted, st.rejected

    def profile_ratio(self, num_electrons: int) -> float:
        ms = C.c_double()
        check(self.L.qmcg_profile_ratio(self.handle, num_electrons, C.byref(ms)))
        return ms.value

    def profile_sweep(self, nsweeps: int):
        """(ms per resident-kernel launch, ms per flush launch, resident launches per sweep, flushes per sweep)"""
        out = np.zeros(4)
        check(self.L.qmcg_profile_sweep(self.handle, nsweeps, _p(out)))
        return float(out[0]), float(out[1]), int(out[2]), int(out[3])

    def sweep_info(self, flush: int = 0):
        """How the walker-resident sweep runs with this flush kind: threads per walker,
        segment rows staged, delayed-update sets per spin and walker, block-lazy updates."""
        out = np.zeros(4, np.int32)
        check(self.L.qmcg_sweep_info(self.handle, flush, _p(out, _ip)))
        return {"threads": int(out[0]), "rows_staged": bool(out[1]), "sets": int(out[2]), "block_lazy": bool(out[3])}

    def profile_recompute(self) -> float:
        """Device ms of one periodic FP64 recompute of every walker."""
        ms = C.c_double()
        check(self.L.qmcg_profile_recompute(self.handle, C.byref(ms)))
        return ms.value

    def stream(self) -> int:
        p = C.c_void_p()
        check(self.L.qmcg_crowd_stream(self.handle, C.byref(p)))
        return p.value or 0


def dmc_comb(weights, u: float):
    """Population control with a fixed walker count (no GPU needed): (sources, walkers kept)."""
    w = np.ascontiguousarray(weights, np.float64)
    src = np.zeros(w.size, np.int32)
    kept = C.c_int()
    L = _lib.load()
    check(L.qmcg_dmc_comb(w.size, _p(w), float(u), _p(src, _ip), C.byref(kept)))
    return src, kept.value


def group_seed(seed: int, index: int) -> int:
    """The counter-based stream seed a group gives its index-th crowd."""
    return (seed ^ ((0x9E3779B97F4A7C15 * (index + 1)) & 0xFFFFFFFFFFFFFFFF)) & 0xFFFFFFFFFFFFFFFF


class Group:
    """Crowds of different systems swept together, one persistent launch per stage."""

    def __init__(self, crowds):
        self.L = _lib.load()
        self.crowds = list(crowds)
        arr = (C.c_void_p * len(self.crowds))(*[c.handle.value for c in self.crowds])
        self.handle = C.c_void_p()
        check(self.L.qmcg_group_create(arr, len(self.crowds), C.byref(self.handle)))

    def close(self):
        if getattr(self, "handle", None) and self.handle.value:
            self.L.qmcg_group_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        self.close()

    def sweeps(self, nsweeps: int, tau: float, seed: int, use_drift: bool = True, recompute_every: int = 0,
               flush: int = 0):
        """[(accepted, rejected, repaired) per crowd]"""
        p = SweepParams(tau=tau, use_drift=int(use_drift), rng_mode=1, seed=seed,
                        recompute_every=recompute_every, path=0, flush=flush)
        st = (SweepStats * len(self.crowds))()
        check(self.L.qmcg_group_sweeps(self.handle, C.byref(p), nsweeps, st))
        return [(x.accepted, x.rejected, x.repaired) for x in st]

    def info(self):
        out = np.zeros(4, np.int32)
        check(self.L.qmcg_group_info(self.handle, _p(out, _ip)))
        return {"stages": int(out[0]), "ctas": int(out[1]), "smem_bytes": int(out[2]), "threads": int(out[3])}
