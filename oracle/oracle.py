"""ctypes binding of the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs import
this module.  The oracle is the checker, never the product path.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_lp = C.POINTER(C.c_long)

# fields of one move record: position xyz, ratio, grad at R' xyz, grad at R xyz, accepted, self ratio
TRACE_FIELDS = 12


def build(force: bool = False) -> str:
    so = os.path.join(_HERE, "liboracle.so")
    srcs = [os.path.join(_HERE, f) for f in ("qmc_oracle.cpp", "ewald_oracle.cpp", "Makefile")]
    if force or not os.path.exists(so) or os.path.getmtime(so) < max(os.path.getmtime(f) for f in srcs):
        subprocess.check_call(["make", "-s", "-C", _HERE, "liboracle.so"])
    return so


def lib():
    global _LIB
    if _LIB is None:
        _LIB = C.CDLL(build())
        L = _LIB
        L.orc_crowd_create.restype = C.c_void_p
        L.orc_crowd_create.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _dp, C.c_int, _dp, _ip, C.c_int,
                                       _ip, _dp, C.c_int, C.c_double, _dp, _dp, C.c_int, C.c_double, _dp, _dp,
                                       C.c_int, C.c_int]
        L.orc_crowd_destroy.argtypes = [C.c_void_p]
        L.orc_load_walkers.argtypes = [C.c_void_p, _dp]
        L.orc_get_positions.argtypes = [C.c_void_p, _dp]
        L.orc_evaluate_log.argtypes = [C.c_void_p, _dp, _ip, C.c_int]
        L.orc_evaluate_log.restype = C.c_int
        L.orc_get_log.argtypes = [C.c_void_p, _dp, _ip, _dp]
        L.orc_eval_grad.argtypes = [C.c_void_p, C.c_int, _dp]
        L.orc_make_move.argtypes = [C.c_void_p, C.c_int, _dp]
        L.orc_ratio_grad.argtypes = [C.c_void_p, C.c_int, _dp, _dp]
        L.orc_accept_reject.argtypes = [C.c_void_p, C.c_int, _ip]
        L.orc_complete_updates.argtypes = [C.c_void_p]
        L.orc_get_ainv.argtypes = [C.c_void_p, C.c_int, _dp]
        L.orc_get_jastrow_state.argtypes = [C.c_void_p, _dp, _dp]
        L.orc_get_phi_vgl.argtypes = [C.c_void_p, C.c_int, _dp]
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_rng_create.restype = C.c_void_p
        L.orc_rng_create.argtypes = [C.c_uint]
        L.orc_rng_destroy.argtypes = [C.c_void_p]
        L.orc_rng_uniform.argtypes = [C.c_void_p, _dp, C.c_long]
        L.orc_rng_gauss.argtypes = [C.c_void_p, _dp, C.c_long]
        L.orc_vmc_sweeps.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_double, C.c_int, _lp, _lp, _ip]
        L.orc_vmc_sweeps_philox.argtypes = [C.c_void_p, C.c_uint64, C.c_uint, C.c_int, C.c_double, C.c_int, _lp,
                                            _lp, _dp]
        L.orc_replay_trace.argtypes = [C.c_void_p, C.c_int, _dp, _dp]
        L.orc_replay_trace_philox.argtypes = [C.c_void_p, C.c_uint64, C.c_uint, C.c_int, C.c_double, C.c_int,
                                              C.c_int, _dp, _dp, _dp]
        L.orc_copy_walkers.argtypes = [C.c_void_p, _ip]
        L.orc_evaluate_ratios.argtypes = [C.c_void_p, C.c_int, _ip, _ip, _dp, _dp]
        L.orc_prefactors.argtypes = [C.c_double, _dp, _dp, _dp]
        L.orc_spline_vgh.argtypes = [_ip, C.c_int, _dp, C.c_int, _dp, _dp, _dp, _dp]
        L.orc_functor_eval.argtypes = [C.c_int, C.c_double, _dp, C.c_double, C.c_int, _dp, _dp, _dp, _dp]
        L.orc_invert.argtypes = [_dp, C.c_int, _dp, _ip]
        L.orc_invert.restype = C.c_int
        L.orc_distance_row.argtypes = [_dp, C.c_int, _dp, _dp, _dp, _dp]
        L.orc_det_create.restype = C.c_void_p
        L.orc_det_create.argtypes = [C.c_int, C.c_int]
        L.orc_det_destroy.argtypes = [C.c_void_p]
        L.orc_det_recompute.argtypes = [C.c_void_p, _dp, _dp, _ip]
        L.orc_det_recompute.restype = C.c_int
        L.orc_det_ratio.argtypes = [C.c_void_p, C.c_int, _dp]
        L.orc_det_ratio.restype = C.c_double
        L.orc_det_accept_reject.argtypes = [C.c_void_p, C.c_int, _dp, C.c_double, C.c_int]
        L.orc_det_complete.argtypes = [C.c_void_p]
        L.orc_det_get_ainv.argtypes = [C.c_void_p, _dp]
        L.orc_kinetic.argtypes = [C.c_void_p, _dp, _dp]
        L.orc_ewald_ref_energy.argtypes = [_dp, C.c_int, _dp, _dp, C.c_double]
        L.orc_ewald_ref_energy.restype = C.c_double
        L.orc_madelung.argtypes = [_dp, C.c_double]
        L.orc_madelung.restype = C.c_double
        L.orc_ewald_split_energy.argtypes = [_dp, C.c_int, _dp, _dp, C.c_double, _dp]
    return _LIB


def _d(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _ptr(a, t=_dp):
    return a.ctypes.data_as(t)


# ---------------------------------------------------------------- unit functions
def prefactors(t: float):
    a, da, d2a = np.zeros(4), np.zeros(4), np.zeros(4)
    lib().orc_prefactors(t, _ptr(a), _ptr(da), _ptr(d2a))
    return a, da, d2a


def spline_vgh(coefs: np.ndarray, norb: int, u):
    """coefs: (gx+3, gy+3, gz+3, npad) ghost layout; u: unit-cube point."""
    c = _d(coefs)
    grid = np.array([c.shape[0] - 3, c.shape[1] - 3, c.shape[2] - 3], np.int32)
    npad = c.shape[3]
    v, g, h = np.zeros(norb), np.zeros((3, norb)), np.zeros((6, norb))
    uu = _d(u)
    lib().orc_spline_vgh(_ptr(grid, _ip), npad, _ptr(c), norb, _ptr(uu), _ptr(v), _ptr(g), _ptr(h))
    return v, g, h


def functor_eval(params, rcut: float, cusp: float, r):
    p = _d(params)
    rr = _d(np.atleast_1d(r))
    u, du, d2u = np.zeros_like(rr), np.zeros_like(rr), np.zeros_like(rr)
    lib().orc_functor_eval(len(p), rcut, _ptr(p), cusp, len(rr), _ptr(rr), _ptr(u), _ptr(du), _ptr(d2u))
    return u, du, d2u


def invert(a):
    m = _d(a).copy()
    la = C.c_double()
    sg = C.c_int()
    rc = lib().orc_invert(_ptr(m), m.shape[0], C.byref(la), C.byref(sg))
    if rc != 0:
        raise ValueError("singular matrix")
    return m, la.value, sg.value


def distance_row(lattice, R, r):
    R = _d(R)
    n = R.shape[0]
    dist, dr = np.zeros(n), np.zeros((3, n))
    lat = _d(lattice)
    rr = _d(r)
    lib().orc_distance_row(_ptr(lat), n, _ptr(R), _ptr(rr), _ptr(dist), _ptr(dr))
    return dist, dr


def ewald_ref_energy(cell_rows, R, Q, tol: float = 1e-10) -> float:
    """Total Ewald energy of point charges (EwaldRef restatement); cell_rows: 3x3, rows = cell vectors."""
    a = _d(cell_rows).reshape(9)
    R = _d(R).reshape(-1, 3)
    Q = _d(Q)
    return lib().orc_ewald_ref_energy(_ptr(a), len(Q), _ptr(R), _ptr(Q), tol)


def madelung(cell_rows, tol: float = 1e-12) -> float:
    a = _d(cell_rows).reshape(9)
    return lib().orc_madelung(_ptr(a), tol)


def ewald_split_energy(lattice, R, Q, eps: float = 1e-14):
    """Same energy by the real/reciprocal split of the GPU kernel (orthorhombic cell, FP64).
    Returns (real-space, reciprocal, constant, total)."""
    L = _d(lattice)
    R = _d(R).reshape(-1, 3)
    Q = _d(Q)
    out = np.zeros(4)
    lib().orc_ewald_split_energy(_ptr(L), len(Q), _ptr(R), _ptr(Q), eps, _ptr(out))
    return out


def set_threads(n: int):
    lib().orc_set_threads(int(n))


class Det:
    """One determinant with its delayed-update engine (rank k; k = 1 is SM-1)."""

    def __init__(self, n: int, k: int):
        self.n, self.k = n, k
        self.h = lib().orc_det_create(n, k)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_det_destroy(self.h)
            self.h = None

    def recompute(self, psiM):
        p = _d(psiM)
        la = C.c_double()
        sg = C.c_int()
        if lib().orc_det_recompute(self.h, _ptr(p), C.byref(la), C.byref(sg)) != 0:
            raise ValueError("singular")
        return la.value, sg.value

    def ratio(self, row: int, phi) -> float:
        p = _d(phi)
        return lib().orc_det_ratio(self.h, row, _ptr(p))

    def accept_reject(self, row: int, phi, ratio: float, accepted: bool):
        p = _d(phi)
        lib().orc_det_accept_reject(self.h, row, _ptr(p), ratio, int(bool(accepted)))

    def complete(self):
        lib().orc_det_complete(self.h)

    def ainv(self):
        out = np.zeros((self.n, self.n))
        lib().orc_det_get_ainv(self.h, _ptr(out))
        return out


class Rng:
    def __init__(self, seed: int):
        self.h = lib().orc_rng_create(seed)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_rng_destroy(self.h)
            self.h = None

    def uniform(self, n):
        out = np.zeros(n)
        lib().orc_rng_uniform(self.h, _ptr(out), n)
        return out

    def gauss(self, n):
        out = np.zeros(n)
        lib().orc_rng_gauss(self.h, _ptr(out), n)
        return out


class Crowd:
    """The oracle's batched crowd, same call sequence as the mw_ API."""

    def __init__(self, system, nw: int, delay: int, precision: int):
        s = system
        self.system, self.nw, self.delay, self.prec = s, nw, delay, precision
        self.ne = s.n_elec
        self.norb = s.norb
        self._keep = [_d(s.lattice), _d(s.ion_pos), np.ascontiguousarray(s.ion_species, np.int32),
                      np.ascontiguousarray(s.grid, np.int32), _d(s.coefs), _d(s.j1_params), _d(s.j1_cusp),
                      _d(s.j2_params), _d(s.j2_cusp)]
        lat, ions, spec, grid, coefs, j1p, j1c, j2p, j2c = self._keep
        self.h = lib().orc_crowd_create(precision, s.spec.n_up, s.spec.n_dn, s.norb, s.npad, _ptr(lat),
                                        len(ions), _ptr(ions), _ptr(spec, _ip), s.n_ion_species, _ptr(grid, _ip),
                                        _ptr(coefs), j1p.shape[1], s.spec.j1_rcut, _ptr(j1p), _ptr(j1c),
                                        j2p.shape[1], s.spec.j2_rcut, _ptr(j2p), _ptr(j2c), nw, delay)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_crowd_destroy(self.h)
            self.h = None

    def load_walkers(self, R):
        R = _d(R)
        assert R.shape == (self.nw, self.ne, 3)
        lib().orc_load_walkers(self.h, _ptr(R))

    def positions(self):
        R = np.zeros((self.nw, self.ne, 3))
        lib().orc_get_positions(self.h, _ptr(R))
        return R

    def evaluate_log(self, nthreads: int = 1):
        lp = np.zeros(self.nw)
        sg = np.zeros(self.nw, np.int32)
        if lib().orc_evaluate_log(self.h, _ptr(lp), _ptr(sg, _ip), nthreads) != 0:
            raise ValueError("singular Slater matrix")
        return lp, sg

    def get_log(self):
        lp = np.zeros(self.nw)
        sg = np.zeros(self.nw, np.int32)
        parts = np.zeros((self.nw, 4))
        lib().orc_get_log(self.h, _ptr(lp), _ptr(sg, _ip), _ptr(parts))
        return lp, sg, parts

    def eval_grad(self, iat):
        g = np.zeros((self.nw, 3))
        lib().orc_eval_grad(self.h, iat, _ptr(g))
        return g

    def make_move(self, iat, displ):
        d = _d(displ)
        lib().orc_make_move(self.h, iat, _ptr(d))

    def ratio_grad(self, iat):
        r = np.zeros(self.nw)
        g = np.zeros((self.nw, 3))
        lib().orc_ratio_grad(self.h, iat, _ptr(r), _ptr(g))
        return r, g

    def accept_reject(self, iat, accepted):
        a = np.ascontiguousarray(accepted, np.int32)
        lib().orc_accept_reject(self.h, iat, _ptr(a, _ip))

    def complete_updates(self):
        lib().orc_complete_updates(self.h)

    def ainv(self, spin):
        out = np.zeros((self.nw, self.norb, self.norb))
        lib().orc_get_ainv(self.h, spin, _ptr(out))
        return out

    def jastrow_state(self):
        j2 = np.zeros((self.nw, 5, self.ne))
        j1 = np.zeros((self.nw, 5, self.ne))
        lib().orc_get_jastrow_state(self.h, _ptr(j2), _ptr(j1))
        return j2, j1

    def phi_vgl(self, spin):
        out = np.zeros((self.nw, 5, self.norb))
        lib().orc_get_phi_vgl(self.h, spin, _ptr(out))
        return out

    def vmc_sweeps(self, rng: Rng, nsteps: int, tau: float, use_drift: bool = True, log_accepts: bool = False):
        na, nr = C.c_long(0), C.c_long(0)
        acc = np.zeros((nsteps, self.ne, self.nw), np.int32) if log_accepts else None
        lib().orc_vmc_sweeps(self.h, rng.h, nsteps, tau, int(use_drift), C.byref(na), C.byref(nr),
                             _ptr(acc, _ip) if acc is not None else None)
        return na.value, nr.value, acc

    def vmc_sweeps_philox(self, seed: int, nsteps: int, tau: float, use_drift: bool = True, sweep0: int = 0,
                          trace: bool = False):
        """Sweeps on the device's counter-based stream (Philox4x32-10, counter (walker, electron,
        sweep, j)): (accepted, rejected, trace [nsteps][ne][nw][12] or None)."""
        na, nr = C.c_long(0), C.c_long(0)
        tr = np.zeros((nsteps, self.ne, self.nw, TRACE_FIELDS)) if trace else None
        lib().orc_vmc_sweeps_philox(self.h, seed, sweep0, nsteps, tau, int(use_drift), C.byref(na), C.byref(nr),
                                    _ptr(tr) if tr is not None else None)
        return na.value, nr.value, tr

    def replay(self, trace_in):
        """Follow a recorded trajectory (proposed positions and decisions of trace_in
        [nsteps][ne][nw][12]); returns this crowd's records on the same moves."""
        ti = _d(trace_in)
        assert ti.shape[1:] == (self.ne, self.nw, TRACE_FIELDS)
        to = np.zeros_like(ti)
        lib().orc_replay_trace(self.h, ti.shape[0], _ptr(ti), _ptr(to))
        return to

    def replay_philox(self, trace_in, seed: int, tau: float, use_drift: bool = True, sweep0: int = 0,
                      dmc: bool = False):
        """Follow a recorded trajectory on the counter-based stream and form, at every move,
        this crowd's own proposal, ratio, gradients and decision from the shared state:
        (trace_out with TR_POS = own proposal, TR_ACCEPT = own decision and TR_SELF = tau |xi|^2,
        margin (u - P) / P).  dmc: fixed-node moves (a sign change of psi is rejected)."""
        ti = _d(trace_in)
        assert ti.shape[1:] == (self.ne, self.nw, TRACE_FIELDS)
        to = np.zeros_like(ti)
        margin = np.zeros(ti.shape[:3])
        lib().orc_replay_trace_philox(self.h, seed, sweep0, ti.shape[0], tau, int(use_drift), int(dmc), _ptr(ti),
                                      _ptr(to), _ptr(margin))
        return to, margin

    def evaluate_ratios(self, walker, electron, pos):
        """Ratios psi(R, electron at pos) / psi(R) of a flat list of virtual moves."""
        wk = np.ascontiguousarray(walker, np.int32).ravel()
        el = np.ascontiguousarray(electron, np.int32).ravel()
        ps = _d(pos).reshape(-1, 3)
        r = np.zeros(wk.size)
        lib().orc_evaluate_ratios(self.h, wk.size, _ptr(wk, _ip), _ptr(el, _ip), _ptr(ps), _ptr(r))
        return r

    def copy_walkers(self, src):
        """Walker i takes the state of walker src[i] (population control)."""
        a = np.ascontiguousarray(src, np.int32)
        lib().orc_copy_walkers(self.h, _ptr(a, _ip))

    def kinetic(self, with_gl: bool = False):
        """Kinetic energy per walker from the tracked state (call complete_updates first);
        with_gl also returns [nw][ne][4] = grad log psi (xyz) and Laplacian of log psi."""
        ke = np.zeros(self.nw)
        gl = np.zeros((self.nw, self.ne, 4)) if with_gl else None
        lib().orc_kinetic(self.h, _ptr(ke), _ptr(gl) if gl is not None else None)
        return (ke, gl) if with_gl else ke

    def potential(self, eps: float = 1e-14):
        """Ewald energy of electrons (charge -1) and ions (the system's charges) per walker."""
        s = self.system
        R = self.positions()
        Q = np.concatenate([-np.ones(self.ne), s.ion_charges[s.ion_species]])
        return np.array([ewald_split_energy(s.lattice, np.concatenate([R[iw], s.ion_pos]), Q, eps)[3]
                         for iw in range(self.nw)])

    def local_energy(self, eps: float = 1e-14):
        ke = self.kinetic()
        v = self.potential(eps)
        return ke + v, ke, v
