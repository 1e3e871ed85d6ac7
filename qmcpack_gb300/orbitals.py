"""Orbital input from plane waves: the spline coefficient table of a system from the bands'
plane-wave coefficients, on the GPU (qmcg_spline_from_planewaves; QMCPACK's ESHDF orbital
path, OneSplineOrbData::fft_spline, for real Gamma-point orbitals).  Reading the ESHDF file
itself needs HDF5, which this image lacks: callers pass the arrays they read."""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import check, load

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def spline_from_planewaves(gvecs: np.ndarray, coefs_g: np.ndarray, mesh, precision: int = 8,
                           num_orbitals_padded: int | None = None, with_phases: bool = False):
    """gvecs [num_g][3] int Miller indices, coefs_g [num_orbitals][num_g] complex, mesh (nx, ny, nz).
    Returns the table [nx+3][ny+3][nz+3][num_orbitals_padded] (float32 for precision 4, float64
    for 8) and, with with_phases, the [num_orbitals][2] phase rotations."""
    L = load()
    g = np.ascontiguousarray(gvecs, np.int32)
    cg = np.ascontiguousarray(np.stack([np.real(coefs_g), np.imag(coefs_g)], axis=-1), np.float64)
    norb, ng = cg.shape[0], cg.shape[1]
    assert g.shape == (ng, 3)
    lda = num_orbitals_padded or (norb + 15) // 16 * 16
    m = np.ascontiguousarray(mesh, np.int32)
    out = np.zeros((m[0] + 3, m[1] + 3, m[2] + 3, lda), np.float32 if precision == 4 else np.float64)
    ph = np.zeros((norb, 2))
    check(L.qmcg_spline_from_planewaves(precision, norb, ng, g.ctypes.data_as(_ip), cg.ctypes.data_as(_dp),
                                        m.ctypes.data_as(_ip), lda, out.ctypes.data_as(C.c_void_p),
                                        ph.ctypes.data_as(_dp)))
    return (out, ph) if with_phases else out


def synthetic_planewaves(num_orbitals: int, mesh, gmax: float, seed: int = 0, real_orbitals: bool = False):
    """Seeded synthetic bands: every Miller index G with |G| <= gmax (in grid units of the
    reciprocal lattice), coefficients complex normal damped by exp(-|G|^2 / gmax^2).  With
    real_orbitals the coefficients satisfy c(-G) = conj(c(G)), as real Gamma-point orbitals
    written by a plane-wave code do."""
    rng = np.random.default_rng(seed)
    r = int(np.floor(gmax))
    gv = np.array([(a, b, c) for a in range(-r, r + 1) for b in range(-r, r + 1) for c in range(-r, r + 1)
                   if a * a + b * b + c * c <= gmax * gmax], np.int32)
    damp = np.exp(-(gv ** 2).sum(axis=1) / gmax ** 2)
    cg = (rng.normal(size=(num_orbitals, len(gv))) + 1j * rng.normal(size=(num_orbitals, len(gv)))) * damp
    if real_orbitals:
        index = {tuple(x): i for i, x in enumerate(gv)}
        partner = np.array([index[tuple(-x)] for x in gv])
        cg = 0.5 * (cg + np.conj(cg[:, partner]))
    return gv, cg
