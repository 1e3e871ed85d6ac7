"""Virtual moves of a non-local pseudopotential evaluation.

For every electron and every ion within the pseudopotential's cutoff radius, the
electron is moved to the quadrature points on the sphere through it around that ion:
r' = R_I + |r - R_I| u_j, u_j the points of the angular rule, randomly rotated at
every evaluation (NonLocalECPComponent::buildQuadraturePointDeltaPositions,
src/QMCHamiltonians/NonLocalECPComponent.cpp:826-832, with the random rotation of
randomize_grid).  The rule here is the 12-point icosahedral one.  The moves of all
walkers form one flat list for qmcg_mw_evaluate_ratios.
"""
from __future__ import annotations

import numpy as np


def icosahedron() -> np.ndarray:
    """The 12 vertices of a regular icosahedron on the unit sphere."""
    phi = (1 + np.sqrt(5.0)) / 2
    v = []
    for s1 in (-1, 1):
        for s2 in (-1, 1):
            v += [(0, s1, s2 * phi), (s1, s2 * phi, 0), (s2 * phi, 0, s1)]
    v = np.array(v, dtype=np.float64)
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def random_rotation(rng: np.random.Generator) -> np.ndarray:
    """A uniformly random proper rotation (QR of a Gaussian matrix, signs fixed)."""
    q, r = np.linalg.qr(rng.normal(size=(3, 3)))
    q = q * np.sign(np.diag(r))
    if np.linalg.det(q) < 0:
        q[:, 0] = -q[:, 0]
    return q


def quadrature_moves(system, R: np.ndarray, rcut: float, rng: np.random.Generator, rule: np.ndarray = None):
    """(walker, electron, pos [n][3], ion) of every virtual move of the walkers R [nw][ne][3]."""
    rule = icosahedron() if rule is None else rule
    L = np.asarray(system.lattice, np.float64)
    ions = np.asarray(system.ion_pos, np.float64)
    R = np.asarray(R, np.float64)
    nw, ne, _ = R.shape
    walkers, elecs, pos, which = [], [], [], []
    for w in range(nw):
        d = ions[None, :, :] - R[w][:, None, :]
        d -= L * np.round(d / L)
        dist = np.linalg.norm(d, axis=-1)
        e_idx, i_idx = np.nonzero(dist < rcut)
        for e, I in zip(e_idx, i_idx):
            rot = random_rotation(rng)
            centre = R[w, e] + d[e, I]
            pts = centre + dist[e, I] * (rule @ rot.T)
            walkers.append(np.full(len(rule), w))
            elecs.append(np.full(len(rule), e))
            pos.append(pts)
            which.append(np.full(len(rule), I))
    if not walkers:
        z = np.zeros(0, np.int32)
        return z, z, np.zeros((0, 3)), z
    return (np.concatenate(walkers).astype(np.int32), np.concatenate(elecs).astype(np.int32),
            np.concatenate(pos), np.concatenate(which).astype(np.int32))
