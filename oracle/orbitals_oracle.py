"""CPU restatement of QMCPACK's plane-wave orbital input for real Gamma-point orbitals —
test infrastructure only: the checker of qmcg_spline_from_planewaves.

Per band (OneSplineOrbData::fft_spline, src/QMCWaveFunctions/BsplineFactory/OneSplineOrbData.cpp:62-95):
  unpack4fftw            src/QMCWaveFunctions/BsplineFactory/einspline_helper.hpp:34-59
  backward 3-D FFT       the FFTW plan of OneSplineOrbData.cpp:30-31 (sign +1, unnormalized)
  fix_phase_rotate_c2r   einspline_helper.hpp:70-127, twist 0
  einspline::set         set_multi_UBspline_3d_d, src/einspline/multi_bspline_create.c:1186-1240,
                         find_coefs_1d_d and solve_periodic_interp_1d_d,
                         src/einspline/bspline_create.c:991-1043 and 1095-1118
"""
from __future__ import annotations

import numpy as np


def unpack(gvecs: np.ndarray, cg: np.ndarray, mesh) -> np.ndarray:
    """unpack4fftw: [norb][nx][ny][nz] complex box, c_G at (G + n) mod n for G inside the mesh's
    [lower, upper] bounds per axis (einspline_helper.hpp:39-58)."""
    n = np.asarray(mesh)
    up = (n - 1) // 2
    lo = up - n + 1
    inside = np.all((gvecs <= up) & (gvecs >= lo), axis=1)
    idx = (gvecs[inside] + n) % n
    box = np.zeros((cg.shape[0],) + tuple(n), np.complex128)
    box[:, idx[:, 0], idx[:, 1], idx[:, 2]] = cg[:, inside]
    return box


def backward_transform(box: np.ndarray) -> np.ndarray:
    """psi(r) = sum_G c_G exp(+2 pi i G.r / n): numpy's ifftn times the point count."""
    npts = box.shape[1] * box.shape[2] * box.shape[3]
    return np.fft.ifftn(box, axes=(1, 2, 3)) * npts


def phase_rotate(psi: np.ndarray):
    """fix_phase_rotate_c2r at twist 0 (einspline_helper.hpp:81-126): per band the phase from
    the sums of Re^2, Im^2 and Re Im; returns (real orbitals, [norb][2] phases)."""
    re, im = psi.real, psi.imag
    rn = (re * re).sum(axis=(1, 2, 3))
    inn = (im * im).sum(axis=(1, 2, 3))
    ri = (re * im).sum(axis=(1, 2, 3))
    with np.errstate(divide="ignore", invalid="ignore"):
        x = (rn - inn) / ri
    y = 1.0 / np.sqrt(x * x + 4.0)
    phs = np.sqrt(0.5 - y)
    pi = np.where(x < 0, np.sqrt(1.0 - phs * phs), -np.sqrt(1.0 - phs * phs))
    out = phs[:, None, None, None] * re - pi[:, None, None, None] * im
    return out, np.stack([phs, pi], axis=1)


def periodic_coefs(data: np.ndarray, axis: int) -> np.ndarray:
    """find_coefs_1d_d with periodic boundaries along `axis` for every line at once: the bands
    (1/6, 2/3, 1/6 | data) through solve_periodic_interp_1d_d (bspline_create.c:991-1043), step
    for step; M points in, M + 3 coefficients out with c[0] = c[M], c[M+1] = c[1], c[M+2] = c[2]."""
    d = np.moveaxis(np.asarray(data, np.float64), axis, 0)
    M = d.shape[0]
    b0 = np.full(M, 1.0 / 6.0)
    b1 = np.full(M, 2.0 / 3.0)
    b2 = np.full(M, 1.0 / 6.0)
    lc = np.zeros(M)
    b3 = [d[i].copy() for i in range(M)]
    b2[0] /= b1[0]
    b0[0] /= b1[0]
    b3[0] = b3[0] / b1[0]
    b1[0] = 1.0
    b1[M - 1] -= b2[M - 1] * b0[0]
    b3[M - 1] = b3[M - 1] - b2[M - 1] * b3[0]
    b2[M - 1] = -b2[M - 1] * b2[0]
    lc[0] = b0[0]
    for row in range(1, M - 1):
        b1[row] -= b0[row] * b2[row - 1]
        b3[row] = b3[row] - b0[row] * b3[row - 1]
        lc[row] = -b0[row] * lc[row - 1]
        b0[row] = 0.0
        b2[row] /= b1[row]
        b3[row] = b3[row] / b1[row]
        lc[row] /= b1[row]
        b1[row] = 1.0
        if row < M - 2:
            b3[M - 1] = b3[M - 1] - b2[M - 1] * b3[row]
            b1[M - 1] -= b2[M - 1] * lc[row]
            b2[M - 1] = -b2[M - 1] * b2[row]
    b0[M - 1] += b2[M - 1]
    b1[M - 1] -= b0[M - 1] * (b2[M - 2] + lc[M - 2])
    b3[M - 1] = b3[M - 1] - b0[M - 1] * b3[M - 2]
    b3[M - 1] = b3[M - 1] / b1[M - 1]
    c = np.empty((M + 3,) + d.shape[1:])
    c[M] = b3[M - 1]
    for row in range(M - 2, -1, -1):
        c[row + 1] = b3[row] - b2[row] * c[row + 2] - lc[row] * c[M]
    c[0] = c[M]
    c[M + 1] = c[1]
    c[M + 2] = c[2]
    return np.moveaxis(c, 0, axis)


def spline_coefs_3d(data: np.ndarray) -> np.ndarray:
    """set_multi_UBspline_3d_d for every band: [norb][nx][ny][nz] -> [norb][nx+3][ny+3][nz+3],
    the periodic solves along x, then y, then z."""
    c = periodic_coefs(data, 1)
    c = periodic_coefs(c, 2)
    return periodic_coefs(c, 3)


def spline_from_planewaves(gvecs, cg, mesh, num_orbitals_padded: int):
    """The whole path: the coefficient table [nx+3][ny+3][nz+3][num_orbitals_padded] (FP64) and
    the phases."""
    psi = backward_transform(unpack(np.asarray(gvecs), np.asarray(cg), mesh))
    real, phases = phase_rotate(psi)
    c = spline_coefs_3d(real)
    out = np.zeros(c.shape[1:] + (num_orbitals_padded,))
    out[..., : c.shape[0]] = np.moveaxis(c, 0, -1)
    return out, phases, real


def values_at_grid_points(table: np.ndarray, norb: int) -> np.ndarray:
    """The spline's values at the grid points (weights 1/6, 2/3, 1/6 of the three coefficients
    around each point along every axis): [norb][nx][ny][nz]; equals the interpolated data."""
    w = (1.0 / 6.0, 2.0 / 3.0, 1.0 / 6.0)
    nx, ny, nz = table.shape[0] - 3, table.shape[1] - 3, table.shape[2] - 3
    v = np.zeros((nx, ny, nz, norb))
    for a in range(3):
        for b in range(3):
            for c in range(3):
                v += w[a] * w[b] * w[c] * table[a:a + nx, b:b + ny, c:c + nz, :norb]
    return np.moveaxis(v, -1, 0)
