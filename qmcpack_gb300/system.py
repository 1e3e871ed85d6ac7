"""Seeded synthetic Slater-Jastrow systems for the batched move loop.

A system is what QMCPACK builds from its XML input for the particle-by-particle
loop: an orthorhombic periodic cell, ions, a multi-orbital periodic tricubic
B-spline table of real orbitals (ghost layout of
src/spline2/MultiBsplineBase.hpp:75-130 and src/einspline/bspline_create.c:1032-1034),
one-body (electron-ion) and two-body (electron-electron) B-spline Jastrow
parameters with the cusp values RadialJastrowBuilder assigns
(src/QMCWaveFunctions/Jastrow/RadialJastrowBuilder.cpp:200-207), and walkers.

No public dataset is involved: every array is drawn from
numpy.random.Generator(PCG64(seed)) with the shapes and distributions of the
workloads named below.
"""
from __future__ import annotations

import dataclasses
from typing import Optional

import numpy as np


def padded(n: int, multiple: int = 16) -> int:
    """Orbital padding (elements); 16 keeps rows 64-byte aligned in FP32."""
    return ((n + multiple - 1) // multiple) * multiple


@dataclasses.dataclass
class SystemSpec:
    name: str
    cell: float                 # cubic cell length (bohr)
    n_ions: int
    ion_layout: str             # "uniform" or "jittered:nx,ny,nz"
    n_up: int
    n_dn: int
    grid: int                   # spline grid points per axis (unique, periodic)
    coef_dist: str              # "uniform0.5" (U(-0.5,0.5)) or "normal0.1" (N(0,0.1))
    j1_size: int
    j1_rcut: float
    j2_size: int
    j2_rcut: float
    walkers: int
    delay: int                  # delay rank k (1 = Sherman-Morrison rank-1)
    precision: int              # 8 = FP64 everywhere, 4 = FP32 move loop + FP64 recompute
    tau: float = 0.3
    steps: int = 100
    recompute_every: int = 0    # sweeps between FP64 recomputes (0 = never)


# The workloads of the benchmark plan (seeded synthetic systems).
SPECS = {
    "c0_32e": SystemSpec("c0_32e", 10.0, 8, "uniform", 16, 16, 32, "uniform0.5", 8, 4.0, 8, 5.0,
                         64, 1, 8, tau=0.3, steps=100),
    "c1_384e": SystemSpec("c1_384e", 15.8, 32, "jittered:4,2,4", 192, 192, 48, "normal0.1", 10, 4.0, 10, 5.0,
                          512, 32, 4, tau=0.3, steps=200, recompute_every=100),
    "c2_1536e": SystemSpec("c2_1536e", 25.0, 128, "jittered:8,4,4", 768, 768, 60, "normal0.1", 10, 4.0, 10, 5.0,
                           256, 64, 4, tau=0.3, steps=200, recompute_every=100),
    "c3_768e": SystemSpec("c3_768e", 20.0, 64, "jittered:4,4,4", 384, 384, 40, "normal0.1", 10, 4.0, 10, 5.0,
                          204, 32, 4, tau=0.3, steps=200, recompute_every=100),
}


@dataclasses.dataclass
class System:
    spec: SystemSpec
    lattice: np.ndarray          # (3,) orthorhombic lengths
    ion_pos: np.ndarray          # (n_ions, 3)
    ion_species: np.ndarray      # (n_ions,) int32
    n_ion_species: int
    grid: np.ndarray             # (3,) int32
    norb: int
    npad: int
    coefs: np.ndarray            # ((gx+3),(gy+3),(gz+3), npad) float64 or float32
    j1_params: np.ndarray        # (n_ion_species, j1_size)
    j1_cusp: np.ndarray          # (n_ion_species,)
    j2_params: np.ndarray        # (2, j2_size): same spin, opposite spin
    j2_cusp: np.ndarray          # (2,)
    ion_charges: np.ndarray = None  # (n_ion_species,) valence charge; neutral cell by default

    @property
    def n_elec(self) -> int:
        return self.spec.n_up + self.spec.n_dn


def _ions(spec: SystemSpec, rng: np.random.Generator) -> np.ndarray:
    a = spec.cell
    if spec.ion_layout == "uniform":
        return rng.uniform(0.0, a, size=(spec.n_ions, 3))
    kind, dims = spec.ion_layout.split(":")
    assert kind == "jittered"
    nx, ny, nz = (int(x) for x in dims.split(","))
    assert nx * ny * nz == spec.n_ions
    idx = np.stack(np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij"), -1).reshape(-1, 3)
    spacing = np.array([a / nx, a / ny, a / nz])
    jitter = rng.uniform(-0.1, 0.1, size=(spec.n_ions, 3)) * spacing
    return (idx + 0.5) * spacing + jitter


def ghost_wrap(unique: np.ndarray) -> np.ndarray:
    """Periodic ghost layout: c[0]=c[M], c[M+1]=c[1], c[M+2]=c[2] on every axis.

    ``unique`` holds the M coefficients of each axis in einspline order
    (index m of the unique array is ghost index m+1).
    """
    out = unique
    for ax in range(3):
        m = out.shape[ax]
        last = np.take(out, [m - 1], axis=ax)
        first2 = np.take(out, [0, 1], axis=ax)
        out = np.concatenate([last, out, first2], axis=ax)
    return out


def make_system(spec: SystemSpec | str, seed: int = 2024) -> System:
    if isinstance(spec, str):
        spec = SPECS[spec]
    rng = np.random.Generator(np.random.PCG64(seed))
    ions = _ions(spec, rng)
    norb = spec.n_up
    assert spec.n_up == spec.n_dn, "closed-shell systems: both spins share the orbital set"
    npad = padded(norb)
    g = spec.grid
    dtype = np.float64 if spec.precision == 8 else np.float32
    if spec.coef_dist == "uniform0.5":
        uniq = rng.uniform(-0.5, 0.5, size=(g, g, g, norb))
    else:
        uniq = rng.normal(0.0, 0.1, size=(g, g, g, norb))
    uniq = uniq.astype(dtype)
    if npad > norb:
        uniq = np.concatenate([uniq, np.zeros((g, g, g, npad - norb), dtype)], axis=-1)
    coefs = np.ascontiguousarray(ghost_wrap(uniq))
    j1 = rng.uniform(-0.3, 0.0, size=(1, spec.j1_size))
    j2 = rng.uniform(-0.3, 0.0, size=(2, spec.j2_size))
    return System(spec=spec, lattice=np.full(3, spec.cell), ion_pos=ions,
                  ion_species=np.zeros(spec.n_ions, np.int32), n_ion_species=1,
                  grid=np.full(3, g, np.int32), norb=norb, npad=npad, coefs=coefs,
                  j1_params=j1, j1_cusp=np.zeros(1),
                  j2_params=j2, j2_cusp=np.array([-0.25, -0.5]),
                  ion_charges=np.array([float(spec.n_up + spec.n_dn) / spec.n_ions]))


def make_walkers(system: System, nw: Optional[int] = None, seed: int = 7) -> np.ndarray:
    """Initial walkers, uniform in the cell: (nw, n_elec, 3) float64."""
    nw = system.spec.walkers if nw is None else nw
    rng = np.random.Generator(np.random.PCG64(seed))
    return rng.uniform(0.0, 1.0, size=(nw, system.n_elec, 3)) * system.lattice


def scaled_spec(name: str, **over) -> SystemSpec:
    """A copy of a named spec with fields replaced (used for small parity cases)."""
    return dataclasses.replace(SPECS[name], **over)
