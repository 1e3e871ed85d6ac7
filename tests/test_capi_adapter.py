"""A compiled C++ caller of the C ABI: tests/capi/adapter_crowd.cpp includes
include/qmcg.h, links libqmcg.so and drives a crowd through the adapter a QMCPACK
maintainer adds (the mw_ call sequence electron by electron, mw_evaluateGL, then
one device-resident sweep).  The CPU test checks that it compiles and links; the
GPU test runs it and compares every output with the oracle driven the same way.
"""
import os
import subprocess

import numpy as np
import pytest

from qmcpack_gb300.system import make_system, make_walkers, scaled_spec

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "capi", "adapter_crowd.cpp")


def compile_adapter(out_dir):
    from qmcpack_gb300 import build
    lib = build.build()
    exe = os.path.join(str(out_dir), "adapter_crowd")
    libdir = os.path.dirname(lib)
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), SRC,
                           "-o", exe, "-L", libdir, "-lqmcg", f"-Wl,-rpath,{libdir}"])
    return exe


def test_adapter_compiles_and_links(tmp_path):
    exe = compile_adapter(tmp_path)
    assert os.access(exe, os.X_OK)


def write_input(path, s, nw, k, R, displ, acc, tau):
    hdr = np.array([s.spec.precision, s.spec.n_up, s.spec.n_dn, s.norb, s.npad, len(s.ion_pos), *s.grid,
                    s.j1_params.shape[1], s.j2_params.shape[1], nw, k, displ.shape[0]], np.int32)
    with open(path, "wb") as f:
        f.write(hdr.tobytes())
        f.write(np.array([*s.lattice, s.spec.j1_rcut, s.spec.j2_rcut, tau], np.float64).tobytes())
        for a in (s.ion_pos, s.j1_params[0], s.j1_cusp[:1], s.j2_params, s.j2_cusp, s.coefs, R, displ):
            f.write(np.ascontiguousarray(a, np.float64).tobytes())
        f.write(np.ascontiguousarray(acc, np.int32).tobytes())


@pytest.mark.gpu
@pytest.mark.parametrize("delay", [1, 3])
def test_adapter_against_oracle(tmp_path, delay):
    from oracle import oracle as orc
    spec = scaled_spec("c0_32e", n_up=8, n_dn=8, grid=12, walkers=5, delay=delay, precision=8)
    s = make_system(spec, seed=13)
    nw, ne, nsw, tau = 5, s.n_elec, 2, 0.3
    R = make_walkers(s, nw, seed=14)
    rng = np.random.default_rng(15)
    displ = rng.normal(size=(nsw, ne, nw, 3)) * 0.4
    acc = rng.integers(0, 2, size=(nsw, ne, nw))
    exe = compile_adapter(tmp_path)
    inp, outp = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    write_input(inp, s, nw, delay, R, displ, acc, tau)
    subprocess.check_call([exe, inp, outp], timeout=300)
    out = np.fromfile(outp, np.float64)
    pos = 0

    def take(n, shape):
        nonlocal pos
        v = out[pos:pos + n].reshape(shape)
        pos += n
        return v

    o = orc.Crowd(s, nw, delay, 8)
    o.load_walkers(R)
    lo, _ = o.evaluate_log()
    np.testing.assert_allclose(take(nw, (nw,)), lo, rtol=1e-10)
    for sw in range(nsw):
        for iat in range(ne):
            gn = o.eval_grad(iat)
            o.make_move(iat, displ[sw, iat])
            r, g = o.ratio_grad(iat)
            o.accept_reject(iat, acc[sw, iat])
            np.testing.assert_allclose(take(nw * 3, (nw, 3)), gn, rtol=1e-10, atol=1e-10)
            np.testing.assert_allclose(take(nw, (nw,)), r, rtol=1e-10, atol=1e-12)
            np.testing.assert_allclose(take(nw * 3, (nw, 3)), g, rtol=1e-10, atol=1e-10)
        o.complete_updates()
    lg = take(nw, (nw,))
    G = take(nw * ne * 3, (nw, ne, 3))
    L = take(nw * ne, (nw, ne))
    P = take(nw * ne * 3, (nw, ne, 3))
    lo, _, _ = o.get_log()
    _, gl = o.kinetic(with_gl=True)
    np.testing.assert_allclose(lg, lo, rtol=1e-10)
    np.testing.assert_allclose(G, gl[..., 0:3], rtol=1e-9, atol=1e-10)
    np.testing.assert_allclose(L, gl[..., 3], rtol=1e-9, atol=1e-10)
    np.testing.assert_allclose(P, o.positions(), rtol=0, atol=1e-13)
    counts = take(2, (2,))
    assert counts.sum() == nw * ne and counts[0] > 0
    acc2, rej2, dpos, dlog = take(4, (4,))
    assert acc2 + rej2 == nw * ne and dpos == 0 and dlog == 0
    assert pos == out.size
