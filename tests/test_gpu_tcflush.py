"""The delayed-update flush on tcgen05 tensor cores (qmcg_mw_update_inv_mat_ex).

Checked against the NumPy FP64 restatement of DelayedUpdate::updateInvMat
(src/QMCWaveFunctions/Fermion/DelayedUpdate.h:145-215) used in
tests/test_gpu_det_engine.py.  Tolerances (max error over the largest element):
3xTF32 1e-5, TF32 5e-3 (TF32 keeps 10 mantissa bits, unit roundoff 2^-11).  The C2 shape
(n = 768, k = 64) reports both errors against FP64.
"""
import numpy as np
import pytest

from tests.test_gpu_det_engine import call_flush, flush_case, flush_reference

pytestmark = pytest.mark.gpu


def call_ex(method, arrays, dc):
    import ctypes as C
    import torch
    from qmcpack_gb300 import _lib
    L = _lib.load()
    A, U, V, B, dl = arrays
    nw, n, lda = A.shape
    k = U.shape[1]
    tA, tU, tV, tB = (torch.tensor(x, dtype=torch.float32, device="cuda") for x in (A, U, V, B))
    tD = torch.tensor(dl, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    rc = L.qmcg_mw_update_inv_mat_ex(4, nw, n, lda, k, dc, C.c_void_p(tA.data_ptr()), C.c_void_p(tU.data_ptr()),
                                     C.c_void_p(tV.data_ptr()), C.c_void_p(tB.data_ptr()),
                                     C.c_void_p(tD.data_ptr()), method, None)
    torch.cuda.synchronize()
    return rc, tA.double().cpu().numpy(), L


@pytest.mark.parametrize("method,tol", [(3, 1e-5), (1, 5e-3)])
@pytest.mark.parametrize("nw,n,lda,k,dc", [(3, 20, 32, 4, 4), (2, 64, 64, 16, 9), (4, 192, 192, 32, 32),
                                           (2, 200, 208, 32, 17), (2, 256, 256, 32, 5), (3, 96, 100, 8, 8),
                                           # N-tiled kernel: k > 32 or n_pad > 256 (one MMA's largest N)
                                           (3, 192, 192, 64, 37), (2, 300, 304, 48, 41), (2, 520, 528, 16, 9),
                                           (2, 384, 384, 32, 32),
                                           (2, 768, 768, 64, 64)])
def test_tensor_core_flush(method, tol, nw, n, lda, k, dc):
    arrays = flush_case(nw, n, lda, k, dc, seed=7 * n + dc)
    rc, got, L = call_ex(method, arrays, dc)
    assert rc == 0, L.qmcg_last_error()
    ref = flush_reference(*arrays, dc)
    err = np.max(np.abs(got[:, :, :n] - ref[:, :, :n])) / np.max(np.abs(ref[:, :, :n]))
    print(f"tcgen05 flush method {method} n={n} k={k}: max error {err:.2e}")
    assert err < tol, err


def test_tensor_core_flush_rejects_fp64():
    from qmcpack_gb300 import _lib
    L = _lib.load()
    assert L.qmcg_mw_update_inv_mat_ex(8, 1, 16, 16, 4, 2, None, None, None, None, None, 3, None) == -1


def test_tensor_core_flush_rejects_misaligned_buffers():
    """Rows are moved as 16-byte vectors: a base off a 16-byte boundary is an argument error."""
    import ctypes as C
    import torch
    from qmcpack_gb300 import _lib
    L = _lib.load()
    A, U, V, B, dl = flush_case(1, 16, 16, 4, 4, seed=1)
    tA, tU, tV, tB = (torch.tensor(x, dtype=torch.float32, device="cuda") for x in (A, U, V, B))
    tD = torch.tensor(dl, dtype=torch.int32, device="cuda")
    before = tA.clone()
    rc = L.qmcg_mw_update_inv_mat_ex(4, 1, 12, 16, 4, 4, C.c_void_p(tA.data_ptr() + 4), C.c_void_p(tU.data_ptr()),
                                     C.c_void_p(tV.data_ptr()), C.c_void_p(tB.data_ptr()),
                                     C.c_void_p(tD.data_ptr()), 3, None)
    assert rc == -1 and b"16-byte" in L.qmcg_last_error()
    assert torch.equal(before, tA)


def test_fullsize_sweeps_with_tensor_core_flush():
    from qmcpack_gb300.crowd import Crowd, DeviceSystem
    from qmcpack_gb300.system import make_system, make_walkers
    s = make_system("c1_384e")
    g = Crowd(DeviceSystem(s), 512, 32)
    g.load_walkers(make_walkers(s, 512, seed=31))
    g.mw_evaluateLog()
    acc, rej, _ = g.vmc_sweeps(2, 0.3, 4, rng_mode=1, flush=3)
    tracked, _, _ = g.get_log()
    fresh, _ = g.mw_evaluateLog()
    dl = np.abs(tracked - fresh)
    print("tensor-core flush, full size: median", np.median(dl), "max", dl.max(), "repaired", g.last_repaired)
    assert 0.05 < acc / (acc + rej) < 0.95
    assert np.median(dl) < 1e-3
    assert (dl < 1e-3 * np.abs(fresh)).all()
