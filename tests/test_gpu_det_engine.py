"""The delayed-update flush on caller device buffers (qmcg_mw_update_inv_mat).

Checked against a NumPy FP64 restatement of DelayedUpdate::updateInvMat
(src/QMCWaveFunctions/Fermion/DelayedUpdate.h:145-215):
    Ainv <- Ainv - (Ainv U^T - E) (Binv V),  E[delay_list[c], c] = 1, slots with -1 skipped.
Tolerance: 1e-12 relative to the largest element in FP64, 2e-5 in FP32.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def flush_case(nw, n, lda, k, dc, seed):
    rng = np.random.default_rng(seed)
    A = np.zeros((nw, n, lda))
    A[:, :, :n] = rng.normal(size=(nw, n, n))
    U = np.zeros((nw, k, lda))
    U[:, :, :n] = rng.normal(size=(nw, k, n))
    V = np.zeros((nw, k, lda))
    V[:, :, :n] = rng.normal(size=(nw, k, n))
    B = rng.normal(size=(nw, k, k)) * 0.3
    dl = np.full((nw, k), -1, np.int32)
    for w in range(nw):
        rows = rng.choice(n, size=dc, replace=False)
        mask = rng.random(dc) < 0.8
        dl[w, :dc] = np.where(mask, rows, -1)
    return A, U, V, B, dl


def flush_reference(A, U, V, B, dl, dc):
    out = A.copy()
    nw, n, lda = A.shape
    for w in range(nw):
        a = A[w, :, :n]
        T1 = a @ U[w, :dc, :n].T
        for c in range(dc):
            if dl[w, c] >= 0:
                T1[dl[w, c], c] -= 1.0
        W = B[w, :dc, :dc] @ V[w, :dc, :n]
        out[w, :, :n] = a - T1 @ W
    return out


def call_flush(fn_name, prec, arrays, dc, stream=None):
    import torch
    from qmcpack_gb300 import _lib
    L = _lib.load()
    A, U, V, B, dl = arrays
    nw, n, lda = A.shape
    k = U.shape[1]
    dt = torch.float64 if prec == 8 else torch.float32
    tA, tU, tV, tB = (torch.tensor(x, dtype=dt, device="cuda") for x in (A, U, V, B))
    tD = torch.tensor(dl, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    fn = getattr(L, fn_name)
    rc = fn(prec, nw, n, lda, k, dc, C.c_void_p(tA.data_ptr()), C.c_void_p(tU.data_ptr()),
            C.c_void_p(tV.data_ptr()), C.c_void_p(tB.data_ptr()), C.c_void_p(tD.data_ptr()), None)
    torch.cuda.synchronize()
    return rc, tA.double().cpu().numpy()


@pytest.mark.parametrize("prec,tol", [(8, 1e-12), (4, 2e-5)])
@pytest.mark.parametrize("nw,n,lda,k,dc", [(3, 20, 32, 4, 4), (5, 50, 64, 8, 5), (2, 192, 192, 32, 32)])
def test_update_inv_mat_matches_restatement(prec, tol, nw, n, lda, k, dc):
    arrays = flush_case(nw, n, lda, k, dc, seed=n + dc)
    rc, got = call_flush("qmcg_mw_update_inv_mat", prec, arrays, dc)
    assert rc == 0
    ref = flush_reference(*arrays, dc)
    err = np.max(np.abs(got[:, :, :n] - ref[:, :, :n])) / np.max(np.abs(ref))
    assert err < tol, err


def test_update_inv_mat_rejects_bad_sizes():
    from qmcpack_gb300 import _lib
    L = _lib.load()
    rc = L.qmcg_mw_update_inv_mat(8, 1, 10, 5, 4, 2, None, None, None, None, None, None)
    assert rc == -1
    assert b"lda" in L.qmcg_last_error()
