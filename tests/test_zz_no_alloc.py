"""The allocation-free delayed-update flush (qmcg_mw_update_inv_mat_noalloc).

It serves callers that cannot allocate device memory themselves or through a
stream-ordered pool (their device memory belongs to another allocator, or they
cannot take the synchronisation that freeing implies); its scratch is a fixed
16 MiB device array instead.  Two calls in a row, with different data and sizes,
must each give the same result as the allocating entry point
qmcg_mw_update_inv_mat on the same inputs, within the tolerances of
tests/test_gpu_det_engine.py (1e-12 FP64, 2e-5 FP32, relative to the largest
element), and the second call must not change the free device memory.
This file is collected last so that a run stopping at the first failure has
already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _case(nw, n, lda, k, dc, seed):
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
        dl[w, :dc] = np.where(rng.random(dc) < 0.8, rng.choice(n, size=dc, replace=False), -1)
    return A, U, V, B, dl


def _device(arrays, prec):
    import torch
    dt = torch.float64 if prec == 8 else torch.float32
    A, U, V, B, dl = arrays
    out = [torch.tensor(x, dtype=dt, device="cuda") for x in (A, U, V, B)]
    out.append(torch.tensor(dl, dtype=torch.int32, device="cuda"))
    return out


def _call(L, name, prec, dev, dc):
    tA, tU, tV, tB, tD = dev
    nw, n, lda = tA.shape
    k = tU.shape[1]
    return getattr(L, name)(prec, nw, n, lda, k, dc, C.c_void_p(tA.data_ptr()), C.c_void_p(tU.data_ptr()),
                            C.c_void_p(tV.data_ptr()), C.c_void_p(tB.data_ptr()), C.c_void_p(tD.data_ptr()), None)


@pytest.mark.parametrize("prec,tol", [(8, 1e-12), (4, 2e-5)])
def test_noalloc_flush_matches_allocating_flush_twice(prec, tol):
    import torch
    from qmcpack_gb300 import _lib
    L = _lib.load()
    # second case: the production shape (384 electrons, delay rank 32); 12.6 MB of scratch either way
    cases = [((4, 40, 48, 8, 6), 1), ((512 if prec == 4 else 256, 192, 192, 32, 32), 2)]
    results = []
    free_before_second = None
    for i, (shape, seed) in enumerate(cases):
        arrays = _case(*shape, seed=seed)
        dev = _device(arrays, prec)
        torch.cuda.synchronize()
        if i == 1:
            free_before_second = torch.cuda.mem_get_info()[0]
        rc = _call(L, "qmcg_mw_update_inv_mat_noalloc", prec, dev, shape[4])
        torch.cuda.synchronize()
        assert rc == 0, L.qmcg_last_error()
        if i == 1:
            assert torch.cuda.mem_get_info()[0] == free_before_second
        results.append((arrays, dev[0].double().cpu().numpy(), shape))
    # the allocating entry point on the same inputs, after the allocation-free calls
    for arrays, got, shape in results:
        dev = _device(arrays, prec)
        rc = _call(L, "qmcg_mw_update_inv_mat", prec, dev, shape[4])
        torch.cuda.synchronize()
        assert rc == 0, L.qmcg_last_error()
        ref = dev[0].double().cpu().numpy()
        n = shape[1]
        err = np.max(np.abs(got[:, :, :n] - ref[:, :, :n])) / np.max(np.abs(ref[:, :, :n]))
        assert err <= tol, err


def test_noalloc_flush_rejects_oversized_batches():
    from qmcpack_gb300 import _lib
    L = _lib.load()
    # 1024 walkers x k=64 x lda=768 x 4 B = 192 MiB > 16 MiB
    rc = L.qmcg_mw_update_inv_mat_noalloc(4, 1024, 768, 768, 64, 64, None, None, None, None, None, None)
    assert rc == -1
    msg = L.qmcg_last_error().decode()
    assert "exceeds" in msg and "16777216" in msg
