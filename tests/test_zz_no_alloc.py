"""The allocation-free delayed-update flush (qmcg_mw_update_inv_mat_noalloc).

It serves callers that cannot allocate device memory themselves or through a
stream-ordered pool (their device memory belongs to another allocator, or they
cannot take the synchronisation that freeing implies).  Shapes whose tiles fit in
shared memory need no scratch; the others use a fixed 16 MiB device array instead.
Per precision, three calls in a row: a large batch on the scratch path with every
delay slot used, then a smaller one on the scratch path with fewer slots used than
the delay rank (so stale scratch from the first call would show), then a shape
that needs no scratch.  Each must give the same result as the allocating entry
point qmcg_mw_update_inv_mat on the same inputs, within the tolerances of
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


# (num_walkers, n, lda, delay_rank, delay_count): scratch path with dc = k, scratch path with
# dc < k, then a shape whose shared-memory tiles fit (no scratch)
CASES = {
    8: [(256, 192, 192, 32, 32), (64, 192, 208, 32, 20), (4, 40, 48, 8, 6)],
    4: [(80, 768, 768, 64, 64), (16, 768, 784, 64, 40), (512, 192, 192, 32, 32)],
}


@pytest.mark.parametrize("prec,tol", [(8, 1e-12), (4, 2e-5)])
def test_noalloc_flush_matches_allocating_flush(prec, tol):
    import torch
    from qmcpack_gb300 import _lib
    L = _lib.load()
    results = []
    for i, shape in enumerate(CASES[prec]):
        arrays = _case(*shape, seed=i + 1)
        dev = _device(arrays, prec)
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        rc = _call(L, "qmcg_mw_update_inv_mat_noalloc", prec, dev, shape[4])
        torch.cuda.synchronize()
        assert rc == 0, L.qmcg_last_error()
        if i == 1:
            assert torch.cuda.mem_get_info()[0] == free_before
        results.append((arrays, dev[0].double().cpu().numpy(), shape))
        del dev
    # the allocating entry point on the same inputs, after the allocation-free calls
    for arrays, got, shape in results:
        dev = _device(arrays, prec)
        rc = _call(L, "qmcg_mw_update_inv_mat", prec, dev, shape[4])
        torch.cuda.synchronize()
        assert rc == 0, L.qmcg_last_error()
        ref = dev[0].double().cpu().numpy()
        n = shape[1]
        err = np.max(np.abs(got[:, :, :n] - ref[:, :, :n])) / np.max(np.abs(ref[:, :, :n]))
        assert err <= tol, (shape, err)
        del dev


def test_noalloc_flush_rejects_oversized_batches():
    from qmcpack_gb300 import _lib
    L = _lib.load()
    # 1024 walkers x k=64 x lda=768 x 4 B = 192 MiB > 16 MiB
    rc = L.qmcg_mw_update_inv_mat_noalloc(4, 1024, 768, 768, 64, 64, None, None, None, None, None, None)
    assert rc == -1
    msg = L.qmcg_last_error().decode()
    assert "exceeds" in msg and "16777216" in msg
