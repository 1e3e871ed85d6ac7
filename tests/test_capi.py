"""The C ABI library loads and exports every symbol include/qmcg.h declares (no GPU needed)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    text = open(os.path.join(ROOT, "include", "qmcg.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(qmcg_[a-z_0-9]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from qmcpack_gb300 import build
    path = build.build()
    return ctypes.CDLL(path)


def test_exports_every_declared_symbol(lib):
    syms = header_symbols()
    assert len(syms) >= 20
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_binding_lists_every_symbol():
    from qmcpack_gb300._lib import EXPORTS
    assert sorted(EXPORTS) == header_symbols()


def test_no_device_error_path(lib):
    """Without a GPU the library reports QMCG_ERR_NO_DEVICE instead of crashing."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib.qmcg_last_error.restype = ctypes.c_char_p
    n = ctypes.c_int(-1)
    rc = lib.qmcg_device_count(ctypes.byref(n))
    assert rc == -7 and n.value == 0
    assert b"device" in lib.qmcg_last_error()


def test_missing_library_fails_loudly(tmp_path, monkeypatch):
    from qmcpack_gb300 import _lib
    monkeypatch.setattr(_lib, "_LIB", None)
    with pytest.raises(ImportError):
        _lib.load(str(tmp_path / "libqmcg.so"))
