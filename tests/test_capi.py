"""The C-ABI library builds, loads and exports every declared symbol (CPU)."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "exh_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(exh_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    from exshalos_gb300 import _capi
    L = _capi.load()
    syms = declared_symbols()
    assert len(syms) >= 15
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing
    assert set(syms) == set(_capi.SIGNATURES), set(syms) ^ set(_capi.SIGNATURES)


def test_precision_and_strerror():
    from exshalos_gb300 import _capi
    L = _capi.load()
    assert L.exh_check_precision() == 4
    assert L.exh_strerror(_capi.EXH_E_RANGE)


def test_no_device_raises_instead_of_falling_back():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from exshalos_gb300 import _capi
    with pytest.raises(_capi.ExhError):
        _capi.context()


def test_host_output_pool_never_aliases_live_arrays():
    """Large outputs come from a per-thread pool; a buffer returns only after
    every reference to it (views included) is gone."""
    import numpy as np
    from exshalos_gb300 import _capi
    shape = (64, 64, 64)
    a = _capi.host_empty(shape, np.float32)
    b = _capi.host_empty(shape, np.float32)
    assert a.ctypes.data != b.ctypes.data
    pa = a.ctypes.data
    v = a.reshape(-1)
    del a
    c = _capi.host_empty(shape, np.float32)          # a is still alive through v
    assert c.ctypes.data not in (pa, b.ctypes.data)
    del v, c
    d = _capi.host_empty(shape, np.float32)
    assert d.ctypes.data != b.ctypes.data
    small = _capi.host_empty(10, np.float32)
    assert small.shape == (10,) and small.dtype == np.float32
