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
