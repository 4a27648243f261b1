"""The allocation-free power spectrum (GPU).

exh_power_compute_noalloc serves callers that cannot allocate device memory
(real-time loops that must not stall in the allocator, hosts whose device
memory belongs to a pool they do not own).  Its temporaries live in
one static device array shared by every call.  This test calls it through
the C ABI twice in a row, with different sizes so that the second call runs
on what the first left behind, and checks both results against
exh_power_compute.  The file sorts last so that a run stopping at the first
failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _reference(L_, grid, nd, L, window, Nk, kmin, kmax):
    from exshalos_gb300 import _capi
    k = np.zeros(Nk, dtype=np.float32)
    P = np.zeros(Nk, dtype=np.float32)
    n = np.zeros(Nk, dtype=np.int64)
    _capi.check(L_.exh_power_compute(_capi.context(), _capi.ptr(grid), nd, C.c_float(L), window, Nk, C.c_float(kmin),
                                     C.c_float(kmax), _capi.ptr(k), _capi.ptr(P), _capi.ptr(n), _capi.EXH_MEM_HOST,
                                     None))
    return k, P, n


def _noalloc(L_, grid, nd, L, window, Nk, kmin, kmax):
    import torch
    from exshalos_gb300 import _capi
    g = torch.from_numpy(grid).cuda()
    k = torch.empty(Nk, dtype=torch.float32, device="cuda")
    P = torch.empty(Nk, dtype=torch.float32, device="cuda")
    n = torch.empty(Nk, dtype=torch.int64, device="cuda")
    _capi.check(L_.exh_power_compute_noalloc(_capi.ptr(g), nd, C.c_float(L), window, Nk, C.c_float(kmin),
                                             C.c_float(kmax), _capi.ptr(k), _capi.ptr(P), _capi.ptr(n), None))
    torch.cuda.synchronize()
    return k.cpu().numpy(), P.cpu().numpy(), n.cpu().numpy()


def test_noalloc_power_matches_allocating_entry_point():
    from exshalos_gb300 import _capi
    L_ = _capi.load()
    rng = np.random.default_rng(2024)
    cases = [(64, 256.0, 2, 32), (48, 96.0, 0, 20)]
    for nd, L, window, Nk in cases:
        grid = rng.standard_normal((nd, nd, nd)).astype(np.float32)
        kmin, kmax = np.float32(2 * np.pi / L), np.float32(np.pi / L * nd)
        k0, P0, n0 = _reference(L_, grid, nd, L, window, Nk, kmin, kmax)
        k1, P1, n1 = _noalloc(L_, grid, nd, L, window, Nk, kmin, kmax)
        np.testing.assert_array_equal(n1, n0)
        m = n0 > 0
        np.testing.assert_allclose(P1[m], P0[m], rtol=1e-6)
        np.testing.assert_allclose(k1[m], k0[m], rtol=1e-6)


def test_noalloc_rejects_sizes_beyond_its_limit():
    import torch
    from exshalos_gb300 import _capi
    L_ = _capi.load()
    g = torch.zeros(96 ** 3, dtype=torch.float32, device="cuda")
    out = torch.zeros(300, dtype=torch.float32, device="cuda")
    cnt = torch.zeros(300, dtype=torch.int64, device="cuda")
    st = L_.exh_power_compute_noalloc(_capi.ptr(g), 96, C.c_float(100.0), 2, 16, C.c_float(0.1), C.c_float(1.0),
                                      _capi.ptr(out), _capi.ptr(out), _capi.ptr(cnt), None)
    assert st == _capi.EXH_E_INVALID
    st = L_.exh_power_compute_noalloc(_capi.ptr(g), 32, C.c_float(100.0), 2, 300, C.c_float(0.1), C.c_float(1.0),
                                      _capi.ptr(out), _capi.ptr(out), _capi.ptr(cnt), None)
    assert st == _capi.EXH_E_INVALID
    # windows beyond CIC are not built, as in the allocating entry point
    st = L_.exh_power_compute_noalloc(_capi.ptr(g), 32, C.c_float(100.0), 3, 16, C.c_float(0.1), C.c_float(1.0),
                                      _capi.ptr(out), _capi.ptr(out), _capi.ptr(cnt), None)
    assert st == _capi.EXH_E_UNSUPPORTED
    # kernel-class timing would create CUDA events: refused while it is on
    _capi.timing_enable(True)
    try:
        st = L_.exh_power_compute_noalloc(_capi.ptr(g), 32, C.c_float(100.0), 2, 16, C.c_float(0.1),
                                          C.c_float(1.0), _capi.ptr(out), _capi.ptr(out), _capi.ptr(cnt), None)
    finally:
        _capi.timing_enable(False)
    assert st == _capi.EXH_E_UNSUPPORTED
