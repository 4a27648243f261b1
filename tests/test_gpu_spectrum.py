"""FFT, CIC and P(k) kernels against the oracle (GPU)."""
import numpy as np
import pytest

from conftest import rel_rms

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("shape", [(32, 32, 32), (48, 48, 48), (64, 64, 64), (96, 96, 96), (16, 24, 36),
                                   (128, 128, 128), (64, 32, 16), (512, 512, 8), (16, 512, 36), (512, 24, 1024),
                                   (256, 256, 256), (512, 512, 512)])
def test_fft_roundtrip_vs_numpy(shape):
    import torch
    from exshalos_gb300 import _capi
    L = _capi.load()
    ctx = _capi.context()
    rng = np.random.default_rng(7)
    x = rng.standard_normal(shape).astype(np.float32)
    xd = _dev(x)
    nc = shape[2] // 2 + 1
    kd = torch.empty((shape[0], shape[1], nc, 2), dtype=torch.float32, device="cuda")
    _capi.check(L.exh_fft_r2c_3d(ctx, *shape, _capi.ptr(xd), _capi.ptr(kd), None))
    torch.cuda.synchronize()
    got = kd.cpu().numpy()
    got = got[..., 0] + 1j * got[..., 1]
    want = np.fft.rfftn(x.astype(np.float64))
    assert rel_rms(np.abs(got - want), np.abs(want)) < 2e-6 or rel_rms(got.real, want.real) < 2e-6
    assert np.sqrt(np.mean(np.abs(got - want) ** 2) / np.mean(np.abs(want) ** 2)) < 1e-6
    back = torch.empty(shape, dtype=torch.float32, device="cuda")
    _capi.check(L.exh_fft_c2r_3d(ctx, *shape, _capi.ptr(kd), _capi.ptr(back), None))
    torch.cuda.synchronize()
    assert rel_rms(back.cpu().numpy() / np.prod(shape), x) < 1e-6


def test_cic_matches_oracle(orc):
    from exshalos_gb300.lib import spectrum
    rng = np.random.default_rng(11)
    nd, L = 64, 256.0
    pos = rng.uniform(-10.0, L + 10.0, (20000, 3)).astype(np.float32)
    pos[:5] = [0.0, L - 1e-4, L / 2]
    g = spectrum.grid_compute(pos, None, None, 0, None, 1, nd, L, 0.31, 0.0, -1, 2, 4.0, 5.0, 0, 1, 0, 1)
    want = orc.cic(pos.astype(np.float64), nd, L)
    assert g.shape == (1, 1, nd, nd, nd)
    assert rel_rms(g[0, 0], want) < 1e-5
    assert np.abs(g[0, 0] - want).max() < 1e-3


@pytest.mark.parametrize("window", [0, 1, 2])
def test_power_matches_oracle(orc, window):
    from exshalos_gb300.lib import spectrum
    rng = np.random.default_rng(12)
    nd, L, Nk = 64, 256.0, 32
    grid = rng.standard_normal((nd, nd, nd)).astype(np.float32)
    kmin, kmax = np.float32(2 * np.pi / L), np.float32(np.pi / L * nd)
    r = spectrum.power_compute(grid, 1, nd, np.float32(L), window, 4.0, 0, Nk, kmin, kmax, 0, -1, 0, 1)
    want = orc.power(grid.astype(np.float64), L, window=window, Nk=Nk, kmin=kmin, kmax=kmax)
    np.testing.assert_array_equal(r["Nk"], want["Nk"])
    m = want["Nk"] > 0
    assert np.abs(r["Pk"][0, 0][m] / want["Pk"][m] - 1).max() < 1e-5
    assert np.abs(r["k"][m] / want["k"][m] - 1).max() < 1e-6


def test_density_grid_matches_oracle(orc, pk):
    from exshalos_gb300 import _capi
    k, P = pk
    nd, Lc, seed = 64, 4.0, 21
    prm = _capi.default_params(ndx=nd, ndy=nd, ndz=nd, Lc=Lc, seed=seed)
    out = np.empty((nd, nd, nd), dtype=np.float32)
    L = _capi.load()
    _capi.check(L.exh_density_grid_compute(_capi.context(), _capi.ptr(k), _capi.ptr(P), k.size, prm,
                                           _capi.ptr(out), _capi.EXH_MEM_HOST, None))
    p = orc.make_params(nd, Lc, seed=seed)
    want = orc.field_real(p, orc.field_modes(p, k, P, stream=0))
    assert rel_rms(out, want) < 1e-5
