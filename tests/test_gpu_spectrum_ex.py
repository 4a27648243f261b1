"""General tracer grids and power spectra (NGP/CIC/Sphere/Exp windows,
masses, several types, interlacing, redshift-space shifts, folds, cross
spectra, multipoles) against the FP64 oracle restatement (GPU)."""
import numpy as np
import pytest

from conftest import rel_rms

pytestmark = pytest.mark.gpu


def _tracers(n, L, ntype, seed):
    rng = np.random.default_rng(seed)
    pos = rng.uniform(0.0, L, (n, 3)).astype(np.float32)
    vel = rng.normal(0.0, 300.0, (n, 3)).astype(np.float32)
    mass = rng.lognormal(0.0, 0.5, n).astype(np.float32)
    types = rng.integers(0, ntype, n).astype(np.int32)
    return pos, vel, mass, types


@pytest.mark.parametrize("window,R,interlacing,direction,folds,weighted,ntype", [
    (1, 4.0, 0, -1, 1, True, 2),
    (2, 4.0, 1, 2, 1, True, 2),
    (2, 4.0, 0, 0, 2, False, 1),
    (3, 6.0, 1, -1, 1, True, 1),
    (4, 3.0, 0, 1, 1, False, 3),
])
def test_grid_ex_matches_oracle(window, R, interlacing, direction, folds, weighted, ntype):
    from exshalos_gb300.lib import spectrum
    from oracle import spectrum_f64 as sp
    nd, L, n = 32, 128.0, 4000
    pos, vel, mass, types = _tracers(n, L, ntype, 10 + window)
    m = mass if weighted else None
    t = types if ntype > 1 else None
    g = spectrum.grid_compute(pos, vel, m, int(weighted), t, ntype, nd, L, 0.31, 0.5, direction, window, R, 2.0,
                              interlacing, folds, 0, 1)
    want = sp.tracer_grid(pos.astype(np.float64), nd, L, vel=vel, mass=m, types=t, ntype=ntype, Om0=0.31, z=0.5,
                          direction=direction, window=window, R=R, R_times=2.0, interlacing=interlacing, folds=folds)
    assert g.shape == want.shape
    assert rel_rms(g, want) < 1e-5
    assert np.max(np.abs(g - want)) < 1e-3


@pytest.mark.parametrize("window,interlacing,ntype,l_max,direction", [
    (2, 1, 2, 4, 2),
    (1, 0, 3, 2, 0),
    (3, 0, 1, 0, -1),
    (4, 1, 1, 2, 1),
    (0, 0, 2, 0, -1),
])
def test_power_ex_matches_oracle(window, interlacing, ntype, l_max, direction):
    from exshalos_gb300.lib import spectrum
    from oracle import spectrum_f64 as sp
    nd, L, Nk, R = 32, 128.0, 12, 3.0
    rng = np.random.default_rng(30 + window)
    grid = rng.standard_normal((ntype, interlacing + 1, nd, nd, nd)).astype(np.float32)
    kmin, kmax = np.float32(2 * np.pi / L), np.float32(np.pi / L * nd)
    r = spectrum.power_compute(grid, ntype, nd, np.float32(L), window, np.float32(R), interlacing, Nk, kmin, kmax,
                               l_max, direction, 0, 1)
    want = sp.power(grid.astype(np.float64), L, ntype=ntype, window=window, R=R, interlacing=interlacing, Nk=Nk,
                    kmin=kmin, kmax=kmax, l_max=l_max, direction=direction)
    np.testing.assert_array_equal(r["Nk"], want["Nk"])
    m = want["Nk"] > 0
    assert r["Pk"].shape == want["Pk"].shape
    # multipoles and cross spectra cross zero: errors against each pair's monopole scale
    scale = np.max(np.abs(want["Pk"][:, :1, :]), axis=(1, 2))[:, None, None]
    assert np.max(np.abs(r["Pk"] - want["Pk"])[..., m] / scale) < 1e-4
    assert np.max(np.abs(r["k"][m] / want["k"][m] - 1)) < 1e-6


def test_public_api_types_interlacing_multipoles():
    from exshalos_gb300 import simulation
    nd, L = 32, 128.0
    pos, vel, mass, types = _tracers(5000, L, 2, 3)
    g = simulation.Compute_Density_Grid(pos, vel=vel, mass=mass, types=types + 7, nd=nd, L=L, direction="z",
                                        window="CIC", interlacing=True)
    assert g.shape == (2, 2, nd, nd, nd)
    assert np.all(np.abs(g.reshape(4, -1).mean(axis=1)) < 1e-4)      # every grid is a contrast
    p = simulation.Compute_Power_Spectrum(g, L=L, window="CIC", Nk=10, l_max=2, direction="z", ntypes=2)
    assert p["Pk"].shape == (3, 2, 10)
    assert np.all(np.isfinite(p["Pk"]))
    # the single-type path and the general one agree on one CIC grid
    g1 = simulation.Compute_Density_Grid(pos, nd=nd, L=L, window="CIC")
    a = simulation.Compute_Power_Spectrum(g1, L=L, window="CIC", Nk=10)
    b = simulation.Compute_Power_Spectrum(g1, L=L, window="CIC", Nk=10, l_max=2, direction="x")
    np.testing.assert_array_equal(a["Nk"], b["Nk"])
    assert np.max(np.abs(b["Pk"][0, 0] / a["Pk"] - 1)) < 1e-5
