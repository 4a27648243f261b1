"""Halo finder and the halo pipeline against the oracle (GPU).

The catalogue (centre cells, member counts, masses, order and the per-cell
flags) must be bit-identical to the oracle's Find_Halos run on the same float
grid with the same sigma/barrier/mass-function tables."""
import numpy as np
import pytest

from conftest import rel_rms

pytestmark = pytest.mark.gpu


def _field(nd, Lc, seed, pk):
    # the cases below were chosen on Philox fields (the reference's stream has
    # its own tests, test_gpu_taus_field.py)
    from exshalos_gb300.lib import exshalos
    k, P = pk
    return exshalos.density_grid_compute(k, P, 1e5, nd, nd, nd, Lc, 0, seed, 0, 0.0, 1e5, 0, 1,
                                         field_stream="philox")["grid"]


def _compare(orc, delta, pk, Lc, Om0=0.31, z=0.0, dc=-1.0, Nmin=1, a=1.0, beta=0.0, alpha=0.0, fp64=0):
    from exshalos_gb300.lib import exshalos
    k, P = pk
    got = exshalos.find_halos(delta, k, P, Lc, Om0, z, dc, Nmin, a, beta, alpha, 1, 0, 0, _catalogue=True,
                              setup_fp64=fp64)
    tab = exshalos.halo_tables()
    nd = delta.shape
    p = orc.make_params(nd, Lc, Om0=Om0, z=z, dc=dc, Nmin=Nmin, a=a, beta=beta, alpha=alpha, seed=12345)
    otab = orc.sigma_tables(p, k, P, prec64=fp64)
    # the product's set-up tables are the oracle's, bit for bit
    np.testing.assert_array_equal(tab["Sig_grid"], otab["Sig_grid"])
    np.testing.assert_array_equal(tab["Btab"], otab["Btab"])
    np.testing.assert_array_equal(tab["M"], otab["M"])
    np.testing.assert_array_equal(tab["Int"], otab["Int"])
    want = orc.find_halos(p, delta, tab)
    assert got["Mh"].size == want["nh"]
    np.testing.assert_array_equal(got["x"], want["x"])
    np.testing.assert_array_equal(got["count"], want["count"])
    np.testing.assert_array_equal(got["Mh"].view(np.uint32), want["Mh"].view(np.uint32))
    np.testing.assert_array_equal(got["flag"].reshape(-1), want["flag"])
    Lc32 = np.float32(Lc)
    np.testing.assert_array_equal(got["posh"], (Lc32 * (want["x"] + 0.5)).astype(np.float32))
    return got, want


@pytest.mark.parametrize("nd,Lc,seed", [(32, 4.0, 1), (64, 4.0, 2), (48, 2.0, 3), (96, 3.0, 4), (64, 2.0, 11),
                                        (64, 2.0, 12), (64, 2.0, 13), (128, 2.0, 14), (128, 4.0, 15)])
def test_find_halos_bit_exact(orc, pk, nd, Lc, seed):
    delta = _field(nd, Lc, seed, pk)
    got, want = _compare(orc, delta, pk, Lc)
    assert want["nh"] > 10


def test_find_halos_ellipsoidal_barrier_and_nmin(orc, pk):
    delta = _field(64, 2.0, 7, pk)
    _compare(orc, delta, pk, 2.0, a=1.0, beta=0.12, alpha=0.0, Nmin=5)
    _compare(orc, delta, pk, 2.0, a=0.9, beta=0.3, alpha=0.4, Nmin=2, fp64=1)


def test_find_halos_many_ties(orc, pk):
    # quantised densities: many peaks share a value, so the order depends on
    # the reference quicksort's handling of equal keys
    delta = _field(64, 4.0, 9, pk)
    q = (np.round(delta * 8.0) / 8.0).astype(np.float32)
    got, want = _compare(orc, q, pk, 4.0)
    dens = q.reshape(-1)[(want["x"][:, 0] * 64 + want["x"][:, 1]) * 64 + want["x"][:, 2]]
    assert np.unique(dens).size < dens.size / 4       # ties do occur


def test_find_halos_edge_cases(orc, pk):
    k, P = pk
    from exshalos_gb300.lib import exshalos
    flat = np.zeros((16, 16, 16), dtype=np.float32)           # no peaks at all
    r = exshalos.find_halos(flat, k, P, 4.0, 0.31, 0.0, -1.0, 1, 1.0, 0.0, 0.0, 1, 0, 0)
    assert r["Mh"].size == 0 and np.all(r["flag"] == 16 ** 3)
    one = flat.copy()
    one[3, 4, 5] = 10.0                                       # one peak: the reference loop never runs
    r = exshalos.find_halos(one, k, P, 4.0, 0.31, 0.0, -1.0, 1, 1.0, 0.0, 0.0, 1, 0, 0)
    assert r["Mh"].size == 0
    two = one.copy()
    two[10, 10, 10] = 20.0
    _compare(orc, two, pk, 4.0)
    with pytest.raises(ValueError):
        exshalos.find_halos(flat, k, P, -1.0, 0.31, 0.0, -1.0, 1, 1.0, 0.0, 0.0, 1, 0, 0)


@pytest.mark.parametrize("do2", [0, 1])
def test_halos_box_from_pk_vs_oracle(orc, pk, do2):
    from exshalos_gb300.lib import exshalos
    k, P = pk
    nd, Lc, seed = 64, 4.0, 1
    r = exshalos.halos_box_from_pk(k, P, 1e5, nd, nd, nd, Lc, seed, 1e4, 0.31, 0.0, -1.0, 1, 1.0, 0.0, 0.0, 0, 0.0,
                                   1, 1, 1, do2, 1, 0, 0, 1, _catalogue=True)
    p = orc.make_params(nd, Lc, seed=seed)
    want_field = orc.field_real(p, orc.field_modes(p, k, P, stream=0))
    assert rel_rms(r["grid"], want_field) < 1e-5
    # the catalogue of the GPU field, bit for bit
    tab = orc.sigma_tables(p, k, P)
    ref = orc.find_halos(p, r["grid"], tab)
    np.testing.assert_array_equal(r["x"], ref["x"])
    np.testing.assert_array_equal(r["count"], ref["count"])
    np.testing.assert_array_equal(r["Mh"].view(np.uint32), ref["Mh"].view(np.uint32))
    np.testing.assert_array_equal(r["flag"].reshape(-1), ref["flag"])
    # displacements against the FP64 oracle on the same labelling
    lp = orc.lpt_posh(p, k, P, ref["flag"], ref["x"], ref["count"], do_2lpt=do2, keep_pos=True, stream=0)
    L = nd * Lc
    d = np.abs(r["posh"] - lp["posh"])
    d = np.minimum(d, L - d)
    assert d.max() < 2e-3
    dp = np.abs(r["pos"] - lp["pos"])
    dp = np.minimum(dp, L - dp)
    assert dp.max() < 2e-3
    assert np.all(np.isfinite(r["velh"]))


@pytest.mark.parametrize("do2", [0, 1])
def test_halos_box_from_grid_vs_oracle(orc, pk, do2):
    """Generate_Halos_Box_from_Grid: the catalogue of a given grid bit for bit
    (mass draws seeded 1234), LPT from Normk r2c(grid) against the FP64 oracle."""
    from exshalos_gb300.lib import exshalos
    k, P = pk
    nd, Lc = 64, 4.0
    p = orc.make_params(nd, Lc, seed=5)
    grid = orc.field_real(p, orc.field_modes(p, k, P, stream=1)).astype(np.float32)
    r = exshalos.halos_box_from_grid(k, P, grid, None, None, Lc, 1e4, 0.31, 0.0, -1.0, 1, 1.0, 0.0, 0.0, 1, 1, do2,
                                     1, 0, 0, 0, 1, _catalogue=True)
    pm = orc.make_params(nd, Lc, seed=1234)
    ref = orc.find_halos(pm, grid, orc.sigma_tables(pm, k, P))
    np.testing.assert_array_equal(r["x"], ref["x"])
    np.testing.assert_array_equal(r["count"], ref["count"])
    np.testing.assert_array_equal(r["Mh"].view(np.uint32), ref["Mh"].view(np.uint32))
    np.testing.assert_array_equal(r["flag"].reshape(-1), ref["flag"])
    lp = orc.lpt_posh(pm, k, P, ref["flag"], ref["x"], ref["count"], do_2lpt=do2, keep_pos=True,
                      modes=orc.grid_modes(pm, grid.astype(np.float64)))
    L = nd * Lc
    d = np.abs(r["posh"] - lp["posh"])
    assert np.minimum(d, L - d).max() < 2e-3
    dp = np.abs(r["pos"] - lp["pos"])
    assert np.minimum(dp, L - dp).max() < 2e-3
    assert np.all(np.isfinite(r["velh"])) and np.all(np.isfinite(r["vel"]))


def test_halos_box_from_grid_given_displacements(orc, pk):
    """With S given, posh = cysumf(Lc (x + 1/2), sum of the members' S / count)
    (box.c:89-105, lpt.c:245-255) and velh = sum of V / count."""
    from exshalos_gb300 import mock
    k, P = pk
    nd, Lc = 48, 4.0
    ng = nd ** 3
    p = orc.make_params(nd, Lc, seed=9)
    grid = orc.field_real(p, orc.field_modes(p, k, P, stream=1)).astype(np.float32)
    rng = np.random.default_rng(4)
    S = rng.normal(0, 3.0, (ng, 3)).astype(np.float32)
    V = rng.normal(0, 100.0, (ng, 3)).astype(np.float32)
    r = mock.Generate_Halos_Box_from_Grid(grid, k, P, S=S, V=V, Lc=Lc, OUT_VEL=True, OUT_FLAG=True)
    flag = r["flag"].reshape(-1)
    nh = r["posh"].shape[0]
    owner = np.abs(flag)
    m = owner < ng
    sS = np.stack([np.bincount(owner[m], weights=S[m, a].astype(np.float64), minlength=nh) for a in range(3)], 1)
    sV = np.stack([np.bincount(owner[m], weights=V[m, a].astype(np.float64), minlength=nh) for a in range(3)], 1)
    pm = orc.make_params(nd, Lc, seed=1234)
    ref = orc.find_halos(pm, grid, orc.sigma_tables(pm, k, P))
    assert ref["nh"] == nh
    cnt = ref["count"].astype(np.float64)          # Compute_Posh divides by the halo's count
    L = nd * Lc
    want = np.mod(Lc * (ref["x"] + 0.5) + sS / cnt[:, None], L)
    d = np.abs(r["posh"] - want)
    assert np.minimum(d, L - d).max() < 1e-3
    np.testing.assert_allclose(r["velh"], sV / cnt[:, None], rtol=1e-4, atol=1e-3)
    with pytest.raises(ValueError):
        mock.Generate_Halos_Box_from_Grid(grid, k, P, S=S[:-1], Lc=Lc)
