"""Halo abundance, repeated halo finding on one grid (peaks and sort found
once) and the barrier fit built on them (GPU)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _grid(orc, pk, nd, Lc, seed):
    k, P = pk
    p = orc.make_params(nd, Lc, seed=seed)
    return orc.field_real(p, orc.field_modes(p, k, P, stream=1)).astype(np.float32)


def test_abundance_matches_restatement():
    from exshalos_gb300 import simulation
    from oracle import spectrum_f64 as sp
    rng = np.random.default_rng(5)
    M = np.exp(rng.uniform(np.log(1e12), np.log(1e15), 20000)).astype(np.float32)
    for Mmin, Mmax in ((None, None), (2e12, 5e14)):
        r = simulation.Compute_Abundance(M, Mmin=Mmin, Mmax=Mmax, Nm=20, Lc=2.0, nd=128)
        w = sp.abundance(M, -1.0 if Mmin is None else np.float32(Mmin), -1.0 if Mmax is None else np.float32(Mmax),
                         20, 2.0, 128, 128, 128)
        np.testing.assert_array_equal(r["dn"], w["dn"])
        np.testing.assert_array_equal(r["dn_err"], w["dn_err"])
        np.testing.assert_allclose(r["Mh"], w["Mh"], rtol=1e-6)
        assert r["dn"][0] == 0.0                   # the reference never fills the first bin


def test_repeated_barriers_on_one_grid(orc, pk):
    """Three barriers on one grid, then another grid, then the first again:
    every catalogue bit for bit against the oracle (the cached peaks must
    follow the grid)."""
    from exshalos_gb300.lib import exshalos
    k, P = pk
    nd, Lc = 64, 4.0
    g1, g2 = _grid(orc, pk, nd, Lc, 3), _grid(orc, pk, nd, Lc, 4)
    cases = [(g1, 1.0, 0.0, 0.0), (g1, 0.8, 0.3, 0.5), (g1, 1.2, 0.1, 0.2), (g2, 0.8, 0.3, 0.5), (g1, 1.0, 0.0, 0.0)]
    for g, a, beta, alpha in cases:
        r = exshalos.find_halos(g, k, P, Lc, 0.31, 0.0, -1.0, 1, a, beta, alpha, 1, 0, 0, _catalogue=True)
        p = orc.make_params(nd, Lc, seed=12345, a=a, beta=beta, alpha=alpha)
        ref = orc.find_halos(p, g, orc.sigma_tables(p, k, P))
        np.testing.assert_array_equal(r["x"], ref["x"])
        np.testing.assert_array_equal(r["Mh"].view(np.uint32), ref["Mh"].view(np.uint32))
        np.testing.assert_array_equal(r["flag"].reshape(-1), ref["flag"])


def test_fit_barrier_improves_chi2(orc, pk):
    from exshalos_gb300 import simulation, utils
    k, P = pk
    nd, Lc = 64, 4.0
    g = _grid(orc, pk, nd, Lc, 6)
    truth = (0.8, 0.3, 0.5)
    h = utils.Find_Halos_from_Grid(g, k, P, Lc=Lc, Nmin=10, a=truth[0], beta=truth[1], alpha=truth[2],
                                   delta_c=utils.Get_deltac())
    target = simulation.Compute_Abundance(h["Mh"], Nm=12, Lc=Lc, nd=nd)
    m = target["dn"] > 0
    best = utils.Fit_Barrier(k, P, target["Mh"][m], target["dn"][m], dn_err=target["dn_err"][m], grid=g, Nm=12,
                             nd=nd, Lc=Lc, Nmin=10, Max_iter=25)
    lo, hi = np.array([0.1, 0.0, 0.0]), np.array([2.0, 1.0, 1.0])
    assert np.all(best >= lo) and np.all(best <= hi)

    def chi2(theta):
        x = utils.Find_Halos_from_Grid(g, k, P, Lc=Lc, Nmin=10, a=theta[0], beta=theta[1], alpha=theta[2],
                                       delta_c=utils.Get_deltac())
        d = simulation.Compute_Abundance(x["Mh"], Nm=12, Lc=Lc, nd=nd)
        mm = (d["dn"] > 0) & (target["dn"] > 0)
        return np.sum((d["dn"][mm] - target["dn"][mm]) ** 2 / (target["dn_err"][mm] ** 2 + 1e-30))

    assert chi2(best) <= chi2([0.55, 0.4, 0.7])
