"""Batched realisations: lane-count independence, equality with the plain
public-API chain, and the P(k) error against the FP64 oracle (GPU)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NDS = [64, 32, 48, 64, 32, 96, 48, 32, 64, 48]
SEEDS = list(range(len(NDS)))


@pytest.fixture(scope="module")
def plain(pk):
    from exshalos_gb300.lib import exshalos as ex
    k, P = pk
    return ex.batch_run(k, P, NDS, SEEDS, Lc=2.0, Nk_pk=64, lanes=1)


@pytest.mark.parametrize("lanes", [2, 4, 7])
def test_batch_independent_of_lanes(pk, plain, lanes):
    from exshalos_gb300.lib import exshalos as ex
    k, P = pk
    r = ex.batch_run(k, P, NDS, SEEDS, Lc=2.0, Nk_pk=64, lanes=lanes)
    for key in ("nh", "k", "Pk", "Nk", "status"):
        assert np.array_equal(r[key], plain[key]), key
    assert np.all(plain["nh"] > 0)


def test_batch_equals_public_api_chain(pk, plain):
    from exshalos_gb300 import mock, simulation
    k, P = pk
    for i in (0, 5, 7):
        nd, L = NDS[i], 2.0 * NDS[i]
        h = mock.Generate_Halos_Box_from_Pk(k, P, nd=nd, Lc=2.0, seed=SEEDS[i], field_stream="philox")
        assert h["posh"].shape[0] == plain["nh"][i]
        g = simulation.Compute_Density_Grid(h["posh"], nd=nd, L=L, window="CIC")
        p = simulation.Compute_Power_Spectrum(g, L=L, window="CIC", Nk=64, k_min=2 * np.pi / L, k_max=np.pi * nd / L)
        assert np.array_equal(np.asarray(p["Pk"]).ravel(), plain["Pk"][i])
        assert np.array_equal(np.asarray(p["k"]).ravel(), plain["k"][i])
        assert np.array_equal(np.asarray(p["Nk"]).ravel(), plain["Nk"][i])


def test_batch_pk_vs_fp64_oracle(orc, pk, plain):
    """P(k) of the batch against the FP64 oracle's CIC + P(k) of the same halo
    positions: relative error below 1e-4 in every populated bin."""
    from exshalos_gb300 import mock
    k, P = pk
    for i in (1, 5):
        nd, L = NDS[i], 2.0 * NDS[i]
        h = mock.Generate_Halos_Box_from_Pk(k, P, nd=nd, Lc=2.0, seed=SEEDS[i], field_stream="philox")
        g = orc.cic(h["posh"].astype(np.float64), nd, L)
        want = orc.power(g, L, window=2, Nk=64, kmin=2 * np.pi / L, kmax=np.pi * nd / L)
        m = want["Nk"] > 0
        got = plain["Pk"][i][m]
        ref = np.asarray(want["Pk"]).ravel()[m]
        assert np.max(np.abs(got - ref) / np.abs(ref)) < 1e-4
        assert np.array_equal(plain["Nk"][i][m], np.asarray(want["Nk"]).ravel()[m])


def test_batch_rejects_bad_items(pk):
    from exshalos_gb300.lib import exshalos as ex
    k, P = pk
    with pytest.raises(ValueError):
        ex.batch_run(k, P, [64, 33], [1, 2])
    with pytest.raises(ValueError):
        ex.batch_run(k, P, [64], [1], lanes=0)
    r = ex.batch_run(k, P, [], [])
    assert r["nh"].size == 0


def test_many_lanes_mixed_sizes_match_one_lane(pk):
    """More lanes than items of one size, sizes interleaved, 2LPT on: every
    lane thread launches the same kernels with different shared-memory sizes,
    and the results equal the one-lane loop."""
    from exshalos_gb300.lib import exshalos as ex
    k, P = pk
    nds = np.array([32, 96, 64, 128, 48, 96, 32, 128, 64, 48, 96, 32] * 4)
    seeds = np.arange(100, 100 + nds.size)
    kw = dict(Lc=2.0, Nk_pk=32, DO_2LPT=1, beta=0.12)
    one = ex.batch_run(k, P, nds, seeds, lanes=1, **kw)
    many = ex.batch_run(k, P, nds, seeds, lanes=32, **kw)
    for key in ("nh", "k", "Pk", "Nk", "status"):
        assert np.array_equal(many[key], one[key]), key
