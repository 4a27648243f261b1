"""The oracle against the reference's own C (CPU).

oracle/ref_build.py compiles the reference's mock-path sources unmodified,
from the reference tree, against project-written stand-ins for the FFTW3 and
GSL entry points they call (oracle/ref_shim/); the stand-ins use the oracle's
own FFT, taus stream, polar Gaussian and spline.  With the library arithmetic
identical on both sides, every stage of the oracle's restatement must equal
the reference's loops bit for bit: the field (Compute_Den), the sigma and
barrier tables (Compute_Sig, Barrier), the halo catalogue (Find_Halos: peaks,
quicksort, growth, masses), 1LPT/2LPT halo and particle positions, the CIC
grid and the binned P(k), and the whole Generate_Halos_Box_from_Pk on the
workloads' configurations.  What this does not pin is FFTW's and GSL's own
round-off.  Skipped where the reference tree is absent.
"""
import numpy as np
import pytest

ref = pytest.importorskip("oracle.ref")
if not ref.available():
    pytest.skip("the reference tree is not available", allow_module_level=True)

BAR = dict(a=1.0, beta=0.12, alpha=0.0)


def _same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return a.shape == b.shape and np.array_equal(a.view(np.uint8), b.view(np.uint8))


@pytest.mark.parametrize("nd,Lc,seed,fixed,phase", [(32, 4.0, 3, 0, 0.0), (48, 2.0, 12345, 0, 0.0),
                                                     (64, 4.0, 1, 1, 0.0), (36, 3.0, 7, 0, 0.4)])
def test_field_equals_reference(orc, pk, nd, Lc, seed, fixed, phase):
    k, P = pk
    d, m = ref.density_grid(k, P, nd, Lc, seed, fixed=fixed, phase=phase)
    p = orc.make_params(nd, Lc, seed=seed, prec="f32")
    om = orc.field_modes(p, k, P, stream=0, fixed=fixed, phase=phase, prec="f32")
    assert _same(om, m)
    assert _same(orc.field_real(p, om, prec="f32"), d)


@pytest.mark.parametrize("nd,Lc,bar", [(64, 4.0, dict(a=1.0, beta=0.0, alpha=0.0)), (256, 2.0, BAR),
                                       (64, 2.0, dict(a=0.9, beta=0.3, alpha=0.4))])
def test_sigma_and_barrier_tables_equal_reference(orc, pk, nd, Lc, bar):
    k, P = pk
    p = orc.make_params(nd, Lc, **bar)
    tab = orc.sigma_tables(p, k, P)
    sig, btab = ref.sigma_barrier(k, P, nd, Lc, tab["Ncells"], **bar)
    assert _same(tab["Sig_grid"], sig)
    assert _same(tab["Btab"], btab)


@pytest.mark.parametrize("quantise,bar,Nmin", [(False, BAR, 1), (True, dict(a=1.0, beta=0.0, alpha=0.0), 1),
                                               (False, dict(a=0.9, beta=0.3, alpha=0.4), 5)])
def test_catalogue_equals_reference(orc, pk, quantise, bar, Nmin):
    k, P = pk
    nd, Lc, seed = 64, 4.0, 2
    d, _ = ref.density_grid(k, P, nd, Lc, seed)
    if quantise:                                   # many equal peak densities: the quicksort's tie order
        d = (np.round(d * 8.0) / 8.0).astype(np.float32)
    p = orc.make_params(nd, Lc, seed=seed, Nmin=Nmin, **bar)
    got = orc.find_halos(p, d, orc.sigma_tables(p, k, P))
    want = ref.find_halos(d, k, P, Lc, seed, Nmin=Nmin, **bar)
    assert got["nh"] == want["nh"] > 100
    for key in ("x", "count", "Mh", "flag"):
        assert _same(got[key], want[key]), key


@pytest.mark.parametrize("do2", [0, 1])
def test_lpt_equals_reference(orc, pk, do2):
    k, P = pk
    nd, Lc, seed = 48, 4.0, 5
    d, m = ref.density_grid(k, P, nd, Lc, seed)
    p = orc.make_params(nd, Lc, seed=seed)
    h = orc.find_halos(p, d, orc.sigma_tables(p, k, P))
    p32 = orc.make_params(nd, Lc, seed=seed, prec="f32")
    got = orc.lpt_posh(p32, k, P, h["flag"], h["x"], h["count"], do_2lpt=do2, keep_pos=True, prec="f32", modes=m)
    want = ref.lpt(m, nd, Lc, h["flag"], h["x"], h["count"], do_2lpt=do2)
    assert _same(got["posh"], want["posh"])
    assert _same(got["pos"], want["pos"])


@pytest.mark.parametrize("window", [0, 1, 2])
def test_cic_and_power_equal_reference(orc, window):
    rng = np.random.default_rng(3)
    nd, L, Nk = 48, 192.0, 20
    pos = rng.uniform(-5.0, L + 5.0, (30000, 3)).astype(np.float32)
    g = ref.cic(pos, nd, L)
    assert _same(orc.cic(pos, nd, L, prec="f32"), g)
    want = ref.power(g, L, window=window, Nk=Nk)
    got = orc.power(g, L, window=window, Nk=Nk, prec="f32")
    assert np.array_equal(got["Nk"], want["Nk"])
    assert _same(got["Pk"], want["Pk"]) and _same(got["k"], want["k"])


@pytest.mark.parametrize("nd,Lc,seed,bar,do2", [(64, 4.0, 1, dict(a=1.0, beta=0.0, alpha=0.0), 0),
                                                (256, 2.0, 1, BAR, 1)])
def test_pipeline_equals_reference(orc, pk, nd, Lc, seed, bar, do2):
    """Generate_Halos_Box_from_Pk on the small-box workload (nd = 64, Lc = 4,
    seed 1, defaults) and the box_256 workload (nd = 256, Lc = 2, 2LPT,
    barrier a = 1, beta = 0.12): field, catalogue and halo positions."""
    k, P = pk
    got = orc.halos_box_from_pk(k, P, nd=nd, Lc=Lc, seed=seed, stream=0, do_2lpt=do2, prec="f32", **bar)
    want = ref.halos_box_from_pk(k, P, nd, Lc, seed, do_2lpt=do2, nthreads=8, **bar)
    assert got["nh"] == want["Mh"].size > 1000
    assert _same(got["delta"], want["delta"])
    assert _same(got["flag"], want["flag"])
    for key in ("x", "count", "Mh", "posh"):
        assert _same(got[key], want[key]), key


def test_range_error_where_the_reference_fails(orc, pk):
    """Seed 8 of the box_256 workload: a halo mass beyond the mass-function
    splines, where the reference's GSL aborts; both raise their range error."""
    k, P = pk
    with pytest.raises(ref.RangeError):
        ref.halos_box_from_pk(k, P, 256, 2.0, 8, nthreads=8, **BAR)
    with pytest.raises(orc.RangeError):
        orc.halos_box_from_pk(k, P, nd=256, Lc=2.0, seed=8, stream=0, prec="f32", **BAR)
