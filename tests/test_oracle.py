"""The oracle against the reference's own golden data and known answers (CPU)."""
import os

import numpy as np
import pytest

from conftest import rel_rms

HERE = os.path.dirname(os.path.abspath(__file__))


def test_cells_in_spheres_matches_reference_table(orc):
    ref = np.loadtxt(os.path.join(HERE, "golden", "cells_in_spheres.txt"), dtype=np.int64)
    got = orc.cells_in_spheres()
    assert ref.size == 8335
    np.testing.assert_array_equal(got, ref)


def test_philox_known_answers(orc):
    import ctypes as C
    L = orc.lib()
    kat = [((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
           ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
           ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
            (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1))]
    for ctr, key, want in kat:
        c = (C.c_uint32 * 4)(*ctr)
        k = (C.c_uint32 * 2)(*key)
        o = (C.c_uint32 * 4)()
        L.orc_philox4x32(c, k, o)
        assert tuple(o) == want


@pytest.mark.parametrize("shape", [(8, 8, 8), (12, 16, 18), (6, 9, 24), (16, 8, 32)])
@pytest.mark.parametrize("prec,tol", [("f64", 1e-13), ("f32", 2e-6)])
def test_fft_matches_numpy(orc, shape, prec, tol):
    rng = np.random.default_rng(1)
    x = rng.standard_normal(shape)
    want = np.fft.rfftn(x)
    got = orc.fft_r2c_3d(x, prec=prec)
    assert np.abs(got - want).max() / np.abs(want).max() < tol
    back = orc.fft_c2r_3d(want, shape[2], prec=prec)
    assert rel_rms(back, x * np.prod(shape)) < tol


def test_spline_is_natural_cubic(orc):
    scipy_interp = pytest.importorskip("scipy.interpolate")
    import ctypes as C
    x = np.sort(np.random.default_rng(2).uniform(0, 10, 40))
    y = np.sin(x) + 0.1 * x
    s = orc.lib()
    sp = (C.c_byte * 64)()
    assert s.orc_spline_init(sp, x.ctypes.data_as(C.c_void_p), y.ctypes.data_as(C.c_void_p), x.size) == 0
    ref = scipy_interp.CubicSpline(x, y, bc_type="natural")
    q = np.linspace(x[0], x[-1], 301)
    st = C.c_int(0)
    got = np.array([s.orc_spline_eval(sp, C.c_double(v), C.byref(st)) for v in q])
    assert st.value == 0
    np.testing.assert_allclose(got, ref(q), rtol=1e-12, atol=1e-12)
    s.orc_spline_free(sp)


def _lomuto_py(keys):
    a = list(range(len(keys)))
    stack = [(0, len(a) - 1)]
    while stack:
        lo, hi = stack.pop()
        if lo >= hi:
            continue
        piv = keys[a[hi]]
        i = lo - 1
        for j in range(lo, hi):
            if keys[a[j]] <= piv:
                i += 1
                a[i], a[j] = a[j], a[i]
        a[i + 1], a[hi] = a[hi], a[i + 1]
        stack.append((i + 2, hi))
        stack.append((lo, i))
    return a


def test_quicksort_tie_order(orc):
    rng = np.random.default_rng(3)
    keys = rng.integers(0, 12, 300).astype(np.float32)       # many ties
    pk = np.zeros(keys.size, dtype=[("x", np.int32, 3), ("den", np.float32)])
    pk["den"] = keys
    pk["x"][:, 0] = np.arange(keys.size)
    got = orc.quicksort_peaks(pk)["x"][:, 0]
    np.testing.assert_array_equal(got, np.array(_lomuto_py(list(keys))))


def test_cic_single_particle_known_answer(orc):
    nd, L = 8, 16.0
    pos = np.array([[3.0, 5.0, 7.0]])        # the centre of cell (1, 2, 3)
    g = orc.cic(pos, nd, L)
    want = np.full((nd, nd, nd), -1.0)
    want[1, 2, 3] = nd ** 3 - 1.0
    np.testing.assert_allclose(g, want, atol=1e-12)


def test_power_mode_counts_closed_form(orc):
    nd, L, Nk = 16, 100.0, 6
    p = orc.power(np.zeros((nd, nd, nd)), L, window=0, Nk=Nk)
    kf = 2 * np.pi / L
    kmin, kmax = np.float32(kf), np.float32(np.pi / L * nd)
    dk = np.float32((kmax - kmin) / np.float32(Nk))
    cnt = np.zeros(Nk, dtype=np.int64)
    for i in range(nd):
        for j in range(nd):
            for k in range(nd // 2 + 1):
                if k in (0, nd // 2) and (i == 0 or i == nd // 2 or j == 0 or j == nd // 2 or i > nd // 2):
                    continue
                q = [np.float32((v if 2 * v < nd else v - nd)) * np.float32(kf) for v in (i, j, k)]
                km = np.float32(np.sqrt(np.float32(q[0] * q[0] + q[1] * q[1] + q[2] * q[2])))
                b = int(np.floor(np.float32(km - kmin) / dk))
                if 0 <= b < Nk:
                    cnt[b] += 1
    np.testing.assert_array_equal(p["Nk"], cnt)


def test_field_power_recovers_input(orc, pk):
    k, P = pk
    p = orc.make_params(64, 4.0, seed=5)
    means = []
    for s in range(4):
        p.seed = s + 5
        d = orc.field_real(p, orc.field_modes(p, k, P, stream=1))
        res = orc.power(d, 256.0, window=0, Nk=16)
        means.append(res["Pk"])
    Pm = np.mean(means, axis=0)
    kk = res["k"]
    want = np.interp(np.log(kk), np.log(k), P)
    assert np.all(np.abs(Pm / want - 1.0)[2:] < 0.15)


def test_pipeline_consistency(orc, pk):
    k, P = pk
    r = orc.halos_box_from_pk(k, P, nd=32, Lc=4.0, seed=3, stream=0, prec="f32")
    assert r["nh"] > 0
    flag = r["flag"]
    ng = 32 ** 3
    # member cells per halo equal the counted cells, centres flagged -h
    members = np.bincount(np.abs(flag[np.abs(flag) < ng]), minlength=r["nh"])
    np.testing.assert_array_equal(members, r["count"])
    x = r["x"]
    centre = (x[:, 0] * 32 + x[:, 1]) * 32 + x[:, 2]
    np.testing.assert_array_equal(flag[centre[1:]], -np.arange(1, r["nh"]))
    assert np.all(np.isfinite(r["Mh"])) and np.all(r["Mh"] > 0)
    assert np.all((r["posh"] >= 0) & (r["posh"] < 128.0))


def test_ladder_matches_numpy_restatement(orc, pk):
    """The oracle ladder against an independent numpy irfftn of W(kR) delta_k."""
    k, P = pk
    nd, Lc = 32, 4.0
    p = orc.make_params(nd, Lc, seed=3)
    modes = orc.field_modes(p, k, P, stream=1)
    dk = modes[..., 0] + 1j * modes[..., 1]
    R = np.array([4.0, 9.0, 20.0], dtype=np.float32)
    kf = 2 * np.pi / (nd * Lc)
    f = np.fft.fftfreq(nd, 1.0 / nd)
    fz = np.arange(nd // 2 + 1, dtype=np.float64)
    fz[-1] = -(nd // 2)
    kk = kf * np.sqrt(f[:, None, None] ** 2 + f[None, :, None] ** 2 + fz[None, None, :] ** 2)
    fields = []
    for r in R:
        x = kk * float(r)
        with np.errstate(invalid="ignore", divide="ignore"):
            w = np.where(x > 0, 3 * (np.sin(x) - x * np.cos(x)) / np.where(x > 0, x, 1) ** 3, 1.0)
        fields.append(np.fft.irfftn(dk * w, s=(nd, nd, nd), axes=(0, 1, 2)) * nd ** 3 * p.Normx_d)
    # barriers at the 90th percentile of each smoothed field
    B = np.array([np.percentile(fl, 90) for fl in fields], dtype=np.float32)
    want = np.full((nd, nd, nd), 255, dtype=np.uint8)
    for i in range(len(R) - 1, -1, -1):
        want[(want == 255) & (fields[i] >= float(B[i]))] = i
    got = orc.ladder(p, modes, R, B)
    assert np.mean(got != want) < 1e-4
    assert np.mean(got == 2) > 0.05


def test_diff_oracle_recovers_input_spectrum(orc, pk):
    """The FP64 differentiable-model oracle: with no displacement beyond first
    order, the particles' CIC P(k) follows the knot spectrum on large scales."""
    from oracle import diff_f64
    k, P = pk
    nd, L = 32, 256.0
    knot_k = np.geomspace(2 * np.pi / L, np.sqrt(3) * np.pi * nd / L * 1.01, 20)
    knot_P = np.exp(np.interp(np.log(knot_k), np.log(k.astype(np.float64)), np.log(P.astype(np.float64))))
    Nk = 8
    ps = []
    for seed in range(4):
        w = np.random.default_rng(seed).standard_normal((nd, nd, nd))
        _, Pb, n = diff_f64.forward(w, knot_k, knot_P, L, np.ones(Nk), Nk, 2 * np.pi / L, np.pi * nd / L / 4,
                                    do_2lpt=False)
        ps.append(Pb)
    Pm = np.mean(ps, axis=0)
    kc = 2 * np.pi / L + (np.arange(Nk) + 0.5) * (np.pi * nd / L / 4 - 2 * np.pi / L) / Nk
    want = np.exp(np.interp(np.log(kc), np.log(knot_k), np.log(knot_P)))
    assert np.all(np.abs(Pm[1:] / want[1:] - 1) < 0.35)


@pytest.mark.parametrize("do_2lpt", [False, True])
def test_diff_oracle_adjoint_vs_finite_differences(orc, pk, do_2lpt):
    """The FP64 adjoint restatement against FP64 central differences (nd = 16)."""
    from oracle import diff_f64
    k, P = pk
    nd, L, Nk = 16, 64.0, 8
    knot_k = np.geomspace(2 * np.pi / L, np.sqrt(3) * np.pi * nd / L * 1.01, 20)
    knot_P = np.exp(np.interp(np.log(knot_k), np.log(k.astype(np.float64)), np.log(P.astype(np.float64))))
    kmin, kmax = np.float32(2 * np.pi / L), np.float32(np.pi * nd / L)
    w8 = np.random.default_rng(8).standard_normal((nd,) * 3)
    _, T, _ = diff_f64.forward(w8, knot_k, knot_P, L, np.ones(Nk), Nk, kmin, kmax, do_2lpt=do_2lpt)
    w = np.random.default_rng(7).standard_normal((nd,) * 3)
    loss, gw, gk = diff_f64.gradient(w, knot_k, knot_P, L, T, Nk, kmin, kmax, do_2lpt=do_2lpt)

    def f(ww, kk):
        return diff_f64.forward(ww, knot_k, kk, L, T, Nk, kmin, kmax, do_2lpt=do_2lpt)[0]

    assert abs(loss / f(w, knot_P) - 1) < 1e-5
    v = np.random.default_rng(1).standard_normal(w.shape)
    eps = 1e-6
    fd = (f(w + eps * v, knot_P) - f(w - eps * v, knot_P)) / (2 * eps)
    assert abs(np.sum(gw * v) - fd) < 1e-5 * abs(fd)
    fdk = np.array([(f(w, knot_P * (1 + 1e-6 * (np.arange(20) == i))) -
                     f(w, knot_P * (1 - 1e-6 * (np.arange(20) == i)))) / (2e-6 * knot_P[i]) for i in range(20)])
    assert np.max(np.abs((gk - fdk) * knot_P)) < 1e-5 * np.max(np.abs(fdk * knot_P))


def test_spectrum_oracle_general_matches_basic(orc):
    """The FP64 general-grid / general-P(k) restatement reduces to the C
    oracle's CIC and P(k) for one unit-mass type without interlacing."""
    from oracle import spectrum_f64 as sp
    rng = np.random.default_rng(21)
    nd, L = 16, 64.0
    pos = rng.uniform(0, L, (3000, 3))
    g = sp.tracer_grid(pos, nd, L, window=2)[0, 0]
    want = orc.cic(pos, nd, L)
    assert np.max(np.abs(g - want)) < 1e-5          # float offsets (the reference's) vs FP64
    kmin, kmax = np.float32(2 * np.pi / L), np.float32(np.pi / L * nd)
    p = sp.power(g, L, window=2, Nk=8, kmin=kmin, kmax=kmax)
    q = orc.power(g, L, window=2, Nk=8, kmin=kmin, kmax=kmax)
    np.testing.assert_array_equal(p["Nk"], q["Nk"])
    m = q["Nk"] > 0
    assert np.max(np.abs(p["Pk"][0, 0][m] / q["Pk"][m] - 1)) < 1e-6     # float vs double window
    # multipoles of an isotropic field: l = 2 small against l = 0 in the populated bins
    p4 = sp.power(g, L, window=2, Nk=8, kmin=kmin, kmax=kmax, l_max=2, direction=2)
    assert np.allclose(p4["Pk"][0, 0], p["Pk"][0, 0])
