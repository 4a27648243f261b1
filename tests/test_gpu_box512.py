"""Large box, nd = 512 (L = 1024 Mpc/h): halos, the 2LPT particle catalogue
of 512^3 positions, their CIC grid and the 256-bin P(k), checked at full size
through properties, against the FP64 oracle's P(k) of the same grid, and the
particle positions (the 512-point passes, among them the 2LPT Poisson x pass
k_fft8_x_poisson512) against the FP64 oracle's 2LPT (lpt.c:4-242) on the same
field stream (the reference's, GPU)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_box512_particles_cic_pk(orc, pk):
    import torch
    from exshalos_gb300 import _capi
    k, P = pk
    nd, Lc, Nk = 512, 2.0, 256
    L = nd * Lc
    ng = nd ** 3
    L_ = _capi.load()
    ctx = _capi.context()
    prm = _capi.default_params(ndx=nd, ndy=nd, ndz=nd, Lc=Lc, seed=1, DO_2LPT=1, OUT_LPT=1, a=1.0, beta=0.12,
                               alpha=0.0)
    nh = C.c_int64(0)
    _capi.check(L_.exh_halos_box_from_pk(ctx, _capi.ptr(k), _capi.ptr(P), k.size, prm, C.byref(nh), None))
    assert nh.value > 100000
    pos = torch.empty(3 * ng, dtype=torch.float32, device="cuda")
    posh = torch.empty(3 * nh.value, dtype=torch.float32, device="cuda")
    _capi.check(L_.exh_halos_fetch(ctx, _capi.ptr(posh), None, None, None, None, None, _capi.ptr(pos), None, None,
                                   _capi.EXH_MEM_DEVICE, None))
    torch.cuda.synchronize()
    # cysumf (exshalos_h.c:13-21) wraps into [0, L]: a tiny negative sum
    # plus L can round to L itself
    for a in (pos, posh):
        assert bool(torch.isfinite(a).all())
        assert float(a.min()) >= 0.0 and float(a.max()) <= L
    # the displacements move particles by a few cells at most
    q = (torch.arange(nd, device="cuda", dtype=torch.float32) + 0.5) * Lc
    x = pos.view(nd, nd, nd, 3)[:, 0, 0, 0]
    d = torch.remainder(x - q + L / 2, L) - L / 2
    assert float(d.abs().max()) < 20 * Lc and float(d.abs().mean()) > 0.1
    grid = torch.empty(ng, dtype=torch.float32, device="cuda")
    _capi.check(L_.exh_grid_compute(ctx, _capi.ptr(pos), ng, nd, float(L), 2, 1, _capi.ptr(grid),
                                    _capi.EXH_MEM_DEVICE, None))
    kmin, kmax = np.float32(2 * np.pi / L), np.float32(np.pi / L * nd)
    k_out = np.zeros(Nk, dtype=np.float32)
    P_out = np.zeros(Nk, dtype=np.float32)
    c_out = np.zeros(Nk, dtype=np.int64)
    _capi.check(L_.exh_power_compute(ctx, _capi.ptr(grid), nd, float(L), 2, Nk, float(kmin), float(kmax),
                                     _capi.ptr(k_out), _capi.ptr(P_out), _capi.ptr(c_out), _capi.EXH_MEM_DEVICE,
                                     None))
    g = grid.cpu().numpy().reshape(nd, nd, nd)
    # every particle lands on the grid: the contrast averages to zero
    assert abs(float(g.astype(np.float64).mean())) < 1e-5
    want = orc.power(g.astype(np.float64), L, window=2, Nk=Nk, kmin=kmin, kmax=kmax)
    np.testing.assert_array_equal(c_out, want["Nk"])
    m = want["Nk"] > 0
    assert np.max(np.abs(P_out[m] / want["Pk"][m] - 1)) < 1e-4
    assert np.max(np.abs(k_out[m] / want["k"][m] - 1)) < 1e-6
    del g, grid, posh
    # particle positions against the FP64 2LPT of the same field (no halo
    # labelling needed for the particles), compared slab by slab
    got = pos.cpu().numpy().reshape(nd, nd * nd, 3)
    del pos
    p = orc.make_params(nd, Lc, seed=1, a=1.0, beta=0.12, alpha=0.0)
    lp = orc.lpt_posh(p, k, P, np.full(ng, ng, dtype=np.int64), np.zeros((0, 3), np.int32), np.zeros(0, np.int32),
                      do_2lpt=1, keep_pos=True, stream=0)
    want_pos = lp["pos"].reshape(nd, nd * nd, 3)
    num = den = worst = 0.0
    jk = (np.indices((nd, nd), dtype=np.float64).reshape(2, -1).T + 0.5) * Lc
    for i in range(nd):
        a = got[i].astype(np.float64)
        b = want_pos[i]
        d = np.remainder(a - b + L / 2, L) - L / 2
        q = np.concatenate([np.full((nd * nd, 1), (i + 0.5) * Lc), jk], axis=1)
        s_ = np.remainder(b - q + L / 2, L) - L / 2
        num += float(np.sum(d * d))
        den += float(np.sum(s_ * s_))
        worst = max(worst, float(np.abs(d).max()))
    e = np.sqrt(num / den)
    print(f"512^3 particles vs FP64: rel rms {e:.2e}, max {worst:.2e} Mpc/h")
    assert e < 1e-5 and worst < 2e-3
