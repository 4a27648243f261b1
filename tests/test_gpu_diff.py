"""Differentiable forward and its hand-written adjoint against the FP64
oracle: forward P(k) parity, and gradients w.r.t. the noise field and the
knot amplitudes against FP64 central finite differences at nd = 32 (GPU)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ND, L, NK, NKNOT = 32, 128.0, 16, 20


def _setup(pk, do_2lpt=True):
    import torch
    from exshalos_gb300 import diff
    k, P = pk
    kf = 2 * np.pi / L
    knot_k, knot_P = diff.knots_from_spectrum(k, P, NKNOT, kf, np.sqrt(3) * np.pi * ND / L * 1.01)
    model = diff.pk_chi2_model(ND, L, knot_k, Nk=NK, do_2lpt=do_2lpt)
    g = torch.Generator(device="cpu").manual_seed(8)
    w_t = torch.randn((ND, ND, ND), generator=g, dtype=torch.float64).numpy().astype(np.float32)
    wt = torch.from_numpy(w_t).cuda()
    _, target, _, _ = model.forward(wt, knot_P, np.ones(NK, dtype=np.float32))
    g = torch.Generator(device="cpu").manual_seed(7)
    w = torch.randn((ND, ND, ND), generator=g, dtype=torch.float64).numpy().astype(np.float32)
    return model, knot_k, knot_P, w, target.astype(np.float64)


@pytest.mark.parametrize("do_2lpt", [True, False])
def test_diff_forward_matches_fp64(orc, pk, do_2lpt):
    import torch
    from oracle import diff_f64
    model, knot_k, knot_P, w, target = _setup(pk, do_2lpt)
    loss, P, kb, cnt = model.forward(torch.from_numpy(w).cuda(), knot_P, target.astype(np.float32))
    want_loss, want_P, want_n = diff_f64.forward(w, knot_k, knot_P, L, target.astype(np.float32), NK,
                                                 model.prm.k_min, model.prm.k_max, do_2lpt=do_2lpt)
    np.testing.assert_array_equal(cnt, want_n)
    m = want_n > 0
    assert np.max(np.abs(P[m] / want_P[m] - 1)) < 1e-4
    assert abs(loss / want_loss - 1) < 1e-3


@pytest.mark.parametrize("do_2lpt", [True, False])
def test_diff_adjoint_vs_fp64_finite_differences(orc, pk, do_2lpt):
    import torch
    from exshalos_gb300 import diff
    from oracle import diff_f64
    model, knot_k, knot_P, w, target = _setup(pk, do_2lpt)
    T32 = target.astype(np.float32)
    noise = torch.from_numpy(w).cuda().requires_grad_(True)
    kP = torch.tensor(knot_P, dtype=torch.float64, requires_grad=True)
    loss = diff.pk_chi2(noise, kP, model, T32)
    loss.backward()
    gw = noise.grad.cpu().numpy().astype(np.float64)
    gk = kP.grad.numpy()

    def f(ww, kk):
        return diff_f64.forward(ww, knot_k, kk, L, T32, NK, model.prm.k_min, model.prm.k_max, do_2lpt=do_2lpt)[0]

    # the FP64 adjoint of the oracle on the same inputs
    _, gw64, gk64 = diff_f64.gradient(w, knot_k, knot_P, L, T32, NK, model.prm.k_min, model.prm.k_max,
                                      do_2lpt=do_2lpt)
    rr = np.sqrt(np.mean((gw - gw64) ** 2) / np.mean(gw64 ** 2))
    print(f"noise gradient: FP32 GPU vs FP64 adjoint rel rms {rr:.2e}")
    assert rr < 1e-3
    kr = np.max(np.abs((gk - gk64) * knot_P)) / np.max(np.abs(gk64 * knot_P))
    print(f"knot gradient: FP32 GPU vs FP64 adjoint max rel {kr:.2e}")
    assert kr < 1e-3
    # directional derivatives along random directions of the noise; the CIC
    # weights are piecewise linear in the positions, so the step must be
    # small enough that almost no particle crosses a cell centre
    rng = np.random.default_rng(3)
    for trial in range(3):
        v = rng.standard_normal(w.shape)
        eps = 1e-5
        fd = (f(w + eps * v, knot_P) - f(w - eps * v, knot_P)) / (2 * eps)
        ad = float(np.sum(gw * v))
        # tolerance on the scale of the summed terms (the dot product of a
        # gradient with a random direction cancels)
        assert abs(ad - fd) <= 2e-3 * float(np.sum(np.abs(gw64 * v))), (trial, ad, fd)
    # every knot amplitude
    kd = np.asarray(knot_P, dtype=np.float64)
    fdk = np.zeros(NKNOT)
    for i in range(NKNOT):
        h = 1e-6 * kd[i]
        kp, km = kd.copy(), kd.copy()
        kp[i] += h
        km[i] -= h
        fdk[i] = (f(w, kp) - f(w, km)) / (2 * h)
    scale = np.max(np.abs(fdk * kd))
    assert np.max(np.abs((gk - fdk) * kd)) <= 1e-3 * scale, np.c_[gk * kd, fdk * kd]
