"""ORACLE — test infrastructure only.

FP64 numpy restatement of the differentiable forward model (noise -> knot
P(k) -> 1LPT/2LPT particles -> CIC -> P(k) bins -> chi^2) used to check the
GPU forward and, by central finite differences, its hand-written adjoint.
The LPT steps follow src/exshalos/lpt.c:4-242 (sixth-order differences over
60 Lc, Poisson solves in Fourier space, cysumf wrap of exshalos_h.c:13-21);
CIC and the binned P(k) are the oracle's C restatements of
src/spectrum/gridmodule.c:21-53 and src/spectrum/powermodule.c:4-108.
FFTs are numpy's (unnormalised forward, like FFTW r2c; the inverse is
rescaled by nd^3 to FFTW's unnormalised c2r).
"""
import numpy as np

from . import orc


def _k2(nd, L):
    kf = 2.0 * np.pi / L
    f = np.fft.fftfreq(nd, 1.0 / nd)
    fz = np.arange(nd // 2 + 1, dtype=np.float64)
    fz[-1] = -(nd // 2)
    return kf * kf * (f[:, None, None] ** 2 + f[None, :, None] ** 2 + fz[None, None, :] ** 2)


def knot_power(k, knot_k, knot_P):
    """log-linear interpolation in log k, constant beyond the end knots"""
    lk = np.log(np.maximum(k, 1e-300))
    return np.exp(np.interp(lk, np.log(knot_k), np.log(knot_P)))


def _d6(f, axis, Lc):
    r = lambda s: np.roll(f, -s, axis=axis)      # r(s)[i] = f[i + s]
    return (r(3) - 9.0 * r(2) + 45.0 * r(1) - 45.0 * r(-1) + 9.0 * r(-2) - r(-3)) / (60.0 * Lc)


def particles(w, knot_k, knot_P, L, Om0=0.31, z=0.0, do_2lpt=True):
    nd = w.shape[0]
    ng = nd ** 3
    Lc = L / nd
    k2 = _k2(nd, L)
    W = np.fft.rfftn(w)
    A = np.sqrt(knot_power(np.sqrt(k2), knot_k, knot_P) / ng)
    A[0, 0, 0] = 0.0
    inv = np.zeros_like(k2)
    inv[k2 > 0] = 1.0 / k2[k2 > 0]
    phi1 = np.fft.irfftn(-W * A * inv, s=(nd,) * 3, axes=(0, 1, 2)) * ng
    Normx = 1.0 / np.sqrt(L ** 3)
    Normk = np.sqrt(L ** 3) / ng
    S = [-Normx * _d6(phi1, a, Lc) for a in range(3)]
    if do_2lpt:
        xx, yy, zz = _d6(S[0], 0, Lc), _d6(S[1], 1, Lc), _d6(S[2], 2, Lc)
        xy, xz, yz = _d6(S[0], 1, Lc), _d6(S[0], 2, Lc), _d6(S[1], 2, Lc)
        sig = xx * yy + xx * zz + yy * zz - xy ** 2 - xz ** 2 - yz ** 2
        phi2 = np.fft.irfftn(-np.fft.rfftn(sig) * Normk * inv, s=(nd,) * 3, axes=(0, 1, 2)) * ng
        Omz = Om0 * (1 + z) ** 3 / (Om0 * (1 + z) ** 3 + 1 - Om0)
        c2 = -3.0 / 7.0 * Omz ** (-1.0 / 143.0)
        S = [S[a] + c2 * Normx * _d6(phi2, a, Lc) for a in range(3)]
    q = (np.arange(nd) + 0.5) * Lc
    pos = np.empty((nd, nd, nd, 3))
    pos[..., 0] = q[:, None, None] + S[0]
    pos[..., 1] = q[None, :, None] + S[1]
    pos[..., 2] = q[None, None, :] + S[2]
    pos = np.where(pos >= L, pos - L, pos)
    pos = np.where(pos < 0, pos + L, pos)
    return pos.reshape(-1, 3)


def forward(w, knot_k, knot_P, L, target, Nk, kmin, kmax, Om0=0.31, z=0.0, do_2lpt=True, var=None):
    """chi^2, P(k) bins and mode counts of the model in FP64"""
    nd = w.shape[0]
    pos = particles(np.asarray(w, dtype=np.float64), np.asarray(knot_k, dtype=np.float64),
                    np.asarray(knot_P, dtype=np.float64), L, Om0, z, do_2lpt)
    grid = orc.cic(pos, nd, L)
    pk = orc.power(grid, L, window=2, Nk=Nk, kmin=kmin, kmax=kmax)
    n = pk["Nk"].astype(np.float64)
    T = np.asarray(target, dtype=np.float64)
    v = np.asarray(var, dtype=np.float64) if var is not None else np.where(n > 0, 2.0 * T * T / np.maximum(n, 1), 0.0)
    m = (n > 0) & (v > 0)
    loss = float(np.sum((pk["Pk"][m] - T[m]) ** 2 / v[m]))
    return loss, pk["Pk"], pk["Nk"]


def _bins(nd, L, Nk, kmin, kmax):
    """per-mode bin index (-1: not binned) and CIC factor of the half-complex
    grid, in the reference's float arithmetic (powermodule.c:26-56)"""
    f32 = np.float32
    kn = f32(2 * np.pi / L)
    i = np.arange(nd)
    s = np.where(2 * i < nd, i, i - nd).astype(f32)
    kx = (s * kn)[:, None, None]
    ky = (s * kn)[None, :, None]
    kz = (s[: nd // 2 + 1] * kn)[None, None, :].copy()
    kz[..., nd // 2] = f32(-(nd // 2)) * kn
    k2 = (kx * kx + ky * ky).astype(f32) + (kz * kz).astype(f32)
    kmod = np.sqrt(k2.astype(f32)).astype(f32)
    dk = f32((f32(kmax) - f32(kmin)) / f32(Nk))
    b = np.floor(((kmod - f32(kmin)).astype(f32) / dk).astype(f32)).astype(np.int64)
    I, J, K = np.meshgrid(np.arange(nd), np.arange(nd), np.arange(nd // 2 + 1), indexing="ij")
    skip = ((K == 0) | (K == nd // 2)) & (((I > nd // 2) & (J > nd // 2)) | (I == 0) | (I == nd // 2) | (J == 0) |
                                        (J == nd // 2) | ((I > nd // 2) & (J < nd // 2)))
    b[skip | (b < 0) | (b >= Nk)] = -1
    Lb = L / nd
    sinc = lambda x: np.where(x != 0, np.sin(x) / np.where(x != 0, x, 1), 1.0)
    w = (sinc(kx * Lb / 2) * sinc(ky * Lb / 2) * sinc(kz * Lb / 2)) ** 2
    return b, np.broadcast_to(w, b.shape)


def gradient(w, knot_k, knot_P, L, target, Nk, kmin, kmax, Om0=0.31, z=0.0, do_2lpt=True):
    """chi^2 and its FP64 adjoint gradients w.r.t. the noise and the knot
    amplitudes (the same chain of transposes as the CUDA adjoint)"""
    w = np.asarray(w, dtype=np.float64)
    knot_k = np.asarray(knot_k, dtype=np.float64)
    knot_P = np.asarray(knot_P, dtype=np.float64)
    nd = w.shape[0]
    ng = nd ** 3
    Lc = L / nd
    k2 = _k2(nd, L)
    inv = np.zeros_like(k2)
    inv[k2 > 0] = 1.0 / k2[k2 > 0]
    kmod = np.sqrt(k2)
    lk = np.log(np.maximum(kmod, 1e-300))
    W = np.fft.rfftn(w)
    p = knot_power(kmod, knot_k, knot_P)
    A = np.sqrt(p / ng)
    A[0, 0, 0] = 0.0
    irf = lambda X: np.fft.irfftn(X, s=(nd,) * 3, axes=(0, 1, 2)) * ng
    Normx, Normk = 1.0 / np.sqrt(L ** 3), np.sqrt(L ** 3) / ng
    phi1 = irf(-W * A * inv)
    S1 = [-Normx * _d6(phi1, a, Lc) for a in range(3)]
    S = list(S1)
    if do_2lpt:
        xx, yy, zz = _d6(S1[0], 0, Lc), _d6(S1[1], 1, Lc), _d6(S1[2], 2, Lc)
        xy, xz, yz = _d6(S1[0], 1, Lc), _d6(S1[0], 2, Lc), _d6(S1[1], 2, Lc)
        sig = xx * yy + xx * zz + yy * zz - xy ** 2 - xz ** 2 - yz ** 2
        phi2 = irf(-np.fft.rfftn(sig) * Normk * inv)
        Omz = Om0 * (1 + z) ** 3 / (Om0 * (1 + z) ** 3 + 1 - Om0)
        c2 = -3.0 / 7.0 * Omz ** (-1.0 / 143.0)
        S = [S1[a] + c2 * Normx * _d6(phi2, a, Lc) for a in range(3)]
    q = (np.arange(nd) + 0.5) * Lc
    pos = np.stack(np.broadcast_arrays(q[:, None, None] + S[0], q[None, :, None] + S[1], q[None, None, :] + S[2]), -1)
    pos = np.where(pos >= L, pos - L, pos)
    pos = np.where(pos < 0, pos + L, pos).reshape(-1, 3)
    grid = orc.cic(pos, nd, L)
    X = np.fft.rfftn(grid)
    b, wc = _bins(nd, L, Nk, kmin, kmax)
    Nrm = (L / nd ** 2) ** 1.5
    F2 = np.abs(X * Nrm / wc) ** 2
    m = b >= 0
    n = np.bincount(b[m], minlength=Nk).astype(np.float64)
    Pb = np.bincount(b[m], weights=F2[m], minlength=Nk) / np.maximum(n, 1)
    T = np.asarray(target, dtype=np.float64)
    var = np.where(n > 0, 2 * T * T / np.maximum(n, 1), 0.0)
    ok = (n > 0) & (var > 0)
    loss = float(np.sum((Pb[ok] - T[ok]) ** 2 / var[ok]))
    gP = np.where(ok, 2 * (Pb - T) / np.where(ok, var, 1), 0.0)
    # P(k) and r2c adjoints
    gX = np.zeros_like(X)
    gX[m] = (2 * gP[b[m]] / n[b[m]]) * (Nrm / wc[m]) ** 2 * X[m]
    h = np.ones(X.shape)
    h[..., 1:nd // 2] = 0.5
    ggrid = irf(gX * h)
    # CIC adjoint
    Ld = L / nd
    qd = pos / Ld
    c = np.minimum(np.floor(qd).astype(np.int64), nd - 1)
    d = qd - (c + 0.5)
    sg = np.where(d >= 0, 1, -1)
    dx = np.abs(d)
    t = 1 - dx
    lo, hi = c, (c + sg) % nd
    gpos = np.zeros_like(pos)
    G = lambda a, bb, cc: ggrid[a, bb, cc]
    for ax in range(3):
        o = [a for a in range(3) if a != ax]
        acc = 0.0
        for s1 in (0, 1):
            for s2 in (0, 1):
                idx_hi = [None] * 3
                idx_lo = [None] * 3
                idx_hi[ax], idx_lo[ax] = hi[:, ax], lo[:, ax]
                for s, oa in zip((s1, s2), o):
                    idx_hi[oa] = idx_lo[oa] = hi[:, oa] if s else lo[:, oa]
                wgt = (dx[:, o[0]] if s1 else t[:, o[0]]) * (dx[:, o[1]] if s2 else t[:, o[1]])
                acc = acc + (G(*idx_hi) - G(*idx_lo)) * wgt
        gpos[:, ax] = sg[:, ax] / Ld * acc
    gS = [gpos[:, a].reshape(nd, nd, nd) for a in range(3)]
    D = lambda f, a: _d6(f, a, Lc)
    gS1 = list(gS)
    if do_2lpt:
        gphi2 = -c2 * Normx * sum(D(gS[a], a) for a in range(3))
        gsig = irf(-np.fft.rfftn(gphi2) * Normk * inv)
        gxx, gyy, gzz = gsig * (yy + zz), gsig * (xx + zz), gsig * (xx + yy)
        gxy, gxz, gyz = -2 * gsig * xy, -2 * gsig * xz, -2 * gsig * yz
        gS1 = [gS[0] - (D(gxx, 0) + D(gxy, 1) + D(gxz, 2)), gS[1] - (D(gyy, 1) + D(gyz, 2)), gS[2] - D(gzz, 2)]
    gphi1 = Normx * sum(D(gS1[a], a) for a in range(3))
    V = np.fft.rfftn(gphi1)
    cfac = np.ones(V.shape)
    cfac[..., 1:nd // 2] = 2.0
    gdelta = cfac * (-V * inv)
    gw = irf(-A * V * inv)
    gA = np.real(np.conj(W) * gdelta)
    # knots: p = exp(interp(log k)); dA/dP_i = A / 2 dl/dP_i
    lkn = np.log(knot_k)
    gk = np.zeros(knot_k.size)
    msk = A > 0
    l = lk[msk]
    i0 = np.clip(np.searchsorted(lkn, l, side="right") - 1, 0, knot_k.size - 2)
    tt = np.clip((l - lkn[i0]) / (lkn[i0 + 1] - lkn[i0]), 0.0, 1.0)
    cc = 0.5 * gA[msk] * A[msk]
    np.add.at(gk, i0, cc * (1 - tt) / knot_P[i0])
    np.add.at(gk, i0 + 1, cc * tt / knot_P[i0 + 1])
    return loss, gw, gk
