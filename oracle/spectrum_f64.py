"""ORACLE — test infrastructure only.

FP64 numpy restatement of the general tracer grid and power spectrum of the
reference's spectrum module, used to check exh_grid_compute_ex and
exh_power_compute_ex:

* tracer_grid: Tracer_Grid (src/spectrum/gridmodule.c:146-376) with the
  NGP / CIC / Sphere / Exp assignments of gridmodule.c:7-113, masses, tracer
  types, interlacing, the redshift-space shift of gridmodule.c:167-170 and
  folding; positions wrapped by cysumf (src/spectrum/spectrum_h.c:17-27).
* power: Compute_gridk (src/spectrum/spectrum_h.c:83-167) and Power_Spectrum
  (src/spectrum/powermodule.c:4-108): window deconvolution, interlacing,
  every auto and cross spectrum, even Legendre multipoles, the mode-skip
  rule and the float bin index of the reference.
"""
import numpy as np
from numpy.polynomial import legendre


def _wrap(x, L):
    """cysumf in float32: subtract or add L until x is in [0, L)"""
    x = np.asarray(x, dtype=np.float32).copy()
    L = np.float32(L)
    for _ in range(1024):
        hi = x >= L
        if not hi.any():
            break
        x[hi] = x[hi] - L
    for _ in range(1024):
        lo = x < 0
        if not lo.any():
            break
        x[lo] = x[lo] + L
    return x


def _deposit(grid, post, m, nd, L, window, R, R_times):
    """adds the tracers at post (n, 3, float32) with weights m (n,) to grid;
    returns the deposited weight per tracer.  Cell indices, CIC offsets and
    the Sphere/Exp distances follow the reference's float arithmetic; the
    weights are accumulated in FP64"""
    f32 = np.float32
    Ld = f32(f32(L) / f32(nd))
    xt = np.minimum(np.floor((post / Ld).astype(f32)).astype(np.int64), nd - 1)
    flat = grid.reshape(-1)
    if window == 1:
        np.add.at(flat, (xt[:, 0] * nd + xt[:, 1]) * nd + xt[:, 2], m)
        return m.copy()
    if window == 2:
        d = ((post / Ld).astype(f32) - (xt.astype(f32) + f32(0.5))).astype(f32)
        sg = np.where(d >= 0, 1, -1)
        dx = np.abs(d).astype(np.float64)
        t = (f32(1) - np.abs(d)).astype(np.float64)
        for a in (0, 1):
            for b in (0, 1):
                for c in (0, 1):
                    ix = (xt[:, 0] + (sg[:, 0] if a else 0)) % nd
                    iy = (xt[:, 1] + (sg[:, 1] if b else 0)) % nd
                    iz = (xt[:, 2] + (sg[:, 2] if c else 0)) % nd
                    w = (dx[:, 0] if a else t[:, 0]) * (dx[:, 1] if b else t[:, 1]) * (dx[:, 2] if c else t[:, 2])
                    np.add.at(flat, (ix * nd + iy) * nd + iz, m * w)
        return m.copy()
    R, R_times, Lf = f32(R), f32(R_times), f32(L)
    Rr = R if window == 3 else f32(R * R_times)
    times = int(np.floor(f32(0.5) + f32(Rr / Ld)))
    r2max = f32(R * R) if window == 3 else f32(f32(f32(R * R) * R_times) * R_times)
    M = np.zeros(post.shape[0])
    for i in range(-times, times + 1):
        for j in range(-times, times + 1):
            for k in range(-times, times + 1):
                c = (xt + np.array([i, j, k])) % nd
                d = (post - ((c.astype(f32) + f32(0.5)) * Ld).astype(f32)).astype(f32)
                d = np.where(d > Lf / f32(2), (Lf - d).astype(f32), d)
                d = np.where(d < -Lf / f32(2), (Lf + d).astype(f32), d)
                r2 = ((d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]).astype(f32) + d[:, 2] * d[:, 2]).astype(f32)
                ok = r2 <= r2max
                w = m if window == 3 else m * np.exp(-0.5 * r2.astype(np.float64) / float(R) / float(R))
                w = np.where(ok, w, 0.0)
                np.add.at(flat, (c[:, 0] * nd + c[:, 1]) * nd + c[:, 2], w)
                M += w
    return M


def tracer_grid(pos, nd, L, vel=None, mass=None, types=None, ntype=1, Om0=0.31, z=0.0, direction=-1, window=2,
                R=4.0, R_times=5.0, interlacing=0, folds=1):
    """grid[ntype][interlacing + 1][nd][nd][nd] = rho / (M / nd^3) - 1"""
    pos = np.asarray(pos, dtype=np.float32).reshape(-1, 3).copy()
    Lf = np.float32(np.float32(L) / np.float32(folds))
    n = pos.shape[0]
    if direction != -1:
        # float shift vel * ((1 + z)^3 / H(Om0, z)), gridmodule.c:3-5,167-170
        vfac = np.float32((1 + float(z)) ** 3 / (100.0 * np.sqrt(float(Om0) * (1 + float(z)) ** 3 + (1 - float(Om0)))))
        v = np.asarray(vel, dtype=np.float32).reshape(-1, 3)[:, direction]
        pos[:, direction] = (pos[:, direction] + (v * vfac).astype(np.float32)).astype(np.float32)
    post = _wrap(pos, Lf)
    m = np.ones(n) if mass is None else np.asarray(mass, dtype=np.float64).reshape(-1)
    ty = np.zeros(n, dtype=np.int64) if types is None else np.asarray(types, dtype=np.int64).reshape(-1)
    ng = nd ** 3
    out = np.zeros((ntype, interlacing + 1, nd, nd, nd))
    for t in range(ntype):
        sel = ty == t
        Mt = _deposit(out[t, 0], post[sel], m[sel], nd, Lf, window, R, R_times).sum()
        out[t, 0] = out[t, 0] / (Mt / ng) - 1.0
        if interlacing:
            ps = _wrap((post[sel] + (-(Lf / np.float32(nd)) / np.float32(2))).astype(np.float32), Lf)
            M2 = _deposit(out[t, 1], ps, m[sel], nd, Lf, window, R, R_times).sum()
            out[t, 1] = out[t, 1] / (M2 / ng) - 1.0
    return out


def _modes(nd, L):
    f32 = np.float32
    kn = f32(2 * np.pi / L)
    i = np.arange(nd)
    s = np.where(2 * i < nd, i, i - nd).astype(f32)
    kx = (s * kn)[:, None, None]
    ky = (s * kn)[None, :, None]
    kz = (s[: nd // 2 + 1] * kn)[None, None, :].copy()
    kz[..., nd // 2] = f32(-(nd // 2)) * kn
    return kx, ky, kz


def _window(kx, ky, kz, Lb, R, window):
    kx, ky, kz = (np.asarray(a, dtype=np.float64) for a in (kx, ky, kz))
    sinc = lambda x: np.where(x != 0, np.sin(x) / np.where(x != 0, x, 1), 1.0)
    if window == 0:
        return np.ones(np.broadcast(kx, ky, kz).shape)
    if window == 1:
        return sinc(kx * Lb / 2) * sinc(ky * Lb / 2) * sinc(kz * Lb / 2)
    if window == 2:
        return (sinc(kx * Lb / 2) * sinc(ky * Lb / 2) * sinc(kz * Lb / 2)) ** 2
    km = np.sqrt(kx * kx + ky * ky + kz * kz)
    if window == 3:
        with np.errstate(divide="ignore", invalid="ignore"):
            return 3.0 / km / km / R / R * (sinc(km * R) - np.cos(km * R))
    return np.exp(-(kx * kx + ky * ky + kz * kz) * R * R / 2)


def power(grid, L, ntype=1, window=2, R=4.0, interlacing=0, Nk=25, kmin=None, kmax=None, l_max=0, direction=-1):
    """{"k", "Pk" [npairs][l_max/2+1][Nk], "Nk"} in FP64"""
    nd = grid.shape[-1]
    f32 = np.float32
    if kmin is None:
        kmin = 2 * np.pi / L
    if kmax is None:
        kmax = np.pi / L * nd
    g = np.asarray(grid, dtype=np.float64).reshape(ntype, interlacing + 1, nd, nd, nd)
    kx, ky, kz = _modes(nd, L)
    # the reference's float wave numbers in Compute_gridk use kz = k kn for k < nd/2 and (k - nd) kn
    Lb = L / nd
    Nrm = (L / nd ** 2) ** 1.5
    W = _window(kx, ky, kz, Lb, R, window)
    gk = []
    with np.errstate(divide="ignore", invalid="ignore"):
        for t in range(ntype):
            o1 = np.fft.rfftn(g[t, 0])
            if interlacing:
                o2 = np.fft.rfftn(g[t, 1])
                th = (np.asarray(kx, dtype=np.float64) + ky + kz) * Lb / 2
                v = (o1 + o2 * np.exp(-1j * th)) / 2 * Nrm / W
            else:
                v = o1 * Nrm / W
            gk.append(v)
    k2 = (kx * kx + ky * ky).astype(f32) + (kz * kz).astype(f32)
    kmod = np.sqrt(k2.astype(f32)).astype(f32)
    dk = f32((f32(kmax) - f32(kmin)) / f32(Nk))
    b = np.floor(((kmod - f32(kmin)).astype(f32) / dk).astype(f32)).astype(np.int64)
    I, J, K = np.meshgrid(np.arange(nd), np.arange(nd), np.arange(nd // 2 + 1), indexing="ij")
    skip = ((K == 0) | (K == nd // 2)) & (((I > nd // 2) & (J > nd // 2)) | (I == 0) | (I == nd // 2) | (J == 0) |
                                        (J == nd // 2) | ((I > nd // 2) & (J < nd // 2)))
    ok = (~skip) & (b >= 0) & (b < Nk)
    with np.errstate(divide="ignore", invalid="ignore"):
        kd = np.broadcast_to([kx, ky, kz][direction], kmod.shape).astype(np.float64) if direction >= 0 else None
        mu = kd / kmod.astype(np.float64) if direction >= 0 else np.zeros(kmod.shape)
    ls = l_max // 2 + 1
    n = np.bincount(b[ok], minlength=Nk).astype(np.float64)
    kmean = np.bincount(b[ok], weights=kmod[ok].astype(np.float64), minlength=Nk)
    pairs = [(l, m) for l in range(ntype) for m in range(l + 1)]
    P = np.zeros((len(pairs), ls, Nk))
    for q, (l, m) in enumerate(pairs):
        c = (gk[l].real * gk[m].real + gk[l].imag * gk[m].imag)
        for s in range(ls):
            coef = np.zeros(2 * s + 1)
            coef[2 * s] = 1.0
            w = c * legendre.legval(mu, coef)
            P[q, s] = np.bincount(b[ok], weights=w[ok], minlength=Nk)
    for s in range(ls):
        P[:, s] = np.where(n > 0, (4 * s + 1) * P[:, s] / np.maximum(n, 1), 0.0)
    return {"k": np.where(n > 0, kmean / np.maximum(n, 1), 0.0), "Pk": P, "Nk": n.astype(np.int64)}


def abundance(Mh, Mmin, Mmax, Nm, Lc, ndx, ndy, ndz):
    """Measure_Abundance (src/spectrum/abundance.c:4-36) with the range rule
    of abundance_compute (src/spectrum/spectrum.c:566-578); the mean masses in
    FP64"""
    f32 = np.float32
    M = np.asarray(Mh, dtype=f32).reshape(-1)
    if Mmin < 0:
        Mmin = f32(min(float(M.min()) if M.size else 1e20, 1e20) * 0.9999)
    if Mmax < 0:
        Mmax = f32(float(M.max()) * 1.0001)
    dlnM = f32((np.log(float(Mmax)) - np.log(float(Mmin))) / Nm)
    ind = np.floor((np.log(M.astype(np.float64)) - np.log(float(Mmin))) / float(dlnM)).astype(np.int64)
    ok = (ind > 0) & (ind < Nm)
    N = np.bincount(ind[ok], minlength=Nm)[:Nm]
    S = np.bincount(ind[ok], weights=M[ok].astype(np.float64), minlength=Nm)[:Nm]
    V = f32(f32(f32(Lc) * f32(ndx)) * f32(f32(Lc) * f32(ndy))) * f32(f32(Lc) * f32(ndz))
    dn = (N.astype(f32) / V / dlnM).astype(f32)
    err = (np.sqrt(N.astype(np.float64)) / float(V) / float(dlnM)).astype(f32)
    Mm = np.where(N > 0, S / np.maximum(N, 1), 0.0).astype(f32)
    return {"Mh": Mm, "dn": dn, "dn_err": err}
