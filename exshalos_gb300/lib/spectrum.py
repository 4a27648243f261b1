"""Mirror of the reference extension pyexshalos.lib.spectrum
(src/spectrum/spectrum.c) for the functions on the mock path.

Arguments keep the reference's positional order and meaning.
"""
import numpy as np

from .. import _capi


def check_precision():
    """sizeof(fft_real): 4, the grids are float32 (spectrum.c:41-43)."""
    return int(_capi.load().exh_check_precision())


def grid_compute(pos, vel, mass, nmass, type, ntype, nd, L, Om0, z, direction, window, R, R_times,
                 interlacing, folds, verbose, nthreads, stream=None):
    """Density contrast grid [ntype, interlacing+1, nd, nd, nd] (spectrum.c:46-108).

    One unit-mass tracer type with CIC, no interlacing and no redshift-space
    shift runs the dedicated CIC kernel; every other combination (NGP, CIC,
    Sphere, Exp windows, masses, several types, interlacing, a shift along
    x/y/z, folds) runs the general assignment.  The positions passed in are
    not modified (the reference shifts them in place for redshift space).
    stream: a CUDA stream handle (int) for the device work, None for the
    default stream."""
    pos = np.ascontiguousarray(pos, dtype=np.float32).reshape(-1, 3)
    npart = pos.shape[0]
    nd, ntype, interlacing, direction = int(nd), int(ntype), int(interlacing), int(direction)
    window, folds = int(window), int(folds)
    weighted = int(nmass) != 0 and mass is not None
    if window not in (1, 2, 3, 4):
        raise ValueError("window must be 1 (NGP), 2 (CIC), 3 (Sphere) or 4 (Exp)")
    L_ = _capi.load()
    grid = _capi.host_empty((ntype, interlacing + 1, nd, nd, nd), np.float32)
    if ntype == 1 and interlacing == 0 and direction == -1 and window == 2 and not weighted:
        _capi.check(L_.exh_grid_compute(_capi.context(), _capi.ptr(pos), npart, nd, float(L) / folds, 2, 1,
                                        _capi.ptr(grid), _capi.EXH_MEM_HOST, stream))
        return grid
    v = np.ascontiguousarray(vel, dtype=np.float32).reshape(-1, 3) if direction != -1 else None
    if direction != -1 and (v is None or v.shape[0] != npart):
        raise ValueError("a redshift-space shift needs one velocity per tracer")
    m = np.ascontiguousarray(mass, dtype=np.float32).reshape(-1) if weighted else None
    t = np.ascontiguousarray(type, dtype=np.int32).reshape(-1) if ntype > 1 else None
    if (m is not None and m.size != npart) or (t is not None and t.size != npart):
        raise ValueError("mass and type need one entry per tracer")
    _capi.check(L_.exh_grid_compute_ex(_capi.context(), _capi.ptr(pos), _capi.ptr(v), _capi.ptr(m), _capi.ptr(t),
                                       npart, ntype, nd, float(L), float(Om0), float(z), direction, window, float(R),
                                       float(R_times), interlacing, folds, _capi.ptr(grid), _capi.EXH_MEM_HOST,
                                       stream))
    return grid


def power_compute(grid, ntype, nd, L, window, R, interlacing, Nk, k_min, k_max, l_max, direction, verbose,
                  nthreads, stream=None):
    """{"k", "Pk", "Nk"} (spectrum.c:111-197); Pk shaped [ntype (ntype + 1) / 2, l_max / 2 + 1, Nk]
    (auto and cross spectra in the order (0,0), (1,0), (1,1), ...; even
    multipoles).  One grid, l_max = 0, no interlacing and windows 0-2 run
    the fused single-spectrum kernel; other options the general one.  stream:
    a CUDA stream handle (int) for the device work, None for the default
    stream."""
    g = np.ascontiguousarray(grid, dtype=np.float32)
    nd, ntype, interlacing, l_max = int(nd), int(ntype), int(interlacing), int(l_max)
    window, direction, Nk = int(window), int(direction), int(Nk)
    if g.size != ntype * (interlacing + 1) * nd ** 3:
        raise ValueError("grid size does not match ntype, interlacing and nd")
    nps, ls = ntype * (ntype + 1) // 2, l_max // 2 + 1
    k = np.zeros(Nk, dtype=np.float32)
    P = np.zeros((nps, ls, Nk), dtype=np.float32)
    cnt = np.zeros(Nk, dtype=np.int64)
    L_ = _capi.load()
    if ntype == 1 and interlacing == 0 and l_max == 0 and window in (0, 1, 2):
        _capi.check(L_.exh_power_compute(_capi.context(), _capi.ptr(g), nd, float(L), window, Nk, float(k_min),
                                         float(k_max), _capi.ptr(k), _capi.ptr(P), _capi.ptr(cnt),
                                         _capi.EXH_MEM_HOST, stream))
    else:
        _capi.check(L_.exh_power_compute_ex(_capi.context(), _capi.ptr(g), ntype, nd, float(L), window, float(R),
                                            interlacing, Nk, float(k_min), float(k_max), l_max, direction,
                                            _capi.ptr(k), _capi.ptr(P), _capi.ptr(cnt), _capi.EXH_MEM_HOST, stream))
    return {"k": k, "Pk": P, "Nk": cnt}


def abundance_compute(Mh_array, Mmin, Mmax, Nm, Lc, ndx, ndy, ndz, verbose):
    """{"Mh", "dn", "dn_err"}: differential abundance of a halo catalogue
    (spectrum.c:535-600, abundance.c:4-36) in Nm log-mass bins; Mmin or
    Mmax < 0 take the catalogue's range widened by 1e-4."""
    M = np.ascontiguousarray(Mh_array, dtype=np.float32).reshape(-1)
    Nm = int(Nm)
    out = {"Mh": np.zeros(Nm, dtype=np.float32), "dn": np.zeros(Nm, dtype=np.float32),
           "dn_err": np.zeros(Nm, dtype=np.float32)}
    _capi.check(_capi.load().exh_abundance_compute(_capi.context(), _capi.ptr(M), M.size, float(Mmin), float(Mmax),
                                                   Nm, float(Lc), int(ndx), int(ndy), int(ndz),
                                                   _capi.ptr(out["Mh"]), _capi.ptr(out["dn"]),
                                                   _capi.ptr(out["dn_err"]), _capi.EXH_MEM_HOST, None))
    return out
