"""Mirror of the reference extension pyexshalos.lib.spectrum
(src/spectrum/spectrum.c) for the functions on the mock path.

Arguments keep the reference's positional order and meaning.  Options the
GPU path does not build (other windows, several tracer types, interlacing,
redshift-space shifts, multipoles, folding) raise NotImplementedError instead
of silently changing the result.
"""
import numpy as np

from .. import _capi


def check_precision():
    """sizeof(fft_real): 4, the grids are float32 (spectrum.c:41-43)."""
    return int(_capi.load().exh_check_precision())


def grid_compute(pos, vel, mass, nmass, type, ntype, nd, L, Om0, z, direction, window, R, R_times,
                 interlacing, folds, verbose, nthreads):
    """Density contrast grid [ntype, interlacing+1, nd, nd, nd] (spectrum.c:46-108)."""
    if int(nmass) != 0 or mass is not None:
        raise NotImplementedError("weighted tracers are not built")
    if int(ntype) != 1 or int(interlacing) != 0:
        raise NotImplementedError("one tracer type without interlacing is built")
    if int(direction) != -1:
        raise NotImplementedError("redshift-space shifts are not built")
    pos = np.ascontiguousarray(pos, dtype=np.float32).reshape(-1, 3)
    nd = int(nd)
    grid = np.empty((1, 1, nd, nd, nd), dtype=np.float32)
    L_ = _capi.load()
    _capi.check(L_.exh_grid_compute(_capi.context(), _capi.ptr(pos), pos.shape[0], nd, float(L), int(window),
                                    int(folds), _capi.ptr(grid), _capi.EXH_MEM_HOST, None))
    return grid


def power_compute(grid, ntype, nd, L, window, R, interlacing, Nk, k_min, k_max, l_max, direction, verbose,
                  nthreads):
    """{"k", "Pk", "Nk"} of one grid (spectrum.c:111-197); Pk shaped [1, 1, Nk]."""
    if int(ntype) != 1 or int(interlacing) != 0 or int(l_max) != 0:
        raise NotImplementedError("one tracer type, no interlacing and l_max = 0 are built")
    g = np.ascontiguousarray(grid, dtype=np.float32)
    nd = int(nd)
    if g.size != nd ** 3:
        raise ValueError("grid size does not match nd")
    Nk = int(Nk)
    k = np.zeros(Nk, dtype=np.float32)
    P = np.zeros((1, 1, Nk), dtype=np.float32)
    cnt = np.zeros(Nk, dtype=np.int64)
    L_ = _capi.load()
    _capi.check(L_.exh_power_compute(_capi.context(), _capi.ptr(g), nd, float(L), int(window), Nk, float(k_min),
                                     float(k_max), _capi.ptr(k), _capi.ptr(P), _capi.ptr(cnt),
                                     _capi.EXH_MEM_HOST, None))
    return {"k": k, "Pk": P, "Nk": cnt}
