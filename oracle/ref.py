"""REFERENCE BUILD ctypes binding — test infrastructure only.

Calls into the reference's own C (oracle/_ref/, built by oracle/ref_build.py
from the reference tree against the FFTW3/GSL stand-ins of oracle/ref_shim/)
so that tests/test_oracle_ref.py can check the oracle's restatement against
the reference's loops.  Nothing in the product package imports this module.
"""
import ctypes as C

import numpy as np

from . import ref_build

_LIBS = {}
_P = C.c_void_p


class RangeError(RuntimeError):
    """A spline evaluated outside its knots, where the reference's GSL aborts."""


def available():
    """True when the reference tree is present and the libraries build."""
    try:
        return ref_build.build() is not None
    except RuntimeError:
        return False


def lib(name):
    if name not in _LIBS:
        paths = ref_build.build()
        if paths is None:
            raise RuntimeError("the reference tree is not available")
        _LIBS[name] = C.CDLL(paths[name])
    return _LIBS[name]


def _ptr(a):
    return a.ctypes.data_as(_P) if a is not None else None


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _status(st):
    if st == 5:
        raise RangeError("the reference evaluated a spline outside its knots")
    if st:
        raise RuntimeError(f"reference call failed ({st})")


def halos_box_from_pk(k, P, nd, Lc, seed, Om0=0.31, z=0.0, dc=-1.0, Nmin=1, a=1.0, beta=0.0, alpha=0.0, fixed=0,
                      phase=0.0, k_smooth=10000.0, do_2lpt=0, keep_pos=False, nthreads=1):
    """Generate_Halos_Box_from_Pk (box.c:4-68): {"delta", "flag", "x",
    "count", "Mh", "posh"} and "pos" with keep_pos."""
    L = lib("exshalos")
    k, P = _f32(k), _f32(P)
    ng = nd ** 3
    delta = np.zeros(ng, dtype=np.float32)
    flag = np.zeros(ng, dtype=np.int64)
    S = np.zeros(3 * ng, dtype=np.float32) if keep_pos else None
    cap = ng // 2 + 1
    hx = np.zeros(3 * cap, dtype=np.int32)
    hc = np.zeros(cap, dtype=np.int32)
    Mh = np.zeros(cap, dtype=np.float32)
    posh = np.zeros(3 * cap, dtype=np.float32)
    nh = C.c_size_t(0)
    st = L.ref_halos_box_from_pk(_ptr(k), _ptr(P), k.size, nd, C.c_float(Lc), C.c_float(Om0), C.c_float(z),
                                 C.c_float(dc), Nmin, C.c_float(a), C.c_float(beta), C.c_float(alpha), seed, fixed,
                                 C.c_float(phase), C.c_float(k_smooth), do_2lpt, nthreads, _ptr(delta), _ptr(flag),
                                 _ptr(S), C.c_size_t(cap), C.byref(nh), _ptr(hx), _ptr(hc), _ptr(Mh), _ptr(posh))
    _status(st)
    n = nh.value
    out = {"delta": delta.reshape(nd, nd, nd), "flag": flag, "x": hx[:3 * n].reshape(n, 3), "count": hc[:n],
           "Mh": Mh[:n], "posh": posh[:3 * n].reshape(n, 3)}
    if keep_pos:
        out["pos"] = S.reshape(ng, 3)
    return out


def density_grid(k, P, nd, Lc, seed, fixed=0, phase=0.0, k_smooth=100000.0, nthreads=1):
    """Compute_Den (density_grid.c:71-217): (delta, modes [nd, nd, nd/2+1, 2])."""
    L = lib("exshalos")
    k, P = _f32(k), _f32(P)
    delta = np.zeros((nd, nd, nd), dtype=np.float32)
    modes = np.zeros((nd, nd, nd // 2 + 1, 2), dtype=np.float32)
    _status(L.ref_density_grid(_ptr(k), _ptr(P), k.size, nd, C.c_float(Lc), seed, fixed, C.c_float(phase),
                               C.c_float(k_smooth), nthreads, _ptr(delta), _ptr(modes)))
    return delta, modes


def find_halos(delta, k, P, Lc, seed, Om0=0.31, z=0.0, dc=-1.0, Nmin=1, a=1.0, beta=0.0, alpha=0.0, nthreads=1):
    """Find_Halos (find_halos.c:479-563) on a given grid."""
    L = lib("exshalos")
    delta = _f32(delta)
    nd = delta.shape[0]
    k, P = _f32(k), _f32(P)
    ng = delta.size
    flag = np.zeros(ng, dtype=np.int64)
    cap = ng // 2 + 1
    hx = np.zeros(3 * cap, dtype=np.int32)
    hc = np.zeros(cap, dtype=np.int32)
    Mh = np.zeros(cap, dtype=np.float32)
    nh = C.c_size_t(0)
    _status(L.ref_find_halos(_ptr(delta), _ptr(k), _ptr(P), k.size, nd, C.c_float(Lc), C.c_float(Om0), C.c_float(z),
                             C.c_float(dc), Nmin, C.c_float(a), C.c_float(beta), C.c_float(alpha), seed, nthreads,
                             _ptr(flag), C.c_size_t(cap), C.byref(nh), _ptr(hx), _ptr(hc), _ptr(Mh)))
    n = nh.value
    return {"nh": n, "flag": flag, "x": hx[:3 * n].reshape(n, 3), "count": hc[:n], "Mh": Mh[:n]}


def sigma_barrier(k, P, nd, Lc, Ncells, Om0=0.31, z=0.0, dc=-1.0, a=1.0, beta=0.0, alpha=0.0):
    """Compute_Sig (find_halos.c:16-44) and Barrier (:200-212): (Sig_grid, Btab)."""
    L = lib("exshalos")
    k, P = _f32(k), _f32(P)
    sig = np.zeros(Ncells, dtype=np.float32)
    btab = np.zeros(Ncells, dtype=np.float32)
    _status(L.ref_sigma_barrier(_ptr(k), _ptr(P), k.size, nd, C.c_float(Lc), C.c_float(Om0), C.c_float(z),
                                C.c_float(dc), C.c_float(a), C.c_float(beta), C.c_float(alpha), Ncells, _ptr(sig),
                                _ptr(btab)))
    return sig, btab


def lpt(modes, nd, Lc, flag, x, count, do_2lpt=1, Om0=0.31, z=0.0, k_smooth=10000.0, nthreads=1):
    """Compute_1LPT / Compute_2LPT / Compute_Posh / Compute_Pos (lpt.c:4-255)
    on given modes and labelling: {"posh", "pos"}."""
    L = lib("exshalos")
    modes = _f32(modes)
    flag = np.ascontiguousarray(flag, dtype=np.int64).reshape(-1)
    x = np.ascontiguousarray(x, dtype=np.int32).reshape(-1)
    count = np.ascontiguousarray(count, dtype=np.int32)
    nh = count.size
    posh = np.zeros(3 * max(nh, 1), dtype=np.float32)
    S = np.zeros(3 * nd ** 3, dtype=np.float32)
    _status(L.ref_lpt(_ptr(modes), nd, C.c_float(Lc), C.c_float(Om0), C.c_float(z), do_2lpt, C.c_float(k_smooth),
                      nthreads, _ptr(flag), C.c_size_t(nh), _ptr(x), _ptr(count), _ptr(posh), _ptr(S)))
    return {"posh": posh[:3 * nh].reshape(nh, 3), "pos": S.reshape(-1, 3)}


def cic(pos, nd, L):
    """Tracer_Grid with the CIC window (gridmodule.c:146-211), one thread."""
    pos = _f32(pos).reshape(-1)
    grid = np.zeros((nd, nd, nd), dtype=np.float32)
    lib("spectrum").ref_cic(_ptr(pos), C.c_size_t(pos.size // 3), nd, C.c_float(L), _ptr(grid))
    return grid


def power(grid, L, window=2, Nk=25, kmin=None, kmax=None, nthreads=1):
    """Power_Spectrum (powermodule.c:4-108), one grid, l_max = 0."""
    grid = _f32(grid)
    nd = grid.shape[-1]
    kmin = np.float32(2 * np.pi / L) if kmin is None else np.float32(kmin)
    kmax = np.float32(np.pi / L * nd) if kmax is None else np.float32(kmax)
    km = np.zeros(Nk)
    Pk = np.zeros(Nk)
    cnt = np.zeros(Nk, dtype=np.int64)
    lib("spectrum").ref_power(_ptr(grid), nd, C.c_float(L), window, Nk, C.c_float(kmin), C.c_float(kmax), nthreads,
                              _ptr(km), _ptr(Pk), _ptr(cnt))
    return {"k": km, "Pk": Pk, "Nk": cnt}
