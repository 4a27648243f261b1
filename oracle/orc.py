"""ORACLE ctypes binding — test infrastructure only.

Loads the C restatement built by oracle/build.py and exposes numpy-level
helpers to tests/, __graft_entry__.smoke() and bench.py.  Nothing in the
product package imports this module.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

_LIBS = {}


class RangeError(RuntimeError):
    """A halo mass outside the mass-function splines: the reference's
    gsl_spline_eval aborts there (find_halos.c:472-474)."""


class Params(C.Structure):
    _fields_ = [
        ("Om0", C.c_float), ("redshift", C.c_float), ("dc", C.c_float), ("rhoc", C.c_float),
        ("Hz", C.c_float), ("Omz", C.c_float), ("rhomz", C.c_float), ("Dv", C.c_float),
        ("Lc", C.c_float), ("Mcell", C.c_float), ("L", C.c_float * 3), ("Mtot", C.c_float),
        ("kl", C.c_float * 3), ("Normx", C.c_float), ("Normk", C.c_float),
        ("nd", C.c_int * 3), ("nz2", C.c_int), ("nmin", C.c_int),
        ("ng", C.c_size_t),
        ("Nmin", C.c_int), ("seed", C.c_int), ("DO_EB", C.c_int),
        ("a", C.c_float), ("beta", C.c_float), ("alpha", C.c_float),
        ("Lc_d", C.c_double), ("L_d", C.c_double * 3), ("kl_d", C.c_double * 3),
        ("Normx_d", C.c_double), ("Normk_d", C.c_double), ("Omz_d", C.c_double),
        ("Hz_d", C.c_double),
    ]


class Result(C.Structure):
    _fields_ = [
        ("nh", C.c_size_t), ("np", C.c_size_t),
        ("Mh", C.c_void_p), ("posh", C.c_void_p), ("hx", C.c_void_p), ("hcount", C.c_void_p),
        ("delta", C.c_void_p), ("flag", C.c_void_p), ("S", C.c_void_p),
        ("t_field", C.c_double), ("t_halos", C.c_double), ("t_lpt", C.c_double),
    ]


def lib(prec="f64"):
    if prec not in _LIBS:
        paths = _build.build()
        L = C.CDLL(paths[prec])
        L.orc_spline_eval.restype = C.c_double
        L.orc_taus_uniform.restype = C.c_double
        L.orc_gaussian.restype = C.c_double
        L.orc_taus_get.restype = C.c_uint32
        L.orc_count_peaks.restype = C.c_size_t
        L.orc_find_peaks.restype = C.c_size_t
        L.orc_grow_halos.restype = C.c_size_t
        L.orc_find_halos.restype = C.c_size_t
        L.orc_barrier.restype = C.c_float
        _LIBS[prec] = L
    return _LIBS[prec]


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def real_dtype(prec):
    return np.float32 if prec == "f32" else np.float64


def set_threads(n, prec="f64"):
    lib(prec).orc_set_threads(int(n))


def make_params(nd, Lc, Om0=0.31, z=0.0, dc=-1.0, Nmin=1, a=1.0, beta=0.0, alpha=0.0, seed=12345,
                prec="f64"):
    L = lib(prec)
    p = Params()
    nd3 = nd if isinstance(nd, (tuple, list)) else (nd, nd, nd)
    L.orc_set_cosmology(C.byref(p), C.c_float(Om0), C.c_float(z), C.c_float(dc))
    if L.orc_set_box(C.byref(p), int(nd3[0]), int(nd3[1]), int(nd3[2]), C.c_float(Lc)):
        raise ValueError("unsupported cell size")
    L.orc_set_barrier(C.byref(p), int(Nmin), C.c_float(a), C.c_float(beta), C.c_float(alpha), int(seed))
    return p


def cells_in_spheres(lmax=10000):
    out = np.zeros(9000, dtype=np.int32)
    n = lib().orc_cells_in_spheres(int(lmax), _ptr(out), out.size)
    return out[:n].copy()


def fft_r2c_3d(x, prec="f64"):
    x = np.ascontiguousarray(x, dtype=real_dtype(prec))
    nx, ny, nz = x.shape
    out = np.zeros((nx, ny, nz // 2 + 1, 2), dtype=real_dtype(prec))
    lib(prec).orc_fft_r2c_3d(nx, ny, nz, _ptr(x), _ptr(out))
    return out[..., 0] + 1j * out[..., 1]


def fft_c2r_3d(xk, nz, prec="f64"):
    nx, ny, nc = xk.shape
    a = np.ascontiguousarray(np.stack([xk.real, xk.imag], axis=-1), dtype=real_dtype(prec))
    out = np.zeros((nx, ny, nz), dtype=real_dtype(prec))
    lib(prec).orc_fft_c2r_3d(nx, ny, nz, _ptr(a), _ptr(out))
    return out


def sigma_tables(p, k, P, prec64=0, prec="f64"):
    L = lib(prec)
    k = np.ascontiguousarray(k, dtype=np.float32)
    P = np.ascontiguousarray(P, dtype=np.float32)
    nc = L.orc_ncells(C.byref(p))
    sig = np.zeros(nc, dtype=np.float32)
    M = np.zeros(k.size, dtype=np.float64)
    Int = np.zeros(k.size, dtype=np.float64)
    r = L.orc_sigma_tables(C.byref(p), _ptr(k), _ptr(P), k.size, int(prec64), _ptr(sig), _ptr(M), _ptr(Int))
    if r < 0:
        raise RuntimeError("sigma tables failed")
    btab = np.zeros(nc, dtype=np.float32)
    L.orc_barrier_table(C.byref(p), _ptr(sig), nc, _ptr(btab))
    return {"Sig_grid": sig, "M": M, "Int": Int, "Btab": btab, "Ncells": nc}


def field_modes(p, k, P, stream=1, fixed=0, phase=0.0, prec="f64"):
    L = lib(prec)
    nd = tuple(p.nd)
    k = np.ascontiguousarray(k, dtype=np.float32)
    P = np.ascontiguousarray(P, dtype=np.float32)
    out = np.zeros((nd[0], nd[1], nd[2] // 2 + 1, 2), dtype=real_dtype(prec))
    r = L.orc_field_modes(C.byref(p), _ptr(k), _ptr(P), k.size, int(stream), int(fixed),
                          C.c_float(phase), C.c_float(1e5), _ptr(out))
    if r:
        raise RuntimeError(f"field synthesis failed ({r})")
    return out


def field_real(p, modes, prec="f64"):
    nd = tuple(p.nd)
    out = np.zeros(nd, dtype=real_dtype(prec))
    lib(prec).orc_field_real(C.byref(p), _ptr(np.ascontiguousarray(modes)), _ptr(out))
    return out


def find_halos(p, delta, tables, prec="f64"):
    """Find_Halos on a given float32 grid with given tables."""
    L = lib(prec)
    delta = np.ascontiguousarray(delta, dtype=np.float32)
    ng = delta.size
    npk = L.orc_count_peaks(C.byref(p), _ptr(delta))
    cap = max(int(npk), 1)
    flag = np.zeros(ng, dtype=np.int64)
    hx = np.zeros(3 * cap, dtype=np.int32)
    hc = np.zeros(cap, dtype=np.int32)
    Mh = np.zeros(cap, dtype=np.float32)
    npo = C.c_size_t(0)
    btab = np.ascontiguousarray(tables["Btab"], dtype=np.float32)
    M = np.ascontiguousarray(tables["M"], dtype=np.float64)
    Int = np.ascontiguousarray(tables["Int"], dtype=np.float64)
    nh = L.orc_find_halos(C.byref(p), _ptr(delta), _ptr(btab), int(tables["Ncells"]), _ptr(M), _ptr(Int),
                          M.size, _ptr(flag), _ptr(hx), _ptr(hc), _ptr(Mh), C.c_size_t(cap), C.byref(npo))
    if nh == (1 << 64) - 2:
        raise RangeError("oracle halo finder: a halo mass outside the mass-function splines")
    if nh >= (1 << 63):
        raise RuntimeError("oracle halo finder failed")
    return {"nh": nh, "np": npo.value, "x": hx[:3 * nh].reshape(nh, 3), "count": hc[:nh],
            "Mh": Mh[:nh], "flag": flag}


def peaks_sorted(p, delta, prec="f64"):
    """Peaks in the reference's quicksort order (ascending density)."""
    L = lib(prec)
    delta = np.ascontiguousarray(delta, dtype=np.float32)
    npk = L.orc_count_peaks(C.byref(p), _ptr(delta))
    pk = np.zeros(max(npk, 1), dtype=[("x", np.int32, 3), ("den", np.float32)])
    L.orc_find_peaks(C.byref(p), _ptr(delta), _ptr(pk))
    unsorted = pk[:npk].copy()
    if npk > 0:
        L.orc_quicksort_peaks(_ptr(pk), C.c_longlong(0), C.c_longlong(npk - 1))
    return unsorted, pk[:npk]


def quicksort_peaks(pk):
    pk = np.ascontiguousarray(pk.copy())
    if pk.size > 0:
        lib().orc_quicksort_peaks(_ptr(pk), C.c_longlong(0), C.c_longlong(pk.size - 1))
    return pk


def cic(pos, nd, L, prec="f64"):
    pos = np.ascontiguousarray(pos, dtype=real_dtype(prec)).reshape(-1, 3)
    grid = np.zeros((nd, nd, nd), dtype=real_dtype(prec))
    lib(prec).orc_cic(_ptr(pos), C.c_size_t(pos.shape[0]), int(nd), C.c_float(L), _ptr(grid))
    return grid


def power(grid, L, window=2, Nk=25, kmin=None, kmax=None, prec="f64"):
    nd = grid.shape[-1]
    if kmin is None:
        kmin = 2.0 * np.pi / L
    if kmax is None:
        kmax = np.pi / L * nd
    g = np.ascontiguousarray(grid, dtype=real_dtype(prec))
    km = np.zeros(Nk)
    Pk = np.zeros(Nk)
    cnt = np.zeros(Nk, dtype=np.int64)
    lib(prec).orc_power(_ptr(g), int(nd), C.c_float(L), int(window), int(Nk), C.c_float(np.float32(kmin)),
                        C.c_float(np.float32(kmax)), _ptr(km), _ptr(Pk), _ptr(cnt))
    return {"k": km, "Pk": Pk, "Nk": cnt}


def halos_box_from_pk(k, P, nd=64, Lc=4.0, Om0=0.31, z=0.0, dc=-1.0, Nmin=1, a=1.0, beta=0.0,
                      alpha=0.0, seed=12345, stream=0, fixed=0, phase=0.0, k_smooth=10000.0,
                      do_2lpt=0, prec64=0, keep_S=0, prec="f32"):
    L = lib(prec)
    k = np.ascontiguousarray(k, dtype=np.float32)
    P = np.ascontiguousarray(P, dtype=np.float32)
    r = Result()
    st = L.orc_halos_box_from_pk(_ptr(k), _ptr(P), k.size, int(nd), C.c_float(Lc), C.c_float(Om0),
                                 C.c_float(z), C.c_float(dc), int(Nmin), C.c_float(a), C.c_float(beta),
                                 C.c_float(alpha), int(seed), int(stream), int(fixed), C.c_float(phase),
                                 C.c_float(k_smooth), int(do_2lpt), int(prec64), int(keep_S), C.byref(r))
    if st == 5:
        raise RangeError("oracle pipeline: a halo mass outside the mass-function splines")
    if st:
        raise RuntimeError(f"oracle pipeline failed ({st})")
    nh, ng = r.nh, nd ** 3
    rt = real_dtype(prec)

    def arr(ptr, n, dt):
        if not ptr or n == 0:
            return np.zeros(0, dtype=dt)
        return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(np.ctypeslib.as_ctypes_type(dt))), shape=(n,)).copy()

    out = {"nh": nh, "np": r.np, "Mh": arr(r.Mh, nh, np.float32),
           "posh": arr(r.posh, 3 * nh, rt).reshape(nh, 3), "x": arr(r.hx, 3 * nh, np.int32).reshape(nh, 3),
           "count": arr(r.hcount, nh, np.int32), "delta": arr(r.delta, ng, np.float32).reshape(nd, nd, nd),
           "flag": arr(r.flag, ng, np.int64),
           "t_field": r.t_field, "t_halos": r.t_halos, "t_lpt": r.t_lpt}
    if keep_S:
        out["pos"] = arr(r.S, 3 * ng, rt).reshape(ng, 3)
    L.orc_result_free(C.byref(r))
    return out


def grid_modes(p, delta, prec="f64"):
    """Compute_Denk (density_grid.c:220-235): Normk r2c(delta), as modes"""
    xk = fft_r2c_3d(delta, prec=prec) * (p.Normk_d if prec == "f64" else p.Normk)
    out = np.zeros(xk.shape + (2,), dtype=real_dtype(prec))
    out[..., 0] = xk.real
    out[..., 1] = xk.imag
    return out


def lpt_posh(p, k, P, flag, hx, hcount, do_2lpt=1, k_smooth=10000.0, stream=1, keep_pos=False, prec="f64",
             modes=None):
    """Compute_1LPT/Compute_2LPT/Compute_Posh (lpt.c) for a given halo
    labelling, on the field modes of the given stream (or given modes)."""
    L = lib(prec)
    rt = real_dtype(prec)
    if modes is None:
        modes = field_modes(p, k, P, stream=stream, prec=prec)
    # orc_lpt1 turns the modes into the potential in place: work on a copy
    modes = np.array(modes, dtype=rt, order="C", copy=True)
    nh = int(hcount.size)
    ng = int(p.ng)
    flag = np.ascontiguousarray(flag, dtype=np.int64).reshape(-1)
    posh = np.zeros((max(nh, 1), 3), dtype=rt)
    S = np.zeros((ng, 3), dtype=rt)
    L.orc_lpt1(C.byref(p), _ptr(modes), _ptr(flag), C.c_size_t(nh), C.c_float(k_smooth), _ptr(S), _ptr(posh))
    if do_2lpt:
        L.orc_lpt2(C.byref(p), _ptr(S), _ptr(flag), C.c_size_t(nh), C.c_float(k_smooth), int(keep_pos), _ptr(posh))
    hx = np.ascontiguousarray(hx, dtype=np.int32).reshape(-1)
    hc = np.ascontiguousarray(hcount, dtype=np.int32)
    L.orc_posh(C.byref(p), C.c_size_t(nh), _ptr(hx), _ptr(hc), _ptr(posh))
    out = {"posh": posh[:nh]}
    if keep_pos:
        L.orc_pos(C.byref(p), _ptr(S))
        out["pos"] = S
    return out


def ladder(p, modes, R, B, prec="f64"):
    """First-crossing map of the smoothing ladder on given modes."""
    R = np.ascontiguousarray(R, dtype=np.float32)
    B = np.ascontiguousarray(B, dtype=np.float32)
    out = np.zeros(tuple(p.nd), dtype=np.uint8)
    if lib(prec).orc_ladder(C.byref(p), _ptr(np.ascontiguousarray(modes)), R.size, _ptr(R), _ptr(B), _ptr(out)):
        raise RuntimeError("oracle ladder failed")
    return out


def populate_halos(posh, Mh, velh=None, Ch=None, Lc=2.0, z=0.0, nd=(0, 0, 0), logMmin=13.25424743,
                   siglogM=0.26461332, logM0=13.28383025, logM1=14.32465146, alpha=1.00811277, sigma=0.5,
                   seed=12345, out_vel=False, prec="f32"):
    """Galaxies of a halo catalogue on the reference's sequential taus stream:
    {"posg", "velg", "flag", "nsat", "ncen"} (nsat, ncen per halo)."""
    rt = real_dtype(prec)
    cr = C.c_float if prec == "f32" else C.c_double
    L = lib(prec)
    L.orc_populate_halos.restype = C.c_longlong
    posh = np.ascontiguousarray(posh, dtype=rt).reshape(-1, 3)
    Mh = np.ascontiguousarray(Mh, dtype=rt).reshape(-1)
    nh = Mh.size
    v = np.ascontiguousarray(velh, dtype=rt).reshape(-1, 3) if out_vel else None
    c = np.ascontiguousarray(Ch, dtype=rt).reshape(-1) if Ch is not None else None
    cap = 64 * max(nh, 1) + 1024
    while True:
        posg = np.zeros((cap, 3), dtype=rt)
        velg = np.zeros((cap, 3), dtype=rt) if out_vel else None
        flag = np.zeros(cap, dtype=np.int64)
        nsat = np.zeros(max(nh, 1), dtype=np.int32)
        ncen = np.zeros(max(nh, 1), dtype=np.int32)
        ng = L.orc_populate_halos(_ptr(posh), _ptr(v) if v is not None else None, _ptr(Mh),
                                  _ptr(c) if c is not None else None, C.c_longlong(nh), cr(Lc), cr(z),
                                  int(nd[0]), int(nd[1]), int(nd[2]), cr(logMmin), cr(siglogM), cr(logM0),
                                  cr(logM1), cr(alpha), cr(sigma), int(seed), int(bool(out_vel)),
                                  C.c_longlong(cap), _ptr(posg), _ptr(velg) if velg is not None else None,
                                  _ptr(flag), _ptr(nsat), _ptr(ncen))
        if ng == -1:
            cap *= 4
            continue
        if ng < 0:
            raise RuntimeError("oracle r(Eps) tables failed")
        out = {"posg": posg[:ng], "flag": flag[:ng], "nsat": nsat[:nh], "ncen": ncen[:nh]}
        if out_vel:
            out["velg"] = velg[:ng]
        return out


def split_galaxies(Mh, flag, params_cen, params_sat, seed=12345, prec="f32"):
    """Galaxy types (signed, as split_galaxies.c) on the reference's taus stream."""
    rt = real_dtype(prec)
    Mh = np.ascontiguousarray(Mh, dtype=rt).reshape(-1)
    flag = np.ascontiguousarray(flag, dtype=np.int64).reshape(-1)
    pc = np.ascontiguousarray(np.atleast_2d(params_cen), dtype=rt)
    ps = np.ascontiguousarray(np.atleast_2d(params_sat), dtype=rt)
    out = np.zeros(flag.size, dtype=np.int32)
    if lib(prec).orc_split_galaxies(C.c_longlong(flag.size), _ptr(Mh), C.c_longlong(Mh.size), _ptr(flag), _ptr(pc),
                                    _ptr(ps), pc.shape[0] + 1, pc.shape[1], ps.shape[1], int(seed), _ptr(out)):
        raise ValueError("a flag names a halo outside the catalogue")
    return out
