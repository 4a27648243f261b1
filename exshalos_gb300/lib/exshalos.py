"""Mirror of the reference extension pyexshalos.lib.exshalos
(src/exshalos/exshalos.c) for the functions on the mock path.

Arguments keep the reference's positional order and meaning
(exshalos.c:52, 518, 718).  Failures raise exceptions where the reference
prints and exits: ValueError for invalid sizes, MemoryError, RuntimeError for
CUDA errors and for halos that outgrow the sigma(M) table, and
NotImplementedError for options the GPU path does not build (R_max < 1e5,
OUT_PROF).
"""
import numpy as np

from .. import _capi


def check_precision():
    """sizeof(fft_real): 4, the grids are float32 (exshalos.c:41-43)."""
    return int(_capi.load().exh_check_precision())


def _params(**kw):
    return _capi.default_params(**kw)


def _fetch_catalogue(nh, ng, want_vel=False, want_grid=False, want_pos=False, want_flag=False, nd=None, stream=None):
    L = _capi.load()
    # every array is filled completely by exh_halos_fetch
    he = _capi.host_empty
    out = {
        "posh": he((nh, 3), np.float32),
        "Mh": he(nh, np.float32),
        "x": he((nh, 3), np.int32),
        "count": he(nh, np.int32),
    }
    velh = he((nh, 3), np.float32) if want_vel else None
    grid = he(nd, np.float32) if want_grid else None
    pos = he((ng, 3), np.float32) if want_pos else None
    vel = he((ng, 3), np.float32) if (want_pos and want_vel) else None
    flag = he(nd, np.int64) if want_flag else None
    _capi.check(L.exh_halos_fetch(_capi.context(), _capi.ptr(out["posh"]), _capi.ptr(velh), _capi.ptr(out["Mh"]),
                                  _capi.ptr(out["x"]), _capi.ptr(out["count"]), _capi.ptr(grid), _capi.ptr(pos),
                                  _capi.ptr(vel), _capi.ptr(flag), _capi.EXH_MEM_HOST, stream))
    if velh is not None:
        out["velh"] = velh
    if grid is not None:
        out["grid"] = grid
    if pos is not None:
        out["pos"] = pos
    if vel is not None:
        out["vel"] = vel
    if flag is not None:
        out["flag"] = flag
    return out


def halos_box_from_pk(k, P, R_max, Ndx, Ndy, Ndz, Lc, seed, k_smooth, Om0, redshift, dc, Nmin, a, beta, alpha,
                      fixed, phase, OUT_DEN, OUT_LPT, OUT_VEL, DO_2LPT, OUT_FLAG, OUT_PROF, verbose, nthreads,
                      _catalogue=False, field_stream="taus", stream=None):
    """Halo catalogue from a linear P(k) (exshalos.c:710-940 / box.c:4-68).

    Returns the reference's dictionary: "posh", "Mh" always; "velh" with
    OUT_VEL; "pos" (and "vel" with OUT_VEL) with OUT_LPT; "flag" with OUT_FLAG;
    "grid" with OUT_DEN.  The reference returns an empty dict for a few flag
    combinations it does not list (e.g. OUT_DEN alone); here every requested
    output is returned.  With _catalogue=True the Lagrangian centre cells "x"
    and member counts "count" are added.  field_stream: "taus" (default: the
    reference's own gsl_rng_taus stream, the reference's realisation for this
    seed) or "philox" (one counter-based block per Fourier mode).  stream: a
    CUDA stream handle (int) for the device work, None for the default
    stream; the call returns with the host outputs filled either way.
    """
    k = np.ascontiguousarray(k, dtype=np.float32)
    P = np.ascontiguousarray(P, dtype=np.float32)
    if k.shape != P.shape or k.ndim != 1:
        raise ValueError("k and P must be 1-D arrays of the same length")
    prm = _params(R_max=float(R_max), ndx=int(Ndx), ndy=int(Ndy), ndz=int(Ndz), Lc=float(Lc), seed=int(seed),
                  k_smooth=float(k_smooth), Om0=float(Om0), redshift=float(redshift), dc=float(dc), Nmin=int(Nmin),
                  a=float(a), beta=float(beta), alpha=float(alpha), fixed=int(fixed), phase=float(phase),
                  OUT_DEN=int(OUT_DEN), OUT_LPT=int(OUT_LPT), OUT_VEL=int(OUT_VEL), DO_2LPT=int(DO_2LPT),
                  OUT_FLAG=int(OUT_FLAG), OUT_PROF=int(OUT_PROF), verbose=int(verbose), nthreads=int(nthreads),
                  field_stream=_capi.field_stream_code(field_stream))
    L = _capi.load()
    import ctypes as C
    nh = C.c_int64(0)
    _capi.check(L.exh_halos_box_from_pk(_capi.context(), _capi.ptr(k), _capi.ptr(P), k.size, prm, C.byref(nh),
                                        stream))
    nd = (int(Ndx), int(Ndy), int(Ndz))
    ng = nd[0] * nd[1] * nd[2]
    out = _fetch_catalogue(nh.value, ng, want_vel=bool(OUT_VEL), want_grid=bool(OUT_DEN), want_pos=bool(OUT_LPT),
                           want_flag=bool(OUT_FLAG), nd=nd, stream=stream)
    if not _catalogue:
        out.pop("x")
        out.pop("count")
    return out


def halos_box_from_grid(k, P, grid, S, V, Lc, k_smooth, Om0, redshift, dc, Nmin, a, beta, alpha, OUT_LPT, OUT_VEL,
                        DO_2LPT, OUT_FLAG, IN_disp, OUT_PROF, verbose, nthreads, _catalogue=False):
    """Halo catalogue of a given density grid (exshalos.c:943-1103 /
    box.c:71-150): the halos of `grid`, displaced by (2)LPT computed from the
    grid or, with IN_disp, by the given displacements S[ng, 3] (and
    velocities V with OUT_VEL).  Returns "posh", "Mh"; "velh" with OUT_VEL;
    "pos" (and "vel") with OUT_LPT; "flag" with OUT_FLAG."""
    if int(OUT_PROF):
        raise NotImplementedError("Lagrangian profiles (OUT_PROF) are not built")
    d = np.ascontiguousarray(grid, dtype=np.float32)
    if d.ndim != 3:
        raise ValueError("grid must be a 3-D array")
    k = np.ascontiguousarray(k, dtype=np.float32)
    P = np.ascontiguousarray(P, dtype=np.float32)
    nd = tuple(int(x) for x in d.shape)
    ng = nd[0] * nd[1] * nd[2]
    Sd = Vd = None
    if int(IN_disp):
        Sd = np.ascontiguousarray(S, dtype=np.float32).reshape(ng, 3)
        if int(OUT_VEL):
            if V is None:
                raise ValueError("OUT_VEL with given displacements needs V")
            Vd = np.ascontiguousarray(V, dtype=np.float32).reshape(ng, 3)
    prm = _params(ndx=nd[0], ndy=nd[1], ndz=nd[2], Lc=float(Lc), k_smooth=float(k_smooth), Om0=float(Om0),
                  redshift=float(redshift), dc=float(dc), Nmin=int(Nmin), a=float(a), beta=float(beta),
                  alpha=float(alpha), OUT_LPT=int(OUT_LPT), OUT_VEL=int(OUT_VEL), DO_2LPT=int(DO_2LPT),
                  OUT_FLAG=int(OUT_FLAG), verbose=int(verbose), nthreads=int(nthreads))
    import ctypes as C
    nh = C.c_int64(0)
    _capi.check(_capi.load().exh_halos_box_from_grid(_capi.context(), _capi.ptr(d), nd[0], nd[1], nd[2], _capi.ptr(k),
                                                     _capi.ptr(P), k.size, _capi.ptr(Sd), _capi.ptr(Vd), prm,
                                                     _capi.EXH_MEM_HOST, C.byref(nh), None))
    out = _fetch_catalogue(nh.value, ng, want_vel=bool(OUT_VEL), want_pos=bool(OUT_LPT), want_flag=bool(OUT_FLAG),
                           nd=nd)
    if not _catalogue:
        out.pop("x")
        out.pop("count")
    return out


def find_halos(delta, k, P, Lc, Om0, redshift, dc, Nmin, a, beta, alpha, OUT_FLAG, OUT_PROF, verbose,
               _catalogue=False, setup_fp64=0):
    """Halos of a given density grid (exshalos.c:509-610): "posh" are the
    Lagrangian centres Lc (x + 1/2), "Mh" the masses, "flag" with OUT_FLAG."""
    if int(OUT_PROF):
        raise NotImplementedError("Lagrangian profiles (OUT_PROF) are not built")
    d = np.ascontiguousarray(delta, dtype=np.float32)
    if d.ndim != 3:
        raise ValueError("delta must be a 3-D grid")
    k = np.ascontiguousarray(k, dtype=np.float32)
    P = np.ascontiguousarray(P, dtype=np.float32)
    prm = _params(Lc=float(Lc), Om0=float(Om0), redshift=float(redshift), dc=float(dc), Nmin=int(Nmin),
                  a=float(a), beta=float(beta), alpha=float(alpha), verbose=int(verbose), setup_fp64=int(setup_fp64))
    L = _capi.load()
    import ctypes as C
    nh = C.c_int64(0)
    nd = d.shape
    _capi.check(L.exh_find_halos(_capi.context(), _capi.ptr(d), nd[0], nd[1], nd[2], _capi.ptr(k), _capi.ptr(P),
                                 k.size, prm, _capi.EXH_MEM_HOST, C.byref(nh), None))
    out = _fetch_catalogue(nh.value, d.size, want_flag=bool(OUT_FLAG), nd=nd)
    if not _catalogue:
        out.pop("x")
        out.pop("count")
    return out


def density_grid_compute(k, P, R_max, Ndx, Ndy, Ndz, Lc, outk, seed, fixed, phase, k_smooth, verbose, nthreads,
                         field_stream="taus"):
    """Gaussian density grid (exshalos.c:46-121): {"grid"}.  The Fourier
    modes are regenerated where they are needed and are not returned
    (outk raises NotImplementedError).  field_stream as halos_box_from_pk."""
    if int(outk):
        raise NotImplementedError("returning the Fourier-space grid (outk) is not built")
    k = np.ascontiguousarray(k, dtype=np.float32)
    P = np.ascontiguousarray(P, dtype=np.float32)
    prm = _params(R_max=float(R_max), ndx=int(Ndx), ndy=int(Ndy), ndz=int(Ndz), Lc=float(Lc), seed=int(seed),
                  fixed=int(fixed), phase=float(phase), k_smooth=float(k_smooth),
                  field_stream=_capi.field_stream_code(field_stream))
    grid = _capi.host_empty((int(Ndx), int(Ndy), int(Ndz)), np.float32)
    _capi.check(_capi.load().exh_density_grid_compute(_capi.context(), _capi.ptr(k), _capi.ptr(P), k.size, prm,
                                                      _capi.ptr(grid), _capi.EXH_MEM_HOST, None))
    return {"grid": grid}


def smoothing_ladder(k, P, R_max, Ndx, Ndy, Ndz, Lc, seed=12345, n_radii=50, Om0=0.31, z=0.0, dc=1.686, a=1.0,
                     beta=0.0, alpha=0.0, fixed=0, phase=0.0, k_smooth=100000.0, out=None, stream=None,
                     field_stream="taus"):
    """First-crossing map of the top-hat smoothing ladder of the Gaussian
    field that density_grid_compute makes with the same arguments.

    Returns {"cross": u8 (Ndx, Ndy, Ndz) (index of the largest crossing
    radius, 255 = none), "R": radii, "B": barriers}.  With ``out`` a CUDA
    uint8 tensor of ng elements, the map is written there on the device.
    """
    k = np.ascontiguousarray(k, dtype=np.float32)
    P = np.ascontiguousarray(P, dtype=np.float32)
    prm = _params(R_max=float(R_max), ndx=int(Ndx), ndy=int(Ndy), ndz=int(Ndz), Lc=float(Lc), seed=int(seed),
                  Om0=float(Om0), redshift=float(z), dc=float(dc), a=float(a), beta=float(beta), alpha=float(alpha),
                  fixed=int(fixed), phase=float(phase), k_smooth=float(k_smooth),
                  field_stream=_capi.field_stream_code(field_stream))
    R = np.zeros(int(n_radii), dtype=np.float32)
    B = np.zeros(int(n_radii), dtype=np.float32)
    if out is None:
        cross = _capi.host_empty((int(Ndx), int(Ndy), int(Ndz)), np.uint8)
        dst, mem = _capi.ptr(cross), _capi.EXH_MEM_HOST
    else:
        cross, dst, mem = out, out.data_ptr(), _capi.EXH_MEM_DEVICE
    _capi.check(_capi.load().exh_smoothing_ladder(_capi.context(), _capi.ptr(k), _capi.ptr(P), k.size, prm,
                                                  int(n_radii), float(R_max), dst, _capi.ptr(R), _capi.ptr(B), mem,
                                                  stream))
    return {"cross": cross, "R": R, "B": B}


def batch_run(k, P, nds, seeds, Lc=2.0, Nk_pk=64, lanes=8, field_stream="philox", **params):
    """Halos and the 64-bin (Nk_pk) CIC power spectrum of the halos for many
    boxes of uneven size, each from its own Philox seed (field_stream
    "taus": the reference's stream instead), scheduled over ``lanes``
    streams (1 = the plain loop).  ``params`` are fields of the halo
    parameters shared by every box (Om0, DO_2LPT, a, beta, ...).

    Returns {"nh": i64[n], "k": f32[n, Nk_pk], "Pk": f32[n, Nk_pk], "Nk": i64[n, Nk_pk],
    "status": i32[n]}: a box whose halo masses leave the mass-function
    tables (where the reference aborts) has status 4 (EXH_E_RANGE) and nh -1;
    the others still run.
    """
    k = np.ascontiguousarray(k, dtype=np.float32)
    P = np.ascontiguousarray(P, dtype=np.float32)
    nds = np.asarray(nds, dtype=np.int64).ravel()
    seeds = np.asarray(seeds, dtype=np.int64).ravel()
    if nds.shape != seeds.shape:
        raise ValueError("nds and seeds must have the same length")
    n = nds.size
    items = (_capi.BatchItem * max(n, 1))()
    for i in range(n):
        items[i].nd = int(nds[i])
        items[i].seed = int(seeds[i])
    prm = _params(Lc=float(Lc), field_stream=_capi.field_stream_code(field_stream), **params)
    out = {"nh": np.zeros(n, dtype=np.int64), "k": np.zeros((n, Nk_pk), dtype=np.float32),
           "Pk": np.zeros((n, Nk_pk), dtype=np.float32), "Nk": np.zeros((n, Nk_pk), dtype=np.int64),
           "status": np.zeros(n, dtype=np.int32)}
    _capi.check(_capi.load().exh_batch_run(_capi.context(), _capi.ptr(k), _capi.ptr(P), k.size, prm, items, n,
                                           int(Nk_pk), int(lanes), _capi.ptr(out["nh"]), _capi.ptr(out["k"]),
                                           _capi.ptr(out["Pk"]), _capi.ptr(out["Nk"]), _capi.ptr(out["status"])))
    return out


def halo_tables():
    """Sigma(M), barrier and mass-function tables of the last halo call."""
    import ctypes as C
    L = _capi.load()
    nc, nr = C.c_int(0), C.c_int(0)
    ctx = _capi.context()
    _capi.check(L.exh_halo_tables(ctx, C.byref(nc), C.byref(nr), None, None, None, None))
    sig = np.zeros(nc.value, dtype=np.float32)
    btab = np.zeros(nc.value, dtype=np.float32)
    M = np.zeros(nr.value)
    Int = np.zeros(nr.value)
    _capi.check(L.exh_halo_tables(ctx, C.byref(nc), C.byref(nr), _capi.ptr(sig), _capi.ptr(btab), _capi.ptr(M),
                                  _capi.ptr(Int)))
    return {"Sig_grid": sig, "Btab": btab, "M": M, "Int": Int, "Ncells": nc.value}
