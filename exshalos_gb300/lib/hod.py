"""Mirror of the reference extension pyexshalos.lib.hod (src/hod/hod.c).

Arguments keep the reference's keyword list and meaning; the work runs in
libexh_gb300.so (exh_hod_populate / exh_hod_fetch / exh_hod_split).
"""
import numpy as np

from .. import _capi


def check_precision():
    """sizeof(fft_real): 4, the catalogues are float32 (hod.c:27-29)."""
    return int(_capi.load().exh_check_precision())


def populate_halos(posh_array, velh_array, Mh_array, Ch_array, Lc, Om0, redshift, ndx, ndy, ndz, logMmin, siglogM,
                   logM0, logM1, alpha, sigma, Deltah, seed, OUT_VEL, OUT_FLAG, IN_C, verbose):
    """{"posg"[, "velg"][, "flag"]} (hod.c:31-160): centrals at the halo
    centres (flag -i), satellites around them (flag i), halo by halo."""
    posh = np.ascontiguousarray(posh_array, dtype=np.float32).reshape(-1, 3)
    Mh = np.ascontiguousarray(Mh_array, dtype=np.float32).reshape(-1)
    nh = Mh.size
    if posh.shape[0] != nh:
        raise ValueError("posh needs one row per halo")
    out_vel = int(OUT_VEL) != 0
    vel = None
    if out_vel:
        if velh_array is None:
            raise ValueError("OUT_VEL needs the halo velocities")
        vel = np.ascontiguousarray(velh_array, dtype=np.float32).reshape(-1, 3)
        if vel.shape[0] != nh:
            raise ValueError("velh needs one row per halo")
    C = None
    if int(IN_C) != 0:
        C = np.ascontiguousarray(Ch_array, dtype=np.float32).reshape(-1)
        if C.size != nh:
            raise ValueError("Ch needs one entry per halo")
    p = _capi.HodParams(float(Lc), float(Om0), float(redshift), int(ndx), int(ndy), int(ndz), float(logMmin),
                        float(siglogM), float(logM0), float(logM1), float(alpha), float(sigma), float(Deltah),
                        int(seed))
    L_ = _capi.load()
    ctx = _capi.context()
    ng = _capi.C.c_int64(0)
    _capi.check(L_.exh_hod_populate(ctx, _capi.ptr(posh), _capi.ptr(vel), _capi.ptr(Mh), _capi.ptr(C), nh,
                                    _capi.C.byref(p), int(out_vel), _capi.C.byref(ng), _capi.EXH_MEM_HOST, None))
    n = int(ng.value)
    out = {"posg": np.zeros((n, 3), dtype=np.float32)}
    if out_vel:
        out["velg"] = np.zeros((n, 3), dtype=np.float32)
    if int(OUT_FLAG) != 0:
        out["flag"] = np.zeros(n, dtype=np.int64)
    _capi.check(L_.exh_hod_fetch(ctx, _capi.ptr(out["posg"]), _capi.ptr(out.get("velg")), _capi.ptr(out.get("flag")),
                                 _capi.EXH_MEM_HOST, None))
    if int(verbose):
        print("%d galaxies in %d halos" % (n, nh))
    return out


def split_galaxies(Mh_array, Flag_array, params_cen_array, params_sat_array, seed, verbose):
    """int32 type per galaxy (hod.c:163-211): +-(1..ntypes), negative for
    centrals; ntypes = rows of the parameter arrays + 1."""
    Mh = np.ascontiguousarray(Mh_array, dtype=np.float32).reshape(-1)
    flag = np.ascontiguousarray(Flag_array, dtype=np.int64).reshape(-1)
    pc = np.ascontiguousarray(params_cen_array, dtype=np.float32)
    ps = np.ascontiguousarray(params_sat_array, dtype=np.float32)
    if pc.ndim != 2 or ps.ndim != 2 or pc.shape[0] != ps.shape[0]:
        raise ValueError("Different number of types of galaxies for the centrals and satellites!")
    out = np.zeros(flag.size, dtype=np.int32)
    _capi.check(_capi.load().exh_hod_split(_capi.context(), _capi.ptr(Mh), Mh.size, _capi.ptr(flag), flag.size,
                                           _capi.ptr(pc), _capi.ptr(ps), pc.shape[0] + 1, pc.shape[1], ps.shape[1],
                                           int(seed), _capi.ptr(out), _capi.EXH_MEM_HOST, None))
    return out
