"""Halo mocks on the GPU — mirror of pyexshalos.mock (pyexshalos/mock.py).

Generate_Halos_Box_from_Pk (mock.py:11-184) and Generate_Halos_Box_from_Grid
(mock.py:188-353) keep the reference's signatures, defaults, input checks,
float32 casting and return dictionaries; the work runs in libexh_gb300.so.
"""
from typing import Dict, Optional

import numpy as np

from .lib import exshalos as _ext


def Generate_Halos_Box_from_Pk(
    k: np.ndarray,
    P: np.ndarray,
    R_max: float = 100000.0,
    nd: int = 256,
    ndx: int = 0,
    ndy: int = 0,
    ndz: int = 0,
    Lc: float = 2.0,
    Om0: float = 0.31,
    z: float = 0.0,
    k_smooth: float = 10000.0,
    delta_c: float = -1.0,
    Nmin: int = 1,
    a: float = 1.0,
    beta: float = 0.0,
    alpha: float = 0.0,
    seed: int = 12345,
    fixed: bool = False,
    phase: float = 0.0,
    OUT_DEN: bool = False,
    OUT_LPT: bool = False,
    OUT_VEL: bool = False,
    OUT_PROF: bool = False,
    DO_2LPT: bool = False,
    OUT_FLAG: bool = False,
    verbose: bool = False,
    nthreads: int = 1,
) -> Dict[str, np.ndarray]:
    """Halo catalogue in a periodic box from a linear power spectrum.

    Keys: "posh" (halo positions, Mpc/h), "Mh" (masses, Msun/h), and with the
    flags "velh", "pos", "vel", "flag", "grid".  The Gaussian field is drawn
    from a counter-based Philox stream keyed by `seed` (one block per Fourier
    mode), so a realisation is reproducible and independent of the launch
    shape; it is not the reference's GSL taus stream.
    """
    precision = _ext.check_precision()
    if precision == 4:
        k = np.asarray(k).astype("float32")
        P = np.asarray(P).astype("float32")
        R_max, Lc, Om0, z = np.float32(R_max), np.float32(Lc), np.float32(Om0), np.float32(z)
        k_smooth, delta_c = np.float32(k_smooth), np.float32(delta_c)
        a, beta, alpha, phase = np.float32(a), np.float32(beta), np.float32(alpha), np.float32(phase)
    if ndx <= 0:
        ndx = nd
    if ndy <= 0:
        ndy = nd
    if ndz <= 0:
        ndz = nd
    return _ext.halos_box_from_pk(
        k, P, R_max, np.int32(ndx), np.int32(ndy), np.int32(ndz), Lc, np.int32(seed), k_smooth, Om0, z,
        delta_c, np.int32(Nmin), a, beta, alpha, np.int32(fixed), phase, np.int32(OUT_DEN), np.int32(OUT_LPT),
        np.int32(OUT_VEL), np.int32(DO_2LPT), np.int32(OUT_FLAG), np.int32(OUT_PROF), np.int32(verbose),
        np.int32(nthreads))


def Generate_Halos_Box_from_Grid(
    grid: np.ndarray,
    k: np.ndarray,
    P: np.ndarray,
    S: Optional[np.ndarray] = None,
    V: Optional[np.ndarray] = None,
    Lc: float = 2.0,
    Om0: float = 0.31,
    z: float = 0.0,
    k_smooth: float = 10000.0,
    delta_c: float = -1.0,
    Nmin: int = 1,
    a: float = 1.0,
    beta: float = 0.0,
    alpha: float = 0.0,
    OUT_LPT: bool = False,
    OUT_VEL: bool = False,
    DO_2LPT: bool = False,
    OUT_FLAG: bool = False,
    OUT_PROF: bool = False,
    verbose: bool = False,
    nthreads: int = 1,
) -> Dict[str, np.ndarray]:
    """Halo catalogue of a given density grid.

    The halos of `grid` are displaced by (2)LPT computed from the grid or, if
    `S` is given, by those displacements (one row per grid cell; `V` the
    velocities, needed with OUT_VEL).  Keys: "posh", "Mh"; "velh" with
    OUT_VEL; "pos" (and "vel") with OUT_LPT; "flag" with OUT_FLAG.
    """
    In_disp = S is not None
    ng = grid.shape[0] * grid.shape[1] * grid.shape[2]
    if In_disp:
        if S.shape[0] != ng:
            raise ValueError("The number of particles in S is different of the number of grid cells!")
        if S.shape[1] != 3:
            raise ValueError("The number of components of S is different from 3!")
        if V is not None:
            if V.shape[0] != ng:
                raise ValueError("The number of particles in V is different of the number of grid cells!")
            if V.shape[1] != 3:
                raise ValueError("The number of components of V is different from 3!")
    precision = _ext.check_precision()
    if precision == 4:
        grid = np.asarray(grid).astype("float32")
        k = np.asarray(k).astype("float32")
        P = np.asarray(P).astype("float32")
        Lc, Om0, z = np.float32(Lc), np.float32(Om0), np.float32(z)
        k_smooth, delta_c = np.float32(k_smooth), np.float32(delta_c)
        a, beta, alpha = np.float32(a), np.float32(beta), np.float32(alpha)
        if S is not None:
            S = np.asarray(S).astype("float32")
        if V is not None:
            V = np.asarray(V).astype("float32")
    return _ext.halos_box_from_grid(
        k, P, grid, S, V, Lc, k_smooth, Om0, z, delta_c, np.int32(Nmin), a, beta, alpha, np.int32(OUT_LPT),
        np.int32(OUT_VEL), np.int32(DO_2LPT), np.int32(OUT_FLAG), np.int32(In_disp), np.int32(OUT_PROF),
        np.int32(verbose), np.int32(nthreads))
