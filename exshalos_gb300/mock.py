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
    field_stream: str = "taus",
    stream: Optional[int] = None,
) -> Dict[str, np.ndarray]:
    """Halo catalogue in a periodic box from a linear power spectrum.

    Keys: "posh" (halo positions, Mpc/h), "Mh" (masses, Msun/h), and with the
    flags "velh", "pos", "vel", "flag", "grid".  field_stream picks the random
    stream of the Gaussian field: "taus" (default: the reference's
    gsl_rng_taus stream seeded with `seed`, drawn in its loop order, so the
    reference's realisation for that seed, up to float rounding of the
    transforms) or "philox" (a counter-based Philox block per Fourier mode
    keyed by `seed`).  stream: a CUDA stream handle (int) for the device work
    (None: the default stream); the call returns with the outputs filled.
    """
    precision = _ext.check_precision()
    if precision == 4:
        k = np.asarray(k, dtype=np.float32)
        P = np.asarray(P, dtype=np.float32)
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
        np.int32(nthreads), field_stream=field_stream, stream=stream)


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
        grid = np.asarray(grid, dtype=np.float32)
        k = np.asarray(k, dtype=np.float32)
        P = np.asarray(P, dtype=np.float32)
        Lc, Om0, z = np.float32(Lc), np.float32(Om0), np.float32(z)
        k_smooth, delta_c = np.float32(k_smooth), np.float32(delta_c)
        a, beta, alpha = np.float32(a), np.float32(beta), np.float32(alpha)
        if S is not None:
            S = np.asarray(S, dtype=np.float32)
        if V is not None:
            V = np.asarray(V, dtype=np.float32)
    return _ext.halos_box_from_grid(
        k, P, grid, S, V, Lc, k_smooth, Om0, z, delta_c, np.int32(Nmin), a, beta, alpha, np.int32(OUT_LPT),
        np.int32(OUT_VEL), np.int32(DO_2LPT), np.int32(OUT_FLAG), np.int32(In_disp), np.int32(OUT_PROF),
        np.int32(verbose), np.int32(nthreads))


def Generate_Galaxies_from_Halos(
    posh: np.ndarray,
    Mh: np.ndarray,
    velh: Optional[np.ndarray] = None,
    Ch: Optional[np.ndarray] = None,
    nd: int = 256,
    ndx: int = 0,
    ndy: int = 0,
    ndz: int = 0,
    Lc: float = 2.0,
    Om0: float = 0.31,
    z: float = 0.0,
    logMmin: float = 13.25424743,
    siglogM: float = 0.26461332,
    logM0: float = 13.28383025,
    logM1: float = 14.32465146,
    alpha: float = 1.00811277,
    sigma: float = 0.5,
    Deltah: float = -1.0,
    seed: int = 12345,
    OUT_VEL: bool = False,
    OUT_FLAG: bool = False,
    verbose: bool = False,
) -> Dict[str, np.ndarray]:
    """Galaxy catalogue of a halo catalogue (mock.py:357-507): Zheng (2005)
    occupations, centrals at the halo centres, satellites around them.

    Returns {"posg"[, "velg" with OUT_VEL][, "flag" with OUT_FLAG]}; flag is
    -i for the central of halo i and i for its satellites.  As in the
    reference, ndx/ndy/ndz fall back to nd only when None: with the default 0
    the box length along that axis is 0 and satellite positions are not
    wrapped into the box.
    """
    from .lib import hod as _hod

    In_C = Ch is not None
    posh = np.asarray(posh, dtype=np.float32)
    if velh is not None:
        velh = np.asarray(velh, dtype=np.float32)
    Mh = np.asarray(Mh, dtype=np.float32)
    if In_C:
        Ch = np.asarray(Ch, dtype=np.float32)
    if ndx is None:
        ndx = nd
    if ndy is None:
        ndy = nd
    if ndz is None:
        ndz = nd
    return _hod.populate_halos(
        posh, velh, Mh, Ch, np.float32(Lc), np.float32(Om0), np.float32(z), np.int32(ndx), np.int32(ndy),
        np.int32(ndz), np.float32(logMmin), np.float32(siglogM), np.float32(logM0), np.float32(logM1),
        np.float32(alpha), np.float32(sigma), np.float32(Deltah), np.int32(seed), np.int32(OUT_VEL),
        np.int32(OUT_FLAG), np.int32(In_C), np.int32(verbose))


def Split_Galaxies(
    Mh: np.ndarray,
    Flag: np.ndarray,
    params_cen: np.ndarray = np.array([37.10265321, -5.07596644, 0.17497771]),
    params_sat: np.ndarray = np.array([19.84341938, -2.8352781, 0.10443049]),
    seed: int = 12345,
    verbose: bool = False,
) -> np.ndarray:
    """Type of each galaxy from polynomial occupations in log10(Mh)
    (mock.py:519-576): int32, +-(1..ntypes), negative for centrals."""
    from .lib import hod as _hod

    Mh = np.asarray(Mh, dtype=np.float32)
    params_cen = np.asarray(params_cen, dtype=np.float32)
    params_sat = np.asarray(params_sat, dtype=np.float32)
    if len(params_cen.shape) == 1:
        params_cen = params_cen.reshape([1, len(params_cen)])
    if len(params_sat.shape) == 1:
        params_sat = params_sat.reshape([1, len(params_sat)])
    if params_cen.shape[0] != params_sat.shape[0]:
        raise ValueError(
            "Different number of types of galaxies for the centrals and satellites! %d != %d!"
            % (params_cen.shape[0], params_sat.shape[0]))
    return _hod.split_galaxies(Mh, Flag, params_cen, params_sat, np.int32(seed), np.int32(verbose))
