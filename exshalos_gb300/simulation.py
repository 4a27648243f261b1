"""Density grids and power spectra on the GPU — mirror of
pyexshalos.simulation (pyexshalos/simulation.py:9-311)."""
from typing import Dict, Optional, Union

import numpy as np

from .lib import spectrum as _spec


def _window_code(window, allow_none):
    if window in ("NO", "no", "No", 0):
        return 0 if allow_none else None
    if window in ("NGP", "ngp", 1):
        return 1
    if window in ("CIC", "cic", 2):
        return 2
    if window in ("SPHERICAL", "spherical", 3):
        return 3
    if window in ("EXPONENTIAL", "exponential", 4):
        return 4
    return window


def _direction_code(direction):
    if direction is None or direction == -1:
        return -1
    if direction in ("x", "X", 0):
        return 0
    if direction in ("y", "Y", 1):
        return 1
    if direction in ("z", "Z", 2):
        return 2
    raise ValueError("Direction must be None, x, y or z!")


def Compute_Density_Grid(
    pos: np.ndarray,
    vel: Optional[np.ndarray] = None,
    mass: Optional[np.ndarray] = None,
    types: Optional[np.ndarray] = None,
    nd: int = 256,
    L: float = 1000.0,
    Om0: float = 0.31,
    z: float = 0.0,
    direction: Optional[int] = None,
    window: Union[str, int] = "CIC",
    R: float = 4.0,
    R_times: float = 5.0,
    interlacing: bool = False,
    folds: int = 1,
    verbose: bool = False,
    nthreads: int = 1,
    stream: Optional[int] = None,
) -> np.ndarray:
    """Density contrast of a tracer set on an nd^3 grid (simulation.py:9-166).

    Windows NGP, CIC, SPHERICAL (R), EXPONENTIAL (R, R_times); masses;
    several tracer types; interlacing; redshift-space shifts along x/y/z;
    folds.  Returns [nd, nd, nd] float32 for one type without interlacing,
    else [ntypes, interlacing + 1, nd, nd, nd].  stream: a CUDA stream handle
    (int) for the device work, None for the default stream."""
    pos = np.asarray(pos, dtype=np.float32)
    L, R, R_times = np.float32(L), np.float32(R), np.float32(R_times)
    Om0, z = np.float32(Om0), np.float32(z)
    nmass = 0
    if mass is not None:
        mass = np.asarray(mass, dtype=np.float32)
        nmass = 1
    ntypes = 1
    if types is not None:
        types = np.fabs(types)
        types = (types - np.min(types)).astype("int32")
        ntypes = len(np.unique(types))
    direction = _direction_code(direction)
    window = _window_code(window, allow_none=False)
    if window is None:
        print("You need to choose some density assigment method to construct the density grid!")
        return None
    grid = _spec.grid_compute(pos, vel, mass, np.int32(nmass), types, np.int32(ntypes), np.int32(nd), L, Om0, z,
                              np.int32(direction), np.int32(window), R, R_times, np.int32(interlacing),
                              np.int32(folds), np.int32(verbose), np.int32(nthreads), stream=stream)
    if not interlacing and ntypes == 1:
        grid = grid.reshape([nd, nd, nd])
    return grid


def Compute_Power_Spectrum(
    grid: np.ndarray,
    L: float = 1000.0,
    window: Union[str, int] = "CIC",
    R: float = 4.0,
    Nk: int = 25,
    k_min: Optional[float] = None,
    k_max: Optional[float] = None,
    l_max: int = 0,
    direction: Optional[Union[str, int]] = None,
    folds: int = 1,
    verbose: bool = False,
    nthreads: int = 1,
    ntypes: int = 1,
    stream: Optional[int] = None,
) -> Dict[str, np.ndarray]:
    """Shell-binned power spectrum of a grid (simulation.py:170-311):
    {"k": mean |k| per bin, "Pk": P(k), "Nk": modes per bin}.  stream: a
    CUDA stream handle (int) for the device work, None for the default stream."""
    if grid.ndim == 3:
        interlacing, ntypes = 0, 1
    elif grid.ndim == 5:
        interlacing, ntypes = 1, grid.shape[0]
    elif grid.ndim == 4 and ntypes == 1:
        interlacing = 1
    else:
        interlacing = 0
    nd = grid.shape[-1]
    L = L / folds
    if k_min is None:
        k_min = 2.0 * np.pi / L
    if k_max is None:
        k_max = np.pi / L * nd
    grid = np.asarray(grid, dtype=np.float32)
    L, R = np.float32(L), np.float32(R)
    k_min, k_max = np.float32(k_min), np.float32(k_max)
    window = _window_code(window, allow_none=True)
    direction = _direction_code(direction)
    x = _spec.power_compute(grid, np.int32(ntypes), np.int32(nd), L, np.int32(window), R, np.int32(interlacing),
                            np.int32(Nk), k_min, k_max, np.int32(l_max), np.int32(direction), np.int32(verbose),
                            np.int32(nthreads), stream=stream)
    if ntypes == 1 and l_max == 0:
        x["Pk"] = x["Pk"].reshape([Nk])
    return x


def Compute_Abundance(
    Mh: np.ndarray,
    Mmin: Optional[float] = None,
    Mmax: Optional[float] = None,
    Nm: int = 25,
    Lc: float = 2.0,
    nd: int = 256,
    ndx: Optional[int] = None,
    ndy: Optional[int] = None,
    ndz: Optional[int] = None,
    verbose: bool = False,
) -> Dict[str, np.ndarray]:
    """Differential abundance of a halo catalogue (simulation.py:719-806):
    {"Mh": mean mass per bin, "dn": dn/dlnM, "dn_err": Poisson error}."""
    Mmin = -1.0 if Mmin is None else Mmin
    Mmax = -1.0 if Mmax is None else Mmax
    ndx = nd if ndx is None else ndx
    ndy = nd if ndy is None else ndy
    ndz = nd if ndz is None else ndz
    return _spec.abundance_compute(np.asarray(Mh, dtype=np.float32), np.float32(Mmin), np.float32(Mmax), np.int32(Nm),
                                   np.float32(Lc), np.int32(ndx), np.int32(ndy), np.int32(ndz), np.int32(verbose))
