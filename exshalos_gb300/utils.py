"""Sub-stage hooks of the mock path and the barrier fit — mirror of
pyexshalos.utils (pyexshalos/utils.py:8-209, 291-455)."""
from typing import Optional

import numpy as np

from .lib import exshalos as _ext


def Generate_Density_Grid(k, P, R_max=100000.0, nd=256, ndx: Optional[int] = None, ndy: Optional[int] = None,
                          ndz: Optional[int] = None, Lc=2.0, outk=False, seed=12345, fixed=False, phase=0.0,
                          k_smooth=100000.0, verbose=False, nthreads=1):
    """Gaussian density grid from P(k) (utils.py:8-109): {"grid"}."""
    k = np.asarray(k).astype("float32")
    P = np.asarray(P).astype("float32")
    ndx = nd if ndx is None else ndx
    ndy = nd if ndy is None else ndy
    ndz = nd if ndz is None else ndz
    return _ext.density_grid_compute(k, P, np.float32(R_max), np.int32(ndx), np.int32(ndy), np.int32(ndz),
                                     np.float32(Lc), np.int32(outk), np.int32(seed), np.int32(fixed),
                                     np.float32(phase), np.float32(k_smooth), np.int32(verbose), np.int32(nthreads))


def Find_Halos_from_Grid(grid, k, P, Lc=2.0, Om0=0.31, z=0.0, delta_c=-1.0, Nmin=1, a=1.0, beta=0.0, alpha=0.0,
                         OUT_FLAG=False, verbose=False):
    """Halos of a given density grid (utils.py:113-209): {"posh", "Mh"[, "flag"]}."""
    k = np.asarray(k).astype("float32")
    P = np.asarray(P).astype("float32")
    return _ext.find_halos(np.asarray(grid).astype("float32"), k, P, np.float32(Lc), np.float32(Om0),
                           np.float32(z), np.float32(delta_c), np.int32(Nmin), np.float32(a), np.float32(beta),
                           np.float32(alpha), np.int32(OUT_FLAG), np.int32(False), verbose)


def Get_Omz(z: float = 0.0, Om0: float = 0.31) -> float:
    """Omega_m(z) = Om0 (1+z)^3 / (Om0 (1+z)^3 + 1 - Om0)."""
    a3 = np.power(1.0 + z, 3.0)
    return Om0 * a3 / (Om0 * a3 + (1.0 - Om0))


def Get_deltac(z: float = 0.0, Om0: float = 0.31) -> float:
    """delta_c = 1.686 Omega_m(z)^0.0055 (the fit of pyexshalos/theory.py:55-67)."""
    return 1.686 * np.power(Get_Omz(z, Om0), 0.0055)


def Fit_Barrier(k, P, M, dndlnM, dn_err=None, grid=None, R_max=100000.0, Mmin=None, Mmax=None, Nm=25, nd=256,
                Lc=2.0, Om0=0.31, z=0.0, delta_c=None, Nmin=10, seed=12345, x0=None, verbose=False, nthreads=1,
                Max_iter=100, tol=None):
    """Best-fit (a, beta, alpha) of the ellipsoidal barrier for a target mass
    function (utils.py:291-455): Nelder-Mead over chi^2 between the abundance
    of the halos of one Gaussian grid and the interpolated target.  Every
    trial runs the GPU halo finder on the same grid; the peaks and their
    sorted order are found once and reused for the later trials."""
    from scipy.interpolate import interp1d
    from scipy.optimize import minimize

    from .simulation import Compute_Abundance
    if grid is None:
        grid = Generate_Density_Grid(k, P, R_max, nd=nd, Lc=Lc, seed=seed, verbose=False, nthreads=nthreads)["grid"]
    M = np.asarray(M)
    dndlnM = np.asarray(dndlnM)
    dn_err = np.zeros(len(M)) if dn_err is None else np.asarray(dn_err)
    Mmin = -1.0 if Mmin is None else Mmin
    Mmax = -1.0 if Mmax is None else Mmax
    fdn = interp1d(np.log(M[M > 0.0]), dndlnM[M > 0.0], bounds_error=False, fill_value=0.0)
    fdn_err = interp1d(np.log(M[M > 0.0]), dn_err[M > 0.0], bounds_error=False, fill_value=0.0)
    if delta_c is None:
        delta_c = Get_deltac(z, Om0)
    grid32 = np.ascontiguousarray(grid, dtype=np.float32)

    def Chi2(theta):
        a, beta, alpha = theta
        x = Find_Halos_from_Grid(grid32, k, P, Lc=Lc, Om0=Om0, z=z, delta_c=delta_c, Nmin=Nmin, a=a, beta=beta,
                                 alpha=alpha, verbose=False)
        dnh = Compute_Abundance(x["Mh"], Mmin=Mmin, Mmax=Mmax, Nm=Nm, Lc=Lc, nd=nd, verbose=False)
        mask = dnh["dn"] > 0.0
        # the error term is evaluated at M, not ln M, as in utils.py:414-418
        chi2 = np.sum(np.power(dnh["dn"][mask] - fdn(np.log(dnh["Mh"][mask])), 2.0) /
                      (np.power(dnh["dn_err"][mask], 2.0) + np.power(fdn_err(dnh["Mh"][mask]), 2.0))) / (Nm - 4)
        if verbose:
            print("Current try: (%f, %f, %f) with chi2 = %f" % (a, beta, alpha, chi2))
        return chi2

    if x0 is None:
        x0 = [0.55, 0.4, 0.7]
    bounds = [(0.1, 2.0), (0.0, 1.0), (0.0, 1.0)]
    x = minimize(Chi2, x0=x0, bounds=bounds, method="Nelder-Mead", options={"maxiter": Max_iter}, tol=tol)
    return x.x
