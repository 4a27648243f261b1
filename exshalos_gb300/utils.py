"""Sub-stage hooks of the mock path — mirror of pyexshalos.utils
(pyexshalos/utils.py:8-209)."""
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
