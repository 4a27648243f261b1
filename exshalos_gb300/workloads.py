"""Synthetic inputs for the mock-generation path.

The reference's tutorials read a tabulated MDPL2 linear spectrum; no dataset
is available here, so every workload uses the same synthetic stand-in:

    P(k) = A k^n_s T_BBKS(k)^2,   Omega_m = 0.31, h = 0.68, n_s = 0.965,

normalised to sigma_8 = 0.81 with an FP64 top-hat quadrature and tabulated in
float64 at 1000 log-spaced k in [1e-4, 1e2] h/Mpc.  T_BBKS is the transfer
function of Bardeen, Bond, Kaiser & Szalay (1986, eq. G3) with shape
parameter Gamma = Omega_m h.
"""
import numpy as np


def bbks_transfer(k, Om0=0.31, h=0.68):
    q = np.asarray(k, dtype=np.float64) / (Om0 * h)
    return (np.log1p(2.34 * q) / (2.34 * q) *
            (1.0 + 3.89 * q + (16.1 * q) ** 2 + (5.46 * q) ** 3 + (6.71 * q) ** 4) ** -0.25)


def tophat_sigma2(k, P, R):
    """sigma^2(R) = 1/(2 pi^2) int k^2 P W^2 dk, trapezoid in ln k (FP64)."""
    x = k * R
    W = 3.0 * (np.sin(x) - x * np.cos(x)) / x ** 3
    f = k ** 3 * P * W ** 2 / (2.0 * np.pi ** 2)
    lk = np.log(k)
    return float(np.sum(0.5 * (f[1:] + f[:-1]) * np.diff(lk)))


def synthetic_pk(nk=1000, kmin=1e-4, kmax=1e2, Om0=0.31, h=0.68, ns=0.965, sigma8=0.81):
    """(k, P) float64 arrays of the synthetic linear spectrum."""
    k = np.logspace(np.log10(kmin), np.log10(kmax), nk)
    kf = np.logspace(np.log10(kmin), np.log10(kmax), 200001)
    Pf = kf ** ns * bbks_transfer(kf, Om0, h) ** 2
    A = sigma8 ** 2 / tophat_sigma2(kf, Pf, 8.0)
    P = A * k ** ns * bbks_transfer(k, Om0, h) ** 2
    return k, P


# Box configurations used by the tests and the benchmark (one per line of the
# reference benchmark description): cells per side, cell size in Mpc/h.
CONFIGS = {
    "plain_64": dict(nd=64, Lc=4.0, Om0=0.31, seed=1, Nk_pk=32),
    "box_256": dict(nd=256, Lc=2.0, Om0=0.31, seed=1, a=1.0, beta=0.12, alpha=0.0,
                    DO_2LPT=True, Nk_pk=128, n_radii=50, R_max_ladder=30.0),
    "box_512": dict(nd=512, Lc=2.0, Om0=0.31, seed=1, DO_2LPT=True, Nk_pk=256),
}
