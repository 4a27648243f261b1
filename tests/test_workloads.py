"""The synthetic linear spectrum every workload and benchmark uses
(exshalos_gb300/workloads.py), checked on the CPU: normalised to sigma_8 =
0.81 on the tabulated k grid, the BBKS transfer function's limits, the shape
of the table, and the box configurations' sizes."""
import numpy as np

from exshalos_gb300 import workloads as w


def test_spectrum_is_normalised_to_sigma8():
    k, P = w.synthetic_pk()
    assert k.shape == P.shape == (1000,)
    assert np.all(np.diff(np.log(k)) > 0) and np.all(P > 0)
    assert abs(k[0] - 1e-4) < 1e-12 and abs(k[-1] - 1e2) < 1e-9
    # the 1000-point table integrates to sigma_8 within its quadrature error
    assert abs(np.sqrt(w.tophat_sigma2(k, P, 8.0)) - 0.81) < 2e-3


def test_bbks_limits_and_turnover():
    assert abs(w.bbks_transfer(1e-8) - 1.0) < 1e-4           # T -> 1 on large scales
    ks = np.logspace(-2, 1, 50)
    T = w.bbks_transfer(ks)
    assert np.all(np.diff(T) < 0)                             # falls monotonically
    k, P = w.synthetic_pk()
    kpk = k[np.argmax(P)]
    assert 0.01 < kpk < 0.03                                  # turnover near k_eq for Gamma = 0.21


def test_box_configurations():
    c = w.CONFIGS
    assert c["box_256"]["nd"] * c["box_256"]["Lc"] == 512.0
    assert c["box_512"]["nd"] * c["box_512"]["Lc"] == 1024.0
    assert c["plain_64"]["nd"] * c["plain_64"]["Lc"] == 256.0
    assert c["box_256"]["n_radii"] == 50 and c["box_256"]["Nk_pk"] == 128
