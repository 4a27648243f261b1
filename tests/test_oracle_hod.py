"""The oracle's galaxy population and colour split (CPU): occupation
statistics, the radial profile the r(Eps) tables invert, the reference's
angle convention, and the split fractions.  GSL is absent, so the taus
stream and the Poisson draw are restated, not pinned to a GSL build; these
tests check the distributions they produce."""
import numpy as np
import pytest
from scipy.special import erf

from oracle import orc


def _occupation(M, logMmin=13.25424743, siglogM=0.26461332, logM0=13.28383025, logM1=14.32465146,
                alpha=1.00811277):
    Md = np.float64(M)
    pc = 0.5 * (1 + erf((np.log10(Md) - logMmin) / siglogM))
    M0, M1 = 10 ** logM0, 10 ** logM1
    mu = np.power(max(Md - M0, 0.0) / M1, alpha) * pc if Md >= M0 else 0.0
    return pc, mu


@pytest.mark.parametrize("logM", [13.2, 14.5, 15.3])
def test_occupation_statistics(logM):
    nh = 20000
    M = np.full(nh, 10 ** logM, dtype=np.float32)
    pos = np.zeros((nh, 3), dtype=np.float32)
    r = orc.populate_halos(pos, M, seed=4)
    pc, mu = _occupation(M[0])
    n = r["ncen"].astype(np.float64)
    assert abs(n.mean() - pc) < 5 * np.sqrt(pc * (1 - pc) / nh) + 1e-12
    s = r["nsat"].astype(np.float64)
    assert abs(s.mean() - mu) < 5 * np.sqrt(max(mu, 1e-12) / nh) + 1e-12
    if mu > 0.5:
        assert abs(s.var() / mu - 1) < 0.1             # Poisson: variance = mean
    assert r["posg"].shape[0] == n.sum() + s.sum()


def _profile_cdf(c, sigma, r):
    x = np.logspace(-3, 1, 200001)
    f = 1.0 / (c * x * (1 + c * x) ** 2) / (1 + x ** (2.0 / sigma)) * x * x
    F = np.concatenate([[0.0], np.cumsum(0.5 * (f[1:] + f[:-1]) * np.diff(x))])
    return np.interp(r, x, F / F[-1])


def test_satellite_radii_follow_the_profile():
    """Equal concentrations (one r(Eps) table, weight 1): the offsets of the
    satellites follow the truncated profile; theta is drawn uniform in
    [0, pi] as populate_halos.c:183 does, so <cos^2 theta> = 1/2."""
    nh = 3000
    M = np.full(nh, 10 ** 15.0, dtype=np.float32)
    pos = np.zeros((nh, 3), dtype=np.float32)
    C = np.full(nh, 5.0, dtype=np.float32)
    r = orc.populate_halos(pos, M, Ch=C, seed=9, sigma=0.5)
    sat = r["flag"] > 0
    d = r["posg"][sat].astype(np.float64)
    rad = np.sqrt((d ** 2).sum(axis=1))
    assert rad.size > 10000
    assert rad.min() >= 1e-3 * 0.999 and rad.max() <= 10.0 * 1.001
    rs = np.sort(rad)
    ks = np.max(np.abs(_profile_cdf(5.0, 0.5, rs) - (np.arange(rs.size) + 0.5) / rs.size))
    assert ks < 0.015
    cz2 = np.mean((d[:, 2] / rad) ** 2)
    assert abs(cz2 - 0.5) < 0.01


def test_split_fractions():
    nh = 4000
    M = np.full(nh, 10 ** 14.0, dtype=np.float32)
    flag = np.concatenate([-np.arange(1, nh), np.arange(1, nh)]).astype(np.int64)
    pc = np.array([[0.3, 0.0, 0.0]])
    ps = np.array([[0.8, 0.0, 0.0]])
    t = orc.split_galaxies(M, flag, pc, ps, seed=3)
    cen, sat = t[: nh - 1], t[nh - 1:]
    assert set(np.unique(cen)) <= {-1, -2} and set(np.unique(sat)) <= {1, 2}
    assert abs(np.mean(cen == -1) - 0.3) < 0.04
    assert abs(np.mean(sat == 1) - 0.8) < 0.04
    with pytest.raises(ValueError):
        orc.split_galaxies(M[:5], flag, pc, ps)
