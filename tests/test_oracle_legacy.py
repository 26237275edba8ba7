"""The oracle's legacy algorithms (legacy = true), CPU only.

The spline is Dierckx.Spline1D(x, y; k, s = 0) (src/splines.jl:312-315), which
wraps netlib FITPACK (curfit/fpcurf with s = 0, splev/fpbspl).  scipy's
splrep/splev call the same FITPACK routines, so the restatement is pinned
against them bit for bit.  The sampling grid knots[1]:0.001:knots[end] is a
Julia float range; its elements are checked against the exact decimal values
the TwicePrecision construction is designed to produce."""
from fractions import Fraction

import numpy as np
import pytest


@pytest.mark.parametrize("k", [1, 2, 3])
def test_fitpack_matches_scipy_bitwise(orc, k):
    si = pytest.importorskip("scipy.interpolate")
    rng = np.random.default_rng(10 + k)
    for trial in range(60):
        m = int(rng.integers(k + 1, 40))
        x = np.sort(rng.uniform(-50, 200, m))
        if np.unique(x).size < m:
            continue
        y = rng.normal(size=m) * 10.0 ** rng.integers(-4, 3)
        t, c = orc.fitpack_curfit0(x, y, k)
        ts, cs, ks = si.splrep(x, y, k=k, s=0)
        np.testing.assert_array_equal(t, ts)
        np.testing.assert_array_equal(c, cs[:m])
        xe = np.concatenate([x, np.linspace(x[0], x[-1], 301)])
        np.testing.assert_array_equal(orc.fitpack_splev(t, c, k, xe), si.splev(xe, (ts, cs, ks)))


def test_fitpack_interpolates_flip_angle_grid(orc):
    """Interior knots of the cubic interpolant are the data points 3..m-2
    (not-a-knot), and the spline passes through every point."""
    x = np.linspace(50.0, 180.0, 8)
    y = (x - 141.3) ** 2 / 1e4 + 0.01
    t, c = orc.fitpack_curfit0(x, y, 3)
    np.testing.assert_array_equal(t[4:8], x[2:6])
    assert t[:4].tolist() == [50.0] * 4 and t[-4:].tolist() == [180.0] * 4
    np.testing.assert_allclose(orc.fitpack_splev(t, c, 3, x), y, rtol=1e-13)


def test_julia_float_ranges(orc):
    r = orc.jl_colon(50.0, 0.001, 180.0)
    assert r.size == 130001
    want = np.array([float(Fraction(50000 + i, 1000)) for i in range(r.size)])
    np.testing.assert_array_equal(r, want)
    # the chi2 search's ranges 0:0.001:(1e-3 * 2^j)
    mu = 1e-3
    for j in range(0, 12):
        r = orc.jl_colon(0.0, 0.001, mu)
        assert r.size == 2 ** j + 1 and r[0] == 0.0 and r[-1] == mu
        mu *= 2.0
    # decimal steps land on the decimal values, unlike repeated addition
    r = orc.jl_colon(0.0, 0.1, 1.0)
    assert r.size == 11 and r[3] == 0.3 and r[-1] == 1.0
    r = orc.jl_colon(1.0, -0.1, 0.0)
    assert r.size == 11 and r[7] == 0.3
    # empty and single-element ranges
    assert orc.jl_colon(1.0, 0.001, 0.5).size == 0
    assert orc.jl_colon(2.0, 0.001, 2.0).tolist() == [2.0]


def test_spline_opt_legacy_quadratic(orc):
    """A cubic interpolant reproduces a parabola, so the sampled minimum is the
    0.001 grid point nearest its vertex."""
    x = np.linspace(50.0, 180.0, 8)
    for c0 in (61.23456, 123.4567, 170.0004, 179.9):
        y = (x - c0) ** 2
        xm, ym = orc.spline_opt_legacy(x, y)
        assert abs(xm - c0) <= 0.0005 + 1e-9
        assert ym == pytest.approx((xm - c0) ** 2, abs=1e-8)


def test_spline_opt_legacy_two_points(orc):
    xm, ym = orc.spline_opt_legacy([50.0, 180.0], [2.0, 1.0])  # linear: minimum at the right end
    assert xm == 180.0 and ym == pytest.approx(1.0)


def test_spline_root_legacy_line(orc):
    mu = np.array([0.0, 1e-3, 2e-3, 4e-3, 8e-3])
    r2 = 1.0 + 10.0 * mu   # res2(mu) = 1 + 10 mu; root of res2 = 1.0502 at mu = 0.00502
    x = orc.spline_root_legacy(mu, r2, 1.0502)
    assert x == 0.005


def test_chi2_legacy_hits_target(orc):
    rng = np.random.default_rng(4)
    m, n = 32, 40
    t = np.arange(1, m + 1) * 10e-3
    T2 = np.geomspace(10e-3, 2.0, n)
    A = np.exp(-t[:, None] / T2[None, :])
    for trial in range(5):
        xt = np.zeros(n)
        xt[rng.integers(5, 15)] = 1.0
        xt[rng.integers(20, 30)] = 2.0
        b = A @ xt + rng.normal(scale=0.01, size=m)
        x, mu, chi2 = orc.lsqnonneg_chi2_legacy(A, b, 1.02)
        assert np.all(x >= 0)
        assert mu >= 0 and round(mu * 1000) == pytest.approx(mu * 1000, abs=1e-6)  # on the 0.001 grid
        assert abs(chi2 - 1.02) < 0.02
