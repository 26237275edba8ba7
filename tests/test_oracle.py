"""The oracle against the reference's own known answers and properties
(test/optimization.jl, test/splines.jl, test/nnls.jl, test/epg.jl).  CPU only."""
import math

import numpy as np
import pytest


# ---- test/optimization.jl:1-60 --------------------------------------------
def test_bisect_root(orc):
    x, fx = orc.bisect_root(math.sin, 3.0, 4.5, xatol=1e-6)
    assert abs(x - math.pi) <= 1e-6
    x, fx = orc.bisect_root(math.sin, 2.5, 4.0, xrtol=1e-7)
    assert abs(x - math.pi) <= 1e-7 * math.pi
    x, fx = orc.bisect_root(math.sin, 2.0, 3.5, ftol=1e-8)
    assert abs(fx) <= 1e-8


def test_brent_root(orc):
    x, fx = orc.brent_root(math.sin, 3.0, 4.5, xatol=1e-6)
    assert abs(x - math.pi) <= 1e-6
    x, fx = orc.brent_root(math.sin, 2.5, 4.0, xrtol=1e-7)
    assert abs(x - math.pi) <= 1e-7 * math.pi
    x, fx = orc.brent_root(math.sin, 2.0, 3.5, ftol=1e-8)
    assert abs(fx) <= 1e-8


def test_brent_minimize(orc):
    f = lambda t: math.sin(t) ** 2
    x, fx = orc.brent_minimize(f, 3.0, 4.5, xatol=1e-6, xrtol=0.0)
    assert abs(x - math.pi) <= 1e-6
    x, fx = orc.brent_minimize(f, 2.5, 4.0, xatol=0.0, xrtol=1e-7)
    assert abs(x - math.pi) <= 1e-7 * math.pi


# ---- test/nnls.jl:342-369: corner of (μ, 1/μ) is at log μ = 0 -------------
def test_lcurve_corner(orc):
    x = orc.lcurve_corner(lambda l: (math.exp(l), math.exp(-l)), math.log(0.1), math.log(10.0), 1e-6, 1e-6, 0.0)
    assert abs(x) <= 1e-3


# ---- test/splines.jl:165-203: Hermite surrogate is exact on a cubic ----------
def test_cubic_hermite_exact(orc):
    c = (-2.0, -1.0, -5.0, 3.0)   # 3x^3 - 5x^2 - x - 2
    dc = (-1.0, -10.0, 9.0)
    a, b = -0.5, 2.0
    f = lambda x: np.polyval(c[::-1], x)
    g = lambda x: np.polyval(dc[::-1], x)
    x, u = orc.cubic_hermite_minimize(a, b, f(a), f(b), g(a), g(b))
    # minimize_cubic: local minimum of the cubic on [a, b]
    r = np.roots([9.0, -10.0, -1.0])
    cands = [a, b] + [t for t in r if a < t < b]
    xt = min(cands, key=f)
    assert x == pytest.approx(xt, rel=1e-12)
    assert u == pytest.approx(f(xt), rel=1e-12)


# ---- test/splines.jl:390-435: minimal_bounding_box known answers (1-D slices)
def test_minimal_bounding_box(orc):
    grid = np.arange(1.0, 11.0)
    seen = np.zeros(10, np.uint8)
    seen[[0, 9]] = 1
    assert orc.minimal_bounding_box(grid, seen, 2.0) == (1, 5)
    assert orc.minimal_bounding_box(grid, seen, 6.5) == (5, 10)
    seen[4] = 1
    assert orc.minimal_bounding_box(grid, seen, 6.5) == (5, 7)
    assert orc.minimal_bounding_box(grid, seen, 8.5) == (7, 10)
    assert orc.minimal_bounding_box(grid, seen, 2.0) == (1, 3)
    assert orc.minimal_bounding_box(grid, seen, 4.5) == (3, 5)


# ---- test/epg.jl: kernel variants agree; Jacobian by finite differences ----
@pytest.mark.parametrize("ETL", [4, 5, 6, 7, 8, 16, 32, 48, 64])
def test_epg_default_vs_spec(orc, ETL):
    rng = np.random.default_rng(ETL)
    for _ in range(3):
        a, TE, T2, T1 = rng.uniform(50, 180), rng.uniform(5e-3, 15e-3), rng.uniform(10e-3, 2.0), rng.uniform(0.8, 1.5)
        for beta in (180.0, rng.uniform(50, 179)):
            f = orc.epg_decay_curve(ETL, a, TE, T2, T1, beta)
            s = orc.epg_decay_curve_basic(ETL, a, TE, T2, T1, beta)
            np.testing.assert_allclose(f, s, rtol=math.sqrt(2.220446049250313e-16), atol=10 * 2.220446049250313e-16)


@pytest.mark.parametrize("beta", [180.0, 150.0])
def test_epg_dual_primal_and_jacobian(orc, beta):
    ETL, a, TE, T2, T1 = 32, 163.0, 10e-3, 0.05, 1.0
    v, d = orc.epg_decay_curve_dual(ETL, a, TE, T2, T1, beta)
    f = orc.epg_decay_curve(ETL, a, TE, T2, T1, beta)
    np.testing.assert_array_equal(v, f)  # primal of the dual evaluation is the plain evaluation
    for h in (1e-3, 1e-4):
        fd = (orc.epg_decay_curve(ETL, a + h, TE, T2, T1, beta) - orc.epg_decay_curve(ETL, a - h, TE, T2, T1, beta)) / (2 * h)
        assert np.max(np.abs(fd - d)) <= 5e-8 * (h / 1e-4) ** 2 / 1e-0 + 1e-10


# ---- test/nnls.jl:1-340: KKT conditions of NNLS ----------------------------
def rand_nnls_data(rng, m, n):
    x = rng.uniform(size=n)
    x[rng.integers(0, 2)::2] *= -1
    A = rng.uniform(size=(m, n))
    return A, A @ x


@pytest.mark.parametrize("m,n", [(1, 1), (2, 5), (5, 2), (8, 8), (13, 16), (25, 13), (32, 32), (16, 25)])
@pytest.mark.parametrize("mu", [0.0, 1e-2, 10.0])
def test_nnls_kkt(orc, m, n, mu):
    rng = np.random.default_rng(m * 100 + n)
    A0, b0 = rand_nnls_data(rng, m, n)
    if mu > 0:
        A = np.vstack([A0, mu * np.eye(n)])
        b = np.concatenate([b0, np.zeros(n)])
    else:
        A, b = A0, b0
    x, rnorm, nsetp, mode = orc.nnls(A, b)
    assert mode == 0
    w = -A.T @ (A @ x - b)
    pos = x > 0
    assert np.all(x >= 0)
    assert pos.sum() == nsetp
    assert np.all(w[~pos] <= 1e-10 * max(1.0, np.linalg.norm(A.T @ b)))
    if nsetp > 0:
        Ap = A[:, pos]
        xp = np.linalg.lstsq(Ap, b, rcond=None)[0]
        np.testing.assert_allclose(x[pos], xp, rtol=1e-8, atol=1e-12)
    assert rnorm == pytest.approx(np.linalg.norm(A @ x - b), rel=1e-10, abs=1e-13)


@pytest.mark.parametrize("m,n", [(8, 8), (32, 16), (16, 25), (48, 40)])
def test_lsqnonneg_tikh_matches_padded_nnls(orc, m, n):
    rng = np.random.default_rng(7)
    A0, b0 = rand_nnls_data(rng, m, n)
    mu = 0.3
    x, info = orc.lsqnonneg_tikh(A0, b0, mu)
    A = np.vstack([A0, mu * np.eye(n)])
    b = np.concatenate([b0, np.zeros(n)])
    xr, rn, ns, md = orc.nnls(A, b)
    np.testing.assert_allclose(x, xr, rtol=1e-9, atol=1e-12)  # strictly convex: unique solution
    assert info["resnorm_sq"] == pytest.approx(np.sum((A0 @ x - b0) ** 2), rel=1e-8, abs=1e-14)
    assert info["seminorm_sq"] == pytest.approx(np.sum(x ** 2), rel=1e-12)


# ---- test/nnls.jl:387-434: chi2 hits its target ----------------------------
@pytest.mark.parametrize("m,n", [(8, 5), (16, 16), (32, 25), (25, 32)])
def test_lsqnonneg_chi2(orc, m, n):
    rng = np.random.default_rng(m + 7 * n)
    A, b = rand_nnls_data(rng, m, n)
    x_unreg, rn, _ = orc.lsqnonneg(A, b)
    res2_min, res2_max = rn ** 2, np.sum(b ** 2)
    target = min(math.sqrt(res2_min * res2_max) / res2_min, 1.01 + 0.99 * rng.uniform())
    x, mu, chi2 = orc.lsqnonneg_chi2(A, b, target)
    if res2_min <= 0 or np.sum(x_unreg ** 2) == 0:
        # unregularized solution returned with mu = 0, chi2 = 1
        np.testing.assert_array_equal(x, x_unreg)
        assert mu == 0 and chi2 == 1
    elif res2_min <= 1e-12:
        assert mu >= 0
    else:
        assert mu > 0
        assert chi2 == pytest.approx(target, rel=1e-3)


# ---- test/nnls.jl:483-519: mdp residual --------------------------------------
@pytest.mark.parametrize("m,n", [(16, 8), (32, 16), (13, 25)])
def test_lsqnonneg_mdp(orc, m, n):
    rng = np.random.default_rng(3 * m + n)
    A, b = rand_nnls_data(rng, m, n)
    _, rn, _ = orc.lsqnonneg(A, b)
    r2min, r2max = rn ** 2, np.sum(b ** 2)
    target = r2min + (r2max - r2min) / 10
    x, mu, chi2 = orc.lsqnonneg_mdp(A, b, math.sqrt(target))
    res2 = np.sum((A @ x - b) ** 2)
    if mu <= 0:
        assert res2 == pytest.approx(r2min, abs=1e-12)
    else:
        assert res2 == pytest.approx(target, rel=2e-3, abs=1e-12)


# ---- test/nnls.jl:436-481: GCV singular values and dof identity -------------
@pytest.mark.parametrize("m,n", [(8, 5), (16, 16), (5, 13), (48, 40), (56, 60)])
def test_svdvals_and_gcv_dof(orc, m, n):
    rng = np.random.default_rng(m * n)
    A = rng.uniform(size=(m, n))
    s = orc.svdvals(A)
    np.testing.assert_allclose(s, np.linalg.svd(A, compute_uv=False), rtol=1e-12, atol=1e-13 * s[0])
    mu = 0.37
    dof = max(m - n, 0) + np.sum(mu ** 2 / (s ** 2 + mu ** 2))
    tr = np.trace(np.eye(m) - A @ np.linalg.solve(A.T @ A + mu ** 2 * np.eye(n), A.T))
    assert dof == pytest.approx(tr, rel=1e-9)


@pytest.mark.parametrize("m,n", [(16, 8), (48, 40), (32, 40)])
def test_lcurve_and_gcv_run(orc, m, n):
    rng = np.random.default_rng(11)
    A, b = rand_nnls_data(rng, m, n)
    x, mu, chi2 = orc.lsqnonneg_lcurve(A, b)
    assert np.isfinite(mu) and mu > 0 and np.all(x >= 0)
    x, mu, chi2 = orc.lsqnonneg_gcv(A, b)
    assert np.isfinite(mu) and np.all(x >= 0)


# ---- grids: Julia range semantics ------------------------------------------
def test_grids(orc):
    a = orc.linrange(50.0, 180.0, 32)
    assert a[0] == 50.0 and a[-1] == 180.0
    exact = (50 * (31 - np.arange(32)) + 180 * np.arange(32)) / 31
    np.testing.assert_array_equal(a, exact)  # rational path: correctly rounded
    t = orc.logrange(10e-3, 2.0, 40)
    assert t[0] == 10e-3 and t[-1] == 2.0
    np.testing.assert_allclose(t, np.exp(np.linspace(np.log(10e-3), np.log(2.0), 40)), rtol=4e-16)
    assert orc.sind(30.0) == 0.5 and orc.sind(90.0) == 1.0 and orc.sind(180.0) == 0.0
    assert orc.erfinv(-0.8) == pytest.approx(-0.9061938024368232, rel=1e-15)


# ---- whole path: T2map + T2part smoke on the oracle --------------------------
def test_oracle_pipeline_small(orc):
    rng = np.random.default_rng(0)
    m, X = 32, (2, 2, 1)
    img = np.empty(X + (m,))
    for v in np.ndindex(X):
        dc = 0.15 * orc.epg_decay_curve(m, 165.0, 10e-3, 20e-3, 1.0) + 0.85 * orc.epg_decay_curve(m, 165.0, 10e-3, 70e-3, 1.0)
        img[v] = 1000 * dc + rng.normal(0, 2.0, m)
    o = orc.T2mapOptions(MatrixSize=X, nTE=m, TE=10e-3, nT2=40, T2Range=(10e-3, 2.0), Reg="chi2", Chi2Factor=1.02,
                         nRefAngles=8)
    maps, dist = orc.t2map(img, o)
    assert np.all(np.isfinite(dist)) and np.all(dist >= 0)
    assert np.all((maps["alpha"] > 140) & (maps["alpha"] <= 180))
    parts = orc.t2part(dist, orc.T2partOptions(MatrixSize=X, nT2=40, T2Range=(10e-3, 2.0), SPWin=(10e-3, 25e-3),
                                               MPWin=(25e-3, 200e-3)))
    assert np.all((parts["sfr"] > 0.05) & (parts["sfr"] < 0.3))


# ---- non-finite echoes (bad per-voxel inputs) --------------------------------
@pytest.mark.parametrize("reg,kw", [("none", {}), ("chi2", dict(Chi2Factor=1.02)), ("lcurve", {}), ("gcv", {}),
                                    ("mdp", dict(NoiseLevel=1.0))])
def test_nonfinite_echoes(orc, reg, kw):
    """NaN and Inf echoes end in bounded time and stay within their voxel,
    following src/T2mapSEcorr.jl:201-218: the threshold test `image[I, 1] >
    Threshold` skips a NaN first echo; the running maximum
    `b > max ? b : max` passes over a NaN later echo (the voxel is processed
    with a finite, non-negative distribution); an Inf echo makes the maximum
    Inf and the rescaled distribution NaN (0 * Inf)."""
    rng = np.random.default_rng(1)
    m, X = 32, (4, 1, 1)
    img = np.empty(X + (m,))
    for v in np.ndindex(X):
        img[v] = 1000 * orc.epg_decay_curve(m, 160.0, 10e-3, 60e-3, 1.0) + rng.normal(0, 2.0, m)
    clean = img[3:4].copy()
    img[0, 0, 0, 5] = np.nan
    img[1, 0, 0, 3] = np.inf
    img[2, 0, 0, 0] = np.nan
    o = orc.T2mapOptions(MatrixSize=X, nTE=m, TE=10e-3, nT2=40, T2Range=(10e-3, 2.0), Reg=reg, nRefAngles=8,
                         SaveRegParam=True, **kw)
    maps, dist = orc.t2map(img, o)
    assert np.isfinite(dist[0, 0, 0]).all() and (dist[0, 0, 0] >= 0).all()
    assert np.isnan(dist[1, 0, 0]).all()
    assert np.isnan(dist[2, 0, 0]).all() and np.isnan(maps["alpha"][2, 0, 0])
    o1 = orc.T2mapOptions(MatrixSize=(1, 1, 1), nTE=m, TE=10e-3, nT2=40, T2Range=(10e-3, 2.0), Reg=reg, nRefAngles=8,
                          SaveRegParam=True, **kw)
    maps1, dist1 = orc.t2map(clean, o1)
    np.testing.assert_array_equal(dist[3:4], dist1)
    for k in maps1:
        np.testing.assert_array_equal(maps[k][3:4], maps1[k], err_msg=k)
