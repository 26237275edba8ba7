"""GPU path vs the CPU oracle on the same seeded inputs (run on a GB300).

The oracle restates the reference algorithm in FP64 with the GPU's reduction
order and the same portable transcendentals, so the plain (FP64) method is
expected to agree with it bit for bit; the stated tolerances (1e-8 relative per
distribution bin, 1e-10 absolute MWF) are asserted on top of that."""
import numpy as np
import pytest

from parity import DIST_RTOL, MWF_ATOL, dist_rel_err, orc_opts

pytestmark = pytest.mark.gpu

SPWIN, MPWIN = (10e-3, 25e-3), (25e-3, 200e-3)

CASES = {
    # 32 echoes, chi2 1.02, 8 angles over 50-180 (the reference's small CPU case, sized down in voxels)
    "chi2": dict(X=(8, 8, 2), m=32, TE=10e-3, n=40, T2=(10e-3, 2.0), K=8, Reg="chi2", Chi2Factor=1.02),
    # 48 echoes, 32 angles, lcurve, 35% background below threshold (the 240x240x48 volume's settings)
    "lcurve": dict(X=(8, 8, 2), m=48, TE=10e-3, n=40, T2=(10e-3, 2.0), K=32, Reg="lcurve", bg=0.35, thr=200.0),
    # 56 echoes, TE 7 ms, 60 T2s over 8 ms-2 s, 64 angles, gcv (the 240x240x113 volume's settings)
    "gcv": dict(X=(4, 4, 1), m=56, TE=7e-3, n=60, T2=(8e-3, 2.0), K=64, Reg="gcv"),
    "none": dict(X=(6, 6, 1), m=48, TE=10e-3, n=40, T2=(10e-3, 2.0), K=16, Reg="none"),
    "mdp": dict(X=(6, 6, 1), m=48, TE=10e-3, n=40, T2=(10e-3, 2.0), K=16, Reg="mdp", NoiseLevel=2.0),
    "refcon150": dict(X=(4, 4, 1), m=32, TE=10e-3, n=40, T2=(10e-3, 2.0), K=16, Reg="chi2", Chi2Factor=1.02,
                      RefConAngle=150.0),
    "fixed_angle": dict(X=(6, 6, 1), m=48, TE=10e-3, n=40, T2=(10e-3, 2.0), K=16, Reg="lcurve", SetFlipAngle=165.0),
    "m_lt_n": dict(X=(4, 4, 1), m=24, TE=10e-3, n=48, T2=(10e-3, 2.0), K=8, Reg="gcv"),
}


def run_case(D, orc, ctx, c, dtype=np.float64, seed=11, **extra):
    img = D.mock_image(D.MockImageOptions(MatrixSize=c["X"], nTE=c["m"], TE=c["TE"],
                                          BackgroundFraction=c.get("bg", 0.0)), seed=seed, dtype=dtype)
    o = D.T2mapOptions(MatrixSize=c["X"], nTE=c["m"], TE=c["TE"], nT2=c["n"], T2Range=c["T2"], Reg=c["Reg"],
                       nRefAngles=c["K"], Chi2Factor=c.get("Chi2Factor"), NoiseLevel=c.get("NoiseLevel"),
                       Threshold=c.get("thr", 0.0), RefConAngle=c.get("RefConAngle", 180.0),
                       SetFlipAngle=c.get("SetFlipAngle"), SaveRegParam=True, SaveResidualNorm=True,
                       SaveDecayCurve=True, **extra)
    po = D.T2partOptions.from_t2map(o, SPWin=SPWIN, MPWin=MPWIN)
    maps, dist, parts = D.T2mapSEcorr_T2partSEcorr(img, o, po, ctx=ctx)
    om, od = orc.t2map(img.astype(np.float64), orc_opts(orc, o), nthreads=8)
    op = orc.t2part(od, orc.T2partOptions(MatrixSize=c["X"], nT2=c["n"], T2Range=c["T2"], SPWin=SPWIN, MPWin=MPWIN))
    return img, o, maps, dist, parts, om, od, op


@pytest.mark.parametrize("name", list(CASES))
def test_t2map_matches_oracle(D, orc, ctx, name):
    c = CASES[name]
    img, o, maps, dist, parts, om, od, op = run_case(D, orc, ctx, c)
    # same voxels processed (threshold) and same NaN pattern
    np.testing.assert_array_equal(np.isnan(dist), np.isnan(od))
    err, ok = dist_rel_err(dist, od)
    assert ok.any()
    frac_bitwise = float(np.mean([np.array_equal(dist.reshape(-1, c["n"])[i], od.reshape(-1, c["n"])[i])
                                  for i in np.flatnonzero(ok)]))
    print(f"{name}: voxels={ok.sum()} bitwise={frac_bitwise:.4f} max_rel={err[ok].max():.3g}")
    assert err[ok].max() <= DIST_RTOL
    assert np.nanmax(np.abs(parts["sfr"] - op["sfr"])) <= MWF_ATOL
    for k in ("gdn", "ggm", "gva", "fnr", "snr", "alpha", "resnorm", "mu", "chi2factor"):
        a, b = maps[k], om[k]
        np.testing.assert_array_equal(np.isnan(a), np.isnan(b))
        np.testing.assert_allclose(a[~np.isnan(b)], b[~np.isnan(b)], rtol=1e-8, atol=0, err_msg=k)
    np.testing.assert_allclose(maps["decaycurve"], om["decaycurve"], rtol=1e-8, equal_nan=True)


def test_plain_method_is_bitwise(D, orc, ctx):
    """The FP64 path and the oracle agree bit for bit (dist, alpha, mu, and
    the fused T2part maps)."""
    c = CASES["lcurve"]
    img, o, maps, dist, parts, om, od, op = run_case(D, orc, ctx, c, seed=5)
    np.testing.assert_array_equal(dist, od)
    np.testing.assert_array_equal(maps["alpha"], om["alpha"])
    np.testing.assert_array_equal(maps["mu"], om["mu"])
    for k in ("sfr", "sgm", "mfr", "mgm"):
        np.testing.assert_array_equal(parts[k], op[k], err_msg=k)


def test_float32_input(D, orc, ctx):
    """Float32 images are widened to FP64 on the device; outputs are Float32."""
    c = CASES["chi2"]
    img, o, maps, dist, parts, om, od, op = run_case(D, orc, ctx, c, dtype=np.float32)
    assert dist.dtype == np.float32 and maps["alpha"].dtype == np.float32
    np.testing.assert_array_equal(dist, od.astype(np.float32))


def test_decaybasisset_and_grids(D, orc, ctx):
    c = CASES["lcurve"]
    img, o, maps, dist, parts, om, od, op = run_case(D, orc, ctx, c)
    t2 = orc.logrange(*c["T2"], c["n"])
    np.testing.assert_array_equal(maps["t2times"], t2)
    ang = orc.linrange(50.0, 180.0, c["K"])
    np.testing.assert_array_equal(maps["refangleset"], ang)
    np.testing.assert_array_equal(maps["echotimes"], c["TE"] * np.arange(1, c["m"] + 1))
    for k in (0, 7, c["K"] - 1):
        for j in (0, 13, c["n"] - 1):
            v, _ = orc.epg_decay_curve_dual(c["m"], ang[k], c["TE"], t2[j], 1.0)
            np.testing.assert_array_equal(maps["decaybasisset"][:, j, k], v)


def test_t2part_standalone(D, orc, ctx):
    rng = np.random.default_rng(4)
    X, n = (7, 5, 3), 40
    dist = rng.uniform(0, 1, X + (n,)) * (rng.uniform(size=X + (n,)) < 0.4)
    dist[0, 0, 0, 3] = np.nan
    for sig in (None, 5e-3):
        po = D.T2partOptions(MatrixSize=X, nT2=n, T2Range=(10e-3, 2.0), SPWin=SPWIN, MPWin=MPWIN, Sigmoid=sig)
        got = D.T2partSEcorr(dist, po, ctx=ctx)
        want = orc.t2part(dist, orc.T2partOptions(MatrixSize=X, nT2=n, T2Range=(10e-3, 2.0), SPWin=SPWIN,
                                                 MPWin=MPWIN, Sigmoid=sig))
        for k in ("sfr", "sgm", "mfr", "mgm"):
            np.testing.assert_array_equal(got[k], want[k], err_msg=k)


@pytest.mark.parametrize("thr", [np.inf, -np.inf])
def test_threshold_edges(D, orc, ctx, thr):
    """Threshold=Inf processes nothing (all NaN); -Inf processes every voxel."""
    c = dict(CASES["chi2"], X=(3, 3, 1), thr=thr)
    img, o, maps, dist, parts, om, od, op = run_case(D, orc, ctx, c)
    np.testing.assert_array_equal(np.isnan(dist), np.isnan(od))
    if thr == np.inf:
        assert np.isnan(dist).all() and np.isnan(maps["alpha"]).all()
    else:
        assert not np.isnan(dist).any()
        np.testing.assert_array_equal(dist, od)


def test_zero_and_constant_voxels(D, orc, ctx):
    """All-zero signal (processed with Threshold=-Inf) and a flat signal."""
    X, m = (2, 1, 1), 32
    img = np.zeros(X + (m,))
    img[1, 0, 0, :] = 100.0
    o = D.T2mapOptions(MatrixSize=X, nTE=m, TE=10e-3, nT2=40, T2Range=(10e-3, 2.0), Reg="chi2", Chi2Factor=1.02,
                       nRefAngles=8, Threshold=-np.inf, SaveRegParam=True)
    maps, dist = D.T2mapSEcorr(img, o, ctx=ctx)
    om, od = orc.t2map(img, orc_opts(orc, o))
    np.testing.assert_array_equal(dist, od)
    np.testing.assert_array_equal(np.isnan(maps["ggm"]), np.isnan(om["ggm"]))


def test_b1map(D, orc, ctx):
    c = CASES["chi2"]
    X = (4, 4, 1)
    img = D.mock_image(D.MockImageOptions(MatrixSize=X, nTE=32, TE=10e-3), seed=2)
    b1 = np.random.default_rng(1).uniform(140, 180, X)
    o = D.T2mapOptions(MatrixSize=X, nTE=32, TE=10e-3, nT2=40, T2Range=(10e-3, 2.0), Reg="chi2", Chi2Factor=1.02,
                       nRefAngles=8)
    maps, dist = D.T2mapSEcorr(img, o, b1map=b1, ctx=ctx)
    om, od = orc.t2map(img, orc_opts(orc, o), b1map=b1)
    np.testing.assert_array_equal(maps["alpha"], b1)
    np.testing.assert_array_equal(dist, od)


def test_stats_and_launches(D, orc, ctx):
    c = CASES["chi2"]
    run_case(D, orc, ctx, c)
    st = ctx.stats()
    assert st["voxels"] == 128 and st["voxels_processed"] == 128
    assert st["nnls_cap_hits"] == 0 and st["search_limit_hits"] == 0
    assert st["solve_launches"] == 1 and st["kernel_launches"] >= 3
    assert st["ms_solve"] > 0
