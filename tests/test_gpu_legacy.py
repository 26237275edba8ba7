"""legacy = true on the GPU against the oracle: the spline-surrogate flip-angle
search (spline_opt_legacy on knots[1]:0.001:knots[end]) and the chi2 search by
mu doubling with the legacy spline root.  The FP64 method is bit-exact with the
oracle; the mixed method is held to its MWF gate."""
import numpy as np
import pytest

from parity import DIST_RTOL, MWF_ATOL, dist_rel_err, orc_opts

pytestmark = pytest.mark.gpu

SPWIN, MPWIN = (14e-3, 40e-3), (40e-3, 200e-3)

CASES = {
    # the legacy defaults: chi2 1.02, 8 angles all evaluated, T2 15 ms-2 s, threshold 200
    "chi2_defaults": dict(X=(8, 8, 2), m=32, TE=10e-3, n=40, T2=(15e-3, 2.0), Reg="chi2", Chi2Factor=1.02,
                          thr=200.0, bg=0.3),
    # the legacy search with another regularizer, 48 echoes
    "lcurve_search": dict(X=(6, 6, 1), m=48, TE=10e-3, n=40, T2=(10e-3, 2.0), Reg="lcurve"),
    # a subset of 16 angles evaluated: the knots differ between voxels
    "partial_grid": dict(X=(6, 6, 1), m=32, TE=10e-3, n=40, T2=(15e-3, 2.0), Reg="chi2", Chi2Factor=1.02,
                         K=16, Kmin=5),
    # 150 degree refocusing control angle (DualVector EPG) with the legacy chi2
    "refcon150": dict(X=(4, 4, 1), m=32, TE=10e-3, n=40, T2=(15e-3, 2.0), Reg="chi2", Chi2Factor=1.05,
                      RefConAngle=150.0),
    # fixed angle: only the legacy chi2 search runs
    "fixed_angle": dict(X=(6, 6, 1), m=32, TE=10e-3, n=40, T2=(15e-3, 2.0), Reg="chi2", Chi2Factor=1.02,
                        SetFlipAngle=170.0),
}


def run_case(D, orc, ctx, c, precision="fp64", seed=11):
    img = D.mock_image(D.MockImageOptions(MatrixSize=c["X"], nTE=c["m"], TE=c["TE"],
                                          BackgroundFraction=c.get("bg", 0.0)), seed=seed)
    kw = dict(MatrixSize=c["X"], nTE=c["m"], TE=c["TE"], nT2=c["n"], T2Range=c["T2"], Reg=c["Reg"],
              Chi2Factor=c.get("Chi2Factor"), Threshold=c.get("thr", 0.0), RefConAngle=c.get("RefConAngle", 180.0),
              SetFlipAngle=c.get("SetFlipAngle"), SaveRegParam=True, SaveResidualNorm=True, legacy=True)
    if "K" in c:
        kw.update(nRefAngles=c["K"], nRefAnglesMin=c["Kmin"])
    o = D.T2mapOptions(**kw, precision=precision)
    po = D.T2partOptions.from_t2map(o, SPWin=SPWIN, MPWin=MPWIN)
    maps, dist, parts = D.T2mapSEcorr_T2partSEcorr(img, o, po, ctx=ctx)
    om, od = orc.t2map(img, orc_opts(orc, D.T2mapOptions(**kw)), nthreads=8)
    op = orc.t2part(od, orc.T2partOptions(MatrixSize=c["X"], nT2=c["n"], T2Range=c["T2"], SPWin=SPWIN, MPWin=MPWIN))
    return o, maps, dist, parts, om, od, op


def test_legacy_defaults(D):
    o = D.T2mapOptions(MatrixSize=(2, 2, 1), nTE=32, TE=10e-3, nT2=40, T2Range=(15e-3, 2.0), Reg="chi2",
                       Chi2Factor=1.02, legacy=True)
    assert o.nRefAngles == 8 and o.nRefAnglesMin == 8


@pytest.mark.parametrize("name", list(CASES))
def test_legacy_fp64_bitwise(D, orc, ctx, name):
    c = CASES[name]
    o, maps, dist, parts, om, od, op = run_case(D, orc, ctx, c)
    np.testing.assert_array_equal(np.isnan(dist), np.isnan(od))
    ok = ~np.isnan(od).any(axis=-1)
    assert ok.any()
    np.testing.assert_array_equal(dist, od)
    for k in ("alpha", "mu", "chi2factor", "resnorm", "gdn", "ggm", "gva", "fnr", "snr"):
        np.testing.assert_array_equal(maps[k], om[k], err_msg=k)
    # T2part's window sums run in another order than the oracle's: MWF to MWF_ATOL
    np.testing.assert_array_equal(np.isnan(parts["sfr"]), np.isnan(op["sfr"]))
    assert np.nanmax(np.abs(parts["sfr"] - op["sfr"])) <= MWF_ATOL
    alpha = maps["alpha"][~np.isnan(maps["alpha"])]
    if c.get("SetFlipAngle") is None:
        # the legacy search returns points of the 0.001 degree grid
        np.testing.assert_allclose(alpha * 1000, np.round(alpha * 1000), atol=1e-6)
    if c["Reg"] == "chi2":
        mu = maps["mu"][~np.isnan(maps["mu"])]
        np.testing.assert_allclose(mu * 1000, np.round(mu * 1000), atol=1e-6)
    print(f"{name}: voxels={int(ok.sum())} alpha[:4]={alpha[:4]}")


@pytest.mark.parametrize("name", ["chi2_defaults", "partial_grid"])
def test_legacy_mixed_within_gate(D, orc, ctx, name):
    c = CASES[name]
    o, maps, dist, parts, om, od, op = run_case(D, orc, ctx, c, precision="mixed")
    np.testing.assert_array_equal(np.isnan(dist), np.isnan(od))
    d = np.abs(parts["sfr"] - op["sfr"])
    d = d[~np.isnan(d)]
    err, ok = dist_rel_err(dist, od)
    print(f"{name} mixed: MWF max {d.max():.3g}, alpha max {np.nanmax(np.abs(maps['alpha'] - om['alpha'])):.3g}")
    assert d.max() <= 1e-3
