"""The reference's command-line settings sweep (test/cli.jl:255-287), run
through the API: each case changes one group of settings from the sweep's
defaults (test/cli.jl:2-21) and keeps the others, nTE and nT2 are drawn from
4:64 unless the case sets them (test/cli.jl:121-127), and the 2x2x2 mock
image is scaled to a unit-mean first echo (test/cli.jl:130-139), so
Threshold = 1 skips some voxels, Inf all of them and -Inf none.

The reference compares its CLI against its API on each case, including a rerun
with the fitted flip-angle map passed back as the B1 map (rtol 1e-14,
test/cli.jl:318-328) and a T2part-only run on the saved distribution
(test/cli.jl:339-348).  Here the oracle's outputs are checked for the
invariants of the path on the CPU, and on the GPU the FP64 method is held to
the oracle on every case, the B1 rerun and the standalone T2part to the fused
run, and the saved per-voxel basis to the EPG curves at the fitted angle;
the mixed method is held to its MWF gate on every case.
(`Silent` and `Threaded` change no result and are left out.)"""
import numpy as np
import pytest

from parity import DIST_RTOL, MWF_ATOL, dist_rel_err, orc_opts

DEFAULTS = dict(TE=8e-3, T2Range=(12e-3, 1.8), SPWin=(12e-3, 37e-3), MPWin=(37e-3, 650e-3), Reg="lcurve")
LEGACY_DEFAULTS = dict(TE=10e-3, T2Range=(15e-3, 2.0), SPWin=(14e-3, 40e-3), MPWin=(40e-3, 200e-3), Reg="chi2",
                       RegParams=1.02, Threshold=200.0)

SWEEP = {
    "MPWin": dict(MPWin=(38e-3, 180e-3)),
    "MinRefAngle": dict(MinRefAngle=55.0),
    "RefConAngle": dict(RefConAngle=172.0),
    "Reg_lcurve": dict(Reg="lcurve"),
    "Reg_gcv": dict(Reg="gcv"),
    "Reg_chi2": dict(Reg="chi2", RegParams=1.025),
    "Reg_mdp": dict(Reg="mdp", RegParams=3e-4),
    "Reg_none": dict(Reg="none"),
    "SPWin": dict(SPWin=(13e-3, 37e-3)),
    "SaveResidualNorm": dict(SaveResidualNorm=True),
    "SaveDecayCurve": dict(SaveDecayCurve=True),
    "SaveNNLSBasis": dict(SaveNNLSBasis=True),
    "SaveRegParam": dict(SaveRegParam=True),
    "SetFlipAngle": dict(SetFlipAngle=170.0),
    "SetFlipAngle_basis": dict(SetFlipAngle=170.0, SaveNNLSBasis=True),
    "Sigmoid": dict(Sigmoid=1.0),
    "T1": dict(T1=0.95),
    "T2Range": dict(T2Range=(16e-3, 1.8)),
    "TE": dict(TE=11e-3),
    "Threshold_1": dict(Threshold=1.0),
    "Threshold_Inf": dict(Threshold=np.inf),
    "Threshold_-Inf": dict(Threshold=-np.inf),
    "nRefAngles_9": dict(nRefAngles=9),
    "nRefAngles_10": dict(nRefAngles=10),
    "nRefAnglesMin_4": dict(nRefAnglesMin=4),
    "nRefAnglesMin_7": dict(nRefAnglesMin=7),
    "nTE_4": dict(nTE=4),
    "nTE_5": dict(nTE=5),
    "nTE_8": dict(nTE=8),
    "nTE_47": dict(nTE=47),
    "nT2_2": dict(nT2=2),
    "nT2_3": dict(nT2=3),
    "nT2_8": dict(nT2=8),
    "nT2_47": dict(nT2=47),
    "legacy_gcv": dict(legacy=True, Threshold=1.0, Reg="gcv", RegParams=None),
    "legacy_chi2": dict(legacy=True, Threshold=0.0, Reg="chi2", RegParams=1.025),
}
NAMES = list(SWEEP)
X = (2, 2, 2)


def settings(name):
    """The case's full settings (the defaults, its own values, nTE/nT2 drawn)."""
    p = dict(SWEEP[name])
    base = dict(DEFAULTS)
    if p.get("legacy"):
        base.update(LEGACY_DEFAULTS)
    base.update(p)
    rng = np.random.default_rng(1000 + NAMES.index(name))
    m, n = (int(v) for v in rng.integers(4, 65, size=2))
    base.setdefault("nTE", m)
    base.setdefault("nT2", n)
    return base


def image(D, s, seed):
    img = D.mock_image(D.MockImageOptions(MatrixSize=X, nTE=s["nTE"], TE=s["TE"]), seed=seed)
    return img / img[..., 0].mean()


def options(D, s, precision="fp64"):
    rp = s.get("RegParams")
    mo = D.T2mapOptions(
        MatrixSize=X, nTE=s["nTE"], TE=s["TE"], nT2=s["nT2"], T2Range=s["T2Range"], Reg=s["Reg"],
        legacy=s.get("legacy", False), T1=s.get("T1", 1.0), Threshold=s.get("Threshold", 0.0),
        MinRefAngle=s.get("MinRefAngle", 50.0), nRefAngles=s.get("nRefAngles"), nRefAnglesMin=s.get("nRefAnglesMin"),
        Chi2Factor=rp if s["Reg"] == "chi2" else None, NoiseLevel=rp if s["Reg"] == "mdp" else None,
        RefConAngle=s.get("RefConAngle", 180.0), SetFlipAngle=s.get("SetFlipAngle"),
        SaveResidualNorm=s.get("SaveResidualNorm", False), SaveDecayCurve=s.get("SaveDecayCurve", False),
        SaveRegParam=s.get("SaveRegParam", False), SaveNNLSBasis=s.get("SaveNNLSBasis", False), precision=precision)
    po = D.T2partOptions.from_t2map(mo, SPWin=s["SPWin"], MPWin=s["MPWin"], Sigmoid=s.get("Sigmoid"))
    return mo, po


def oracle_run(orc, img, mo, po):
    om, od = orc.t2map(img, orc_opts(orc, mo))
    op = orc.t2part(od, orc.T2partOptions(MatrixSize=X, nT2=mo.nT2, T2Range=mo.T2Range, SPWin=po.SPWin,
                                          MPWin=po.MPWin, Sigmoid=po.Sigmoid))
    return om, od, op


@pytest.mark.parametrize("name", NAMES)
def test_oracle_sweep_invariants(D, orc, name):
    """On the CPU: the oracle runs every case, processes exactly the voxels
    whose first echo is above Threshold, and its outputs keep the path's
    invariants (non-negative distributions, angles in range, fractions in
    [0, 1], a regularized residual no smaller than the unregularized one)."""
    s = settings(name)
    img = image(D, s, seed=NAMES.index(name))
    mo, po = options(D, s)
    om, od, op = oracle_run(orc, img, mo, po)
    done = img[..., 0] > mo.Threshold
    np.testing.assert_array_equal(~np.isnan(od).any(axis=-1), done)
    np.testing.assert_array_equal(~np.isnan(om["alpha"]), done)
    if mo.Threshold == np.inf:
        assert not done.any()
    if mo.Threshold == -np.inf:
        assert done.all()
    d = od[done]
    assert (d >= 0).all()
    a = om["alpha"][done]
    if mo.SetFlipAngle is not None:
        assert (a == mo.SetFlipAngle).all()
    else:
        assert ((a >= mo.MinRefAngle) & (a <= 180.0)).all()
    ok = done & (od.sum(axis=-1) > 0)
    for k in ("sfr", "mfr"):
        v = op[k][ok]
        assert ((v >= 0) & (v <= 1 + 1e-12)).all(), k
    if mo.SaveRegParam:
        assert (om["mu"][done] >= 0).all()
        assert (om["chi2factor"][done] >= 1 - 1e-8).all()
    if mo.SaveResidualNorm:
        assert (om["resnorm"][done] >= 0).all()
    if mo.SaveDecayCurve:
        assert om["decaycurve"].shape == X + (mo.nTE,)
        np.testing.assert_array_equal(np.isnan(om["decaycurve"]).any(axis=-1), ~done)


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_gpu_sweep_matches_oracle(D, orc, ctx, name):
    s = settings(name)
    img = image(D, s, seed=NAMES.index(name))
    mo, po = options(D, s)
    maps, dist, parts = D.T2mapSEcorr_T2partSEcorr(img, mo, po, ctx=ctx)
    om, od, op = oracle_run(orc, img, mo, po)

    np.testing.assert_array_equal(np.isnan(dist), np.isnan(od))
    err, ok = dist_rel_err(dist, od)
    if ok.any():
        assert err[ok].max() <= DIST_RTOL
    for k in ("gdn", "ggm", "gva", "fnr", "snr", "alpha", "resnorm", "mu", "chi2factor", "decaycurve"):
        if k not in om:
            continue
        a, b = maps[k], om[k]
        np.testing.assert_array_equal(np.isnan(a), np.isnan(b), err_msg=k)
        np.testing.assert_allclose(a[~np.isnan(b)], b[~np.isnan(b)], rtol=1e-8, atol=0, err_msg=k)
    np.testing.assert_array_equal(np.isnan(parts["sfr"]), np.isnan(op["sfr"]))
    if not np.isnan(op["sfr"]).all():
        assert np.nanmax(np.abs(parts["sfr"] - op["sfr"])) <= MWF_ATOL
    for k in ("sgm", "mfr", "mgm"):
        np.testing.assert_array_equal(np.isnan(parts[k]), np.isnan(op[k]), err_msg=k)
        np.testing.assert_allclose(parts[k], op[k], rtol=1e-8, atol=MWF_ATOL, equal_nan=True, err_msg=k)

    # T2part alone on the saved distribution == the T2part fused into the solve
    alone = D.T2partSEcorr(dist, po, ctx=ctx)
    for k in ("sfr", "sgm", "mfr", "mgm"):
        np.testing.assert_allclose(alone[k], parts[k], rtol=1e-12, atol=1e-15, equal_nan=True, err_msg=k)

    if mo.SaveNNLSBasis:
        t2 = orc.logrange(*mo.T2Range, mo.nT2)
        if mo.SetFlipAngle is not None:
            want = np.stack([orc.epg_decay_curve(mo.nTE, mo.SetFlipAngle, mo.TE, t, mo.T1, mo.RefConAngle)
                             for t in t2], axis=1)
            np.testing.assert_allclose(maps["decaybasis"], want, rtol=1e-10, atol=0)
        else:
            B = maps["decaybasis"]
            assert B.shape == X + (mo.nTE, mo.nT2)
            for I in np.ndindex(*X):
                if np.isnan(maps["alpha"][I]):
                    assert np.isnan(B[I]).all()
                    continue
                want = np.stack([orc.epg_decay_curve(mo.nTE, maps["alpha"][I], mo.TE, t, mo.T1, mo.RefConAngle)
                                 for t in t2], axis=1)
                np.testing.assert_allclose(B[I], want, rtol=1e-10, atol=0)

    # the fitted angles passed back as a B1 map reproduce the run
    if mo.SetFlipAngle is None and not np.isnan(maps["alpha"]).all():
        maps_b1, dist_b1, parts_b1 = D.T2mapSEcorr_T2partSEcorr(img, mo, po, b1map=maps["alpha"], ctx=ctx)
        np.testing.assert_array_equal(np.isnan(dist_b1), np.isnan(dist))
        e, okb = dist_rel_err(dist_b1, dist)
        assert e[okb].max() <= DIST_RTOL
        np.testing.assert_array_equal(maps_b1["alpha"], maps["alpha"])
        np.testing.assert_allclose(parts_b1["sfr"], parts["sfr"], rtol=0, atol=MWF_ATOL, equal_nan=True)


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_gpu_sweep_mixed(D, orc, ctx, name):
    """The mixed method on every case: the same voxels processed as the FP64
    oracle, non-negative distributions, MWF within the method's gate (1e-3;
    measured on a GB300: at most 6.3e-5 over the sweep) and flip angles
    within 1e-2 degrees (measured: 1.3e-9)."""
    s = settings(name)
    img = image(D, s, seed=NAMES.index(name))
    mo, po = options(D, s, precision="mixed")
    maps, dist, parts = D.T2mapSEcorr_T2partSEcorr(img, mo, po, ctx=ctx)
    om, od, op = oracle_run(orc, img, mo, po)
    np.testing.assert_array_equal(np.isnan(dist), np.isnan(od))
    np.testing.assert_array_equal(np.isnan(maps["alpha"]), np.isnan(om["alpha"]))
    done = ~np.isnan(od).any(axis=-1)
    assert (dist[done] >= 0).all()
    if done.any():
        d_mwf = np.abs(parts["sfr"] - op["sfr"])[~np.isnan(op["sfr"])]
        d_alpha = np.abs(maps["alpha"] - om["alpha"])[done]
        print(f"SWEEP_MIXED {name} voxels={int(done.sum())} mwf_max={d_mwf.max():.3e} "
              f"mwf_median={np.median(d_mwf):.3e} alpha_max={d_alpha.max():.3e}")
        assert d_mwf.max() <= 1e-3
        assert d_alpha.max() <= 1e-2


# Corners of the supported shapes: the fewest echoes, T2 bins and angles the
# options allow, and the most this library supports (nTE <= 128, nT2 <= 64
# for the mixed method, nRefAngles <= 256).
EXTREMES = {
    "min": dict(nTE=4, nT2=2, nRefAngles=2, nRefAnglesMin=2),
    "min_m_max_n": dict(nTE=4, nT2=64, nRefAngles=8),
    "max_m_min_n": dict(nTE=128, nT2=2, nRefAngles=8),
    "max": dict(nTE=128, nT2=64, nRefAngles=256),
    "max_legacy": dict(nTE=128, nT2=64, nRefAngles=256, legacy=True, Reg="chi2", RegParams=1.02, Threshold=0.0),
}


def extreme_settings(name):
    s = dict(DEFAULTS)
    if EXTREMES[name].get("legacy"):
        s.update(LEGACY_DEFAULTS)
    s.update(EXTREMES[name])
    return s


@pytest.mark.parametrize("name", list(EXTREMES))
def test_oracle_extreme_shapes(D, orc, name):
    s = extreme_settings(name)
    img = image(D, s, seed=7)
    mo, po = options(D, s)
    om, od, op = oracle_run(orc, img, mo, po)
    assert not np.isnan(od).any() and (od >= 0).all()
    assert ((om["alpha"] >= mo.MinRefAngle) & (om["alpha"] <= 180.0)).all()


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(EXTREMES))
def test_gpu_extreme_shapes(D, orc, ctx, name):
    """Both methods at the corners: FP64 within the stated tolerances of the
    oracle, the mixed method within its MWF gate."""
    s = extreme_settings(name)
    img = image(D, s, seed=7)
    mo, po = options(D, s)
    om, od, op = oracle_run(orc, img, mo, po)
    maps, dist, parts = D.T2mapSEcorr_T2partSEcorr(img, mo, po, ctx=ctx)
    err, ok = dist_rel_err(dist, od)
    assert ok.all() and err.max() <= DIST_RTOL
    assert np.abs(parts["sfr"] - op["sfr"]).max() <= MWF_ATOL
    mo_x, po_x = options(D, s, precision="mixed")
    maps_x, dist_x, parts_x = D.T2mapSEcorr_T2partSEcorr(img, mo_x, po_x, ctx=ctx)
    assert not np.isnan(dist_x).any() and (dist_x >= 0).all()
    d_mwf = np.abs(parts_x["sfr"] - op["sfr"])
    print(f"EXTREME {name} mwf_max_mixed={d_mwf.max():.3e}")
    assert d_mwf.max() <= 1e-3
