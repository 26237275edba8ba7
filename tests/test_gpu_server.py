"""The continuous-batching server: requests of different shapes, methods and
dtypes submitted together give, bit for bit, the results of the same requests
run alone; requests larger than a tick are split across ticks; a request
larger than the admission budget fails alone."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SPWIN, MPWIN = (10e-3, 25e-3), (25e-3, 200e-3)

REQS = [
    dict(X=(12, 10, 3), m=48, TE=10e-3, n=40, K=32, Reg="lcurve", prec="mixed", dtype=np.float32, bg=0.35, thr=200.0, seed=1),
    dict(X=(7, 6, 2), m=32, TE=8e-3, n=48, K=16, Reg="chi2", Chi2Factor=1.02, prec="fp64", dtype=np.float64, seed=2),
    dict(X=(5, 5, 1), m=56, TE=7e-3, n=60, K=64, Reg="gcv", prec="mixed", dtype=np.float32, seed=3),
    dict(X=(9, 9, 1), m=24, TE=12e-3, n=40, K=8, Reg="none", prec="fp64", dtype=np.float32, seed=4),
    dict(X=(6, 6, 2), m=48, TE=10e-3, n=40, K=32, Reg="lcurve", prec="fp64", dtype=np.float64, seed=5),
    # legacy = true: ticks holding its chunks run the legacy kernel
    dict(X=(5, 4, 2), m=32, TE=10e-3, n=40, K=8, Reg="chi2", Chi2Factor=1.02, prec="fp64", dtype=np.float32, seed=6,
         legacy=True),
]


def _req(D, c):
    img = D.mock_image(D.MockImageOptions(MatrixSize=c["X"], nTE=c["m"], TE=c["TE"],
                                          BackgroundFraction=c.get("bg", 0.0)), seed=c["seed"], dtype=c["dtype"])
    mo = D.T2mapOptions(MatrixSize=c["X"], nTE=c["m"], TE=c["TE"], nT2=c["n"], T2Range=(10e-3, 2.0), Reg=c["Reg"],
                        nRefAngles=c["K"], Chi2Factor=c.get("Chi2Factor"), Threshold=c.get("thr", 0.0),
                        SaveRegParam=True, SaveResidualNorm=True, precision=c["prec"], legacy=c.get("legacy", False))
    po = D.T2partOptions.from_t2map(mo, SPWin=SPWIN, MPWin=MPWIN)
    return img, mo, po


def _same(a, b):
    ma, da, pa = a
    mb, db, pb = b
    np.testing.assert_array_equal(da, db)
    for k in ("gdn", "ggm", "gva", "fnr", "snr", "alpha", "resnorm", "mu", "chi2factor", "t2times", "echotimes"):
        np.testing.assert_array_equal(ma[k], mb[k], err_msg=k)
    for k in pa:
        np.testing.assert_array_equal(pa[k], pb[k], err_msg=k)


def test_mixed_requests_match_alone(D, ctx):
    from decaes_gb300.server import Server
    reqs = [_req(D, c) for c in REQS]
    alone = [D.T2mapSEcorr_T2partSEcorr(img, mo, po, ctx=ctx) for img, mo, po in reqs]
    srv = Server(ctx, tick_voxels=150)  # small ticks: every request spans several ticks
    try:
        ids = [srv.submit(img, mo, po) for img, mo, po in reqs]
        got = [srv.result(i) for i in ids]
        st = srv.stats()
    finally:
        srv.close()
    for a, b in zip(got, alone):
        _same(a, b)
    total = sum(int(np.prod(c["X"])) for c in REQS)
    assert st["completed"] == len(reqs) and st["failed"] == 0 and st["ticks"] >= -(-total // 150)
    assert st["voxels"] == total
    assert st["p99_ms"] >= st["p50_ms"] > 0 and st["busy_ms"] > 0


def test_admission_by_footprint(D, ctx):
    """A budget below the sum of the requests' footprints still completes every
    request (each admitted as memory frees up); a request larger than the
    whole budget fails on its own."""
    from decaes_gb300.server import Server
    reqs = [_req(D, c) for c in REQS[:3]]
    alone = [D.T2mapSEcorr_T2partSEcorr(img, mo, po, ctx=ctx) for img, mo, po in reqs]
    big = _req(D, dict(REQS[0], X=(60, 60, 20), seed=9))
    srv = Server(ctx, tick_voxels=4096, hbm_budget_bytes=350_000)
    try:
        ids = [srv.submit(img, mo, po) for img, mo, po in reqs]
        bid = srv.submit(*big)
        got = [srv.result(i) for i in ids]
        with pytest.raises(RuntimeError, match="ENOMEM"):
            srv.result(bid)
    finally:
        srv.close()
    for a, b in zip(got, alone):
        _same(a, b)


def test_reset_stats(D, ctx):
    """Counters and latency samples restart after reset_stats (warm-up excluded from percentiles)."""
    from decaes_gb300.server import Server
    img, mo, po = _req(D, REQS[3])
    srv = Server(ctx)
    try:
        srv.result(srv.submit(img, mo, po))
        assert srv.stats()["completed"] == 1
        srv.reset_stats()
        st = srv.stats()
        assert st["completed"] == 0 and st["p50_ms"] == 0 and st["voxels"] == 0
        srv.result(srv.submit(img, mo, po))
        st = srv.stats()
        assert st["completed"] == 1 and st["p50_ms"] > 0 and st["voxels"] == int(np.prod(REQS[3]["X"]))
    finally:
        srv.close()
