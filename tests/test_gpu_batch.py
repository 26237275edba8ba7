"""Batched volumes (decaes_t2map_t2part_batch, decaes_batch_create/run) and
the autotuner, called through the C ABI: every volume of a batch gives the
same outputs, bit for bit, as its own decaes_t2map_t2part_device call, for
both methods, both dtypes and uneven shapes; a captured batch replays to the
same outputs; tuned launch shapes change no result."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SPWIN, MPWIN = (10e-3, 25e-3), (25e-3, 200e-3)
MAPS = ("gdn", "ggm", "gva", "fnr", "snr", "alpha", "resnorm", "mu", "chi2factor")
PARTS = ("sfr", "sgm", "mfr", "mgm")

# uneven volumes: echo counts, nT2, regularizers, methods, dtypes, masks
VOLS = [
    dict(X=(9, 7, 2), m=48, TE=10e-3, n=40, K=32, Reg="lcurve", prec="mixed", dtype=np.float32, bg=0.4, thr=200.0, seed=1),
    dict(X=(6, 5, 3), m=32, TE=8e-3, n=48, K=16, Reg="chi2", Chi2Factor=1.02, prec="fp64", dtype=np.float64, seed=2),
    dict(X=(5, 5, 2), m=24, TE=12e-3, n=40, K=8, Reg="none", prec="fp64", dtype=np.float32, seed=3),
    dict(X=(4, 6, 2), m=56, TE=7e-3, n=60, K=64, Reg="gcv", prec="mixed", dtype=np.float64, bg=0.5, thr=200.0, seed=4),
    dict(X=(3, 3, 1), m=32, TE=10e-3, n=40, K=8, Reg="lcurve", prec="fp64", dtype=np.float32, seed=5, Sigmoid=5e-3),
    # legacy = true: the batch runs on the legacy kernel, the other volumes with it
    dict(X=(4, 4, 2), m=32, TE=10e-3, n=40, K=8, Reg="chi2", Chi2Factor=1.02, prec="fp64", dtype=np.float64, seed=6,
         legacy=True),
]


def _lib():
    from decaes_gb300 import _lib
    return _lib


class Vol:
    def __init__(self, D, c):
        import torch
        self.c = c
        img = D.mock_image(D.MockImageOptions(MatrixSize=c["X"], nTE=c["m"], TE=c["TE"],
                                              BackgroundFraction=c.get("bg", 0.0)), seed=c["seed"], dtype=c["dtype"])
        self.mo = D.T2mapOptions(MatrixSize=c["X"], nTE=c["m"], TE=c["TE"], nT2=c["n"], T2Range=(10e-3, 2.0),
                                 Reg=c["Reg"], nRefAngles=c["K"], Chi2Factor=c.get("Chi2Factor"),
                                 Threshold=c.get("thr", 0.0), SaveRegParam=True, SaveResidualNorm=True,
                                 precision=c["prec"], legacy=c.get("legacy", False))
        self.po = D.T2partOptions.from_t2map(self.mo, SPWin=SPWIN, MPWin=MPWIN, Sigmoid=c.get("Sigmoid"))
        self.d_img = torch.from_numpy(np.asfortranarray(img).reshape(-1, order="F").copy()).cuda()
        V = int(np.prod(c["X"]))
        tdt = torch.float32 if c["dtype"] == np.float32 else torch.float64
        self.out = {"dist": torch.full((V * c["n"],), 7.0, dtype=tdt, device="cuda")}
        for k in MAPS + PARTS:
            self.out[k] = torch.full((V,), 7.0, dtype=tdt, device="cuda")
        L = _lib()
        self.mc = L.T2mapOutC(**{k: self.out[k].data_ptr() for k in ("dist",) + MAPS})
        self.pc = L.T2partOutC(**{k: self.out[k].data_ptr() for k in PARTS})
        self.code = L.F32 if c["dtype"] == np.float32 else L.F64

    def volume_c(self):
        L = _lib()
        return L.VolumeC(mopts=self.mo.to_c(), popts=self.po.to_c(), has_t2part=1, dtype=self.code,
                         d_image=self.d_img.data_ptr(), d_b1map=None, d_mout=self.mc, d_pout=self.pc)

    def host(self):
        return {k: t.double().cpu().numpy() for k, t in self.out.items()}

    def reset(self):
        for t in self.out.values():
            t.fill_(7.0)


def _same(a, b, name):
    for k in a:
        np.testing.assert_array_equal(np.isnan(a[k]), np.isnan(b[k]), err_msg=f"{name}:{k}")
        np.testing.assert_array_equal(np.nan_to_num(a[k], nan=0.0), np.nan_to_num(b[k], nan=0.0), err_msg=f"{name}:{k}")


def _single(D, ctx, v):
    L = D.load()
    ctx.check(L.decaes_t2map_t2part_device(ctx.h, C.byref(v.mo.to_c()), C.byref(v.po.to_c()),
                                           C.c_void_p(v.d_img.data_ptr()), v.code, None, C.byref(v.mc),
                                           C.byref(v.pc), None))
    ctx.check(L.decaes_sync_stats(ctx.h, None))
    return v.host()


def test_batch_matches_single_calls(D, ctx):
    import torch
    vols = [Vol(D, c) for c in VOLS]
    want = []
    for v in vols:
        want.append(_single(D, ctx, v))
        v.reset()
    arr = (_lib().VolumeC * len(vols))(*[v.volume_c() for v in vols])
    ctx.check(D.load().decaes_t2map_t2part_batch(ctx.h, arr, len(vols), None))
    ctx.check(D.load().decaes_sync_stats(ctx.h, None))
    torch.cuda.synchronize()
    for i, v in enumerate(vols):
        got = v.host()
        assert np.isfinite(got["dist"]).any()
        _same(got, want[i], f"vol{i}")


def test_prepared_batch_replays(D, ctx):
    import torch
    vols = [Vol(D, c) for c in VOLS[:3]] + [Vol(D, VOLS[5])]
    want = []
    for v in vols:
        want.append(_single(D, ctx, v))
        v.reset()
    L = D.load()
    arr = (_lib().VolumeC * len(vols))(*[v.volume_c() for v in vols])
    b = L.decaes_batch_create(ctx.h, arr, len(vols))
    assert b, L.decaes_last_error(ctx.h).decode()
    try:
        for rep in range(2):
            for v in vols:
                v.reset()
            assert L.decaes_batch_run(b, None) == 0
            ctx.check(L.decaes_sync_stats(ctx.h, None))
            torch.cuda.synchronize()
            for i, v in enumerate(vols):
                _same(v.host(), want[i], f"rep{rep}:vol{i}")
    finally:
        L.decaes_batch_destroy(b)


def test_autotune_keeps_results(D, ctx):
    v = Vol(D, VOLS[0])
    before = _single(D, ctx, v)
    t = _lib().TuningC()
    ctx.check(D.load().decaes_autotune(ctx.h, C.byref(v.mo.to_c()), C.byref(t)))
    assert t.warps_per_block in (1, 2, 4) and t.us_per_voxel > 0 and t.blocks_per_sm >= 0
    print("tuned:", t.warps_per_block, "warps per block,", t.blocks_per_sm or "all", "blocks per SM,",
          t.us_per_voxel, "us per voxel")
    v.reset()
    _same(_single(D, ctx, v), before, "tuned")


def test_batch_rejects_bad_volume(D, ctx):
    v = Vol(D, VOLS[2])
    bad = v.volume_c()
    bad.d_mout.t2times = 8
    arr = (_lib().VolumeC * 1)(bad)
    rc = D.load().decaes_t2map_t2part_batch(ctx.h, arr, 1, None)
    assert rc == 1
    assert b"constant outputs" in D.load().decaes_last_error(ctx.h)


def test_batch_with_more_shapes_than_resident_bases(D, ctx):
    """More distinct parameter keys than the context keeps resident (8): the
    batch holds every basis it uses until it has run."""
    import torch
    cs = [dict(X=(3, 3, 1), m=24 + 2 * i, TE=10e-3, n=40, K=8, Reg="chi2", Chi2Factor=1.02,
               prec="mixed" if i % 2 else "fp64", dtype=np.float32, seed=20 + i) for i in range(12)]
    vols = [Vol(D, c) for c in cs]
    arr = (_lib().VolumeC * len(vols))(*[v.volume_c() for v in vols])
    ctx.check(D.load().decaes_t2map_t2part_batch(ctx.h, arr, len(vols), None))
    ctx.check(D.load().decaes_sync_stats(ctx.h, None))
    torch.cuda.synchronize()
    got = [v.host() for v in vols]
    for i, v in enumerate(vols):
        v.reset()
        _same(_single(D, ctx, v), got[i], f"vol{i}")
