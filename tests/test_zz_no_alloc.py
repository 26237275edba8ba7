"""decaes_t2map_t2part_noalloc (the entry point that allocates no device
memory, working in a static device array) against decaes_t2map_t2part_device
on the same device-resident inputs, called through the C ABI.

Collected last so that it also runs after every other GPU test has used the
library; it must pass alone in a fresh process as well."""
import ctypes as C

import numpy as np
import pytest

from parity import DIST_RTOL, MWF_ATOL, dist_rel_err

SPWIN, MPWIN = (10e-3, 25e-3), (25e-3, 200e-3)
MAPS = ("gdn", "ggm", "gva", "fnr", "snr", "alpha", "resnorm", "decaycurve", "mu", "chi2factor")
PARTS = ("sfr", "sgm", "mfr", "mgm")

CASES = [
    # 48 echoes, 32 angles, lcurve, 35% background below the threshold, FP64 image
    dict(X=(10, 8, 3), m=48, n=40, K=32, Reg="lcurve", bg=0.35, thr=200.0, dtype=np.float64, seed=3),
    # 32 echoes, 8 angles, chi2, Float32 image, Sigmoid-weighted T2part
    dict(X=(7, 5, 2), m=32, n=40, K=8, Reg="chi2", Chi2Factor=1.02, dtype=np.float32, seed=4, Sigmoid=5e-3),
]


def _setup(D, c):
    import torch
    img = D.mock_image(D.MockImageOptions(MatrixSize=c["X"], nTE=c["m"], BackgroundFraction=c.get("bg", 0.0)),
                       seed=c["seed"], dtype=c["dtype"])
    o = D.T2mapOptions(MatrixSize=c["X"], nTE=c["m"], TE=10e-3, nT2=c["n"], T2Range=(10e-3, 2.0), Reg=c["Reg"],
                       nRefAngles=c["K"], Chi2Factor=c.get("Chi2Factor"), Threshold=c.get("thr", 0.0),
                       SaveRegParam=True, SaveResidualNorm=True, SaveDecayCurve=True)
    po = D.T2partOptions.from_t2map(o, SPWin=SPWIN, MPWin=MPWIN, Sigmoid=c.get("Sigmoid"))
    d_img = torch.from_numpy(np.asfortranarray(img).reshape(-1, order="F").copy()).cuda()
    return o, po, d_img


def _outputs(o, dtype):
    import torch
    V = int(np.prod(o.MatrixSize))
    lens = dict(dist=V * o.nT2, decaycurve=V * o.nTE)
    mo = {k: torch.empty(lens.get(k, V), dtype=dtype, device="cuda") for k in ("dist",) + MAPS}
    po = {k: torch.empty(V, dtype=dtype, device="cuda") for k in PARTS}
    mc = D_lib().T2mapOutC(**{k: t.data_ptr() for k, t in mo.items()})
    pc = D_lib().T2partOutC(**{k: t.data_ptr() for k, t in po.items()})
    return mo, po, mc, pc


def D_lib():
    from decaes_gb300 import _lib
    return _lib


def _host(ts):
    return {k: t.double().cpu().numpy() for k, t in ts.items()}


def run_device(D, ctx, c):
    """The existing context entry point (allocates through its context)."""
    import torch
    o, po, d_img = _setup(D, c)
    mo, pt, mc, pc = _outputs(o, torch.float64 if c["dtype"] == np.float64 else torch.float32)
    L = D.load()
    ctx.check(L.decaes_t2map_t2part_device(ctx.h, C.byref(o.to_c()), C.byref(po.to_c()), C.c_void_p(d_img.data_ptr()),
                                           D_lib().F64 if c["dtype"] == np.float64 else D_lib().F32, None,
                                           C.byref(mc), C.byref(pc), None))
    ctx.check(L.decaes_sync_stats(ctx.h, None))
    return _host(mo), _host(pt)


def run_noalloc(D, c):
    import torch
    o, po, d_img = _setup(D, c)
    mo, pt, mc, pc = _outputs(o, torch.float64)
    # garbage in the outputs: the entry point NaN-fills them itself
    for t in list(mo.values()) + list(pt.values()):
        t.fill_(12345.0)
    err = C.create_string_buffer(512)
    L = D.load()
    rc = L.decaes_t2map_t2part_noalloc(C.byref(o.to_c()), C.byref(po.to_c()), C.c_void_p(d_img.data_ptr()),
                                       D_lib().F64 if c["dtype"] == np.float64 else D_lib().F32, None,
                                       C.byref(mc), C.byref(pc), None, err, len(err))
    assert rc == 0, err.value.decode()
    torch.cuda.synchronize()
    return _host(mo), _host(pt)


def _compare(c, got, want):
    (gm, gp), (wm, wp) = got, want
    narrow = c["dtype"] == np.float32   # the context path returns Float32 outputs for Float32 images
    conv = (lambda a: a.astype(np.float32).astype(np.float64)) if narrow else (lambda a: a)
    n = c["n"]
    np.testing.assert_array_equal(np.isnan(gm["dist"]), np.isnan(wm["dist"]))
    err, ok = dist_rel_err(conv(gm["dist"]).reshape(n, -1).T, wm["dist"].reshape(n, -1).T)
    assert ok.any()
    assert err[ok].max() <= DIST_RTOL
    assert np.nanmax(np.abs(conv(gp["sfr"]) - wp["sfr"])) <= MWF_ATOL
    for k in MAPS + PARTS:
        a, b = (gm[k], wm[k]) if k in gm else (gp[k], wp[k])
        np.testing.assert_array_equal(np.isnan(a), np.isnan(b), err_msg=k)
        np.testing.assert_allclose(conv(a)[~np.isnan(b)], b[~np.isnan(b)], rtol=1e-8, atol=0, err_msg=k)


@pytest.mark.gpu
def test_noalloc_matches_context_path(D, ctx):
    """Two different problems back to back, then the first again: every call
    matches the context entry point, whatever the previous call left in the
    shared static array."""
    want = [run_device(D, ctx, c) for c in CASES]
    for i in (0, 1, 0):
        _compare(CASES[i], run_noalloc(D, CASES[i]), want[i])


@pytest.mark.gpu
def test_noalloc_rejects_oversize(D, ctx):
    """A voxel list that does not fit the static array is refused before any
    work is queued."""
    import torch
    o = D.T2mapOptions(MatrixSize=(4096, 4096, 2), nTE=32, TE=10e-3, nT2=40, T2Range=(10e-3, 2.0), Reg="lcurve", nRefAngles=8)
    dummy = torch.zeros(64, dtype=torch.float64, device="cuda")
    mc = D_lib().T2mapOutC(**{k: dummy.data_ptr() for k in ("dist", "gdn", "ggm", "gva", "fnr", "snr", "alpha")})
    err = C.create_string_buffer(512)
    rc = D.load().decaes_t2map_t2part_noalloc(C.byref(o.to_c()), None, C.c_void_p(dummy.data_ptr()), D_lib().F64,
                                              None, C.byref(mc), None, None, err, len(err))
    assert rc == 3
    assert "static workspace" in err.value.decode()
    assert float(dummy.abs().sum()) == 0.0


def test_noalloc_argument_errors(D):
    """Argument checks happen on the host before any CUDA call (no GPU needed)."""
    L = D.load()
    err = C.create_string_buffer(256)
    o = D.T2mapOptions(MatrixSize=(2, 2, 1), nTE=32, TE=10e-3, nT2=40, T2Range=(10e-3, 2.0), Reg="lcurve")
    assert L.decaes_t2map_t2part_noalloc(C.byref(o.to_c()), None, None, D_lib().F64, None, None, None, None,
                                         err, len(err)) == 1
    assert b"must not be NULL" in err.value
    mc = D_lib().T2mapOutC(dist=8, gdn=8, ggm=8, gva=8, fnr=8, snr=8, alpha=8, t2times=8)
    assert L.decaes_t2map_t2part_noalloc(C.byref(o.to_c()), None, C.c_void_p(8), D_lib().F64, None, C.byref(mc),
                                         None, None, err, len(err)) == 1
    assert b"pass NULL" in err.value
    bad = D.T2mapOptions(MatrixSize=(2, 2, 1), nTE=32, TE=10e-3, nT2=40, T2Range=(10e-3, 2.0), Reg="lcurve").to_c()
    bad.nTE = 3
    assert L.decaes_t2map_t2part_noalloc(C.byref(bad), None, C.c_void_p(8), D_lib().F64, None, C.byref(mc),
                                         None, None, err, len(err)) == 1
    assert err.value.decode() == "At least four echoes are required for T2 mapping, but nTE = 3."


@pytest.mark.parametrize("field,value,msg", [
    ("nTE", 129, "nTE > 128 is not supported by libdecaes_gpu"),
    ("nRefAngles", 257, "nRefAngles > 256 is not supported by libdecaes_gpu"),
])
def test_noalloc_shape_limits(D, field, value, msg):
    """Shapes beyond the library's limits are rejected on the host, before any
    CUDA call (no GPU needed)."""
    L = D.load()
    err = C.create_string_buffer(256)
    o = D.T2mapOptions(MatrixSize=(2, 2, 1), nTE=32, TE=10e-3, nT2=40, T2Range=(10e-3, 2.0), Reg="lcurve").to_c()
    setattr(o, field, value)
    mc = D_lib().T2mapOutC(dist=8, gdn=8, ggm=8, gva=8, fnr=8, snr=8, alpha=8)
    assert L.decaes_t2map_t2part_noalloc(C.byref(o), None, C.c_void_p(8), D_lib().F64, None, C.byref(mc),
                                         None, None, err, len(err)) == 1
    assert err.value.decode() == msg
