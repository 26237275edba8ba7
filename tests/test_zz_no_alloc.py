"""decaes_t2map_t2part_noalloc (the entry point that allocates no device
memory, working in a static device array) against decaes_t2map_t2part_device
on the same device-resident inputs, called through the C ABI.

Collected last so that it also runs after every other GPU test has used the
library; it must pass alone in a fresh process as well."""
import ctypes as C

import numpy as np
import pytest

SPWIN, MPWIN = (10e-3, 25e-3), (25e-3, 200e-3)
REQUIRED = ("dist", "gdn", "ggm", "gva", "fnr", "snr", "alpha")
OPTIONAL = {"resnorm": "SaveResidualNorm", "decaycurve": "SaveDecayCurve", "mu": "SaveRegParam",
            "chi2factor": "SaveRegParam", "decaybasis": "SaveNNLSBasis"}
PARTS = ("sfr", "sgm", "mfr", "mgm")
SAVE_ALL = dict(SaveRegParam=True, SaveResidualNorm=True, SaveDecayCurve=True)

CASES = [
    # 48 echoes, 32 angles, lcurve, 35% background below the threshold, FP64
    # image, every optional output including the per-voxel basis
    dict(X=(10, 8, 3), m=48, n=40, K=32, Reg="lcurve", bg=0.35, thr=200.0, dtype=np.float64, seed=3,
         opts=dict(SAVE_ALL, SaveNNLSBasis=True)),
    # 32 echoes, 8 angles, chi2, Float32 image, Sigmoid-weighted T2part
    dict(X=(7, 5, 2), m=32, n=40, K=8, Reg="chi2", Chi2Factor=1.02, dtype=np.float32, seed=4, Sigmoid=5e-3,
         opts=SAVE_ALL),
    # fixed flip angle (the basis is built once, its work buffer shares the
    # solver scratch) with the saved nTE x nT2 basis
    dict(X=(6, 5, 2), m=32, n=40, K=8, Reg="none", dtype=np.float64, seed=5,
         opts=dict(SetFlipAngle=165.0, SaveNNLSBasis=True, SaveResidualNorm=True)),
    # legacy algorithms (spline-surrogate angle search, chi2 by mu doubling)
    dict(X=(5, 4, 2), m=32, n=40, K=8, Reg="chi2", Chi2Factor=1.02, dtype=np.float64, seed=6,
         opts=dict(legacy=True, SaveRegParam=True)),
    # B1 map in place of the flip-angle search
    dict(X=(6, 6, 1), m=32, n=40, K=16, Reg="lcurve", dtype=np.float64, seed=7, b1=True, opts=SAVE_ALL),
]


def D_lib():
    from decaes_gb300 import _lib
    return _lib


def _setup(D, c):
    import torch
    img = D.mock_image(D.MockImageOptions(MatrixSize=c["X"], nTE=c["m"], BackgroundFraction=c.get("bg", 0.0)),
                       seed=c["seed"], dtype=c["dtype"])
    o = D.T2mapOptions(MatrixSize=c["X"], nTE=c["m"], TE=10e-3, nT2=c["n"], T2Range=(10e-3, 2.0), Reg=c["Reg"],
                       nRefAngles=c["K"], Chi2Factor=c.get("Chi2Factor"), Threshold=c.get("thr", 0.0), **c["opts"])
    po = D.T2partOptions.from_t2map(o, SPWin=SPWIN, MPWin=MPWIN, Sigmoid=c.get("Sigmoid"))
    d_img = torch.from_numpy(np.asfortranarray(img).reshape(-1, order="F").copy()).cuda()
    d_b1 = None
    if c.get("b1"):
        b1 = np.random.default_rng(c["seed"]).uniform(150.0, 180.0, size=int(np.prod(c["X"]))).astype(c["dtype"])
        d_b1 = torch.from_numpy(b1).cuda()
    return o, po, d_img, d_b1


def _outputs(o, dtype):
    """Device buffers of the call dtype: the required outputs and the optional
    ones whose Save* flag is set."""
    import torch
    V = int(np.prod(o.MatrixSize))
    fixed = o.SetFlipAngle is not None
    lens = dict(dist=V * o.nT2, decaycurve=V * o.nTE,
                decaybasis=o.nTE * o.nT2 * (1 if fixed else V))
    keys = REQUIRED + tuple(k for k, flag in OPTIONAL.items() if getattr(o, flag))
    mo = {k: torch.empty(lens.get(k, V), dtype=dtype, device="cuda") for k in keys}
    po = {k: torch.empty(V, dtype=dtype, device="cuda") for k in PARTS}
    mc = D_lib().T2mapOutC(**{k: t.data_ptr() for k, t in mo.items()})
    pc = D_lib().T2partOutC(**{k: t.data_ptr() for k, t in po.items()})
    return mo, po, mc, pc


def _host(ts):
    return {k: t.cpu().numpy() for k, t in ts.items()}


def _code(c):
    return D_lib().F64 if c["dtype"] == np.float64 else D_lib().F32


def _ptr(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def run_device(D, ctx, c):
    """The existing context entry point (allocates through its context); its
    outputs are of the call dtype."""
    import torch
    o, po, d_img, d_b1 = _setup(D, c)
    mo, pt, mc, pc = _outputs(o, torch.float64 if c["dtype"] == np.float64 else torch.float32)
    L = D.load()
    ctx.check(L.decaes_t2map_t2part_device(ctx.h, C.byref(o.to_c()), C.byref(po.to_c()), _ptr(d_img), _code(c),
                                           _ptr(d_b1), C.byref(mc), C.byref(pc), None))
    ctx.check(L.decaes_sync_stats(ctx.h, None))
    return _host(mo), _host(pt)


def run_noalloc(D, c):
    """The entry point that allocates nothing; its outputs are FP64."""
    import torch
    o, po, d_img, d_b1 = _setup(D, c)
    mo, pt, mc, pc = _outputs(o, torch.float64)
    # garbage in the outputs: the entry point NaN-fills them itself
    for t in list(mo.values()) + list(pt.values()):
        t.fill_(12345.0)
    err = C.create_string_buffer(512)
    L = D.load()
    rc = L.decaes_t2map_t2part_noalloc(C.byref(o.to_c()), C.byref(po.to_c()), _ptr(d_img), _code(c), _ptr(d_b1),
                                       C.byref(mc), C.byref(pc), None, err, len(err))
    assert rc == 0, err.value.decode()
    torch.cuda.synchronize()
    return _host(mo), _host(pt)


def _compare(c, got, want):
    """Bit for bit: the FP64 outputs equal the context path's FP64 outputs, or,
    for a Float32 call, round to its Float32 outputs."""
    (gm, gp), (wm, wp) = got, want
    conv = (lambda a: a.astype(np.float32)) if c["dtype"] == np.float32 else (lambda a: a)
    assert set(gm) == set(wm)
    assert (~np.isnan(wm["dist"])).any()
    for k in list(gm) + list(PARTS):
        a, b = (gm[k], wm[k]) if k in gm else (gp[k], wp[k])
        np.testing.assert_array_equal(conv(a), b, err_msg=k)


@pytest.mark.gpu
def test_noalloc_matches_context_path(D, ctx):
    """Different problems back to back, then the first again: every call
    matches the context entry point bit for bit, whatever the previous call
    left in the shared static array."""
    want = [run_device(D, ctx, c) for c in CASES]
    for i in list(range(len(CASES))) + [0]:
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
    # an optional output whose Save* flag is off would never be written
    mc2 = D_lib().T2mapOutC(dist=8, gdn=8, ggm=8, gva=8, fnr=8, snr=8, alpha=8, resnorm=8)
    assert L.decaes_t2map_t2part_noalloc(C.byref(o.to_c()), None, C.c_void_p(8), D_lib().F64, None, C.byref(mc2),
                                         None, None, err, len(err)) == 1
    assert err.value.decode() == "resnorm is written only with SaveResidualNorm; pass NULL or set the flag"
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
