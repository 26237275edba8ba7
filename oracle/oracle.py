"""ctypes wrapper of the CPU oracle (liboracle.so).

TEST INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg use this module as the checker.  The GPU product never imports
it.  The oracle is a plain-C FP64 restatement of DECAES.jl v0.6.1's voxelwise
T2 path; see decaes_oracle.c for the reference files and lines each part
follows.  Parity against the Julia reference itself is unpinned (Julia is not
available); components are pinned by the reference test suite's known answers.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboracle.so")
_lib = None

REG = {"none": 0, "lcurve": 1, "gcv": 2, "chi2": 3, "mdp": 4}
STAGES = ["ensemble", "search_nnls", "search_other", "basis", "reg_nnls", "reg_other", "svd", "save", "t2part"]

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class _T2mapOpts(C.Structure):
    _fields_ = [
        ("nTE", C.c_int), ("TE", C.c_double), ("nT2", C.c_int), ("T2Range", C.c_double * 2),
        ("T1", C.c_double), ("Threshold", C.c_double), ("MinRefAngle", C.c_double),
        ("nRefAngles", C.c_int), ("nRefAnglesMin", C.c_int), ("Reg", C.c_int),
        ("Chi2Factor", C.c_double), ("NoiseLevel", C.c_double), ("RefConAngle", C.c_double),
        ("SetFlipAngle", C.c_double), ("legacy", C.c_int),
    ]


class _T2mapOut(C.Structure):
    _fields_ = [(k, _dp) for k in ("dist", "gdn", "ggm", "gva", "fnr", "snr", "alpha",
                                   "resnorm", "decaycurve", "mu", "chi2factor")]


class _T2partOpts(C.Structure):
    _fields_ = [("nT2", C.c_int), ("T2Range", C.c_double * 2), ("SPWin", C.c_double * 2),
                ("MPWin", C.c_double * 2), ("Sigmoid", C.c_double)]


class _T2partOut(C.Structure):
    _fields_ = [(k, _dp) for k in ("sfr", "sgm", "mfr", "mgm")]


FN = C.CFUNCTYPE(C.c_double, C.c_double, C.c_void_p)
FN2 = C.CFUNCTYPE(None, C.c_double, _dp, C.c_void_p)


class _MockOpts(C.Structure):
    _fields_ = [("nTE", C.c_int), ("TE", C.c_double), ("T1", C.c_double)] + [
        (k, C.c_double * 2) for k in ("FlipAngleRange", "MyelinT2Range", "MyelinFracRange", "IET2Range", "CSFT2Range",
                                     "CSFFracRange", "AmplitudeRange", "SNRRange")] + [
        ("BackgroundFraction", C.c_double), ("BackgroundSigma", C.c_double)]


def build(force: bool = False) -> str:
    """Compile liboracle.so with the Makefile beside this file."""
    src = os.path.join(_HERE, "decaes_oracle.c")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE, "-B" if force else "liboracle.so"], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        L.orc_t2map.argtypes = [C.POINTER(_T2mapOpts), _dp, C.c_long, _dp, C.POINTER(_T2mapOut), C.c_int, _dp]
        L.orc_t2part.argtypes = [C.POINTER(_T2partOpts), _dp, C.c_long, C.POINTER(_T2partOut), C.c_int]
        L.orc_linrange.argtypes = [C.c_double, C.c_double, C.c_int, _dp]
        L.orc_logrange.argtypes = [C.c_double, C.c_double, C.c_int, _dp]
        L.orc_sind.argtypes = [C.c_double]
        L.orc_sind.restype = C.c_double
        L.orc_erfinv.argtypes = [C.c_double]
        L.orc_erfinv.restype = C.c_double
        for f in ("orc_epg_decay_curve", "orc_epg_decay_curve_basic"):
            getattr(L, f).argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double, _dp]
        L.orc_epg_decay_curve_dual.argtypes = [C.c_int] + [C.c_double] * 5 + [_dp, _dp]
        L.orc_nnls.argtypes = [_dp, C.c_int, C.c_int, _dp, _dp, _dp, _ip, _ip]
        L.orc_lsqnonneg.argtypes = [_dp, C.c_int, C.c_int, _dp, _dp, _dp, _ip]
        L.orc_lsqnonneg_tikh.argtypes = [_dp, C.c_int, C.c_int, _dp, C.c_double, _dp, _dp, _dp, _dp, _ip]
        L.orc_lsqnonneg_chi2.argtypes = [_dp, C.c_int, C.c_int, _dp, C.c_double, _dp, _dp, _dp]
        L.orc_lsqnonneg_mdp.argtypes = [_dp, C.c_int, C.c_int, _dp, C.c_double, _dp, _dp, _dp]
        L.orc_lsqnonneg_lcurve.argtypes = [_dp, C.c_int, C.c_int, _dp, _dp, _dp, _dp]
        L.orc_lsqnonneg_gcv.argtypes = [_dp, C.c_int, C.c_int, _dp, _dp, _dp, _dp]
        L.orc_svdvals.argtypes = [_dp, C.c_int, C.c_int, _dp]
        L.orc_brent_root.argtypes = [FN, C.c_void_p] + [C.c_double] * 5 + [C.c_int, _dp, _dp]
        L.orc_bisect_root.argtypes = [FN, C.c_void_p] + [C.c_double] * 5 + [C.c_int, _dp, _dp]
        L.orc_brent_minimize.argtypes = [FN, C.c_void_p] + [C.c_double] * 4 + [C.c_int, _dp, _dp]
        L.orc_lcurve_corner.argtypes = [FN2, C.c_void_p] + [C.c_double] * 5
        L.orc_lcurve_corner.restype = C.c_double
        L.orc_cubic_hermite_minimize.argtypes = [C.c_double] * 6 + [_dp, _dp]
        L.orc_minimal_bounding_box.argtypes = [C.c_int, _dp, C.POINTER(C.c_ubyte), C.c_double, _ip, _ip]
        L.orc_lsqnonneg_chi2_legacy.argtypes = [_dp, C.c_int, C.c_int, _dp, C.c_double, _dp, _dp, _dp]
        L.orc_jl_colon.argtypes = [C.c_double, C.c_double, C.c_double, _dp, C.c_long, C.POINTER(C.c_long)]
        L.orc_fitpack_curfit0.argtypes = [_dp, _dp, C.c_int, C.c_int, _dp, _dp]
        L.orc_fitpack_splev.argtypes = [_dp, C.c_int, _dp, C.c_int, _dp, C.c_int, _dp]
        L.orc_spline_opt_legacy.argtypes = [_dp, _dp, C.c_int, _dp, _dp]
        L.orc_spline_root_legacy.argtypes = [_dp, _dp, C.c_int, C.c_double, _dp]
        L.orc_mock_image.argtypes = [C.POINTER(_MockOpts), C.c_uint64, C.c_long, C.c_void_p, C.c_int, C.c_int]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(_dp) if a is not None else None


def _f64(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


def _fortran(a):
    return np.asfortranarray(np.asarray(a, dtype=np.float64))


# ---------------------------------------------------------------- grids / EPG
def linrange(a, b, n):
    out = np.empty(n)
    lib().orc_linrange(a, b, n, _p(out))
    return out


def logrange(a, b, n):
    out = np.empty(n)
    lib().orc_logrange(a, b, n, _p(out))
    return out


def sind(x):
    return lib().orc_sind(float(x))


def erfinv(x):
    return lib().orc_erfinv(float(x))


def epg_decay_curve(ETL, alpha, TE, T2, T1, beta=180.0):
    out = np.empty(ETL)
    lib().orc_epg_decay_curve(ETL, alpha, TE, T2, T1, beta, _p(out))
    return out


def epg_decay_curve_dual(ETL, alpha, TE, T2, T1, beta=180.0):
    v, d = np.empty(ETL), np.empty(ETL)
    lib().orc_epg_decay_curve_dual(ETL, alpha, TE, T2, T1, beta, _p(v), _p(d))
    return v, d


def epg_decay_curve_basic(ETL, alpha, TE, T2, T1, beta=180.0):
    out = np.empty(ETL)
    lib().orc_epg_decay_curve_basic(ETL, alpha, TE, T2, T1, beta, _p(out))
    return out


# ------------------------------------------------------------ NNLS & friends
def nnls(A, b):
    A, b = _fortran(A), _f64(b)
    m, n = A.shape
    x, rn, ns, md = np.empty(n), C.c_double(), C.c_int(), C.c_int()
    lib().orc_nnls(_p(A), m, n, _p(b), _p(x), C.byref(rn), C.byref(ns), C.byref(md))
    return x, rn.value, ns.value, md.value


def lsqnonneg(A, b):
    A, b = _fortran(A), _f64(b)
    m, n = A.shape
    x, rn, ns = np.empty(n), C.c_double(), C.c_int()
    lib().orc_lsqnonneg(_p(A), m, n, _p(b), _p(x), C.byref(rn), C.byref(ns))
    return x, rn.value, ns.value


def lsqnonneg_tikh(A, b, mu):
    A, b = _fortran(A), _f64(b)
    m, n = A.shape
    x, loss, ssq, rsq, ns = np.empty(n), C.c_double(), C.c_double(), C.c_double(), C.c_int()
    lib().orc_lsqnonneg_tikh(_p(A), m, n, _p(b), mu, _p(x), C.byref(loss), C.byref(ssq), C.byref(rsq), C.byref(ns))
    return x, dict(loss=loss.value, seminorm_sq=ssq.value, resnorm_sq=rsq.value, nsetp=ns.value)


def _reg(fn, A, b, *args):
    A, b = _fortran(A), _f64(b)
    m, n = A.shape
    x, mu, chi2 = np.empty(n), C.c_double(), C.c_double()
    fn(_p(A), m, n, _p(b), *args, _p(x), C.byref(mu), C.byref(chi2))
    return x, mu.value, chi2.value


def lsqnonneg_chi2(A, b, chi2_target):
    return _reg(lib().orc_lsqnonneg_chi2, A, b, chi2_target)


def lsqnonneg_chi2_legacy(A, b, chi2_target):
    """lsqnonneg_chi2!(work, chi2_target, legacy = true)."""
    return _reg(lib().orc_lsqnonneg_chi2_legacy, A, b, chi2_target)


def jl_colon(start, step, stop, maxlen=None):
    """collect(start:step:stop) for Float64 (Julia's TwicePrecision ranges)."""
    n = C.c_long(0)
    lib().orc_jl_colon(start, step, stop, None, 0, C.byref(n))
    out = np.empty(n.value if maxlen is None else min(maxlen, n.value))
    lib().orc_jl_colon(start, step, stop, _p(out), out.size, C.byref(n))
    return out


def fitpack_curfit0(x, y, k):
    """Dierckx.Spline1D(x, y; k, s = 0): (knots t, coefficients c) as FITPACK's curfit."""
    x, y = _f64(x), _f64(y)
    m = x.size
    t, c = np.empty(m + k + 1), np.empty(m)
    if lib().orc_fitpack_curfit0(_p(x), _p(y), m, k, _p(t), _p(c)) != 0:
        raise ValueError("curfit0 needs 1 <= k <= 3 < m")
    return t, c


def fitpack_splev(t, c, k, x):
    t, c, x = _f64(t), _f64(c), _f64(x)
    y = np.empty(x.size)
    lib().orc_fitpack_splev(_p(t), t.size, _p(c), k, _p(x), x.size, _p(y))
    return y


def spline_opt_legacy(X, Y):
    X, Y = _f64(X), _f64(Y)
    x, y = C.c_double(), C.c_double()
    if lib().orc_spline_opt_legacy(_p(X), _p(Y), X.size, C.byref(x), C.byref(y)) != 0:
        raise ValueError("spline_opt_legacy: 2..256 points")
    return x.value, y.value


def spline_root_legacy(X, Y, value=0.0):
    X, Y = _f64(X), _f64(Y)
    x = C.c_double()
    if lib().orc_spline_root_legacy(_p(X), _p(Y), X.size, value, C.byref(x)) != 0:
        raise ValueError("spline_root_legacy: 2..256 points")
    return x.value


def lsqnonneg_mdp(A, b, delta):
    return _reg(lib().orc_lsqnonneg_mdp, A, b, delta)


def lsqnonneg_lcurve(A, b):
    return _reg(lib().orc_lsqnonneg_lcurve, A, b)


def lsqnonneg_gcv(A, b):
    return _reg(lib().orc_lsqnonneg_gcv, A, b)


def svdvals(A):
    A = _fortran(A)
    m, n = A.shape
    s = np.empty(min(m, n))
    lib().orc_svdvals(_p(A), m, n, _p(s))
    return s


def brent_root(f, a, b, xatol=0.0, xrtol=0.0, ftol=0.0, maxiters=100):
    cb = FN(lambda x, _: f(x))
    x, fx = C.c_double(), C.c_double()
    lib().orc_brent_root(cb, None, a, b, xatol, xrtol, ftol, maxiters, C.byref(x), C.byref(fx))
    return x.value, fx.value


def bisect_root(f, a, b, xatol=0.0, xrtol=0.0, ftol=0.0, maxiters=100):
    cb = FN(lambda x, _: f(x))
    x, fx = C.c_double(), C.c_double()
    lib().orc_bisect_root(cb, None, a, b, xatol, xrtol, ftol, maxiters, C.byref(x), C.byref(fx))
    return x.value, fx.value


def brent_minimize(f, a, b, xatol=math.sqrt(2.220446049250313e-16), xrtol=math.sqrt(2.220446049250313e-16), maxiters=100):
    cb = FN(lambda x, _: f(x))
    x, fx = C.c_double(), C.c_double()
    lib().orc_brent_minimize(cb, None, a, b, xatol, xrtol, maxiters, C.byref(x), C.byref(fx))
    return x.value, fx.value


def lcurve_corner(f, xlow=-8.0, xhigh=2.0, xtol=1e-4, Ptol=1e-4, Ctol=1e-4):
    def _cb(x, P, _):
        a, b = f(x)
        P[0], P[1] = a, b
    cb = FN2(_cb)
    return lib().orc_lcurve_corner(cb, None, xlow, xhigh, xtol, Ptol, Ctol)


def cubic_hermite_minimize(a, b, u0, u1, m0, m1):
    x, u = C.c_double(), C.c_double()
    lib().orc_cubic_hermite_minimize(a, b, u0, u1, m0, m1, C.byref(x), C.byref(u))
    return x.value, u.value


def minimal_bounding_box(grid, seen, x):
    g = _f64(grid)
    s = np.ascontiguousarray(np.asarray(seen, dtype=np.uint8))
    lo, hi = C.c_int(), C.c_int()
    lib().orc_minimal_bounding_box(len(g), _p(g), s.ctypes.data_as(C.POINTER(C.c_ubyte)), x, C.byref(lo), C.byref(hi))
    return lo.value, hi.value


# ------------------------------------------------------------------ pipeline
@dataclass
class T2mapOptions:
    """Mirror of T2mapOptions{Float64} (src/types.jl:19-100); None = nothing."""
    MatrixSize: tuple
    nTE: int
    TE: float
    nT2: int
    T2Range: tuple
    Reg: str
    T1: float = 1.0
    Threshold: float = 0.0
    MinRefAngle: float = 50.0
    nRefAngles: int = 64
    nRefAnglesMin: int | None = None
    Chi2Factor: float | None = None
    NoiseLevel: float | None = None
    RefConAngle: float = 180.0
    SetFlipAngle: float | None = None
    SaveResidualNorm: bool = False
    SaveDecayCurve: bool = False
    SaveRegParam: bool = False
    legacy: bool = False


def _nan(v):
    return math.nan if v is None else float(v)


def t2map(image, o: T2mapOptions, b1map=None, nthreads: int = 1, return_flops: bool = False):
    """T2mapSEcorr(image, opts) -> (maps dict, dist) computed by the oracle in FP64."""
    img = np.asarray(image)
    X, Y, Z, m = img.shape
    V = X * Y * Z
    flat = np.asfortranarray(img, dtype=np.float64).reshape((V, m), order="F")
    flat = np.asfortranarray(flat)
    co = _T2mapOpts(m, o.TE, o.nT2, (C.c_double * 2)(*o.T2Range), o.T1, o.Threshold, o.MinRefAngle,
                    o.nRefAngles, o.nRefAnglesMin if o.nRefAnglesMin is not None else
                    (o.nRefAngles if o.legacy else min(5, o.nRefAngles)),
                    REG[o.Reg], _nan(o.Chi2Factor), _nan(o.NoiseLevel), o.RefConAngle, _nan(o.SetFlipAngle),
                    int(o.legacy))
    outs = {k: np.full(V, np.nan) for k in ("gdn", "ggm", "gva", "fnr", "snr", "alpha")}
    dist = np.full((V, o.nT2), np.nan, order="F")
    if o.SaveResidualNorm:
        outs["resnorm"] = np.full(V, np.nan)
    if o.SaveDecayCurve:
        outs["decaycurve"] = np.full((V, m), np.nan, order="F")
    if o.SaveRegParam:
        outs["mu"] = np.full(V, np.nan)
        outs["chi2factor"] = np.full(V, np.nan)
    cout = _T2mapOut(_p(dist), *[_p(outs.get(k)) for k in ("gdn", "ggm", "gva", "fnr", "snr", "alpha", "resnorm",
                                                            "decaycurve", "mu", "chi2factor")])
    b1 = None
    if b1map is not None:
        b1 = np.asfortranarray(np.asarray(b1map, dtype=np.float64)).reshape(V, order="F")
    fl = np.zeros(len(STAGES))
    rc = lib().orc_t2map(C.byref(co), _p(flat), V, _p(b1), C.byref(cout), nthreads, _p(fl))
    if rc != 0:
        raise RuntimeError(f"orc_t2map failed: {rc}")
    maps = {}
    for k, v in outs.items():
        if v.ndim == 1:
            maps[k] = v.reshape((X, Y, Z), order="F")
        else:
            maps[k] = v.reshape((X, Y, Z, v.shape[1]), order="F")
    d = dist.reshape((X, Y, Z, o.nT2), order="F")
    if return_flops:
        return maps, d, dict(zip(STAGES, fl))
    return maps, d


@dataclass
class T2partOptions:
    MatrixSize: tuple
    nT2: int
    T2Range: tuple
    SPWin: tuple
    MPWin: tuple
    Sigmoid: float | None = None


def t2part(dist, o: T2partOptions):
    d = np.asarray(dist)
    X, Y, Z, n = d.shape
    V = X * Y * Z
    flat = np.asfortranarray(np.asfortranarray(d, dtype=np.float64).reshape((V, n), order="F"))
    co = _T2partOpts(n, (C.c_double * 2)(*o.T2Range), (C.c_double * 2)(*o.SPWin), (C.c_double * 2)(*o.MPWin),
                     _nan(o.Sigmoid))
    outs = {k: np.full(V, np.nan) for k in ("sfr", "sgm", "mfr", "mgm")}
    cout = _T2partOut(*[_p(outs[k]) for k in ("sfr", "sgm", "mfr", "mgm")])
    rc = lib().orc_t2part(C.byref(co), _p(flat), V, C.byref(cout), 1)
    if rc != 0:
        raise RuntimeError(f"orc_t2part failed: {rc}")
    return {k: v.reshape((X, Y, Z), order="F") for k, v in outs.items()}


# ---------------------------------------------------------------- synthetic input
MOCK_DEFAULTS = dict(TE=10e-3, T1=1.0, FlipAngleRange=(140.0, 180.0), MyelinT2Range=(15e-3, 25e-3),
                     MyelinFracRange=(0.05, 0.25), IET2Range=(60e-3, 90e-3), CSFT2Range=(1.0, 2.0),
                     CSFFracRange=(0.0, 0.05), AmplitudeRange=(500.0, 2000.0), SNRRange=(50.0, 200.0),
                     BackgroundFraction=0.0, BackgroundSigma=8.0)


def mock_image(MatrixSize, nTE, seed=0, dtype=np.float64, nthreads=0, **kw):
    """The benchmark's synthetic image (x, y, z, echo), byte for byte the
    output of libdecaes_gpu's decaes_mock_image with the same options and seed,
    made without loading the GPU library.  A leading z-slab of a volume equals
    that volume's first slices."""
    o = dict(MOCK_DEFAULTS, **kw)
    co = _MockOpts(nTE, o["TE"], o["T1"], *[(C.c_double * 2)(*o[k]) for k in (
        "FlipAngleRange", "MyelinT2Range", "MyelinFracRange", "IET2Range", "CSFT2Range", "CSFFracRange",
        "AmplitudeRange", "SNRRange")], o["BackgroundFraction"], o["BackgroundSigma"])
    X, Y, Z = (int(v) for v in MatrixSize)
    img = np.empty((X, Y, Z, nTE), dtype=dtype, order="F")
    rc = lib().orc_mock_image(C.byref(co), int(seed), X * Y * Z, img.ctypes.data_as(C.c_void_p),
                              1 if img.dtype == np.float32 else 0, nthreads or (os.cpu_count() or 1))
    if rc != 0:
        raise ValueError("invalid mock image options")
    return img
