"""Python mirror of DECAES.jl's public T2 API over libdecaes_gpu.so.

    T2mapOptions / T2partOptions        src/types.jl:19-100, 139-190
    T2mapSEcorr(image, opts | **kw)     src/T2mapSEcorr.jl:148-196
    T2partSEcorr(dist, opts | **kw)     src/T2partSEcorr.jl:40-71

Arrays follow Julia's layout: a 4D image indexed (x, y, z, echo) with
column-major memory (numpy order='F').  Outputs have the input's dtype; the
plain method computes in FP64 regardless (FP32 input is widened on the GPU).
Option errors raise AssertionError with the reference's messages.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field, fields, replace
from typing import Optional, Tuple

import numpy as np

from . import _lib

__all__ = ["T2mapOptions", "T2partOptions", "T2mapSEcorr", "T2partSEcorr", "T2mapSEcorr_T2partSEcorr", "mock_image",
           "MockImageOptions"]


def _nan(v):
    return math.nan if v is None else float(v)


@dataclass(frozen=True)
class T2mapOptions:
    """Options of T2mapSEcorr (src/types.jl:19-100).  `None` stands for `nothing`."""
    MatrixSize: Tuple[int, int, int]
    nTE: int
    TE: float
    nT2: int
    T2Range: Tuple[float, float]
    Reg: str
    legacy: bool = False
    Threaded: bool = True
    T1: float = 1.0
    Threshold: float = 0.0
    MinRefAngle: float = 50.0
    nRefAngles: Optional[int] = None       # default 64 (8 when legacy)
    nRefAnglesMin: Optional[int] = None    # default min(5, nRefAngles)
    Chi2Factor: Optional[float] = None
    NoiseLevel: Optional[float] = None
    RefConAngle: float = 180.0
    SetFlipAngle: Optional[float] = None
    SaveResidualNorm: bool = False
    SaveDecayCurve: bool = False
    SaveRegParam: bool = False
    SaveNNLSBasis: bool = False
    Silent: bool = True
    precision: str = "fp64"                # extension: "fp64" (plain method) or "mixed"

    def __post_init__(self):
        if self.nRefAngles is None:
            object.__setattr__(self, "nRefAngles", 8 if self.legacy else 64)
        if self.nRefAnglesMin is None:
            object.__setattr__(self, "nRefAnglesMin", self.nRefAngles if self.legacy else min(5, self.nRefAngles))
        object.__setattr__(self, "MatrixSize", tuple(int(v) for v in self.MatrixSize))
        object.__setattr__(self, "T2Range", tuple(float(v) for v in self.T2Range))
        if self.Reg not in _lib.REG:
            raise AssertionError('Reg ∈ ("none", "lcurve", "gcv", "chi2", "mdp")')
        msg = C.create_string_buffer(512)
        rc = _lib.load().decaes_t2map_check_options(C.byref(self.to_c()), msg, 512)
        if rc != 0:
            raise AssertionError(msg.value.decode())

    @classmethod
    def from_image(cls, image, **kw) -> "T2mapOptions":
        """T2mapOptions(image; kwargs...) (src/types.jl:102)."""
        a = np.asarray(image)
        return cls(MatrixSize=a.shape[:3], nTE=a.shape[3], **kw)

    def to_c(self) -> _lib.T2mapOptsC:
        return _lib.T2mapOptsC(
            (C.c_int32 * 3)(*self.MatrixSize), self.nTE, float(self.TE), self.nT2, (C.c_double * 2)(*self.T2Range),
            float(self.T1), float(self.Threshold), float(self.MinRefAngle), int(self.nRefAngles),
            int(self.nRefAnglesMin), _lib.REG.get(self.Reg, -1), _nan(self.Chi2Factor), _nan(self.NoiseLevel),
            float(self.RefConAngle), _nan(self.SetFlipAngle), int(self.SaveResidualNorm), int(self.SaveDecayCurve),
            int(self.SaveRegParam), int(self.SaveNNLSBasis), int(self.legacy), _lib.PREC[self.precision])


@dataclass(frozen=True)
class T2partOptions:
    """Options of T2partSEcorr (src/types.jl:139-172)."""
    MatrixSize: Tuple[int, int, int]
    nT2: int
    T2Range: Tuple[float, float]
    SPWin: Tuple[float, float]
    MPWin: Tuple[float, float]
    legacy: bool = False
    Threaded: bool = True
    Sigmoid: Optional[float] = None
    Silent: bool = True

    def __post_init__(self):
        object.__setattr__(self, "MatrixSize", tuple(int(v) for v in self.MatrixSize))
        for k in ("T2Range", "SPWin", "MPWin"):
            object.__setattr__(self, k, tuple(float(v) for v in getattr(self, k)))
        msg = C.create_string_buffer(512)
        rc = _lib.load().decaes_t2part_check_options(C.byref(self.to_c()), msg, 512)
        if rc != 0:
            raise AssertionError(msg.value.decode())

    @classmethod
    def from_dist(cls, dist, **kw) -> "T2partOptions":
        a = np.asarray(dist)
        return cls(MatrixSize=a.shape[:3], nT2=a.shape[3], **kw)

    @classmethod
    def from_t2map(cls, o: T2mapOptions, **kw) -> "T2partOptions":
        """T2partOptions(::T2mapOptions; kwargs...) (src/types.jl:180-190)."""
        base = dict(legacy=o.legacy, Threaded=o.Threaded, MatrixSize=o.MatrixSize, nT2=o.nT2, T2Range=o.T2Range,
                    Silent=o.Silent)
        base.update(kw)
        return cls(**base)

    def to_c(self) -> _lib.T2partOptsC:
        return _lib.T2partOptsC((C.c_int32 * 3)(*self.MatrixSize), self.nT2, (C.c_double * 2)(*self.T2Range),
                                (C.c_double * 2)(*self.SPWin), (C.c_double * 2)(*self.MPWin), _nan(self.Sigmoid),
                                int(self.legacy))


def _dtype_code(a: np.ndarray) -> int:
    if a.dtype == np.float32:
        return _lib.F32
    if a.dtype == np.float64:
        return _lib.F64
    raise TypeError(f"image must be float32 or float64, got {a.dtype}")


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _t2map_buffers(o: T2mapOptions, dt):
    X, Y, Z = o.MatrixSize
    nan = lambda *shape: np.full(shape, np.nan, dtype=dt, order="F")
    fixed = o.SetFlipAngle is not None
    maps = {
        "echotimes": np.empty(o.nTE, dt),
        "t2times": np.empty(o.nT2, dt),
        "refangleset": np.empty(1 if fixed else o.nRefAngles, dt),
        "decaybasisset": np.empty((o.nTE, o.nT2) if fixed else (o.nTE, o.nT2, o.nRefAngles), dt, order="F"),
        "gdn": nan(X, Y, Z), "ggm": nan(X, Y, Z), "gva": nan(X, Y, Z), "fnr": nan(X, Y, Z), "snr": nan(X, Y, Z),
        "alpha": nan(X, Y, Z),
    }
    if o.SaveResidualNorm:
        maps["resnorm"] = nan(X, Y, Z)
    if o.SaveDecayCurve:
        maps["decaycurve"] = nan(X, Y, Z, o.nTE)
    if o.SaveRegParam:
        maps["mu"] = nan(X, Y, Z)
        maps["chi2factor"] = nan(X, Y, Z)
    if o.SaveNNLSBasis:
        maps["decaybasis"] = np.empty((o.nTE, o.nT2), dt, order="F") if fixed else nan(X, Y, Z, o.nTE, o.nT2)
    dist = nan(X, Y, Z, o.nT2)
    out = _lib.T2mapOutC(*[_ptr(dist if k == "dist" else maps.get(k)) for k, _ in _lib.T2mapOutC._fields_])
    return maps, dist, out


def _finish_maps(maps, o: T2mapOptions):
    if o.SetFlipAngle is not None:
        maps["refangleset"] = maps["refangleset"].dtype.type(maps["refangleset"][0])
    return maps


def T2mapSEcorr(image, opts: Optional[T2mapOptions] = None, *, b1map=None, ctx: Optional[_lib.Context] = None, **kw):
    """T2mapSEcorr(image, opts) -> (maps: dict, dist: ndarray) on the GPU."""
    img = np.asfortranarray(image)
    o = opts if opts is not None else T2mapOptions.from_image(img, **kw)
    if img.shape != (*o.MatrixSize, o.nTE):
        raise AssertionError("size(image) == (opts.MatrixSize..., opts.nTE)")
    dt = img.dtype
    code = _dtype_code(img)
    b1 = None if b1map is None else np.asfortranarray(b1map, dtype=dt)
    maps, dist, out = _t2map_buffers(o, dt)
    c = ctx or _lib.default_context()
    c.check(c.L.decaes_t2map(c.h, C.byref(o.to_c()), _ptr(img), code, _ptr(b1), C.byref(out)))
    return _finish_maps(maps, o), dist


def T2partSEcorr(dist, opts: Optional[T2partOptions] = None, *, ctx: Optional[_lib.Context] = None, **kw):
    """T2partSEcorr(dist, opts) -> dict(sfr, sgm, mfr, mgm) on the GPU."""
    d = np.asfortranarray(dist)
    o = opts if opts is not None else T2partOptions.from_dist(d, **kw)
    if d.shape != (*o.MatrixSize, o.nT2):
        raise AssertionError("size(T2distributions) == (opts.MatrixSize..., opts.nT2)")
    dt = d.dtype
    code = _dtype_code(d)
    parts = {k: np.full(o.MatrixSize, np.nan, dtype=dt, order="F") for k in ("sfr", "sgm", "mfr", "mgm")}
    out = _lib.T2partOutC(*[_ptr(parts[k]) for k, _ in _lib.T2partOutC._fields_])
    c = ctx or _lib.default_context()
    c.check(c.L.decaes_t2part(c.h, C.byref(o.to_c()), _ptr(d), code, C.byref(out)))
    return parts


def T2mapSEcorr_T2partSEcorr(image, mopts: T2mapOptions, popts: T2partOptions, *, b1map=None,
                             ctx: Optional[_lib.Context] = None):
    """T2mapSEcorr followed by T2partSEcorr on its distribution, with the T2part
    window sums fused into the GPU solve.  Returns (maps, dist, parts)."""
    img = np.asfortranarray(image)
    o = mopts
    if img.shape != (*o.MatrixSize, o.nTE):
        raise AssertionError("size(image) == (opts.MatrixSize..., opts.nTE)")
    dt = img.dtype
    code = _dtype_code(img)
    b1 = None if b1map is None else np.asfortranarray(b1map, dtype=dt)
    maps, dist, out = _t2map_buffers(o, dt)
    parts = {k: np.full(o.MatrixSize, np.nan, dtype=dt, order="F") for k in ("sfr", "sgm", "mfr", "mgm")}
    pout = _lib.T2partOutC(*[_ptr(parts[k]) for k, _ in _lib.T2partOutC._fields_])
    c = ctx or _lib.default_context()
    c.check(c.L.decaes_t2map_t2part(c.h, C.byref(o.to_c()), C.byref(popts.to_c()), _ptr(img), code, _ptr(b1),
                                    C.byref(out), C.byref(pout)))
    return _finish_maps(maps, o), dist, parts


@dataclass(frozen=True)
class MockImageOptions:
    """Generator of the synthetic multi-echo images used by the benchmarks."""
    MatrixSize: Tuple[int, int, int] = (2, 2, 2)
    nTE: int = 48
    TE: float = 10e-3
    T1: float = 1.0
    FlipAngleRange: Tuple[float, float] = (140.0, 180.0)
    MyelinT2Range: Tuple[float, float] = (15e-3, 25e-3)
    MyelinFracRange: Tuple[float, float] = (0.05, 0.25)
    IET2Range: Tuple[float, float] = (60e-3, 90e-3)
    CSFT2Range: Tuple[float, float] = (1.0, 2.0)
    CSFFracRange: Tuple[float, float] = (0.0, 0.05)
    AmplitudeRange: Tuple[float, float] = (500.0, 2000.0)
    SNRRange: Tuple[float, float] = (50.0, 200.0)
    BackgroundFraction: float = 0.0
    BackgroundSigma: float = 8.0


def mock_image(o: MockImageOptions = MockImageOptions(), seed: int = 0, dtype=np.float64, nthreads: int = 0):
    """Synthetic image (x, y, z, echo), the counterpart of the reference's mock_image."""
    L = _lib.load()
    X, Y, Z = o.MatrixSize
    img = np.empty((X, Y, Z, o.nTE), dtype=dtype, order="F")
    co = _lib.MockOptsC((C.c_int32 * 3)(*o.MatrixSize), o.nTE, o.TE, o.T1,
                        *[(C.c_double * 2)(*getattr(o, k)) for k in ("FlipAngleRange", "MyelinT2Range", "MyelinFracRange",
                                                                     "IET2Range", "CSFT2Range", "CSFFracRange",
                                                                     "AmplitudeRange", "SNRRange")],
                        o.BackgroundFraction, o.BackgroundSigma)
    rc = L.decaes_mock_image(C.byref(co), seed, _ptr(img), _lib.F32 if img.dtype == np.float32 else _lib.F64, nthreads)
    if rc != 0:
        raise ValueError("invalid mock image options")
    return img
