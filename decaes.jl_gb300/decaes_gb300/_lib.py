"""ctypes binding of libdecaes_gpu.so (the C ABI declared in include/decaes_gpu.h).

Loading never falls back to another implementation: if the library is missing
or a GPU call fails, the error is raised.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

F32, F64 = 0, 1
REG = {"none": 0, "lcurve": 1, "gcv": 2, "chi2": 3, "mdp": 4}
PREC = {"fp64": 0, "mixed": 1, "mixed_tc": 2}
ERRORS = {1: "EINVAL", 2: "ECUDA", 3: "ENOMEM", 4: "ELEGACY"}

_vp = C.c_void_p


class T2mapOptsC(C.Structure):
    _fields_ = [
        ("MatrixSize", C.c_int32 * 3), ("nTE", C.c_int32), ("TE", C.c_double), ("nT2", C.c_int32),
        ("T2Range", C.c_double * 2), ("T1", C.c_double), ("Threshold", C.c_double), ("MinRefAngle", C.c_double),
        ("nRefAngles", C.c_int32), ("nRefAnglesMin", C.c_int32), ("Reg", C.c_int32), ("Chi2Factor", C.c_double),
        ("NoiseLevel", C.c_double), ("RefConAngle", C.c_double), ("SetFlipAngle", C.c_double),
        ("SaveResidualNorm", C.c_int32), ("SaveDecayCurve", C.c_int32), ("SaveRegParam", C.c_int32),
        ("SaveNNLSBasis", C.c_int32), ("legacy", C.c_int32), ("precision", C.c_int32),
    ]


class T2mapOutC(C.Structure):
    _fields_ = [(k, _vp) for k in ("dist", "gdn", "ggm", "gva", "fnr", "snr", "alpha", "resnorm", "decaycurve", "mu",
                                   "chi2factor", "decaybasis", "echotimes", "t2times", "refangleset", "decaybasisset")]


class T2partOptsC(C.Structure):
    _fields_ = [("MatrixSize", C.c_int32 * 3), ("nT2", C.c_int32), ("T2Range", C.c_double * 2),
                ("SPWin", C.c_double * 2), ("MPWin", C.c_double * 2), ("Sigmoid", C.c_double), ("legacy", C.c_int32)]


class T2partOutC(C.Structure):
    _fields_ = [(k, _vp) for k in ("sfr", "sgm", "mfr", "mgm")]


class StatsC(C.Structure):
    _fields_ = [("voxels", C.c_int64), ("voxels_processed", C.c_int64), ("nnls_cap_hits", C.c_int64),
                ("search_limit_hits", C.c_int64), ("ms_total", C.c_double), ("ms_solve", C.c_double),
                ("ms_h2d", C.c_double), ("ms_d2h", C.c_double), ("solve_launches", C.c_int32),
                ("kernel_launches", C.c_int32), ("ms_grid_products", C.c_double),
                ("grid_product_launches", C.c_int32), ("grid_product_failures", C.c_int32)]


class MockOptsC(C.Structure):
    _fields_ = [("MatrixSize", C.c_int32 * 3), ("nTE", C.c_int32), ("TE", C.c_double), ("T1", C.c_double)] + [
        (k, C.c_double * 2) for k in ("FlipAngleRange", "MyelinT2Range", "MyelinFracRange", "IET2Range", "CSFT2Range",
                                      "CSFFracRange", "AmplitudeRange", "SNRRange")] + [
        ("BackgroundFraction", C.c_double), ("BackgroundSigma", C.c_double)]


class VolumeC(C.Structure):
    """decaes_volume: one volume of a batched launch (device pointers)."""
    _fields_ = [("mopts", T2mapOptsC), ("popts", T2partOptsC), ("has_t2part", C.c_int32), ("dtype", C.c_int32),
                ("d_image", _vp), ("d_b1map", _vp), ("d_mout", T2mapOutC), ("d_pout", T2partOutC)]


class TuningC(C.Structure):
    _fields_ = [("warps_per_block", C.c_int32), ("us_per_voxel", C.c_double), ("blocks_per_sm", C.c_int32)]


class ServerOptsC(C.Structure):
    _fields_ = [("tick_voxels", C.c_int64), ("hbm_budget_bytes", C.c_size_t)]


class ServerStatsC(C.Structure):
    _fields_ = [(k, C.c_int64) for k in ("submitted", "completed", "failed", "voxels", "ticks")] + [
        (k, C.c_double) for k in ("p50_ms", "p99_ms", "mean_ms", "max_ms", "busy_ms", "wall_ms")]


# Every symbol include/decaes_gpu.h declares.
EXPORTS = ["decaes_create", "decaes_destroy", "decaes_last_error", "decaes_get_stats", "decaes_t2map_check_options",
           "decaes_t2part_check_options", "decaes_t2map", "decaes_t2part", "decaes_t2map_t2part",
           "decaes_t2map_t2part_device", "decaes_sync_stats", "decaes_mock_image", "decaes_t2map_t2part_noalloc",
           "decaes_t2map_t2part_batch", "decaes_batch_create", "decaes_batch_run", "decaes_batch_destroy",
           "decaes_autotune", "decaes_server_create", "decaes_server_submit", "decaes_server_poll",
           "decaes_server_wait", "decaes_server_get_stats", "decaes_server_reset_stats", "decaes_server_destroy"]

_lib = None


def lib_path() -> str:
    return _build.LIB


def load(build_if_needed: bool = True):
    """Load libdecaes_gpu.so (building it first when sources are newer)."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_needed and _build.needs_build():
        _build.build()
    path = lib_path()
    if not os.path.exists(path):
        raise RuntimeError(f"libdecaes_gpu.so not found at {path}; run decaes_gb300.build.build()")
    L = C.CDLL(path)
    L.decaes_create.argtypes = [C.c_int, C.c_size_t]
    L.decaes_create.restype = _vp
    L.decaes_destroy.argtypes = [_vp]
    L.decaes_last_error.argtypes = [_vp]
    L.decaes_last_error.restype = C.c_char_p
    L.decaes_get_stats.argtypes = [_vp, C.POINTER(StatsC)]
    L.decaes_t2map_check_options.argtypes = [C.POINTER(T2mapOptsC), C.c_char_p, C.c_size_t]
    L.decaes_t2part_check_options.argtypes = [C.POINTER(T2partOptsC), C.c_char_p, C.c_size_t]
    L.decaes_t2map.argtypes = [_vp, C.POINTER(T2mapOptsC), _vp, C.c_int, _vp, C.POINTER(T2mapOutC)]
    L.decaes_t2part.argtypes = [_vp, C.POINTER(T2partOptsC), _vp, C.c_int, C.POINTER(T2partOutC)]
    L.decaes_t2map_t2part.argtypes = [_vp, C.POINTER(T2mapOptsC), C.POINTER(T2partOptsC), _vp, C.c_int, _vp,
                                      C.POINTER(T2mapOutC), C.POINTER(T2partOutC)]
    L.decaes_t2map_t2part_device.argtypes = [_vp, C.POINTER(T2mapOptsC), C.POINTER(T2partOptsC), _vp, C.c_int, _vp,
                                             C.POINTER(T2mapOutC), C.POINTER(T2partOutC), _vp]
    L.decaes_sync_stats.argtypes = [_vp, _vp]
    L.decaes_mock_image.argtypes = [C.POINTER(MockOptsC), C.c_uint64, _vp, C.c_int, C.c_int]
    L.decaes_t2map_t2part_noalloc.argtypes = [C.POINTER(T2mapOptsC), C.POINTER(T2partOptsC), _vp, C.c_int, _vp,
                                              C.POINTER(T2mapOutC), C.POINTER(T2partOutC), _vp, C.c_char_p, C.c_size_t]
    L.decaes_t2map_t2part_batch.argtypes = [_vp, C.POINTER(VolumeC), C.c_int32, _vp]
    L.decaes_batch_create.argtypes = [_vp, C.POINTER(VolumeC), C.c_int32]
    L.decaes_batch_create.restype = _vp
    L.decaes_batch_run.argtypes = [_vp, _vp]
    L.decaes_batch_destroy.argtypes = [_vp]
    L.decaes_autotune.argtypes = [_vp, C.POINTER(T2mapOptsC), C.POINTER(TuningC)]
    L.decaes_server_create.argtypes = [_vp, C.POINTER(ServerOptsC)]
    L.decaes_server_create.restype = _vp
    L.decaes_server_submit.argtypes = [_vp, C.POINTER(T2mapOptsC), C.POINTER(T2partOptsC), _vp, C.c_int,
                                       C.POINTER(T2mapOutC), C.POINTER(T2partOutC)]
    L.decaes_server_submit.restype = C.c_int64
    L.decaes_server_poll.argtypes = [_vp, C.c_int64]
    L.decaes_server_wait.argtypes = [_vp, C.c_int64]
    L.decaes_server_get_stats.argtypes = [_vp, C.POINTER(ServerStatsC)]
    L.decaes_server_reset_stats.argtypes = [_vp]
    L.decaes_server_destroy.argtypes = [_vp]
    _lib = L
    return L


class Context:
    """A decaes_ctx on one device (owns the stream, buffers and resident bases)."""

    def __init__(self, device: int = 0, hbm_budget_bytes: int = 0):
        self.L = load()
        self.h = self.L.decaes_create(device, hbm_budget_bytes)
        if not self.h:
            raise RuntimeError(f"decaes_create failed on device {device} (no usable CUDA device?)")

    def check(self, rc: int):
        if rc != 0:
            msg = self.L.decaes_last_error(self.h).decode()
            if rc == 1:
                raise AssertionError(msg)
            raise RuntimeError(f"{ERRORS.get(rc, rc)}: {msg}")

    def stats(self) -> dict:
        s = StatsC()
        self.L.decaes_get_stats(self.h, C.byref(s))
        return {k: getattr(s, k) for k, _ in StatsC._fields_}

    def close(self):
        if self.h:
            self.L.decaes_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default = None


def default_context() -> Context:
    global _default
    if _default is None:
        _default = Context(0)
    return _default
