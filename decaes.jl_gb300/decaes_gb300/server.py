"""Continuous-batching server on one GPU (the counterpart of the reference's
warm-process request loop, api/decaes_server.jl:69-131, for the voxelwise T2
path): requests are queued and return at once; the library's scheduler thread
admits them by device-memory footprint and solves them in shared ticks.

    srv = Server(ctx, tick_voxels=262144)
    rid = srv.submit(image, T2mapOptions(...), T2partOptions(...))
    maps, dist, parts = srv.result(rid)        # blocks until done
    srv.stats()                                 # p50/p99 latency, voxels, ...
    srv.close()
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import _lib
from .api import T2mapOptions, T2partOptions, _dtype_code, _finish_maps, _ptr, _t2map_buffers


class Server:
    def __init__(self, ctx: Optional[_lib.Context] = None, tick_voxels: int = 0, hbm_budget_bytes: int = 0):
        self.ctx = ctx or _lib.default_context()
        self.L = self.ctx.L
        self.h = self.L.decaes_server_create(self.ctx.h, C.byref(_lib.ServerOptsC(tick_voxels, hbm_budget_bytes)))
        if not self.h:
            raise RuntimeError(self.L.decaes_last_error(self.ctx.h).decode())
        self._req = {}

    def submit(self, image, mopts: T2mapOptions, popts: Optional[T2partOptions] = None) -> int:
        """Queues T2mapSEcorr (+ T2partSEcorr) of a host image; returns a request id."""
        img = np.asfortranarray(image)
        if img.shape != (*mopts.MatrixSize, mopts.nTE):
            raise AssertionError("size(image) == (opts.MatrixSize..., opts.nTE)")
        dt = img.dtype
        maps, dist, out = _t2map_buffers(mopts, dt)
        # per-call constants are filled when the request completes
        parts, pout = None, None
        if popts is not None:
            parts = {k: np.full(mopts.MatrixSize, np.nan, dtype=dt, order="F") for k in ("sfr", "sgm", "mfr", "mgm")}
            pout = _lib.T2partOutC(*[_ptr(parts[k]) for k, _ in _lib.T2partOutC._fields_])
        rid = self.L.decaes_server_submit(self.h, C.byref(mopts.to_c()),
                                          C.byref(popts.to_c()) if popts is not None else None, _ptr(img),
                                          _dtype_code(img), C.byref(out), C.byref(pout) if pout is not None else None)
        if rid < 0:
            msg = self.L.decaes_last_error(self.ctx.h).decode()
            if -rid == 1:
                raise AssertionError(msg)
            raise RuntimeError(f"decaes_server_submit: {_lib.ERRORS.get(-rid, -rid)}: {msg}")
        self._req[rid] = (img, mopts, maps, dist, parts, out, pout)  # keep the buffers alive
        return rid

    def done(self, rid: int) -> bool:
        rc = self.L.decaes_server_poll(self.h, rid)
        if rc < 0:
            raise RuntimeError(f"request {rid} failed: {_lib.ERRORS.get(-rc, -rc)}")
        return rc == 1

    def result(self, rid: int):
        """Waits for a request; returns (maps, dist) or (maps, dist, parts)."""
        rc = self.L.decaes_server_wait(self.h, rid)
        img, mopts, maps, dist, parts, out, pout = self._req.pop(rid)
        if rc != 0:
            raise RuntimeError(f"request {rid} failed: {_lib.ERRORS.get(rc, rc)}")
        maps = _finish_maps(maps, mopts)
        return (maps, dist) if parts is None else (maps, dist, parts)

    def stats(self) -> dict:
        st = _lib.ServerStatsC()
        self.L.decaes_server_get_stats(self.h, C.byref(st))
        return {k: getattr(st, k) for k, _ in _lib.ServerStatsC._fields_}

    def reset_stats(self):
        """Clears the counters and latency samples (after warm-up requests)."""
        self.L.decaes_server_reset_stats(self.h)

    def close(self):
        if getattr(self, "h", None):
            self.L.decaes_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
