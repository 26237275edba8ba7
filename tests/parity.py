"""Shared helpers of the GPU-vs-oracle parity tests: build the same seeded
inputs for both sides and compare outputs with the stated tolerances."""
from __future__ import annotations

import numpy as np

# Tolerances of the plain (FP64) method against the FP64 oracle.
DIST_RTOL = 1e-8     # per distribution bin, relative
MWF_ATOL = 1e-10     # myelin water fraction (sfr), absolute


def orc_opts(orc, o):
    return orc.T2mapOptions(MatrixSize=o.MatrixSize, nTE=o.nTE, TE=o.TE, nT2=o.nT2, T2Range=o.T2Range, Reg=o.Reg,
                            T1=o.T1, Threshold=o.Threshold, MinRefAngle=o.MinRefAngle, nRefAngles=o.nRefAngles,
                            nRefAnglesMin=o.nRefAnglesMin, Chi2Factor=o.Chi2Factor, NoiseLevel=o.NoiseLevel,
                            RefConAngle=o.RefConAngle, SetFlipAngle=o.SetFlipAngle,
                            SaveResidualNorm=o.SaveResidualNorm, SaveDecayCurve=o.SaveDecayCurve,
                            SaveRegParam=o.SaveRegParam, legacy=o.legacy)


def dist_rel_err(d_gpu, d_orc):
    """Per-voxel max over bins of |Δ| / max(|d_orc|, 1e-12 * sum|d_orc|)."""
    n = d_orc.shape[-1]
    a = d_gpu.reshape(-1, n).astype(np.float64)
    b = d_orc.reshape(-1, n)
    ok = ~np.isnan(b).any(axis=1)
    scale = np.maximum(np.abs(b), 1e-12 * np.abs(b).sum(axis=1, keepdims=True))
    err = np.where(scale > 0, np.abs(a - b) / np.where(scale > 0, scale, 1), np.abs(a - b))
    return err.max(axis=1), ok


def summarize(name, err, ok):
    e = err[ok]
    frac = float((e > DIST_RTOL).mean()) if e.size else 0.0
    return dict(name=name, voxels=int(ok.sum()), max_rel=float(e.max()) if e.size else 0.0,
                median_rel=float(np.median(e)) if e.size else 0.0, frac_outside=frac)
