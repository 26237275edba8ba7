"""Philips PAR/REC images (.par + .rec) for the command-line front end.

The PAR header (versions 4.x) describes one line per stored image; its
"IMAGE INFORMATION DEFINITION" block lists the columns (name, count, type), so
the columns are located by name rather than by a fixed version layout.  The
REC file holds the images back to back, each recon_x by recon_y pixels with x
fastest, at the position given by the image's "index in REC file".

Images are arranged as (x, y, slice, echo, dynamic, cardiac phase, image type)
with each key's distinct values in increasing order; the front end then keeps
the first 4-D volume.  Pixel values are converted to floating-point values by
the PAR file's own rule, FP = (PV * RS + RI) / (RS * SS) (rescale slope RS,
rescale intercept RI, scale slope SS).  XML headers (.xml) are not read.
"""
from __future__ import annotations

import os
import re

import numpy as np

_KEYS = ("slice number", "echo number", "dynamic scan number", "cardiac phase number", "image_type_mr")


def _columns(lines):
    """(name, first column, count) of each image-information field."""
    cols, pos, inside = [], 0, False
    for ln in lines:
        s = ln.strip()
        if "IMAGE INFORMATION DEFINITION" in s:
            inside = True
            continue
        if inside and "=== IMAGE INFORMATION ===" in s.replace("  ", " ").upper():
            break
        if not inside or not s.startswith("#"):
            continue
        m = re.match(r"#\s+(.*?)\s+\((?:(\d+)\*)?(integer|float|string)\)\s*$", s)
        if m:
            name, cnt = m.group(1).strip().lower(), int(m.group(2) or 1)
            cols.append((name, pos, cnt))
            pos += cnt
    if not cols:
        raise ValueError("PAR file without an IMAGE INFORMATION DEFINITION block")
    return cols


def _col(cols, name):
    for n, p, c in cols:
        if n == name or n.startswith(name):
            return p, c
    raise ValueError(f"PAR image information lacks the column '{name}'")


def _find(path: str, exts) -> str:
    base = os.path.splitext(path)[0]
    for e in exts:
        for cand in (base + e, base + e.upper()):
            if os.path.exists(cand):
                return cand
    raise FileNotFoundError(f"no {'/'.join(exts)} file next to {path}")


def read(path: str) -> np.ndarray:
    """The PAR/REC image as float64, shape (x, y, slice, echo, dynamic, phase, type)."""
    low = path.lower()
    if low.endswith(".xml"):
        raise ValueError(f"{path}: XML PAR headers are not supported; convert to .par or NIfTI")
    par = path if low.endswith(".par") else _find(path, (".par",))
    rec = path if low.endswith(".rec") else _find(path, (".rec",))
    with open(par, "r", encoding="latin-1") as f:
        lines = f.read().splitlines()
    cols = _columns(lines)
    rows = []
    for ln in lines:
        s = ln.strip()
        if not s or s.startswith("#") or s.startswith("."):
            continue
        rows.append(s.split())
    if not rows:
        raise ValueError(f"{par}: no image lines")
    idx = {k: _col(cols, k)[0] for k in _KEYS}
    p_index = _col(cols, "index in rec file")[0]
    p_bits = _col(cols, "image pixel size")[0]
    p_res = _col(cols, "recon resolution")[0]
    p_ri = _col(cols, "rescale intercept")[0]
    p_rs = _col(cols, "rescale slope")[0]
    p_ss = _col(cols, "scale slope")[0]
    keys = np.array([[int(float(r[idx[k]])) for k in _KEYS] for r in rows])
    nx, ny = int(rows[0][p_res]), int(rows[0][p_res + 1])
    bits = int(rows[0][p_bits])
    dt = {8: np.dtype(np.uint8), 16: np.dtype("<i2"), 32: np.dtype("<i4")}.get(bits)
    if dt is None:
        raise ValueError(f"{par}: unsupported pixel size {bits} bits")
    levels = [np.unique(keys[:, j]) for j in range(len(_KEYS))]
    out = np.full((nx, ny) + tuple(len(l) for l in levels), np.nan, order="F")
    raw = np.fromfile(rec, dtype=dt)
    per = nx * ny
    for r, key in zip(rows, keys):
        if int(r[p_res]) != nx or int(r[p_res + 1]) != ny:
            raise ValueError(f"{par}: images of different sizes")
        k = int(r[p_index])
        if (k + 1) * per > raw.size:
            raise ValueError(f"{rec}: image {k} lies past the end of the file")
        pv = raw[k * per:(k + 1) * per].astype(np.float64).reshape((nx, ny), order="F")
        ri, rs, ss = float(r[p_ri]), float(r[p_rs]), float(r[p_ss])
        pos = tuple(int(np.searchsorted(levels[j], key[j])) for j in range(len(_KEYS)))
        out[(slice(None), slice(None)) + pos] = (pv * rs + ri) / (rs * ss)
    return out
