"""Philips PAR/REC and XML/REC images (.par or .xml header + .rec) for the
command-line front end (the reference reads both through ParXRec.jl,
src/main.jl:601-603).

The PAR header (versions 4.x) describes one line per stored image; its
"IMAGE INFORMATION DEFINITION" block lists the columns (name, count, type), so
the columns are located by name rather than by a fixed version layout.  The
XML header holds one <Image_Info> element per stored image, whose <Key>
(Slice, Echo, Dynamic, Phase, Type, Index, ...) and sibling <Attribute
Name="..."> elements give the same fields (Resolution X/Y, Pixel Size,
Rescale Intercept, Rescale Slope, Scale Slope).  The REC file holds the images
back to back, each x by y pixels with x fastest, at the position given by the
image's index in the REC file.

Images are arranged as (x, y, slice, echo, dynamic, cardiac phase, image type)
with each key's distinct values in increasing order; the front end then keeps
the first 4-D volume.  Pixel values are converted to floating-point values by
the header's own rule, FP = (PV * RS + RI) / (RS * SS) (rescale slope RS,
rescale intercept RI, scale slope SS).
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


def _par_records(par: str):
    """Per stored image: (keys, REC index, bits, nx, ny, RI, RS, SS) from a PAR header."""
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
    return [(tuple(int(float(r[idx[k]])) for k in _KEYS), int(r[p_index]), int(r[p_bits]), int(r[p_res]),
             int(r[p_res + 1]), float(r[p_ri]), float(r[p_rs]), float(r[p_ss])) for r in rows]


_XML_KEYS = ("Slice", "Echo", "Dynamic", "Phase", "Type")


def _xml_records(xml: str):
    """The same records from an XML header: one <Image_Info> per stored image."""
    import xml.etree.ElementTree as ET
    root = ET.parse(xml).getroot()
    infos = root.iter("Image_Info")
    recs, types = [], {}
    for info in infos:
        at = {}
        for a in info.iter("Attribute"):
            at.setdefault(a.get("Name"), (a.text or "").strip())
        try:
            t = at["Type"]
            if t not in types:
                types[t] = len(types)
            keys = tuple(int(float(at[k])) for k in _XML_KEYS[:-1]) + (types[t],)
            recs.append((keys, int(at["Index"]), int(at["Pixel Size"]), int(at["Resolution X"]),
                         int(at["Resolution Y"]), float(at["Rescale Intercept"]), float(at["Rescale Slope"]),
                         float(at["Scale Slope"])))
        except KeyError as e:
            raise ValueError(f"{xml}: <Image_Info> without the attribute {e}") from None
    if not recs:
        raise ValueError(f"{xml}: no <Image_Info> elements")
    return recs


def read(path: str) -> np.ndarray:
    """The PAR/REC or XML/REC image as float64, shape (x, y, slice, echo, dynamic, phase, type)."""
    low = path.lower()
    if low.endswith(".xml"):
        hdr, recs_of = path, _xml_records
    elif low.endswith(".par"):
        hdr, recs_of = path, _par_records
    else:
        try:
            hdr, recs_of = _find(path, (".par",)), _par_records
        except FileNotFoundError:
            hdr, recs_of = _find(path, (".xml",)), _xml_records
    rec = path if low.endswith(".rec") else _find(path, (".rec",))
    recs = recs_of(hdr)
    keys = np.array([r[0] for r in recs])
    nx, ny, bits = recs[0][3], recs[0][4], recs[0][2]
    dt = {8: np.dtype(np.uint8), 16: np.dtype("<i2"), 32: np.dtype("<i4")}.get(bits)
    if dt is None:
        raise ValueError(f"{hdr}: unsupported pixel size {bits} bits")
    levels = [np.unique(keys[:, j]) for j in range(keys.shape[1])]
    out = np.full((nx, ny) + tuple(len(l) for l in levels), np.nan, order="F")
    raw = np.fromfile(rec, dtype=dt)
    per = nx * ny
    for key, k, b, rx, ry, ri, rs, ss in recs:
        if rx != nx or ry != ny or b != bits:
            raise ValueError(f"{hdr}: images of different sizes")
        if (k + 1) * per > raw.size:
            raise ValueError(f"{rec}: image {k} lies past the end of the file")
        pv = raw[k * per:(k + 1) * per].astype(np.float64).reshape((nx, ny), order="F")
        pos = tuple(int(np.searchsorted(levels[j], key[j])) for j in range(len(key)))
        out[(slice(None), slice(None)) + pos] = (pv * rs + ri) / (rs * ss)
    return out
