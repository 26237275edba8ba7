"""NIfTI-1 / NIfTI-2 single-file images (.nii, .nii.gz) for the command-line
front end: the reader returns the raw voxel array (x fastest, as stored) and
the header's scl_slope / scl_inter; the writer stores NIfTI-1.

The front end applies the scaling as the reference does after NIfTI.niread
(src/main.jl:587-595): data = raw * scl_slope + scl_inter, with
scl_slope == 0 meaning "not scaled".  The arithmetic type follows Julia's
promotion of the raw element type with the header's float type (Float32 in
NIfTI-1, Float64 in NIfTI-2): integer and Float32 voxels with Float32 scaling
are scaled in Float32, Float64 voxels in Float64.
"""
from __future__ import annotations

import gzip
import struct
from dataclasses import dataclass

import numpy as np

# NIfTI datatype codes -> numpy element types
_DTYPES = {
    2: np.uint8, 4: np.int16, 8: np.int32, 16: np.float32, 64: np.float64,
    256: np.int8, 512: np.uint16, 768: np.uint32, 1024: np.int64, 1280: np.uint64,
}
_CODES = {np.dtype(v): k for k, v in _DTYPES.items()}


@dataclass
class NiftiImage:
    raw: np.ndarray          # voxel array, shape dim[1..ndim], Fortran order
    scl_slope: float
    scl_inter: float
    header_float: type       # np.float32 (NIfTI-1) or np.float64 (NIfTI-2)
    pixdim: tuple

    def scaled(self) -> np.ndarray:
        """raw .* scl_slope .+ scl_inter (slope 0: unscaled), in Julia's promoted type."""
        slope, inter = self.scl_slope, self.scl_inter
        if slope == 0:
            slope, inter = 1.0, 0.0
        ft = np.float64 if (self.raw.dtype == np.float64 or self.header_float == np.float64) else np.float32
        return self.raw.astype(ft) * ft(slope) + ft(inter)


def _read_bytes(path: str) -> bytes:
    with open(path, "rb") as f:
        head = f.read(2)
        f.seek(0)
        data = f.read()
    if head == b"\x1f\x8b":
        return gzip.decompress(data)
    return data


def read(path: str) -> NiftiImage:
    buf = _read_bytes(path)
    if len(buf) < 348:
        raise ValueError(f"{path}: too short for a NIfTI header")
    for end in ("<", ">"):
        (n1,) = struct.unpack(end + "i", buf[:4])
        if n1 in (348, 540):
            break
    else:
        raise ValueError(f"{path}: not a NIfTI-1/2 file (sizeof_hdr = {n1})")
    if n1 == 348:
        dim = struct.unpack(end + "8h", buf[40:56])
        datatype, _bitpix = struct.unpack(end + "hh", buf[70:74])
        pixdim = struct.unpack(end + "8f", buf[76:108])
        (vox_offset,) = struct.unpack(end + "f", buf[108:112])
        scl_slope, scl_inter = struct.unpack(end + "ff", buf[112:120])
        magic = buf[344:348]
        if magic[:3] != b"n+1":
            raise ValueError(f"{path}: NIfTI-1 header without the single-file magic 'n+1'")
        hf = np.float32
    else:
        magic = buf[4:12]
        if magic[:3] != b"n+2":
            raise ValueError(f"{path}: NIfTI-2 header without the single-file magic 'n+2'")
        datatype, _bitpix = struct.unpack(end + "hh", buf[12:16])
        dim = struct.unpack(end + "8q", buf[16:80])
        pixdim = struct.unpack(end + "8d", buf[104:168])
        (vox_offset,) = struct.unpack(end + "q", buf[168:176])
        scl_slope, scl_inter = struct.unpack(end + "dd", buf[176:192])
        hf = np.float64
    ndim = int(dim[0])
    if not 1 <= ndim <= 7:
        raise ValueError(f"{path}: dim[0] = {ndim}")
    shape = tuple(int(d) for d in dim[1:1 + ndim])
    if datatype not in _DTYPES:
        raise ValueError(f"{path}: unsupported NIfTI datatype {datatype}")
    dt = np.dtype(_DTYPES[datatype]).newbyteorder(end)
    count = int(np.prod(shape))
    off = int(vox_offset)
    need = off + count * dt.itemsize
    if len(buf) < need:
        raise ValueError(f"{path}: {len(buf)} bytes, header describes {need}")
    raw = np.frombuffer(buf, dtype=dt, count=count, offset=off).astype(dt.newbyteorder("="))
    return NiftiImage(raw.reshape(shape, order="F"), float(scl_slope), float(scl_inter), hf, tuple(pixdim[1:1 + ndim]))


def write(path: str, data: np.ndarray, pixdim=None, scl_slope: float = 0.0, scl_inter: float = 0.0) -> None:
    """NIfTI-1 single file (gzip when the name ends in .gz), little-endian."""
    a = np.asarray(data)
    if a.dtype not in _CODES:
        a = a.astype(np.float64)
    if a.ndim > 7:
        raise ValueError("NIfTI holds at most 7 dimensions")
    hdr = bytearray(348)
    struct.pack_into("<i", hdr, 0, 348)
    dim = [a.ndim] + list(a.shape) + [1] * (7 - a.ndim)
    struct.pack_into("<8h", hdr, 40, *dim)
    struct.pack_into("<hh", hdr, 70, _CODES[a.dtype], a.dtype.itemsize * 8)
    pd = [1.0] + (list(pixdim) if pixdim is not None else [1.0] * a.ndim) + [1.0] * (7 - a.ndim)
    struct.pack_into("<8f", hdr, 76, *pd[:8])
    struct.pack_into("<f", hdr, 108, 352.0)
    struct.pack_into("<ff", hdr, 112, scl_slope, scl_inter)
    struct.pack_into("<h", hdr, 252, 0)      # qform_code
    struct.pack_into("<h", hdr, 254, 0)      # sform_code
    hdr[344:348] = b"n+1\x00"
    body = bytes(hdr) + b"\x00" * 4 + np.asfortranarray(a).astype(a.dtype.newbyteorder("<")).tobytes(order="F")
    if path.lower().endswith(".gz"):
        body = gzip.compress(body)
    with open(path, "wb") as f:
        f.write(body)
