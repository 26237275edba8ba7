"""MAT files for the command-line front end (scipy.io).

Reading accepts MATLAB v4/v5/v7 files; v7.3 files are HDF5 containers and
need an HDF5 library, which this environment does not have, so they are
rejected with a message.  Writing produces MATLAB v5 files, which MATLAB,
MAT.jl and scipy read; the reference's MAT.jl writes v7.3 (HDF5).
"""
from __future__ import annotations

import warnings

import numpy as np


def _scipy_io():
    try:
        import scipy.io as sio
    except ImportError as e:  # pragma: no cover - scipy is a dependency of the front end
        raise RuntimeError("reading and writing .mat files needs scipy") from e
    return sio


def read_array(path: str, ndims: int) -> np.ndarray:
    """The first variable of the file that is an ndims-dimensional array, in
    sorted name order when there are several (src/main.jl:577-585)."""
    sio = _scipy_io()
    try:
        data = sio.loadmat(path, squeeze_me=False, mat_dtype=False)
    except NotImplementedError as e:
        raise ValueError(f"{path}: MATLAB v7.3 (HDF5) files are not supported here; save with -v7") from e
    keys = sorted(k for k, v in data.items()
                  if not k.startswith("__") and isinstance(v, np.ndarray) and v.ndim == ndims
                  and v.dtype.kind in "biuf")
    if not keys:
        raise ValueError(f"No {ndims}-D array was found in the input file: {path}")
    if len(keys) > 1:
        warnings.warn(f"Multiple possible images found in file: {path}\nChoosing variable {keys[0]!r} out of the "
                      f"following options: {', '.join(repr(k) for k in keys)}")
    return data[keys[0]]


def write(path: str, variables: dict) -> None:
    sio = _scipy_io()
    out = {}
    for k, v in variables.items():
        out[k] = np.asarray(v)
    sio.savemat(path, out, format="5", do_compression=False, oned_as="column")
