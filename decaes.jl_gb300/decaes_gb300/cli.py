"""Command-line front end on the GPU library: the counterpart of the
reference's `decaes` program (src/main.jl).

    python -m decaes_gb300 image.nii.gz --T2map --T2part --TE 10e-3 --nT2 40 \\
        --T2Range 10e-3 2.0 --SPWin 10e-3 25e-3 --MPWin 25e-3 200e-3 --Reg lcurve -o results/

Same arguments and file conventions as the reference (src/main.jl:8-291):
inputs .mat / .nii / .nii.gz / .par / .xml / .rec (one 4-D image each; masks and B1
maps 3-D), `@file` settings files with one argument per line, outputs
<name>.t2dist.mat ("dist"), <name>.t2maps.mat (the maps dictionary),
<name>.t2parts.mat (the parts dictionary) and <name>.log in the output folder
(next to the input unless --output is given).  Extensions: --precision
(fp64, the reference's arithmetic; or mixed) and --device.  The T2 work runs
on the GPU through decaes_gb300.api; there is no CPU path.
"""
from __future__ import annotations

import argparse
import contextlib
import logging
import os
import shutil
import subprocess
import sys
import tempfile
import threading
import time
import warnings

import numpy as np

ALLOWED_FILE_SUFFIXES = (".mat", ".nii", ".nii.gz", ".par", ".xml", ".rec")
ALLOWED_FILE_SUFFIXES_STRING = ", ".join(ALLOWED_FILE_SUFFIXES[:-1]) + ", and " + ALLOWED_FILE_SUFFIXES[-1]

log = logging.getLogger("decaes_gb300.cli")


# ---------------------------------------------------------------------------
# Arguments (src/main.jl:8-254)
# ---------------------------------------------------------------------------
def build_parser() -> argparse.ArgumentParser:
    p = argparse.ArgumentParser(prog="decaes", fromfile_prefix_chars="@",
                                description="T2 distributions (T2mapSEcorr) and T2 parts (T2partSEcorr) on the GPU.")
    p.add_argument("input", nargs="*", help=f"input images ({ALLOWED_FILE_SUFFIXES_STRING})")
    p.add_argument("--mask", "-m", nargs="+", help="mask files, one per input, multiplied into the images")
    p.add_argument("--output", "-o", nargs="+", help="output folder(s): one for all inputs or one per input")
    p.add_argument("--T2map", action="store_true", help="compute T2 distributions and maps from multi spin-echo images")
    p.add_argument("--T2part", action="store_true",
                   help="compute T2 parts; with --T2map from the computed distributions, else the inputs are distributions")
    p.add_argument("--quiet", "-q", action="store_true", help="print nothing to the terminal (the log file still gets it)")
    p.add_argument("--dry", action="store_true", help="process without saving any results")
    p.add_argument("--legacy", action="store_const", const=True, default=None,
                   help="legacy settings and algorithms of the original MATLAB pipeline (deprecated)")
    g = p.add_argument_group("T2map/T2part required parameters")
    g.add_argument("--MatrixSize", nargs=3, type=int, help="matrix size (default: the image's first three dimensions)")
    g.add_argument("--nTE", type=int, help="number of echoes (default: the image's fourth dimension)")
    g.add_argument("--TE", type=float, help="inter-echo spacing (seconds); required with --T2map")
    g.add_argument("--nT2", type=int, help="number of T2 components; required with --T2map")
    g.add_argument("--T2Range", nargs=2, type=float, help="minimum and maximum T2 (seconds)")
    g.add_argument("--SPWin", nargs=2, type=float, help="short peak window (seconds); required with --T2part")
    g.add_argument("--MPWin", nargs=2, type=float, help="middle peak window (seconds); required with --T2part")
    g.add_argument("--Reg", type=str, help='regularization: "lcurve", "gcv", "chi2", "mdp" or "none"')
    g.add_argument("--RegParams", nargs="+", type=float,
                   help='parameters of --Reg: the chi2 factor for "chi2", the noise level for "mdp"')
    g.add_argument("--Chi2Factor", type=float, help="chi2 factor (deprecated; use --RegParams)")
    g = p.add_argument_group("T2map/T2part optional parameters")
    g.add_argument("--T1", type=float, help="assumed T1 (seconds, default 1.0)")
    g.add_argument("--Sigmoid", type=float, help="smooth the upper short-peak cutoff over this time scale (seconds)")
    g.add_argument("--Threshold", type=float, help="first-echo intensity at or below which a voxel is skipped")
    g = p.add_argument_group("B1 correction and stimulated echo correction")
    g.add_argument("--B1map", nargs="+", help="B1 map files (degrees), one per input")
    g.add_argument("--nRefAngles", type=int, help="maximum number of refocusing angles checked")
    g.add_argument("--nRefAnglesMin", type=int, help="initial number of refocusing angles checked")
    g.add_argument("--MinRefAngle", type=float, help="smallest refocusing angle (degrees, default 50)")
    g.add_argument("--SetFlipAngle", type=float, help="fixed refocusing angle for every voxel (degrees)")
    g.add_argument("--RefConAngle", type=float, help="refocusing pulse control angle (degrees, default 180)")
    g = p.add_argument_group("Additional save options")
    g.add_argument("--SaveDecayCurve", action="store_true", help="save the fitted decay curves")
    g.add_argument("--SaveNNLSBasis", action="store_true", help="save the NNLS basis matrices")
    g.add_argument("--SaveRegParam", action="store_true", help="save the regularization parameters and chi2 factors")
    g.add_argument("--SaveResidualNorm", action="store_true", help="save the residual norms")
    g = p.add_argument_group("BET arguments")
    g.add_argument("--bet", action="store_true", help="make a brain mask with FSL's BET (ignored when --mask is given)")
    g.add_argument("--betargs", type=str, default="-m -n -f 0.25 -R", help="BET arguments, space or comma separated")
    g.add_argument("--betpath", type=str, default="bet", help="path of the BET executable")
    g = p.add_argument_group("GPU")
    g.add_argument("--precision", choices=("fp64", "mixed", "mixed_tc"), default="fp64",
                   help="fp64: the reference's arithmetic; mixed: the mixed-precision method; mixed_tc: the mixed "
                        "method with the flip-angle search's grid products on the tensor cores")
    g.add_argument("--device", type=int, default=0, help="CUDA device")
    return p


_T2MAP_FIELDS = ("MatrixSize", "nTE", "TE", "nT2", "T2Range", "Reg", "legacy", "T1", "Threshold", "MinRefAngle",
                 "nRefAngles", "nRefAnglesMin", "Chi2Factor", "NoiseLevel", "RefConAngle", "SetFlipAngle",
                 "SaveResidualNorm", "SaveDecayCurve", "SaveRegParam", "SaveNNLSBasis")
_T2PART_FIELDS = ("MatrixSize", "nT2", "T2Range", "SPWin", "MPWin", "legacy", "Sigmoid")


def parse_cli(args) -> dict:
    """parse_cli: parse, handle deprecations, verify, clean (src/main.jl:426-485)."""
    opts = vars(build_parser().parse_args(args))
    # deprecations
    if opts.get("legacy") is not None:
        log.warning("The flag --legacy is deprecated and will be removed in future releases.")
    if opts.get("Chi2Factor") is not None:
        if opts.get("RegParams"):
            raise ValueError("The flag --RegParams and the deprecated flag --Chi2Factor were both passed; use --RegParams only.")
        log.warning("The flag --Chi2Factor is deprecated and will be removed in future releases; use --RegParams instead.")
        opts["RegParams"] = [opts["Chi2Factor"]]
    opts.pop("Chi2Factor", None)
    # verification
    if not (opts["T2map"] or opts["T2part"]):
        raise ValueError("At least one of --T2map or --T2part must be passed")
    # cleaning
    opts["betargs"] = clean_bet_args(opts["betargs"])
    if opts.get("Reg") == "chi2":
        if not opts.get("RegParams") or len(opts["RegParams"]) != 1:
            raise AssertionError('Must set chi2 factor via --RegParams when --Reg="chi2"')
        opts["Chi2Factor"] = opts["RegParams"][0]
    elif opts.get("Reg") == "mdp":
        if not opts.get("RegParams") or len(opts["RegParams"]) != 1:
            raise AssertionError('Must set noise level via --RegParams when --Reg="mdp"')
        opts["NoiseLevel"] = opts["RegParams"][0]
    return opts


def clean_bet_args(betargs: str) -> list:
    """Split on spaces and commas; "-m" (binary mask) is always among them (src/main.jl:682-690)."""
    args = [a for a in betargs.replace(",", " ").split() if a]
    if "-m" not in args:
        args.insert(0, "-m")
    return args


def _set(opts, fields, skip=()):
    kw = {}
    for k in fields:
        if k in skip:
            continue
        v = opts.get(k)
        if v is None or (isinstance(v, (list, tuple)) and len(v) == 0):
            continue
        kw[k] = tuple(v) if isinstance(v, (list, tuple)) else v
    return kw


def t2map_options(image: np.ndarray, opts: dict):
    """T2mapOptions(image; the options that were set) (src/main.jl:487-497)."""
    from .api import T2mapOptions
    kw = _set(opts, _T2MAP_FIELDS)
    kw.setdefault("MatrixSize", image.shape[:3])
    kw.setdefault("nTE", image.shape[3])
    return T2mapOptions(**kw, precision=opts.get("precision", "fp64"))


def t2part_options(dist: np.ndarray, opts: dict):
    """T2partOptions(dist; the options that were set); nT2 comes from dist unless
    T2-mapping ran (src/main.jl:499-510)."""
    from .api import T2partOptions
    kw = _set(opts, _T2PART_FIELDS, skip=() if opts["T2map"] else ("nT2",))
    kw.setdefault("MatrixSize", dist.shape[:3])
    kw.setdefault("nT2", dist.shape[3])
    return T2partOptions(**kw)


# ---------------------------------------------------------------------------
# Files (src/main.jl:512-702)
# ---------------------------------------------------------------------------
def maybe_get_suffix(filename: str):
    low = filename.lower()
    for ext in ALLOWED_FILE_SUFFIXES:
        if low.endswith(ext):
            return ext
    return None


def chop_allowed_suffix(filename: str) -> str:
    ext = maybe_get_suffix(filename)
    if ext is None:
        raise ValueError(f"Currently only {ALLOWED_FILE_SUFFIXES_STRING} file types are supported")
    return filename[:-len(ext)]


def get_file_infos(opts: dict) -> list:
    inputs = opts.get("input") or []
    if not inputs:
        raise AssertionError("At least one input file is required")
    files = [f for f in inputs if maybe_get_suffix(f) is not None]
    if not files:
        if os.path.isfile(inputs[0]):
            raise ValueError("No valid file types were found for processing, but a file name was passed.\n"
                             f"Perhaps you meant to prepend an '@' character to a settings file, e.g. '@{inputs[0]}'?\n"
                             f"If not, note that only {ALLOWED_FILE_SUFFIXES_STRING} file types are supported")
        raise ValueError(f"No valid files were found for processing. Note that currently only "
                         f"{ALLOWED_FILE_SUFFIXES_STRING} file types are supported")
    out = opts.get("output") or []
    if not out:
        folders = [os.path.dirname(f) for f in files]
    elif len(out) == len(files):
        folders = list(out)
    elif len(out) == 1:
        folders = [out[0]] * len(files)
    else:
        raise ValueError(f"Incorrect number of output files passed ({len(out)}); must pass either 1 output folder (all "
                         "results are stored in this folder), or the same number of output folders as input image files "
                         f"({len(files)})")
    mask = opts.get("mask") or []
    if not mask:
        masks = [None] * len(files)
    elif len(mask) == len(files):
        masks = list(mask)
    else:
        raise ValueError(f"Number of mask files passed ({len(mask)}) does not equal the number of input image files "
                         f"passed ({len(files)})")
    b1 = opts.get("B1map") or []
    if not b1:
        b1s = [None] * len(files)
    elif len(b1) == len(files):
        if opts.get("SetFlipAngle") is not None:
            raise AssertionError("Cannot set a fixed flip angle using --SetFlipAngle when passing B1 maps using --B1map")
        b1s = list(b1)
    else:
        raise ValueError(f"Number of B1 map files passed ({len(b1)}) does not equal the number of input image files "
                         f"passed ({len(files)})")
    return [dict(inputfile=f, outputfolder=o, maskfile=m, B1mapfile=b, choppedinputfile=chop_allowed_suffix(os.path.basename(f)))
            for f, o, m, b in zip(files, folders, masks, b1s)]


def ensure_ndims(filename: str, data: np.ndarray, n: int) -> np.ndarray:
    if data.ndim < n:
        return data.reshape(data.shape + (1,) * (n - data.ndim), order="F")
    if data.ndim == n:
        return data
    if any(s > 1 for s in data.shape[n:]):
        extra = list(range(n + 1, data.ndim + 1))
        log.warning(f"Input file {filename} has {data.ndim} dimensions, expected {n}; selecting the first {n}-D volume "
                    f"along {'dimension' if len(extra) == 1 else 'dimensions'} {','.join(map(str, extra))}.")
    return data[(slice(None),) * n + (0,) * (data.ndim - n)]


def load_image(filename: str, ndims: int = 4) -> np.ndarray:
    """The file's first ndims-D array as Float64 in Fortran order (src/main.jl:577-616)."""
    ext = maybe_get_suffix(filename)
    if ext == ".mat":
        from . import matfile
        with warnings.catch_warnings(record=True) as caught:
            warnings.simplefilter("always")
            data = matfile.read_array(filename, ndims)
        for w in caught:
            log.warning(str(w.message))
    elif ext in (".nii", ".nii.gz"):
        from . import nifti
        data = nifti.read(filename).scaled()
    elif ext in (".par", ".xml", ".rec"):
        from . import parrec
        data = parrec.read(filename)
    else:
        raise ValueError(f"Currently, only {ALLOWED_FILE_SUFFIXES_STRING} files are supported")
    data = ensure_ndims(filename, np.asarray(data), ndims)
    return np.asfortranarray(data, dtype=np.float64)


def make_bet_mask(image: np.ndarray, betpath: str, betargs: list) -> np.ndarray:
    """Brain mask from BET run on the first echo (src/main.jl:663-680)."""
    from . import nifti
    if image.ndim == 4:
        image = image[:, :, :, 0]
    with tempfile.TemporaryDirectory() as tmp:
        base = os.path.basename(tempfile.mktemp(dir=tmp))
        img_file = os.path.join(tmp, base + ".nii")
        mask_file = os.path.join(tmp, base + ".bet")
        nifti.write(img_file, np.asfortranarray(image))
        subprocess.run([betpath, img_file, mask_file] + list(betargs), check=True,
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
        found = [f for f in os.listdir(tmp) if f.startswith(base + ".bet_mask")]
        if len(found) != 1:
            raise RuntimeError(f"BET produced {len(found)} mask files")
        return load_image(os.path.join(tmp, found[0]), 3)


def _try_apply_mask(image, maskfile):
    try:
        image *= load_image(maskfile, 3)[..., None]
    except Exception as e:  # the reference warns and carries on unmasked
        log.warning(f"Error while loading mask file: {maskfile}")
        log.warning(repr(e))
    return image


def _try_apply_bet(image, betpath, betargs):
    try:
        image *= make_bet_mask(image, betpath, betargs)[..., None]
    except Exception as e:
        log.warning("Error while making mask using BET")
        log.warning(repr(e))
    return image


def _try_load_b1(b1file, shape):
    try:
        b1 = load_image(b1file, 3)
        if b1.shape != tuple(shape):
            raise AssertionError(f"B1 map size {b1.shape} does not match the image matrix size {tuple(shape)}")
        return b1
    except Exception as e:
        log.warning(f"Error while loading B1 map file: {b1file}")
        log.warning(repr(e))
        return None


# ---------------------------------------------------------------------------
# Processing (src/main.jl:272-420)
# ---------------------------------------------------------------------------
class ThisThread(logging.Filter):
    """Passes the records of the thread that made the filter: runs that share
    the process (a daemon serving several clients at once) keep their logs
    apart."""

    def __init__(self):
        super().__init__()
        self.ident = threading.get_ident()

    def filter(self, record):
        return record.thread == self.ident


_level_lock = threading.Lock()
_level_users = [0, logging.NOTSET]  # runs logging at INFO, the level to restore after the last


@contextlib.contextmanager
def _tee(logfile, quiet: bool, dry: bool):
    handlers = []
    if not quiet:
        handlers.append(logging.StreamHandler(sys.stderr))
    if not dry and logfile:
        handlers.append(logging.FileHandler(logfile, mode="w"))
    fmt = logging.Formatter("[%(levelname)s] %(message)s")
    mine = ThisThread()
    for h in handlers:
        h.setFormatter(fmt)
        h.addFilter(mine)
        log.addHandler(h)
    with _level_lock:
        if _level_users[0] == 0:
            _level_users[1] = log.level
        _level_users[0] += 1
        log.setLevel(logging.INFO)
    try:
        yield
    finally:
        for h in handlers:
            log.removeHandler(h)
            h.close()
        with _level_lock:
            _level_users[0] -= 1
            if _level_users[0] == 0:
                log.setLevel(_level_users[1])


def _timed(msg, fn, *a, **kw):
    log.info(msg)
    t = time.time()
    r = fn(*a, **kw)
    log.info(f"Done ({time.time() - t:.2f} seconds)")
    return r


class DirectSolver:
    """The GPU calls of a run, straight on a context (the command line's own
    process)."""

    def __init__(self, ctx):
        self.ctx = ctx

    def t2map_t2part(self, image, mo, po, b1):
        from . import api
        return api.T2mapSEcorr_T2partSEcorr(image, mo, po, b1map=b1, ctx=self.ctx)

    def t2map(self, image, mo, b1):
        from . import api
        return api.T2mapSEcorr(image, mo, b1map=b1, ctx=self.ctx)

    def t2part(self, dist, po):
        from . import api
        return api.T2partSEcorr(dist, po, ctx=self.ctx)


def process_file(info: dict, opts: dict, ctx=None, solver=None) -> None:
    from . import matfile
    solver = solver or DirectSolver(ctx)
    t0 = time.time()
    log.info(f"Starting decaes_gb300 (GPU {opts.get('device', 0)}, precision {opts.get('precision', 'fp64')})")
    image = _timed(f"Loading input file: {info['inputfile']}", load_image, info["inputfile"])
    if info["maskfile"] is not None:
        _timed(f"Applying mask from file: {info['maskfile']}", _try_apply_mask, image, info["maskfile"])
    elif opts["bet"]:
        _timed(f"Making and applying BET mask with args: {' '.join(opts['betargs'])}", _try_apply_bet, image,
               opts["betpath"], opts["betargs"])
    out = info["outputfolder"]
    stem = info["choppedinputfile"]
    save = not opts["dry"]
    if opts["T2map"]:
        mo = t2map_options(image, opts)
        b1 = None
        if info["B1mapfile"] is not None:
            b1 = _timed(f"Loading B1 map from file: {info['B1mapfile']}", _try_load_b1, info["B1mapfile"], mo.MatrixSize)
        if opts["T2part"]:
            po = t2part_options(_dist_shape(mo), opts)
            maps, dist, parts = _timed(f"Running T2mapSEcorr and T2partSEcorr on file: {info['inputfile']}",
                                       solver.t2map_t2part, image, mo, po, b1)
        else:
            maps, dist = _timed(f"Running T2mapSEcorr on file: {info['inputfile']}", solver.t2map, image, mo, b1)
            parts = None
        if save:
            f = os.path.join(out, stem + ".t2dist.mat")
            _timed(f"Saving T2 distribution to file: {f}", matfile.write, f, {"dist": dist})
            f = os.path.join(out, stem + ".t2maps.mat")
            _timed(f"Saving T2 parameter maps to file: {f}", matfile.write, f, maps)
    else:
        dist, parts = image, None
    if opts["T2part"]:
        if parts is None:
            po = t2part_options(dist, opts)
            parts = _timed("Running T2partSEcorr", solver.t2part, dist, po)
        if save:
            f = os.path.join(out, stem + ".t2parts.mat")
            _timed(f"Saving T2 parts maps to file: {f}", matfile.write, f, parts)
    log.info(f"Finished ({time.time() - t0:.2f} seconds)")


class _Shape:
    """Stands for the distribution array when only its shape is needed."""
    def __init__(self, shape):
        self.shape = shape


def _dist_shape(mo):
    return _Shape(tuple(mo.MatrixSize) + (mo.nT2,))


def _under(cwd, path):
    return path if path is None or os.path.isabs(path) else os.path.join(cwd, path)


def run_main(args=None, ctx=None, cwd=None, solver=None) -> None:
    """main(ARGS): every input file in turn; a failing file is logged and the
    next one runs (src/main.jl:272-332).  cwd: the directory relative paths
    (inputs, outputs, masks, B1 maps, @settings files) are taken from, when it
    is not the process's own (a daemon running a client's command line).
    solver: the object that makes the GPU calls (DirectSolver on ctx by
    default)."""
    args = list(sys.argv[1:] if args is None else args)
    if cwd is not None:
        args = ["@" + _under(cwd, a[1:]) if a.startswith("@") else a for a in args]
    opts = parse_cli(args)
    if cwd is not None:
        for k in ("input", "output", "mask", "B1map"):
            if opts.get(k):
                opts[k] = [_under(cwd, f) for f in opts[k]]
    if ctx is None and solver is None:
        from ._lib import Context
        ctx = Context(opts.get("device", 0))
    for info in get_file_infos(opts):
        if not opts["dry"] and info["outputfolder"]:
            os.makedirs(info["outputfolder"], exist_ok=True)
        if not opts["dry"]:
            for a in args:
                if a.startswith("@"):
                    src = a[1:]
                    shutil.copyfile(src, os.path.join(info["outputfolder"], info["choppedinputfile"] + "." + os.path.basename(src)))
        logfile = os.path.join(info["outputfolder"], info["choppedinputfile"] + ".log")
        with _tee(logfile, opts["quiet"], opts["dry"]):
            try:
                process_file(info, opts, ctx, solver)
            except Exception as e:
                log.warning(f"Error during processing of file: {info['inputfile']}")
                log.warning(f"{type(e).__name__}: {e}")


def main() -> None:
    run_main()
