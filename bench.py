#!/usr/bin/env python
"""Throughput of the voxelwise T2mapSEcorr + T2partSEcorr path on GB300.

Workload (the 48-echo configuration of the reference's headline table):
240x240x48 voxels, 48 echoes, TE = 10 ms, nT2 = 40 over 10 ms - 2 s,
nRefAngles = 32 with the spline flip-angle search, Reg = "lcurve", Float32
input; T2part windows SPWin 10-25 ms, MPWin 25-200 ms.  Synthetic, seeded:
three EPG compartments + Rician noise, 35% background voxels excluded by the
threshold.  A step is one pass of T2map+T2part over the whole volume.

  value  voxels/s of the headline method (default: the mixed-precision
         method) with the image resident in HBM (device-pointer C ABI call)
  e2e    the same metric through the host-buffer C ABI call from pinned
         memory (H2D of the image and D2H of all outputs inside the timing)
  mixed_vs_fp64  the FP64 (plain) method on the same volume: its voxels/s,
         the speed-up, and the mixed method's per-output error against it
         over every processed voxel (MWF, distribution L1, flip angle; the
         method's accuracy gate: MWF p99 <= 1e-3)
  parity  the oracle (FP64 CPU restatement of the reference path) on a
         sample of the volume's voxels against the FP64 GPU method (bitwise /
         1e-8 per bin / 1e-10 MWF) and the mixed method (its gate)
  --precision fp64  makes the FP64 method the headline
  --impl reference  times the CPU restatement of the reference path (the
         oracle, all host threads) on a leading z-slab of the same volume,
         generated without loading the GPU library.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "decaes.jl_gb300"))
from decaes_gb300 import replicas  # noqa: E402  (pure Python; no library load)

METRIC = "voxels/s T2map+T2part, 240×240×48×48 echoes: FP64 vs mixed prec @MWF|Δ|≤1e-3; p99"
SPWIN, MPWIN = (10e-3, 25e-3), (25e-3, 200e-3)
THRESHOLD = 200.0


# Workloads: the 48-echo L-curve volume (the headline) and the 56-echo GCV
# volume of the mixed-precision configuration.
WORKLOADS = {
    "lcurve48": dict(matrix=(240, 240, 48), nTE=48, TE=10e-3, nT2=40, T2Range=(10e-3, 2.0), Reg="lcurve", K=32),
    "gcv56": dict(matrix=(240, 240, 113), nTE=56, TE=7e-3, nT2=60, T2Range=(8e-3, 2.0), Reg="gcv", K=64),
    # the 48-echo volume with the MATLAB toolbox's regularization (chi2 1.02) and angle count (8)
    "chi2k8_48": dict(matrix=(240, 240, 48), nTE=48, TE=10e-3, nT2=40, T2Range=(10e-3, 2.0), Reg="chi2",
                      Chi2Factor=1.02, K=8),
}


# z-slices of one --impl reference step (about 5 s of oracle work on 16 cores)
REF_SLICES = {"lcurve48": 2, "gcv56": 1, "chi2k8_48": 4}
# The reference's published whole-dataset figures for these echo counts and
# matrix sizes (README.md:72-73, DECAES on a 32-core AMD Threadripper 3970X;
# real MSE data, settings and mask not stated): voxels / time.
_PUB48 = {"value": 240 * 240 * 48 / 4.3, "unit": "voxels/s", "cores": 32,
          "source": "README.md:73: 48-echo 240x240x48 dataset in 4.3 s on an AMD Threadripper 3970X (32 cores); "
                    "settings and mask not stated"}
PUBLISHED = {"lcurve48": _PUB48, "chi2k8_48": _PUB48,
             "gcv56": {"value": 240 * 240 * 113 / 7.7, "unit": "voxels/s", "cores": 32,
                       "source": "README.md:72: 56-echo 240x240x113 dataset in 7.7 s on an AMD Threadripper 3970X "
                                 "(32 cores); settings and mask not stated"}}


def workload(matrix, precision, name="lcurve48"):
    import decaes_gb300 as D
    w = WORKLOADS[name]
    mo = D.T2mapOptions(MatrixSize=matrix, nTE=w["nTE"], TE=w["TE"], nT2=w["nT2"], T2Range=w["T2Range"], Reg=w["Reg"],
                        nRefAngles=w["K"], MinRefAngle=50.0, Threshold=THRESHOLD, Chi2Factor=w.get("Chi2Factor"),
                        precision=precision)
    po = D.T2partOptions.from_t2map(mo, SPWin=SPWIN, MPWin=MPWIN)
    mock = D.MockImageOptions(MatrixSize=matrix, nTE=w["nTE"], TE=w["TE"], BackgroundFraction=0.35)
    return mo, po, mock


def config_dict(matrix, V, name="lcurve48"):
    """The workload, identical in both arms' lines (nothing measured in it)."""
    w = WORKLOADS[name]
    img_mb = V * w["nTE"] * 4 / 1e6
    return {
        "workload": f"{matrix[0]}x{matrix[1]}x{matrix[2]} voxels x {w['nTE']} echoes, TE={w['TE'] * 1e3:g}ms, "
                    f"nT2={w['nT2']} ({w['T2Range'][0] * 1e3:g}ms-{w['T2Range'][1]:g}s), nRefAngles={w['K']} "
                    f"(spline flip-angle search), Reg={w['Reg']}{' ' + str(w['Chi2Factor']) if 'Chi2Factor' in w else ''}, Float32 input, T2part SPWin 10-25ms MPWin 25-200ms",
        "voxels": V,
        "l2": f"inputs larger than L2 ({img_mb:.0f} MB image vs 129 MB L2); no flush needed",
        "parallelism": "replicas (independent volume per GPU)",
    }


def _oracle():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    return O


def oracle_opts(O, name, V):
    w = WORKLOADS[name]
    return O.T2mapOptions(MatrixSize=(V, 1, 1), nTE=w["nTE"], TE=w["TE"], nT2=w["nT2"], T2Range=w["T2Range"],
                          Reg=w["Reg"], nRefAngles=w["K"], MinRefAngle=50.0, Threshold=THRESHOLD,
                          Chi2Factor=w.get("Chi2Factor"))


def oracle_run(O, name, flat, threads):
    """The oracle on voxel rows flat (V x nTE): T2map + T2part; returns
    (maps, dist V x nT2, parts, FP64 FLOPs per processed voxel, seconds)."""
    w = WORKLOADS[name]
    V = flat.shape[0]
    sub = np.asfortranarray(flat.astype(np.float64)).reshape((V, 1, 1, w["nTE"]), order="F")
    t0 = time.perf_counter()
    maps, dist, fl = O.t2map(sub, oracle_opts(O, name, V), nthreads=threads, return_flops=True)
    parts = O.t2part(dist, O.T2partOptions(MatrixSize=(V, 1, 1), nT2=w["nT2"], T2Range=w["T2Range"], SPWin=SPWIN,
                                           MPWin=MPWIN))
    dt = time.perf_counter() - t0
    nproc = max(1, int((~np.isnan(maps["alpha"].reshape(-1))).sum()))
    flat_maps = {k: v.reshape(V, -1, order="F").squeeze(-1) if v.ndim == 3 else v for k, v in maps.items()}
    return flat_maps, dist.reshape(V, w["nT2"], order="F"), {k: v.reshape(-1, order="F") for k, v in parts.items()}, \
        sum(fl.values()) / nproc, dt


def cpu_baseline(name, flat, Vp, sample, threads):
    """The oracle on a bounded sample of above-threshold voxels (rows of flat,
    V x nTE, evenly spread over the processed voxels); returns the voxel
    indices, the oracle's outputs on them, voxels/s scaled to the whole image
    (its time per processed voxel times the image's processed-voxel count) and
    the FP64 FLOPs per processed voxel."""
    O = _oracle()
    fg = np.flatnonzero(flat[:, 0] > THRESHOLD)
    pick = fg[np.linspace(0, len(fg) - 1, min(sample, len(fg))).astype(np.int64)]
    maps, dist, parts, flv, dt = oracle_run(O, name, flat[pick], threads)
    whole = dt / len(pick) * Vp
    return dict(pick=pick, maps=maps, dist=dist, parts=parts, value=flat.shape[0] / whole, seconds=dt,
                flops_per_voxel=flv)


def run_reference(args):
    """Times the oracle (CPU restatement of the reference path) on the host
    cores.  Each step runs T2map + T2part on a leading z-slab of the
    workload's volume (the first --ref-slices slices: the same voxels the
    whole-volume run sees there), generated by the oracle's copy of the
    synthetic generator, so nothing of the GPU library is loaded."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    O = _oracle()
    w = WORKLOADS[args.workload]
    matrix = tuple(args.matrix) if args.matrix else w["matrix"]
    nz = max(1, min(args.ref_slices or REF_SLICES[args.workload], matrix[2]))
    slab = (matrix[0], matrix[1], nz)
    Vs = int(np.prod(slab))
    threads = os.cpu_count() or 1
    img = O.mock_image(slab, w["nTE"], seed=args.seed, dtype=np.float32, TE=w["TE"], BackgroundFraction=0.35,
                       nthreads=threads)
    flat = img.reshape((Vs, w["nTE"]), order="F")
    nfg = int((flat[:, 0] > THRESHOLD).sum())
    for _ in range(args.warmup):
        oracle_run(O, args.workload, flat, threads)
    secs = []
    for _ in range(args.steps):
        secs.append(oracle_run(O, args.workload, flat, threads)[4])
    ms_per_step = 1e3 * sum(secs) / len(secs)
    value = Vs / (ms_per_step * 1e-3)
    V = int(np.prod(matrix))
    sample = (f"each step: the first {nz} of {matrix[2]} z-slices of the volume ({slab[0]}x{slab[1]}x{nz} = {Vs} "
              f"voxels, {nfg} above threshold), T2map + T2part, {threads} threads; value = slab voxels / step time")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "voxels/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded 3-compartment EPG + Rician noise, 35% background)",
        "config": config_dict(matrix, V, args.workload),
        "method": "oracle: FP64 C restatement of the reference CPU path (Julia is not installed)",
        "cpu_baseline": {"value": value, "unit": "voxels/s", "cores": threads, "kind": "port", "sample": sample,
                         "per_core": value / threads},
        "e2e": {"value": value, "unit": "voxels/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "published_reference": PUBLISHED.get(args.workload),
    }
    print(json.dumps(line), flush=True)


def profile_figure(name, key):
    """A figure (per voxel) from a committed ncu summary, or None."""
    p = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith(key + ":"):
            return float(line.split(":")[1])
    return None


class DeviceRun:
    """Device-resident inputs and outputs (torch owns the memory) and the
    device-pointer C ABI call of one method.  f64: FP64 image and outputs
    (the same values as the Float32 image, widened), for exact comparisons."""

    OUT_KEYS = ["dist", "gdn", "ggm", "gva", "fnr", "snr", "alpha"]

    def __init__(self, D, _lib, ctx, torch, mo, po, img, V, f64=False):
        self.ctx, self.L, self.torch, self._lib = ctx, ctx.L, torch, _lib
        n = mo.nT2
        dt = torch.float64 if f64 else torch.float32
        self.code = _lib.F64 if f64 else _lib.F32
        self.stream = torch.cuda.current_stream()
        h = img.reshape(-1, order="F")
        self.d_img = torch.from_numpy(h.astype(np.float64) if f64 else h.copy()).cuda()
        self.d_out = {"dist": torch.empty(V * n, dtype=dt, device="cuda")}
        for k in self.OUT_KEYS[1:]:
            self.d_out[k] = torch.empty(V, dtype=dt, device="cuda")
        self.d_parts = {k: torch.empty(V, dtype=dt, device="cuda") for k in ("sfr", "sgm", "mfr", "mgm")}
        self.mout = _lib.T2mapOutC(*[C.c_void_p(self.d_out[k].data_ptr()) if k in self.d_out else None
                                     for k, _ in _lib.T2mapOutC._fields_])
        self.pout = _lib.T2partOutC(*[C.c_void_p(self.d_parts[k].data_ptr()) for k, _ in _lib.T2partOutC._fields_])
        self.mo_c, self.po_c = mo.to_c(), po.to_c()
        self.V, self.n = V, n

    def step(self):
        self.ctx.check(self.L.decaes_t2map_t2part_device(
            self.ctx.h, C.byref(self.mo_c), C.byref(self.po_c), C.c_void_p(self.d_img.data_ptr()), self.code, None,
            C.byref(self.mout), C.byref(self.pout), C.c_void_p(self.stream.cuda_stream)))

    def stats(self):
        self.ctx.check(self.L.decaes_sync_stats(self.ctx.h, C.c_void_p(self.stream.cuda_stream)))
        return self.ctx.stats()

    def host(self):
        """dist (V x nT2), alpha and sfr on the host, FP64."""
        return (self.d_out["dist"].double().cpu().numpy().reshape(self.n, self.V).T,
                self.d_out["alpha"].double().cpu().numpy(), self.d_parts["sfr"].double().cpu().numpy())

    def timed(self, steps, warmup, world, clocks=None):
        """W untimed steps, then K steps between barrier + synchronize; returns
        (ms per step as the max over ranks, kernel launches, voxel-solve ms per step)."""
        torch = self.torch
        for _ in range(warmup):
            self.step()
        torch.cuda.synchronize()
        self.stats()
        replicas.barrier(world)
        torch.cuda.synchronize()
        solve_ms, launches = [], 0
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with (clocks if clocks is not None else _Null()):
            e0.record(self.stream)
            for _ in range(steps):
                self.step()
                st = self.stats()
                solve_ms.append(st["ms_solve"])
                launches += st["kernel_launches"]
            e1.record(self.stream)
            torch.cuda.synchronize()
        ms = replicas.max_over_ranks(e0.elapsed_time(e1), world, device="cuda")
        replicas.barrier(world)
        return ms / steps, launches, solve_ms


class _Null:
    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False


def dist_errors(d, ref):
    """Per voxel (rows): the largest per-bin error |d - ref| / max(|ref|,
    1e-12 sum|ref|) and the L1 error sum|d - ref| / sum|ref|."""
    diff = np.abs(d - ref)
    tot = np.abs(ref).sum(axis=1)
    scale = np.maximum(np.abs(ref), 1e-12 * tot[:, None])
    rel = np.where(scale > 0, diff / np.where(scale > 0, scale, 1), diff).max(axis=1)
    l1 = np.where(tot > 0, diff.sum(axis=1) / np.where(tot > 0, tot, 1), diff.sum(axis=1))
    return rel, l1


def _q(x, q):
    return float(np.quantile(x, q)) if x.size else 0.0


def _mx(x):
    return float(x.max()) if x.size else 0.0


def method_errors(dist, alpha, sfr, rdist, ralpha, rsfr, tail=0):
    """A method's per-output errors against reference outputs on the same
    voxels (processed in the reference): MWF, distribution L1 and per-bin
    relative error, flip angle; optionally the voxels with MWF error > 1e-3."""
    ok = ~np.isnan(rsfr)
    same = bool(np.array_equal(ok, ~np.isnan(sfr)))
    dm = np.abs(sfr[ok] - rsfr[ok])
    da = np.abs(alpha[ok] - ralpha[ok])
    rel, l1 = dist_errors(dist[ok], rdist[ok])
    out = {"voxels": int(ok.sum()), "same_processed_voxels": same,
           "mwf_abs": {"max": _mx(dm), "p99": _q(dm, 0.99), "frac_gt_1e-3": float((dm > 1e-3).mean()) if dm.size else 0.0},
           "dist_l1_rel": {"max": _mx(l1), "p99": _q(l1, 0.99)},
           "dist_bin_rel": {"max": _mx(rel), "p99": _q(rel, 0.99)},
           "alpha_abs_deg": {"max": _mx(da), "p99": _q(da, 0.99)}}
    if tail:
        idx = np.flatnonzero(ok)
        big = np.argsort(-dm)[:tail]
        out["largest_mwf_errors"] = [[int(idx[i]), float(dm[i])] for i in big if dm[i] > 1e-3]
    return out


def bitwise_frac(dist, alpha, sfr, rdist, ralpha, rsfr):
    ok = ~np.isnan(rsfr)
    eq = (dist[ok] == rdist[ok]).all(axis=1) & (alpha[ok] == ralpha[ok]) & (sfr[ok] == rsfr[ok])
    return float(eq.mean()) if eq.size else 0.0


class Clocks:
    """Samples nvidia-smi SM clocks and throttle reasons during the timed region."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index, self.rows, self.proc = index, [], None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        rows = [r for r in self.rows if len(r) >= 8]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[4 + i].strip() == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def fp64_pipe_view(torch, ipv, Vp, kern_ms, clocks):
    """The voxel kernel against the unit that binds it: FP64-pipe warp
    instructions per second (ncu's count per voxel on a slab of the same
    generator x voxels processed / kernel time) over the pipe's issue limit,
    one warp instruction per 64 cycles per SM sub-partition (4 per SM) at the
    SM clock sampled during the timed steps."""
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz")
    if not mhz:
        return None
    achieved = ipv * Vp / (kern_ms * 1e-3) / 1e9
    peak = 4 * sms * mhz * 1e6 / 64 / 1e9
    return {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "G FP64 warp instructions/s",
            "frac": achieved / peak, "instructions_per_voxel": ipv,
            "peak_source": f"{sms} SMs x 4 sub-partitions x {mhz:.0f} MHz / 64 cycles per FP64 warp instruction"}


def fp64_peak_tflops(torch):
    """cuBLAS DGEMM throughput on this GPU (the FP64 roofline denominator)."""
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    for _ in range(2):
        a @ b
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    best = 1e30
    for _ in range(5):
        e0.record()
        a @ b
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    del a, b
    return 2 * n ** 3 / (best * 1e-3) / 1e12


def batch_volume_specs(rng, nvol, seed):
    """Volume shapes and options of the uneven-batch configuration: XY ~U{64..240
    step 16}, Z ~U{32..48}, nTE ~U{24..64}, TE ~U(5,12) ms, nT2 in {40,48,60},
    background (mask) fraction ~U(0.3,0.6), chi2 and none alternating."""
    out = []
    for i in range(nvol):
        X = (int(rng.choice(np.arange(64, 241, 16))), int(rng.choice(np.arange(64, 241, 16))), int(rng.integers(32, 49)))
        m, n = int(rng.integers(24, 65)), int(rng.choice([40, 48, 60]))
        TE, bg = float(rng.uniform(5e-3, 12e-3)), float(rng.uniform(0.3, 0.6))
        out.append(dict(X=X, m=m, n=n, TE=TE, bg=bg, reg="chi2" if i % 2 == 0 else "none", seed=seed + i))
    return out


def run_batch_groups(ctx, torch, specs, precision, group, steps, warmup, compare_groups):
    """The volumes in groups of `group`: each group is prepared once
    (decaes_batch_create: validation, buffers, resident bases, captured graph),
    replayed `warmup` times untimed and `steps` times timed with CUDA events on
    its stream, then released before the next group, so device memory holds
    one group at a time.  For the first `compare_groups` groups the same
    volumes are also run as one device call each (timed the same way) and the
    outputs compared.  Returns (voxels, processed voxels, batch ms per pass,
    sequential ms of the compared groups, their voxels, same outputs)."""
    import decaes_gb300 as D
    from decaes_gb300 import _lib
    L = ctx.L
    stream = torch.cuda.Stream()  # an explicit stream: the events see exactly the batch's work
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    V_tot, ms_tot, ms_seq, V_seq, same, Vp = 0, 0.0, 0.0, 0, True, 0
    for g0 in range(0, len(specs), group):
        vols, keep = [], []
        for sp in specs[g0:g0 + group]:
            mo = D.T2mapOptions(MatrixSize=sp["X"], nTE=sp["m"], TE=sp["TE"], nT2=sp["n"], T2Range=(10e-3, 2.0),
                                Reg=sp["reg"], nRefAngles=32, Chi2Factor=1.02 if sp["reg"] == "chi2" else None,
                                Threshold=THRESHOLD, precision=precision)
            po = D.T2partOptions.from_t2map(mo, SPWin=SPWIN, MPWin=MPWIN)
            img = D.mock_image(D.MockImageOptions(MatrixSize=sp["X"], nTE=sp["m"], TE=sp["TE"], BackgroundFraction=sp["bg"]),
                               seed=sp["seed"], dtype=np.float32)
            Vp += int((img[..., 0] > THRESHOLD).sum())
            d_img = torch.from_numpy(img.reshape(-1, order="F").copy()).cuda()
            V = int(np.prod(sp["X"]))
            V_tot += V
            out = {"dist": torch.empty(V * sp["n"], dtype=torch.float32, device="cuda")}
            for k in ("gdn", "ggm", "gva", "fnr", "snr", "alpha", "sfr", "sgm", "mfr", "mgm"):
                out[k] = torch.empty(V, dtype=torch.float32, device="cuda")
            mc = _lib.T2mapOutC(**{k: out[k].data_ptr() for k in ("dist", "gdn", "ggm", "gva", "fnr", "snr", "alpha")})
            pc = _lib.T2partOutC(**{k: out[k].data_ptr() for k in ("sfr", "sgm", "mfr", "mgm")})
            vols.append(_lib.VolumeC(mopts=mo.to_c(), popts=po.to_c(), has_t2part=1, dtype=_lib.F32,
                                     d_image=d_img.data_ptr(), d_b1map=None, d_mout=mc, d_pout=pc))
            keep.append((mo, po, d_img, out, mc, pc, V))
        arr = (_lib.VolumeC * len(vols))(*vols)
        b = L.decaes_batch_create(ctx.h, arr, len(vols))
        if not b:
            raise RuntimeError(L.decaes_last_error(ctx.h).decode())
        for _ in range(warmup):
            L.decaes_batch_run(b, C.c_void_p(stream.cuda_stream))
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(steps):
            L.decaes_batch_run(b, C.c_void_p(stream.cuda_stream))
        e1.record(stream)
        torch.cuda.synchronize()
        ms_tot += e0.elapsed_time(e1) / steps
        L.decaes_batch_destroy(b)
        if g0 // group < compare_groups:
            sfr_batch = [k[3]["sfr"].double().cpu().numpy() for k in keep]
            e0.record(stream)
            for mo, po, d_img, out, mc, pc, V in keep:
                ctx.check(L.decaes_t2map_t2part_device(ctx.h, C.byref(mo.to_c()), C.byref(po.to_c()),
                                                       C.c_void_p(d_img.data_ptr()), _lib.F32, None, C.byref(mc),
                                                       C.byref(pc), C.c_void_p(stream.cuda_stream)))
            e1.record(stream)
            torch.cuda.synchronize()
            ms_seq += e0.elapsed_time(e1)
            V_seq += sum(k[6] for k in keep)
            same = same and all(np.array_equal(np.nan_to_num(a, nan=-1), np.nan_to_num(k[3]["sfr"].double().cpu().numpy(), nan=-1))
                                for a, k in zip(sfr_batch, keep))
        del vols, keep, arr
        torch.cuda.empty_cache()
    return V_tot, Vp, ms_tot, ms_seq, V_seq, same


BATCH_DESC = ("volumes: XY ~U{{64..240 step 16}}, Z ~U{{32..48}} (the 64x64x32..240x240x48 range), nTE ~U{{24..64}}, "
              "TE ~U(5,12) ms, nT2 in {{40,48,60}}, mask ~U(0.3,0.6), Reg alternating chi2/none, 32 angles, Float32, "
              "T2part fused")


def run_batch_workload(args):
    """The batched uneven workload at its stated sizes: many volumes of
    different shapes, each group solved by one graph replay of a prepared
    batch (a persistent launch per occupancy class), against the same volumes
    solved one device call after another."""
    import torch
    import decaes_gb300 as D
    rng = np.random.default_rng(args.seed)
    specs = batch_volume_specs(rng, args.nvol, args.seed)
    ctx = D.Context(0, hbm_budget_bytes=200 << 30)
    clk = Clocks(0)
    with clk:
        V_tot, Vp, ms, ms_seq, V_seq, same = run_batch_groups(ctx, torch, specs, args.precision, args.group, args.steps,
                                                              args.warmup, args.compare_groups)
    line = {
        "metric": f"voxels/s, {args.nvol} uneven volumes, each group of {args.group} in one graph replay "
                  f"(a persistent launch per occupancy class)",
        "value": V_tot / (ms * 1e-3), "unit": "voxels/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else "f64+f32",
        "data": "synthetic (seeded 3-compartment EPG + Rician noise per volume)",
        "config": {"workload": f"{args.nvol} " + BATCH_DESC.replace("{{", "{").replace("}}", "}"),
                   "precision": args.precision, "voxels": V_tot, "voxels_above_threshold": Vp, "group": args.group},
        "sequential_device_calls": {"groups_compared": args.compare_groups, "voxels": V_seq,
                                    "value": V_seq / (ms_seq * 1e-3) if ms_seq else None, "ms": ms_seq,
                                    "same_outputs": bool(same)},
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)


def run_serve_workload(args):
    """The serving mix: Poisson arrivals of single slices (70%, 240x240x1, 48
    echoes), slabs (25%, 240x240x16, 48 echoes) and full volumes (5%,
    240x240x48, 56 echoes), each followed by T2part, through the library's
    continuous-batching server under a 160 GB admission budget; reports p50/p99
    submit-to-result latency and voxels/s at each arrival rate."""
    import threading as th
    import decaes_gb300 as D
    from decaes_gb300.server import Server
    rng = np.random.default_rng(args.seed)
    kinds = [("slice", (240, 240, 1), "lcurve48", 0.70), ("slab", (240, 240, 16), "lcurve48", 0.25),
             ("volume", (240, 240, 48), "gcv56", 0.05)]
    pool = {}
    for name, X, wl, _ in kinds:
        mo, po, mock = workload(X, args.precision, wl)
        pool[name] = [(D.mock_image(mock, seed=args.seed + 17 * i, dtype=np.float32), mo, po)
                      for i in range(4 if name == "slice" else 1)]
    ctx = D.Context(0)
    rates = [float(r) for r in args.rates.split(",")]
    results = []
    for rate in rates:
        srv = Server(ctx, tick_voxels=args.tick_voxels, hbm_budget_bytes=160 << 30)
        # warm the bases and the kernels
        for name in pool:
            srv.result(srv.submit(*pool[name][0]))
        srv.reset_stats()  # latency percentiles over the timed requests only
        st0 = srv.stats()
        ids, t_sub = [], []
        picks = rng.choice(len(kinds), size=args.requests, p=[k[3] for k in kinds])
        gaps = rng.exponential(1.0 / rate, size=args.requests)
        t_start = time.perf_counter()

        def submitter():
            t = time.perf_counter()
            for k, g in zip(picks, gaps):
                t += g
                dt = t - time.perf_counter()
                if dt > 0:
                    time.sleep(dt)
                name = kinds[k][0]
                img, mo, po = pool[name][int(rng.integers(len(pool[name])))]
                ids.append((srv.submit(img, mo, po), name, int(np.prod(mo.MatrixSize))))

        sub = th.Thread(target=submitter)
        with Clocks(0) as clk:
            sub.start()
            sub.join()
            for rid, _, _ in ids:
                srv.result(rid)
        wall = time.perf_counter() - t_start
        st = srv.stats()
        srv.close()
        vox = sum(v for _, _, v in ids)
        results.append({"rate_req_per_s": rate, "requests": len(ids),
                        "mix": {n: sum(1 for _, nn, _ in ids if nn == n) for n, _, _, _ in kinds},
                        "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"], "mean_ms": st["mean_ms"],
                        "max_ms": st["max_ms"], "voxels_per_s": vox / wall, "wall_s": wall,
                        "ticks": st["ticks"] - st0["ticks"], "device_busy_frac": (st["busy_ms"] - st0["busy_ms"]) / (wall * 1e3),
                        "clocks": clk.summary()})
    best = max(results, key=lambda r: r["voxels_per_s"])
    line = {
        "metric": "serving: p50/p99 latency and voxels/s, Poisson mix of slices/slabs/volumes (T2map+T2part)",
        "value": best["voxels_per_s"], "unit": "voxels/s", "n_gpus": 1, "steps": len(rates), "warmup": 1,
        "ms_per_step": best["wall_s"] * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else "f64+f32",
        "data": "synthetic (seeded 3-compartment EPG + Rician noise, 35% background)",
        "config": {"workload": "70% 240x240x1 / 25% 240x240x16 (48 echoes, nT2=40, lcurve) / 5% 240x240x48 "
                               "(56 echoes, nT2=60, GCV), Float32 host buffers, T2part fused, 160 GB admission "
                               f"budget, {args.tick_voxels} voxels per tick",
                   "precision": args.precision},
        "rates": results,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed", "mixed_tc"],
                    help="method of the headline value; with mixed the FP64 method is measured beside it")
    ap.add_argument("--no-fp64-compare", action="store_true",
                    help="skip the FP64 comparison run of the mixed headline")
    ap.add_argument("--no-tc-compare", action="store_true",
                    help="skip the run of the mixed method with tensor-core grid products beside the mixed headline")
    ap.add_argument("--workload", default="lcurve48", choices=sorted(WORKLOADS) + ["batch", "serve"],
                    help="lcurve48 (headline), gcv56, chi2k8_48, batch (uneven volumes in one launch), serve")
    ap.add_argument("--nvol", type=int, default=256, help="volumes of --workload batch")
    ap.add_argument("--group", type=int, default=32, help="volumes per prepared batch (--workload batch)")
    ap.add_argument("--compare-groups", type=int, default=1,
                    help="groups also run as one device call per volume (--workload batch)")
    ap.add_argument("--rates", default="0.5,1,2", help="arrival rates (requests/s) of --workload serve")
    ap.add_argument("--requests", type=int, default=40, help="requests per rate of --workload serve")
    ap.add_argument("--tick-voxels", type=int, default=262144, help="voxels per server tick (--workload serve)")
    ap.add_argument("--matrix", type=int, nargs=3, default=None, help="override the workload's MatrixSize")
    ap.add_argument("--compare-slices", type=int, default=None,
                    help="z-slices of the volume the FP64 comparison runs on (default: all for the 48-echo "
                         "workloads, 8 for gcv56)")
    ap.add_argument("--ref-slices", type=int, default=None,
                    help="z-slices of the volume one --impl reference step runs on")
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--cpu-sample", type=int, default=None,
                    help="above-threshold voxels the CPU oracle runs on for cpu_baseline and parity")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the bounded runs of the other configurations in the headline line")
    args = ap.parse_args()
    if args.cpu_sample is None:
        args.cpu_sample = {"lcurve48": 131072, "chi2k8_48": 131072}.get(args.workload, 16384)
    if args.impl == "reference":
        if args.workload in ("batch", "serve"):
            print(json.dumps({"impl": "reference", "unavailable": "the batched workload is this library's own "
                              "multi-volume launch; the reference runs one volume per call"}), flush=True)
            return
        return run_reference(args)
    if args.workload == "batch":
        return run_batch_workload(args)
    if args.workload == "serve":
        return run_serve_workload(args)

    import torch
    import decaes_gb300 as D
    from decaes_gb300 import _lib

    world, rank, local = replicas.rank_info()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    matrix = tuple(args.matrix) if args.matrix else WORKLOADS[args.workload]["matrix"]
    V = int(np.prod(matrix))
    mo, po, mock = workload(matrix, args.precision, args.workload)
    img = D.mock_image(mock, seed=replicas.replica_seed(args.seed, rank), dtype=np.float32)
    ctx = D.Context(local)

    # ---- headline method, device-resident ----
    run = DeviceRun(D, _lib, ctx, torch, mo, po, img, V)
    clk = Clocks(local)
    ms_per_step, launches, solve_ms = run.timed(args.steps, args.warmup, world, clk)
    Vp = run.stats()["voxels_processed"]
    value = replicas.aggregate_voxels_per_s(V, ms_per_step, world)
    head = run.host()

    # ---- end to end through the host-buffer C ABI from pinned memory ----
    mo_c, po_c = run.mo_c, run.po_c
    h_img = torch.from_numpy(img.reshape(-1, order="F").copy()).pin_memory()
    h_out = {k: torch.empty_like(v, device="cpu").pin_memory() for k, v in run.d_out.items()}
    h_parts = {k: torch.empty_like(v, device="cpu").pin_memory() for k, v in run.d_parts.items()}
    hm = _lib.T2mapOutC(*[C.c_void_p(h_out[k].data_ptr()) if k in h_out else None for k, _ in _lib.T2mapOutC._fields_])
    hp = _lib.T2partOutC(*[C.c_void_p(h_parts[k].data_ptr()) for k, _ in _lib.T2partOutC._fields_])
    del run
    torch.cuda.synchronize()
    replicas.barrier(world)
    t0 = time.perf_counter()
    k_e2e = max(1, min(args.steps, 5))
    for _ in range(k_e2e):
        ctx.check(ctx.L.decaes_t2map_t2part(ctx.h, C.byref(mo_c), C.byref(po_c), C.c_void_p(h_img.data_ptr()),
                                            _lib.F32, None, C.byref(hm), C.byref(hp)))
    e2e_s = replicas.max_over_ranks((time.perf_counter() - t0) / k_e2e, world, device="cuda")
    e2e_st = ctx.stats()  # the last call's own event timings (copies and the whole call on its stream)
    h2d = img.nbytes
    d2h = sum(v.numel() * 4 for v in h_out.values()) + sum(v.numel() * 4 for v in h_parts.values())
    del h_out, h_parts, h_img

    # ---- the mixed method with the search's grid products on the tensor cores ----
    tc = None
    if args.precision == "mixed" and not args.no_tc_compare:
        motc, potc, _ = workload(matrix, "mixed_tc", args.workload)
        runtc = DeviceRun(D, _lib, ctx, torch, motc, potc, img, V)
        ktc = max(1, min(args.steps, 3))
        ms_tc, launches_tc, solve_tc = runtc.timed(ktc, 1, world)
        st_tc = runtc.stats()
        tc = {"ms_per_step": ms_tc, "steps": ktc, "value": replicas.aggregate_voxels_per_s(V, ms_tc, world),
              "grid_products_ms": st_tc["ms_grid_products"], "grid_product_launches": st_tc["grid_product_launches"],
              "grid_product_failures": st_tc["grid_product_failures"], "host": runtc.host()}
        del runtc

    # ---- the FP64 method on the volume (or its leading slices), FP64 outputs ----
    flat = img.reshape((V, -1), order="F")
    nz = matrix[2]
    if args.workload == "gcv56":
        nz = 8
    if args.compare_slices:
        nz = args.compare_slices
    nz = max(1, min(nz, matrix[2]))
    Vs = matrix[0] * matrix[1] * nz
    fp64 = None
    ms64 = None
    if not args.no_fp64_compare:
        sub = (matrix[0], matrix[1], nz)
        img_s = np.ascontiguousarray(flat[:Vs]).reshape((*sub, -1), order="F")
        mo64, po64, _ = workload(sub, "fp64", args.workload)
        run64 = DeviceRun(D, _lib, ctx, torch, mo64, po64, img_s, Vs, f64=True)
        ms64, _, _ = run64.timed(1, 0, world)
        fp64 = run64.host()
        del run64

    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": "voxels/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f64+f32",
        "data": "synthetic (seeded 3-compartment EPG + Rician noise, 35% background)",
        "config": config_dict(matrix, V, args.workload),
        "method": args.precision,
        "voxels_above_threshold": Vp,
        "voxels_above_threshold_per_s": world * Vp / (ms_per_step * 1e-3),
        "e2e": {"value": world * V / e2e_s, "unit": "voxels/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "steps": k_e2e,
                "last_call_ms": {k: round(e2e_st[k], 2) for k in ("ms_h2d", "ms_solve", "ms_d2h", "ms_total")}},
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    pub = PUBLISHED.get(args.workload)
    if pub:
        line["published_reference"] = dict(pub, e2e_ratio=line["e2e"]["value"] / pub["value"],
                                           value_ratio=value / pub["value"])
    if ms64 is not None and args.precision == "mixed":
        hs = tuple(a[:Vs] for a in head)
        line["mixed_vs_fp64"] = {
            "fp64_value": world * Vs / (ms64 * 1e-3), "fp64_ms_per_step": ms64,
            "fp64_volume": f"{matrix[0]}x{matrix[1]}x{nz} (first {nz} of {matrix[2]} z-slices), FP64 image and outputs",
            "speedup_vs_fp64": (world * V / (ms_per_step * 1e-3)) / (world * Vs / (ms64 * 1e-3)),
            "errors": method_errors(*hs, *fp64, tail=32),
            "gate": "MWF |mixed - FP64| p99 <= 1e-3 over every processed voxel of the compared volume",
        }
        e = line["mixed_vs_fp64"]["errors"]
        line["mixed_vs_fp64"]["gate_met"] = bool(e["mwf_abs"]["p99"] <= 1e-3 and e["same_processed_voxels"])

    if tc is not None:
        # the grid-product GEMM's work: 2 x 10 slice-pair products x K*nT2 x nTE per voxel
        w_ = WORKLOADS[args.workload]
        gemm_flops = 2.0 * 10 * w_["K"] * w_["nT2"] * (-(-w_["nTE"] // 16) * 16) * Vp
        gemm_bytes = (w_["K"] * w_["nT2"] * 8.0 + 4.0 + 4.0 * w_["nTE"]) * Vp
        line["tensor_core_grid_products"] = {
            "method": "mixed_tc: the search's A_k'b for every grid angle from one tcgen05 GEMM per 2^19 voxels "
                      "(4 bf16 fixed-point slices per operand, exact FP32 accumulation, float-pair products), "
                      "read by the voxel kernel",
            "value": tc["value"], "ms_per_step": tc["ms_per_step"], "steps": tc["steps"],
            "speedup_vs_mixed": ms_per_step / tc["ms_per_step"],
            "gemm_ms_per_step": tc["grid_products_ms"], "gemm_launches": tc["grid_product_launches"],
            "gemm_failures": tc["grid_product_failures"],
            "gemm_tflops": gemm_flops / (tc["grid_products_ms"] * 1e-3) / 1e12 if tc["grid_products_ms"] else None,
            "gemm_gbs": gemm_bytes / (tc["grid_products_ms"] * 1e-3) / 1e9 if tc["grid_products_ms"] else None,
            "gemm_work": "2 x 10 slice-pair products x K*nT2 x nTE(padded to 16) per above-threshold voxel; "
                         "bytes = K*nT2 float-pair products + exponent + the FP32 echo train per voxel",
        }
        if fp64 is not None:
            line["tensor_core_grid_products"]["errors_vs_fp64"] = method_errors(
                *(a[:Vs] for a in tc["host"]), *fp64)

    # ---- the oracle on a sample: CPU baseline and parity at this scale ----
    peak = fp64_peak_tflops(torch)
    kern_ms = statistics.median(solve_ms)
    cb = None
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        # the sample is drawn from the voxels the FP64 comparison covers
        Vp_s = int((flat[:Vs, 0] > THRESHOLD).sum())
        cb = cpu_baseline(args.workload, flat[:Vs], Vp_s, args.cpu_sample, threads)
        line["cpu_baseline"] = {"value": cb["value"], "unit": "voxels/s", "cores": threads, "kind": "port",
                                "per_core": cb["value"] / threads,
                                "sample": f"{len(cb['pick'])} above-threshold voxels of the same image "
                                          f"({cb['seconds']:.1f} s, FP64 restatement of the reference path); "
                                          f"time per voxel scaled to the whole volume"}
        pk = cb["pick"]
        o_d, o_a, o_s = cb["dist"], cb["maps"]["alpha"], cb["parts"]["sfr"]
        par = {"sample_voxels": int(len(pk)), "oracle": "FP64 C restatement of the reference path (oracle/)"}
        if fp64 is not None:
            d64, a64, s64 = (x[pk] for x in fp64)
            e64 = method_errors(d64, a64, s64, o_d, o_a, o_s)
            par["fp64_vs_oracle"] = {
                "bitwise_frac": bitwise_frac(d64, a64, s64, o_d, o_a, o_s), **e64,
                "gate": "per-bin relative <= 1e-8 and |MWF| <= 1e-10",
                "gate_met": bool(e64["dist_bin_rel"]["max"] <= 1e-8 and e64["mwf_abs"]["max"] <= 1e-10
                                 and e64["same_processed_voxels"])}
        if args.precision in ("mixed", "mixed_tc"):
            dm, am, sm = (x[pk] for x in head)
            em = method_errors(dm, am, sm, o_d, o_a, o_s)
            par["mixed_vs_oracle"] = {**em, "gate": "MWF |mixed - oracle| p99 <= 1e-3",
                                      "gate_met": bool(em["mwf_abs"]["p99"] <= 1e-3 and em["same_processed_voxels"])}
        if tc is not None:
            dm, am, sm = (x[pk] for x in tc["host"])
            em = method_errors(dm, am, sm, o_d, o_a, o_s)
            par["mixed_tc_vs_oracle"] = {**em, "gate": "MWF |mixed_tc - oracle| p99 <= 1e-3",
                                         "gate_met": bool(em["mwf_abs"]["p99"] <= 1e-3 and em["same_processed_voxels"])}
        line["parity"] = par
    if args.precision == "fp64":
        if cb is not None:
            achieved = cb["flops_per_voxel"] * Vp / (kern_ms * 1e-3) / 1e12
            tpv = profile_figure(f"k_voxels_fp64_{args.workload}.md", "dram_bytes_per_voxel")  # ncu on a small slab
            line["roofline"] = {"kernel": "k_voxels_plain (FP64 method)", "bound": "fp64", "achieved": achieved,
                                "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                                "traffic": None if tpv is None else tpv * Vp,
                                "work": f"{cb['flops_per_voxel'] / 1e6:.3f} MFLOP FP64 per above-threshold voxel "
                                        f"(the reference algorithm, counted by the oracle) x {Vp} voxels",
                                "kernel_ms": kern_ms,
                                "peak_source": "cuBLAS DGEMM (torch.matmul float64 4096^3) measured in this run"}
    else:
        fpv = profile_figure(f"k_voxels_mixed_{args.workload}.md", "fp64_flops_per_voxel")
        tpv = profile_figure(f"k_voxels_mixed_{args.workload}.md", "dram_bytes_per_voxel")
        if fpv is not None:
            achieved = fpv * Vp / (kern_ms * 1e-3) / 1e12
            line["roofline"] = {"kernel": "k_voxels_mixed (mixed method)", "bound": "fp64", "achieved": achieved,
                                "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                                "traffic": None if tpv is None else tpv * Vp,
                                "work": f"{fpv / 1e6:.3f} MFLOP FP64 per above-threshold voxel (executed by the "
                                        f"mixed method, ncu thread-instruction counts, FMA = 2) x {Vp} voxels",
                                "kernel_ms": kern_ms,
                                "peak_source": "cuBLAS DGEMM (torch.matmul float64 4096^3) measured in this run"}
            if cb is not None:
                alg = cb["flops_per_voxel"] * Vp / (kern_ms * 1e-3) / 1e12
                line["roofline"]["reference_algorithm_view"] = {
                    "achieved": alg, "frac": alg / peak, "unit": "TFLOP/s",
                    "work": f"{cb['flops_per_voxel'] / 1e6:.3f} MFLOP FP64 per voxel: the reference algorithm's "
                            f"operations (oracle-counted), which the mixed method replaces by fewer"}
    if "roofline" in line:
        line["roofline"]["hbm_view"] = hbm_view(mo, Vp, V, kern_ms)
        method = "fp64" if args.precision == "fp64" else "mixed"
        ipv = profile_figure(f"k_voxels_{method}_{args.workload}.md", "fp64_warp_instructions_per_voxel")
        if ipv is not None:
            line["roofline"]["fp64_pipe_view"] = fp64_pipe_view(torch, ipv, Vp, kern_ms, clk.summary())
    if args.workload == "lcurve48" and args.precision == "mixed" and not args.no_extra and world == 1:
        line["other_configurations"] = other_configurations(args, D, _lib, ctx, torch)
    print(json.dumps(line), flush=True)


def other_configurations(args, D, _lib, ctx, torch):
    """Bounded runs of the other single-GPU configurations beside the headline:
    the 56-echo GCV volume's settings on a slab of it (mixed method; FP64 on
    its first slice for the per-output errors), and a sample of the uneven
    batch at its stated sizes (one graph replay against one device call per
    volume)."""
    out = {}
    nz = 8
    wl = WORKLOADS["gcv56"]
    matrix = (wl["matrix"][0], wl["matrix"][1], nz)
    V = int(np.prod(matrix))
    mo, po, mock = workload(matrix, "mixed", "gcv56")
    img = D.mock_image(mock, seed=args.seed, dtype=np.float32)
    run = DeviceRun(D, _lib, ctx, torch, mo, po, img, V)
    ms, _, _ = run.timed(2, 1, 1)
    Vp = run.stats()["voxels_processed"]
    head = run.host()
    del run
    Vs = matrix[0] * matrix[1]
    sub = (matrix[0], matrix[1], 1)
    mo64, po64, _ = workload(sub, "fp64", "gcv56")
    img_s = np.ascontiguousarray(img.reshape((V, -1), order="F")[:Vs]).reshape((*sub, -1), order="F")
    run64 = DeviceRun(D, _lib, ctx, torch, mo64, po64, img_s, Vs, f64=True)
    ms64, _, _ = run64.timed(1, 0, 1)
    fp64 = run64.host()
    del run64
    out["gcv56_slab"] = {
        "workload": config_dict(matrix, V, "gcv56")["workload"] + f" (the first {nz} of 113 z-slices)",
        "value": V / (ms * 1e-3), "unit": "voxels/s", "ms_per_step": ms, "steps": 2, "voxels_above_threshold": Vp,
        "fp64_value": Vs / (ms64 * 1e-3), "fp64_volume": f"{sub[0]}x{sub[1]}x1 (first z-slice), FP64 image and outputs",
        "speedup_vs_fp64": (V / (ms * 1e-3)) / (Vs / (ms64 * 1e-3)),
        "errors_vs_fp64": method_errors(*(a[:Vs] for a in head), *fp64),
    }
    nvol = 16
    specs = batch_volume_specs(np.random.default_rng(args.seed + 1), nvol, args.seed + 1000)
    V_tot, Vp_b, ms_b, ms_seq, V_seq, same = run_batch_groups(ctx, torch, specs, "mixed", nvol, 1, 0, 1)
    out["batch"] = {
        "workload": f"{nvol} " + BATCH_DESC.replace("{{", "{").replace("}}", "}") + " (mixed method)",
        "value": V_tot / (ms_b * 1e-3), "unit": "voxels/s", "ms_per_step": ms_b, "steps": 1, "warmup": 0,
        "voxels": V_tot, "voxels_above_threshold": Vp_b,
        "sequential_device_calls": {"value": V_seq / (ms_seq * 1e-3), "ms": ms_seq, "speedup_of_batch": ms_seq / ms_b,
                                    "same_outputs": bool(same)},
    }
    return out


def hbm_view(mo, Vp, V, kern_ms):
    """The same kernel against HBM: the bytes it must move (the FP32 echo
    train of every voxel for the threshold test and of each processed voxel
    for its solve, its FP64 distribution, six maps and four T2 parts) over the
    launch time, against the measured HBM copy bandwidth.  It shows how far
    from HBM-bound the path is; the FP64 view above is the binding one."""
    bytes_ = 4.0 * V + 4.0 * mo.nTE * Vp + 8.0 * (mo.nT2 + 10) * Vp
    achieved = bytes_ / (kern_ms * 1e-3) / 1e9
    peak, src = None, None
    try:
        with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "MEASURED_PEAKS.json")) as f:
            peak, src = float(json.load(f)["hbm_gbs"]), "MEASURED_PEAKS.json hbm_gbs (measured copy bandwidth)"
    except (OSError, ValueError, KeyError):
        peak, src = 6800.0, "fallback 6.8 TB/s"
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "algorithmic_bytes_per_step": bytes_, "peak_source": src}


if __name__ == "__main__":
    main()
