"""The per-voxel figures bench.py reads from the committed ncu summaries parse
to the values the summaries state, and the FP64-pipe roofline view is the
instruction rate over 4 x SMs x clock / 64 (no GPU: a stand-in device)."""
import os
import sys
import types

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


@pytest.mark.parametrize("name,key", [
    ("k_voxels_mixed_lcurve48.md", "fp64_flops_per_voxel"),
    ("k_voxels_mixed_lcurve48.md", "fp64_warp_instructions_per_voxel"),
    ("k_voxels_mixed_lcurve48.md", "dram_bytes_per_voxel"),
    ("k_voxels_fp64_lcurve48.md", "dram_bytes_per_voxel"),
])
def test_profile_figures_parse(name, key):
    v = bench.profile_figure(name, key)
    assert v is not None and v > 0
    # exactly one definition line per figure, so the bench cannot pick up a stale one
    lines = [l for l in open(os.path.join(ROOT, "profiles", name)) if l.startswith(key + ":")]
    assert len(lines) == 1


def test_missing_figure_is_none():
    assert bench.profile_figure("k_voxels_mixed_lcurve48.md", "no_such_figure") is None
    assert bench.profile_figure("no_such_profile.md", "fp64_flops_per_voxel") is None


def _device(sms):
    props = types.SimpleNamespace(multi_processor_count=sms)
    return types.SimpleNamespace(cuda=types.SimpleNamespace(get_device_properties=lambda i: props))


def test_fp64_pipe_view_arithmetic():
    v = bench.fp64_pipe_view(_device(152), 32000, 2_000_000, 4000.0, {"sm_mhz": 2000.0, "sm_max_mhz": 2070.0})
    assert v["achieved"] == pytest.approx(32000 * 2_000_000 / 4.0 / 1e9)
    assert v["peak"] == pytest.approx(4 * 152 * 2000e6 / 64 / 1e9)
    assert v["frac"] == pytest.approx(v["achieved"] / v["peak"])
    assert v["bound"] == "fp64"


def test_fp64_pipe_view_uses_max_clock_when_median_missing():
    v = bench.fp64_pipe_view(_device(152), 1, 1, 1.0, {"sm_mhz": None, "sm_max_mhz": 2070.0})
    assert v["peak"] == pytest.approx(4 * 152 * 2070e6 / 64 / 1e9)
    assert bench.fp64_pipe_view(_device(152), 1, 1, 1.0, {"sm_mhz": None, "sm_max_mhz": None}) is None
