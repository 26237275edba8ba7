"""The tensor-core grid-product kernel (decaes.jl_gb300/csrc/decaes_tc.cu) on
its own: tests/tc_kernel_check.cu is compiled with nvcc for sm_103a together
with the kernel's source and compares every product with an exact CPU sum
(within 2e-9 of the sum of the absolute terms) for 4..128 echoes, FP32 and
FP64 images and an uneven voxel list."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "decaes.jl_gb300", "csrc")

pytestmark = pytest.mark.gpu


def test_grid_products_exact(ctx, tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = tmp_path / "tc_kernel_check"
    subprocess.run(["timeout", "300", nvcc, "-O2", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a",
                    "-I", CSRC, "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "tc_kernel_check.cu"),
                    os.path.join(CSRC, "decaes_tc.cu"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    print(r.stdout)
    assert r.returncode == 0 and r.stdout.strip().endswith("PASS"), r.stdout + r.stderr
