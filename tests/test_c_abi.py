"""The C ABI from a plain C program (tests/abi_client.c), compiled against
include/decaes_gpu.h as C99 and as C++ and linked to libdecaes_gpu.so: the
header is usable from both languages, the option checks return the
reference's assertion texts, and the synthetic generator gives the same bytes
as through Python ctypes.  Entry points that need no GPU only."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("lang", ["c", "c++"])
def test_c_client(D, tmp_path, lang):
    D.load()
    from decaes_gb300 import _lib
    so = _lib.lib_path()
    cc = shutil.which("gcc" if lang == "c" else "g++")
    if cc is None:
        pytest.skip(f"no {lang} compiler")
    exe = tmp_path / "abi_client"
    std = ["-std=c99"] if lang == "c" else ["-x", "c++", "-std=c++17"]
    # "-x none" ends the language override before the shared library operand
    subprocess.run(["timeout", "120", cc, *std, "-Wall", "-Wextra", "-Werror", "-O1",
                    "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "abi_client.c"),
                    "-x", "none", "-o", str(exe), so, "-Wl,-rpath," + os.path.dirname(so), "-lm"], check=True)
    out = subprocess.run([str(exe), str(tmp_path / "img.bin")], check=True, capture_output=True, text=True,
                         timeout=60).stdout
    lines = dict(line.split(" ", 1) for line in out.strip().splitlines())
    assert lines["t2map_valid"] == "0"
    assert lines["t2map_invalid"] == "1 Chi2Factor must be greater than 1.0, but Chi2Factor = 0.5."
    assert lines["t2part_valid"] == "0"
    assert lines["t2part_invalid"] == "1 SPWin[1] < SPWin[2]"
    assert lines["mock"] == "0"
    img_c = np.fromfile(tmp_path / "img.bin", dtype=np.float64).reshape((4, 3, 2, 32), order="F")
    img_py = D.mock_image(D.MockImageOptions(MatrixSize=(4, 3, 2), nTE=32, TE=10e-3), seed=11, nthreads=2)
    np.testing.assert_array_equal(img_c, img_py)
