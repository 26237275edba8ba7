"""The C ABI library on the CPU: it loads, exports every symbol the header
declares, validates options with the reference's assertion messages, and the
synthetic generator is deterministic.  No GPU calls."""
import ctypes as C
import math
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "decaes_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(decaes_[a-z0-9_]+)\s*\(", src)))


def test_exports_every_declared_symbol(D):
    L = D.load()
    names = declared_symbols()
    assert len(names) >= 12
    for name in names:
        assert hasattr(L, name), f"libdecaes_gpu.so does not export {name}"
    from decaes_gb300 import _lib
    assert sorted(_lib.EXPORTS) == names


def base(**kw):
    d = dict(MatrixSize=(2, 2, 2), nTE=32, TE=10e-3, nT2=40, T2Range=(10e-3, 2.0), Reg="lcurve")
    d.update(kw)
    return d


@pytest.mark.parametrize("kw,msg", [
    (dict(nTE=3), "At least four echoes are required for T2 mapping, but nTE = 3."),
    (dict(TE=-1e-5), "Echo spacing must be positive, but TE = -1.0e-5."),
    (dict(nT2=1), "At least two T2 components are required for T2 mapping, but nT2 = 1."),
    (dict(T2Range=(2.0, 0.01)), "T2Range must a sorted 2-tuple of positive values, but T2Range = (2.0, 0.01)."),
    (dict(T1=0.0), "T1 must be positive, but T1 = 0.0."),
    (dict(Threshold=-1.0), "First echo signal threshold must be non-negative or -Inf to force processing of every voxel, but Threshold = -1.0."),
    (dict(MinRefAngle=190.0), "Minimum refocusing angle must be in the range [0, 180], but MinRefAngle = 190.0."),
    (dict(nRefAngles=1, nRefAnglesMin=2), "Maximum number of angles to check during flip angle optimization must be at least 2, but nRefAngles = 1."),
    (dict(nRefAngles=8, nRefAnglesMin=9), "Minimum number of angles to check during flip angle optimization must be in the range [2, nRefAngles], but nRefAngles = 8 and nRefAnglesMin = 9."),
    (dict(Reg="chi2"), "Chi2Factor must be greater than 1.0, but Chi2Factor = nothing."),
    (dict(Reg="chi2", Chi2Factor=0.5), "Chi2Factor must be greater than 1.0, but Chi2Factor = 0.5."),
    (dict(Reg="mdp"), "Noise level must be positive, but NoiseLevel = nothing."),
    (dict(RefConAngle=-1.0), "Refocusing control angle must be in the range [0, 180], but RefConAngle = -1.0."),
    (dict(SetFlipAngle=200.0), "Fixed flip angle must be in the range [0, 180], but SetFlipAngle = 200.0."),
    (dict(Reg="tikh"), 'Reg ∈ ("none", "lcurve", "gcv", "chi2", "mdp")'),
    (dict(MatrixSize=(0, 2, 2)), "MatrixSize must be a tuple of 3 positive integers, but MatrixSize = (0, 2, 2)."),
])
def test_t2map_option_messages(D, kw, msg):
    with pytest.raises(AssertionError) as e:
        D.T2mapOptions(**base(**kw))
    assert str(e.value) == msg


def test_option_defaults(D):
    o = D.T2mapOptions(**base())
    assert o.nRefAngles == 64 and o.nRefAnglesMin == 5 and o.MinRefAngle == 50.0 and o.T1 == 1.0
    assert o.RefConAngle == 180.0 and o.Threshold == 0.0 and o.SetFlipAngle is None
    o = D.T2mapOptions(**base(nRefAngles=3))
    assert o.nRefAnglesMin == 3
    p = D.T2partOptions.from_t2map(o, SPWin=(10e-3, 25e-3), MPWin=(25e-3, 200e-3))
    assert p.MatrixSize == o.MatrixSize and p.nT2 == o.nT2 and p.T2Range == o.T2Range and p.Sigmoid is None


def test_legacy_accepted(D):
    """legacy = true is validated like any other option set (src/types.jl:59-63 defaults)."""
    o = D.T2mapOptions(**base(legacy=True))
    assert o.legacy and o.nRefAngles == 8 and o.nRefAnglesMin == 8
    p = D.T2partOptions.from_t2map(o, SPWin=(10e-3, 25e-3), MPWin=(25e-3, 200e-3))
    assert p.legacy


@pytest.mark.parametrize("kw,msg", [
    (dict(nT2=1), "nT2 >= 2"),
    (dict(SPWin=(0.03, 0.01)), "SPWin[1] < SPWin[2]"),
    (dict(MPWin=(0.3, 0.01)), "MPWin[1] < MPWin[2]"),
    (dict(Sigmoid=-1.0), "Sigmoid === nothing || Sigmoid > 0"),
    (dict(T2Range=(0.0, 2.0)), "0.0 < T2Range[1] < T2Range[2]"),
])
def test_t2part_option_messages(D, kw, msg):
    d = dict(MatrixSize=(2, 2, 2), nT2=40, T2Range=(10e-3, 2.0), SPWin=(10e-3, 25e-3), MPWin=(25e-3, 200e-3))
    d.update(kw)
    with pytest.raises(AssertionError) as e:
        D.T2partOptions(**d)
    assert str(e.value) == msg


def test_mock_image_deterministic(D):
    mo = D.MockImageOptions(MatrixSize=(5, 4, 3), nTE=24, BackgroundFraction=0.3)
    a = D.mock_image(mo, seed=9, nthreads=1)
    b = D.mock_image(mo, seed=9, nthreads=7)
    c = D.mock_image(mo, seed=10, nthreads=3)
    np.testing.assert_array_equal(a, b)
    assert not np.array_equal(a, c)
    assert a.shape == (5, 4, 3, 24) and np.all(a >= 0)
    f = D.mock_image(mo, seed=9, dtype=np.float32)
    np.testing.assert_allclose(f, a, rtol=1e-6)


def test_mock_image_signal(D, orc):
    """Noise-free voxels equal the three-compartment EPG mixture of the oracle."""
    mo = D.MockImageOptions(MatrixSize=(3, 1, 1), nTE=32, SNRRange=(1e300, 1e300), CSFFracRange=(0.0, 0.0),
                            MyelinFracRange=(0.0, 0.0), IET2Range=(0.07, 0.07), FlipAngleRange=(160.0, 160.0),
                            AmplitudeRange=(1000.0, 1000.0))
    img = D.mock_image(mo, seed=1)
    want = 1000.0 * orc.epg_decay_curve(32, 160.0, 10e-3, 0.07, 1.0)
    for v in range(3):
        np.testing.assert_allclose(img[v, 0, 0], want, rtol=1e-14)


def test_no_gpu_needed_for_validation(D):
    # validation and generation run without touching CUDA
    L = D.load()
    msg = C.create_string_buffer(256)
    o = D.T2mapOptions(**base()).to_c()
    assert L.decaes_t2map_check_options(C.byref(o), msg, 256) == 0
    assert msg.value == b""
