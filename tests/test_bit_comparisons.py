"""The voxel kernels decide several FP64 comparisons on bit patterns (integer
pipes) instead of the FP64 pipe: Julia's max/min (jmax/jmin,
csrc/nnls_warp.cuh), isapprox with rtol = sqrt(eps) (csrc/t2map_device.cuh),
the argument tests of the portable exp/log (csrc/pmath.h) and the solver's
ordering, positivity and pivot tests (okey, pos_bits, gt_nonneg_bits).  This restates
each bit-pattern rule in Python and checks it against the FP64 comparison it
replaces, over special values (signed zeros, infinities, NaN, subnormals, the
range limits) and random values at and around the tolerances.  The GPU's
subtraction returns a NaN with the sign bit clear (the canonical NaN), which the
old jmax/jmin inherited through signbit(x - y); the rules keep x there as well."""
import itertools
import math
import struct

import numpy as np
import pytest

M = 0x7FFFFFFFFFFFFFFF
INF = 0x7FF0000000000000


def bits(d):
    return struct.unpack("<q", struct.pack("<d", d))[0]


def ubits(d):
    return bits(d) & 0xFFFFFFFFFFFFFFFF


def dbl(i):
    return struct.unpack("<d", struct.pack("<q", i))[0]


def same(a, c):
    return (math.isnan(a) and math.isnan(c)) or bits(a) == bits(c)


# ---- the FP64 forms the kernels used before ---------------------------------
def signbit_gpu(v):
    return False if math.isnan(v) else math.copysign(1.0, v) < 0


def jmax_fp(x, y):
    if math.isnan(x) or math.isnan(y):
        return float("nan")
    return y if signbit_gpu(x - y) else x


def jmin_fp(x, y):
    if math.isnan(x) or math.isnan(y):
        return float("nan")
    return x if signbit_gpu(x - y) else y


def isapprox_fp(x, y):
    if x == y:
        return True
    if not (math.isfinite(x) and math.isfinite(y)):
        return False
    return abs(x - y) <= jmax_fp(0.0, 1.4901161193847656e-08 * jmax_fp(abs(x), abs(y)))


# ---- the bit-pattern forms (same logic as the CUDA code) ---------------------
def tkey(d):
    b = bits(d)
    return b if b >= 0 else b ^ M


def isnan_bits(d):
    return (bits(d) & M) > INF


def jmax_bits(x, y):
    if isnan_bits(x) or isnan_bits(y):
        return float("nan")
    return y if tkey(x) < tkey(y) else x


def jmin_bits(x, y):
    if isnan_bits(x) or isnan_bits(y):
        return float("nan")
    return x if tkey(x) < tkey(y) else y


def isapprox_bits(x, y):
    bx, by = bits(x), bits(y)
    ax, ay = bx & M, by & M
    if (bx == by and ax <= INF) or (ax | ay) == 0:
        return True
    if ax >= INF or ay >= INF:
        return False
    tol = 1.4901161193847656e-08 * dbl(ay if ax < ay else ax)
    return (bits(x - y) & M) <= bits(tol)


def exp_case_fp(x):
    if x != x:
        return "nan"
    if x > 709.782712893384:
        return "inf"
    if x < -745.1332191019412:
        return "zero"
    return "poly"


def exp_case_bits(x):
    u = ubits(x)
    if (u & M) > INF:
        return "nan"
    if not (u >> 63) and u > 0x40862E42FEFA39EF:
        return "inf"
    if (u >> 63) and (u & M) > 0x40874910D52D3052:
        return "zero"
    return "poly"


def log_case_fp(x):
    if x != x:
        return "nan"
    if x < 0:
        return "neg"
    if x == 0:
        return "zero"
    if x == float("inf"):
        return "inf"
    return "poly"


def log_case_bits(x):
    u = ubits(x)
    if (u & M) > INF:
        return "nan"
    if (u & M) == 0:
        return "zero"
    if u >> 63:
        return "neg"
    if u == INF:
        return "inf"
    return "poly"


SPECIAL = [0.0, -0.0, float("inf"), float("-inf"), float("nan"), 5e-324, -5e-324, 2.2250738585072014e-308, 1.0, -1.0,
           1.0 + 2.0 ** -52, 1.0 + 1.49e-8, 1.0 + 1.5e-8, -1.0 - 1.49e-8, 709.782712893384, -745.1332191019412,
           1e308, -1e308]


@pytest.fixture(scope="module")
def values():
    rng = np.random.default_rng(0)
    vals = SPECIAL + [float(v) for v in rng.standard_normal(120) * 10.0 ** rng.integers(-10, 10, 120)]
    vals += [v * (1 + d) for v in vals[len(SPECIAL):len(SPECIAL) + 30]
             for d in (1.4901161193847656e-08, 1.49e-8, 1.5e-8, -1.49e-8, 2.0 ** -52)]
    return vals


def test_jmax_jmin_isapprox_match_fp64(values):
    for x, y in itertools.product(values, repeat=2):
        assert same(jmax_fp(x, y), jmax_bits(x, y)), (x, y)
        assert same(jmin_fp(x, y), jmin_bits(x, y)), (x, y)
        assert isapprox_fp(x, y) == isapprox_bits(x, y), (x, y)


def test_exp_log_argument_tests_match_fp64(values):
    edges = [709.782712893384, math.nextafter(709.782712893384, 1e9), math.nextafter(709.782712893384, 0.0),
             -745.1332191019412, math.nextafter(-745.1332191019412, -1e9), math.nextafter(-745.1332191019412, 0.0)]
    for x in values + edges:
        assert exp_case_fp(x) == exp_case_bits(x), x
        assert log_case_fp(x) == log_case_bits(x), x


def test_log_mantissa_split_matches_fp64():
    s2 = 1.4142135623730951
    fs = [1.0 + k / 4096.0 for k in range(4096)] + [s2, math.nextafter(s2, 2.0), math.nextafter(s2, 0.0)]
    for f in fs:
        assert (f > s2) == (ubits(f) > 0x3FF6A09E667F3BCD), f


# ---- the solver's earlier helpers (csrc/nnls_warp.cuh) -------------------------
def okey(d):
    b = bits(d)
    if (b << 1) & 0xFFFFFFFFFFFFFFFF == 0:
        return 0
    return b if b >= 0 else b ^ M


def pos_bits(d):
    b = bits(d)
    return 0 < b <= INF


def gt_nonneg_bits(d, t):
    b = bits(d)
    return b > bits(t) and b <= INF and not isnan_bits(t)


def test_solver_helpers_match_fp64(values):
    finite_or_inf = [v for v in values if not math.isnan(v)]
    for d in values:
        assert pos_bits(d) == (d > 0), d
    for a, c in itertools.product(finite_or_inf, repeat=2):
        assert (okey(a) < okey(c)) == (a < c), (a, c)
    thresholds = [t for t in values if math.isnan(t) or bits(t) >= 0]  # sign bit clear, as the solver's are
    for d, t in itertools.product(values, thresholds):
        assert gt_nonneg_bits(d, t) == (d > t), (d, t)
