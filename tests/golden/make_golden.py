"""Writes the regression fixtures of tests/golden/ (run from the repository
root: python tests/golden/make_golden.py [names...]).

The reference is a Julia package and Julia is not available, so no outputs of
the reference itself exist here; these fixtures are the oracle's outputs
(oracle/, the FP64 restatement of the reference path) on small seeded inputs,
stored with their inputs.  tests/test_golden.py checks that the oracle still
reproduces them bit for bit (CPU) and that the CUDA path does (GPU)."""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "decaes.jl_gb300"))

SPWIN, MPWIN = (10e-3, 25e-3), (25e-3, 200e-3)
# name: (matrix, nTE, TE, nT2, T2Range, Reg, nRefAngles, extra options)
CASES = {
    "chi2_32echo": ((4, 4, 1), 32, 10e-3, 40, (10e-3, 2.0), "chi2", 8, dict(Chi2Factor=1.02)),
    "lcurve_48echo": ((4, 3, 1), 48, 10e-3, 40, (10e-3, 2.0), "lcurve", 32, {}),
    "gcv_56echo": ((3, 3, 1), 56, 7e-3, 60, (8e-3, 2.0), "gcv", 64, {}),
    "none_refcon150": ((3, 3, 1), 32, 10e-3, 40, (10e-3, 2.0), "none", 16, dict(RefConAngle=150.0)),
    "mdp_fixed_angle": ((3, 3, 1), 48, 10e-3, 40, (10e-3, 2.0), "mdp", 16, dict(NoiseLevel=2.0, SetFlipAngle=165.0)),
    "legacy_chi2": ((3, 3, 1), 32, 10e-3, 40, (15e-3, 2.0), "chi2", 8, dict(Chi2Factor=1.02, legacy=True)),
    # the 13 voxels of the 240x240x48 benchmark volume (48 echoes, lcurve, 32
    # angles; generator seed 2024, 35% background) whose MWF moves by more
    # than 1e-3 between the FP64 and the mixed method: their L-curves have
    # several curvature maxima of nearly equal height
    "lcurve48_tail": ((13, 1, 1), 48, 10e-3, 40, (10e-3, 2.0), "lcurve", 32, {}),
}
# voxel indices of lcurve48_tail in the benchmark volume
TAIL_VOXELS = [1293523, 1137770, 1310933, 1268993, 1347605, 1549362, 1453575, 2010477, 1858108, 1909129, 2752530,
               2394425, 1040029]


def tail_image():
    """The benchmark volume's tail voxels as a 13 x 1 x 1 image (Float32
    values of the benchmark input, widened)."""
    import decaes_gb300 as D
    img = D.mock_image(D.MockImageOptions(MatrixSize=(240, 240, 48), nTE=48, TE=10e-3, BackgroundFraction=0.35),
                       seed=2024, dtype=np.float32)
    flat = img.reshape((-1, 48), order="F")
    return flat[TAIL_VOXELS].astype(np.float64).reshape((len(TAIL_VOXELS), 1, 1, 48), order="F")


def options(orc, name):
    X, m, TE, n, T2, reg, K, extra = CASES[name]
    kw = dict(MatrixSize=X, nTE=m, TE=TE, nT2=n, T2Range=T2, Reg=reg, nRefAngles=K, SaveRegParam=True,
              SaveResidualNorm=True)
    kw.update(extra)
    if kw.get("legacy"):
        kw["nRefAnglesMin"] = K
    return orc.T2mapOptions(**kw), orc.T2partOptions(MatrixSize=X, nT2=n, T2Range=T2, SPWin=SPWIN, MPWin=MPWIN)


def main():
    import oracle as orc
    import decaes_gb300 as D
    orc.build()
    only = sys.argv[1:]
    for i, name in enumerate(CASES):
        if only and name not in only:
            continue
        X, m, TE = CASES[name][:3]
        if name == "lcurve48_tail":
            img = tail_image()
        else:
            img = D.mock_image(D.MockImageOptions(MatrixSize=X, nTE=m, TE=TE), seed=100 + i)
        mo, po = options(orc, name)
        maps, dist = orc.t2map(img, mo, nthreads=4)
        parts = orc.t2part(dist, po)
        out = {"image": np.asarray(img, dtype=np.float64), "dist": dist}
        out.update({"map_" + k: v for k, v in maps.items()})
        out.update({"part_" + k: v for k, v in parts.items()})
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print(name, {k: v.shape for k, v in out.items() if hasattr(v, "shape")})


if __name__ == "__main__":
    main()
