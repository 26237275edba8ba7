"""The oracle's copy of the synthetic benchmark generator makes exactly the
bytes of the library's decaes_mock_image (so the CPU baseline builds its input
without loading libdecaes_gpu), and a leading z-slab equals the first slices
of the whole volume (so a bounded CPU sample sees the same voxels)."""
import numpy as np
import pytest


@pytest.mark.parametrize("X,m,bg,dtype,seed", [
    ((7, 5, 3), 48, 0.35, np.float32, 2024),
    ((4, 4, 2), 32, 0.0, np.float64, 3),
    ((3, 2, 2), 56, 0.5, np.float64, 11),
])
def test_oracle_mock_image_matches_library(D, orc, X, m, bg, dtype, seed):
    lib_img = D.mock_image(D.MockImageOptions(MatrixSize=X, nTE=m, TE=7e-3, BackgroundFraction=bg), seed=seed,
                           dtype=dtype)
    orc_img = orc.mock_image(X, m, seed=seed, dtype=dtype, TE=7e-3, BackgroundFraction=bg, nthreads=3)
    assert orc_img.dtype == lib_img.dtype and orc_img.shape == lib_img.shape
    np.testing.assert_array_equal(orc_img.reshape(-1, order="F").view(np.uint8), lib_img.reshape(-1, order="F").view(np.uint8))


def test_leading_slab_is_the_first_slices(orc):
    whole = orc.mock_image((6, 5, 4), 32, seed=9, dtype=np.float32, BackgroundFraction=0.35)
    slab = orc.mock_image((6, 5, 2), 32, seed=9, dtype=np.float32, BackgroundFraction=0.35)
    np.testing.assert_array_equal(slab, whole[:, :, :2, :])
