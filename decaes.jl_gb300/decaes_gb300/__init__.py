"""decaes_gb300: GB300 (sm_103a) implementation of DECAES.jl's voxelwise
T2-distribution path (T2mapSEcorr + T2partSEcorr) behind a C ABI
(include/decaes_gpu.h), with a Python mirror of the reference API."""
from .api import (MockImageOptions, T2mapOptions, T2mapSEcorr, T2mapSEcorr_T2partSEcorr, T2partOptions, T2partSEcorr,
                  mock_image)
from ._lib import Context, default_context, load

__all__ = ["T2mapOptions", "T2partOptions", "T2mapSEcorr", "T2partSEcorr", "T2mapSEcorr_T2partSEcorr", "mock_image",
           "MockImageOptions", "Context", "default_context", "load"]
