// decaes_legacy.cu -- the voxel-solve kernels with the legacy algorithms
// (T2mapOptions.legacy = true: spline-surrogate flip-angle search and the chi2
// search by mu doubling, src/T2mapSEcorr.jl:401-403, src/lsqnonneg.jl:595-636).
// A separate translation unit, compiled in parallel with decaes_gpu.cu, so the
// default kernels carry none of this code.  The host launches these kernels
// for any launch with a legacy volume; they run non-legacy volumes too.
#define DECAES_LEGACY_KERNEL 1
#include "voxel_kernels.cuh"

namespace dk {

__global__ void __launch_bounds__(128) k_voxels_legacy(const __grid_constant__ Params P) { voxels_body(P); }
__global__ void __launch_bounds__(128) k_voxels_batch_legacy(const __grid_constant__ BatchParams B) { voxels_batch_body(B); }

}  // namespace dk
