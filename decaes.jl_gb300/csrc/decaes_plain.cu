// decaes_plain.cu -- the voxel-solve kernel with the plain FP64 method only (bit-exact with the oracle): single-volume launches
// and batched / served launches whose volumes all use that method run these
// kernels (half the code of the kernels that carry both methods).  A separate
// translation unit, compiled in parallel with the others.
#define DECAES_METHODS 1
#include "voxel_kernels.cuh"

namespace dk {

__global__ void __launch_bounds__(256) k_voxels_plain(const __grid_constant__ Params P) { voxels_body(P); }
__global__ void __launch_bounds__(128) k_voxels_batch_plain(const __grid_constant__ BatchParams B) { voxels_batch_body(B); }

}  // namespace dk
