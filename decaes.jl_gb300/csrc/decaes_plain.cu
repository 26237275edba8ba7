// decaes_plain.cu -- the voxel-solve kernel with the plain FP64 method only (bit-exact with the oracle): single-volume launches
// of that method use it (half the code of the kernel that carries both
// methods, which the batched and served launches keep).  A separate
// translation unit, compiled in parallel with the others.
#define DECAES_METHODS 1
#include "voxel_kernels.cuh"

namespace dk {

__global__ void __launch_bounds__(128) k_voxels_plain(const __grid_constant__ Params P) { voxels_body(P); }

}  // namespace dk
