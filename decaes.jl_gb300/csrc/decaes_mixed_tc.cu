// decaes_mixed_tc.cu -- the mixed method's voxel-solve kernel that reads the
// flip-angle search's grid products A_k'b from the tensor-core GEMM
// (DECAES_PREC_MIXED_TC, decaes_tc.cu) instead of forming them per
// evaluation; launched once per chunk of the voxel list, after that chunk's
// products.  A translation unit of its own, so the other kernels carry none
// of this path.
#define DECAES_METHODS 2
#define DECAES_TC_PRODUCTS 1
#include "voxel_kernels.cuh"

namespace dk {

__global__ void __launch_bounds__(128) k_voxels_mixed_tc(const __grid_constant__ Params P) { voxels_body(P); }

}  // namespace dk
