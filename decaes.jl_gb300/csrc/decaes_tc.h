// decaes_tc.h -- the tensor-core grid products of the mixed method
// (decaes_tc.cu): constants, the operand layout and the host entry points.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>

namespace dk {

constexpr int kTcTileM = 128;    // voxels per tile (MMA M)
constexpr int kTcTileN = 64;     // grid-basis columns per tile (MMA N)
constexpr int kTcSlices = 4;     // bf16 fixed-point slices per operand
constexpr int kTcThreads = 128;  // four warps: one TMEM lane quarter each
constexpr int kTcTmemCols = 256; // TMEM columns per CTA (kTcSlices x kTcTileN used)

__host__ __device__ inline int tc_mpad(int m) { return (m + 15) & ~15; }
__host__ __device__ inline int tc_ntiles(int K, int n) { return (K * n + kTcTileN - 1) / kTcTileN; }
// Bytes of one bf16 slice of a rows x mpad operand tile.
__host__ __device__ inline unsigned tc_slice_bytes(int rows, int mpad) { return (unsigned)rows * mpad * 2u; }
// Byte offset of element (row, k) in the no-swizzle K-major layout: 8 x 8
// core matrices of 16-byte rows, K-adjacent ones 128 B apart, 8-row groups
// mpad * 16 B apart.
__host__ __device__ inline unsigned tc_off(int row, int k, int mpad) {
    return (((unsigned)(row >> 3) * (unsigned)(mpad >> 3) + (unsigned)(k >> 3)) * 8u + (unsigned)(row & 7)) * 16u +
           (unsigned)(k & 7) * 2u;
}

struct TcParams {
    const void *image;             // V x m, column-major, FP32 (f32 != 0) or FP64
    int f32;
    long V;
    int m, mpad;
    const int *vidx;               // compacted voxel list
    const int *nvox;               // its length (device)
    long t0, t1;                   // the list positions of this launch, [t0, min(t1, *nvox))
    const unsigned char *Bsl;      // grid-basis slices: ntiles blocks of kTcSlices x 64 x mpad bf16
    int ntiles;
    float *F;                      // F[(t - t0) * ldF + 2 (k*n + j) + {0, 1}]: the product as a float pair
                                   // (hi, lo), scaled by 2^-e of the voxel
    long ldF;                      // 2 * ntiles * 64
    int *Fexp;                     // per position: e, or INT_MIN when the voxel's row is not usable
    unsigned *err;                 // CTAs whose bounded waits gave up
};

// Basis-tile buffers of one CTA: two when they fit beside the voxel tile in
// the 227 KB of shared memory a block may use, else one.
__host__ __device__ inline int tc_nbuf(int mpad) {
    const unsigned two = kTcSlices * tc_slice_bytes(kTcTileM, mpad) + 2u * kTcSlices * tc_slice_bytes(kTcTileN, mpad) + 64u;
    return two <= 227u * 1024u ? 2 : 1;
}
// Shared memory of one CTA of k_grid_products (before the 100 KB floor).
size_t tc_smem_bytes(int mpad);
// Grid-basis slices (tc_ntiles(K, n) * kTcSlices * tc_slice_bytes(64, mpad)
// bytes) of the K grid bases As (m x n each, FP64).
cudaError_t tc_make_basis_slices(const double *As, int m, int n, int K, unsigned char *out, cudaStream_t st);
// F for the list positions [t0, t1): two CTAs per SM, persistent over tiles.
cudaError_t tc_grid_products(const TcParams &p, int sms, cudaStream_t st);

}  // namespace dk
