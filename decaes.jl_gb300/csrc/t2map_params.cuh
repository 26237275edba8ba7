// t2map_params.cuh -- launch parameters of the voxel-solve kernel and the
// sizes of its per-warp workspaces, shared by the kernel and its host callers.
#pragma once

namespace dk {

constexpr int kCacheCap = 128;   // L-curve cache entries per voxel (the loop needs ~30)
constexpr int kLoopCap = 512;    // hard cap of every data-dependent outer loop
constexpr int kSolCap = 64;      // stored Tikhonov solutions per voxel (keyed by log mu)

struct Params {
    int m, n, K, M, lda;
    int reg;
    double chi2factor, noiselevel;
    int mineval, maxeval;
    int angle_mode;  // 0 search, 1 fixed SetFlipAngle, 2 B1 map
    double fixed_angle;
    int beta180;
    double beta, TE, T1;
    long V;
    const int *nvox;
    const int *vidx;
    const void *image;
    int image_f32;
    const void *b1map;
    const double *t2, *logt2, *angles, *As, *dAs, *basis_fixed;
    double *scratch;
    long scr_stride;  // doubles per warp
    int *counter;
    unsigned long long *stats;  // [0] NNLS cap hits, [1] loop cap hits
    double *dist, *gdn, *ggm, *gva, *fnr, *snr, *alpha, *resnorm, *decaycurve, *mu, *chi2f, *basis_out;
    int fuse_t2part, sp0, sp1, mp0, mp1;
    const double *weights;
    double *sfr, *sgm, *mfr, *mgm;
    int need_chi2;
    int epg_lanes;
    // mixed-precision method (normal-equation NNLS, FP32 EPG at the fitted angle)
    int mixed;
    int legacy;         // legacy algorithms: spline surrogate search, chi2 doubling search
    const double *Gs;   // packed Gram matrices A_k'A_k of the grid bases (K x n(n+1)/2), or of the fixed basis
    const double *AsT;  // the grid (or fixed) bases transposed, K x m x n (row-major per basis)
    int epg_lanes_f32;  // lanes of the FP32 EPG (states in the Gram and factor regions)
    long smem_stride;   // doubles of shared memory per warp (several warps per block)
    // the voxel-list positions of a k_voxels_mixed_tc launch: [tq0, min(tq1, *nvox))
    long tq0, tq1;
    // tensor-core grid products (DECAES_PREC_MIXED_TC): row t - tq0 of F holds
    // A_k' y for every grid angle as float pairs (hi, lo), scaled by
    // 2^-Fexp[t - tq0] (INT_MIN: unusable)
    const float *Fk;
    const int *Fexp;
    long ldF;
};
// Doubles a copy of Params occupies (batched launch: one copy per warp).
constexpr int kParamsDoubles = (int)((sizeof(Params) + 7) / 8);

// The batched launch: many volumes, one persistent kernel.
struct BatchParams {
    const Params *vols;   // per-volume parameters, in queue order (device)
    const int *offsets;   // nvol + 1 prefix offsets of the compacted voxel lists
    int nvol;
    int *counter;         // queue position
    double *scratch;
    long scr_stride;      // doubles of global scratch per warp (maximum over volumes)
    long smem_stride;     // doubles of shared memory per warp (Params copy + largest workspace)
};

// Shared-memory footprint of one warp worker (doubles), mirrored on the host.
__host__ __device__ inline long warp_smem_doubles(int m, int n, int lda) {
    long d = (long)lda * n + 3L * lda + 4L * n + 8;
    long ints = 4L * n;            // idx, posof, zl
    long bytes = (long)n;          // diag
    return d + (ints * 4 + bytes + 7) / 8;
}
// Shared-memory regions of one warp worker of the mixed method (doubles):
// R1 holds the packed Gram matrix, R2 the packed factor, or the basis staged
// in FP32, or (GCV) the tridiagonalization workspace; before the Gram matrix
// is built both hold the FP32 EPG states.
__host__ __device__ inline long mixed_r1_doubles(int m, int n) { return (long)n * (n + 1) / 2; }
__host__ __device__ inline long mixed_r2_doubles(int m, int n, bool gcv) {
    long l = (long)n * (n - 1) / 2, a = ((long)(m | 1) * n + 1) / 2, e = 2L * m;
    long x = l > a ? l : a;
    x = x > e ? x : e;
    if (gcv) {
        long t = (long)n * (n + 1) / 2;
        x = x > t ? x : t;
    }
    return x;
}
__host__ __device__ inline long warp_smem_doubles_mixed(int m, int n, bool gcv) {
    long d = (long)m + 3L * n + mixed_r1_doubles(m, n) + mixed_r2_doubles(m, n, gcv) + 5L * n + 8;
    long ints = 4L * n;  // idx, P, pos, lastP
    return d + (ints * 4 + 7) / 8;
}
// Lanes of the FP64 method's EPG basis (one T2 column per lane, 3m states
// each).  The states use the contiguous C, b and zz regions of the workspace
// (lda * (n + 2) doubles, free while the voxel's basis is built), which hold
// at least one lane's states for every n >= 1 because lda >= m + n.
__host__ __device__ inline int fp64_epg_lanes(int m, int n, int lda) {
    long l = ((long)lda * (n + 2)) / (3L * m);
    return (int)(l < 1 ? 1 : (l > 32 ? 32 : l));
}
// Global scratch of one warp worker (doubles).
// Offset of the mixed method's FP32 basis (m x n floats) in it, after the
// per-voxel basis, surrogate samples, L-curve caches, singular values and the
// stored solutions.
__host__ __device__ inline long warp_scratch_f32_offset(int m, int n, int K) {
    int mn = m < n ? m : n;
    return (long)m * n + 3L * K + (long)kCacheCap * (3 + 4 + 12) + mn + 16 + (long)kSolCap * (n + 1);
}
__host__ __device__ inline long warp_scratch_doubles(int m, int n, int K) {
    return warp_scratch_f32_offset(m, n, K) + ((long)m * n + 1) / 2;
}

}  // namespace dk
