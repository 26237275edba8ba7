// voxel_kernels.cuh -- bodies of the persistent voxel-solve kernels.  Each
// translation unit that includes this header instantiates them as kernels:
// decaes_gpu.cu without the legacy algorithms (k_voxels, k_voxels_batch),
// decaes_legacy.cu with them (k_voxels_legacy, k_voxels_batch_legacy), so the
// default kernel carries no legacy code.
#pragma once

#include "t2map_device.cuh"

namespace dk {

// Points one warp's views at its shared-memory workspace p and global scratch
// scr for the problem shape of P.
static __device__ void warp_setup(Warp &w, const Params &P, double *p, double *scr) {
    w.P = &P;
    w.mixed = P.mixed != 0;
    const int n = P.n, lda = P.lda;
    if (use_mixed(w)) {
        // normal-equation workspace (see warp_smem_doubles_mixed)
        const int m = P.m;
        w.data = p; p += m;
        w.s.x = p; p += n;
        w.s.w = p; p += n;
        w.xout = p; p += n;
        w.g.G = p; p += mixed_r1_doubles(m, n);
        w.g.L = p; p += mixed_r2_doubles(m, n, P.reg == 2);
        w.g.f = p; p += n;
        w.g.y = p; p += n;
        w.g.dd = p; p += n;
        w.g.dinv = p; p += n;
        w.g.xp = p; p += n;
        p += 8;
        int *ip = reinterpret_cast<int *>(p);
        w.s.idx = ip;
        w.g.P = ip + n;
        w.g.pos = ip + 2 * n;
        w.g.lastP = ip + 3 * n;
        w.g.lastk = 0;
        w.As32 = reinterpret_cast<float *>(w.g.L);  // the staged basis is consumed before the first factorization
        w.ldA = m | 1;
        w.s.C = w.g.L;
        w.s.zz = w.g.y;
        w.s.b = nullptr; w.s.rdiag = nullptr; w.s.posof = nullptr; w.s.zl = nullptr; w.s.diag = nullptr;
        w.s.lda = lda;
    } else {
        w.s.C = p; p += (long)lda * n;
        w.s.b = p; p += lda;
        w.s.zz = p; p += lda;
        w.data = p; p += lda;
        w.s.x = p; p += n;
        w.s.w = p; p += n;
        w.xout = p; p += n;
        w.s.rdiag = p; p += n;
        p += 8;
        w.s.idx = reinterpret_cast<int *>(p);
        w.s.posof = w.s.idx + n;
        w.s.zl = w.s.posof + n;
        w.s.diag = reinterpret_cast<unsigned char *>(w.s.zl + 2 * n);
        w.s.lda = lda;
    }
    w.scr = scr;
    const int mn = P.m < P.n ? P.m : P.n;
    w.sol_key = w.scr + (long)P.m * n + 3L * P.K + (long)kCacheCap * 19 + mn + 16;
    w.sol_x = w.sol_key + kSolCap;
    w.nsol = 0;
}

// Persistent voxel solver: one warp per voxel, voxels pulled from a counter;
// blockDim.x / 32 warps per block, each with its own workspace.  P.mixed
// selects the method (warp-uniform for the whole launch).
__device__ __forceinline__ void voxels_body(const Params &P) {
    extern __shared__ double smem[];
    const int wib = threadIdx.x >> 5, wpb = blockDim.x >> 5;
    Warp w;
    w.lane = threadIdx.x & 31;
    w.nnls_caps = 0;
    w.loop_caps = 0;
    warp_setup(w, P, smem + (long)wib * P.smem_stride, P.scratch + ((long)blockIdx.x * wpb + wib) * P.scr_stride);
#if DECAES_TC_PRODUCTS
    // one chunk of the voxel list: positions [tq0, min(tq1, *nvox))
    const long nvox = P.tq1 > 0 && P.tq1 < (long)*P.nvox ? P.tq1 : (long)*P.nvox;
    for (;;) {
        int q = 0;
        if (w.lane == 0) q = atomicAdd(P.counter, 1);
        q = __shfl_sync(FULL, q, 0);
        const long t = P.tq0 + q;
        if (t >= nvox) break;
        process_voxel(w, (long)P.vidx[t], q);
    }
#else
    const int nvox = *P.nvox;
    for (;;) {
        int t = 0;
        if (w.lane == 0) t = atomicAdd(P.counter, 1);
        t = __shfl_sync(FULL, t, 0);
        if (t >= nvox) break;
        process_voxel(w, (long)P.vidx[t]);
    }
#endif
    if (w.lane == 0) {
        if (w.nnls_caps) atomicAdd(&P.stats[0], (unsigned long long)w.nnls_caps);
        if (w.loop_caps) atomicAdd(&P.stats[1], (unsigned long long)w.loop_caps);
    }
}

// Many volumes in one persistent launch (the batched path).  The compacted
// voxel lists of all volumes form one queue in the order of B.offsets (the
// host orders volumes by estimated cost, most expensive first, so the tail of
// the launch is made of cheap voxels).  A warp that moves to another volume
// copies that volume's parameters next to its workspace and re-carves the
// workspace for the volume's (nTE, nT2, method).
__device__ __forceinline__ void voxels_batch_body(const BatchParams &B) {
    extern __shared__ double smem[];
    const int wib = threadIdx.x >> 5, wpb = blockDim.x >> 5;
    double *base = smem + (long)wib * B.smem_stride;
    Params *Pw = reinterpret_cast<Params *>(base);
    double *ws = base + kParamsDoubles;
    double *scr = B.scratch + ((long)blockIdx.x * wpb + wib) * B.scr_stride;
    Warp w;
    w.lane = threadIdx.x & 31;
    w.nnls_caps = 0;
    w.loop_caps = 0;
    int cur = -1;
    const int total = B.offsets[B.nvol];
    for (;;) {
        int t = 0;
        if (w.lane == 0) t = atomicAdd(B.counter, 1);
        t = __shfl_sync(FULL, t, 0);
        if (t >= total) break;
        int lo = 0, hi = B.nvol - 1;  // last volume whose queue segment starts at or before t
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (B.offsets[mid] <= t) lo = mid; else hi = mid - 1;
        }
        if (lo != cur) {
            if (cur >= 0 && w.lane == 0) {
                if (w.nnls_caps) atomicAdd(&Pw->stats[0], (unsigned long long)w.nnls_caps);
                if (w.loop_caps) atomicAdd(&Pw->stats[1], (unsigned long long)w.loop_caps);
            }
            w.nnls_caps = 0;
            w.loop_caps = 0;
            __syncwarp();
            const double *src = reinterpret_cast<const double *>(B.vols + lo);
            for (int q = w.lane; q < kParamsDoubles; q += 32) base[q] = src[q];
            __syncwarp();
            warp_setup(w, *Pw, ws, scr);
            cur = lo;
        }
        process_voxel(w, (long)Pw->vidx[t - B.offsets[lo]]);
    }
    if (cur >= 0 && w.lane == 0) {
        if (w.nnls_caps) atomicAdd(&Pw->stats[0], (unsigned long long)w.nnls_caps);
        if (w.loop_caps) atomicAdd(&Pw->stats[1], (unsigned long long)w.loop_caps);
    }
}

}  // namespace dk
