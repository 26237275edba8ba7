// decaes_tc.cu -- the grid products F = A_k' y of the flip-angle search on the
// tensor cores (tcgen05), for the mixed method's DECAES_PREC_MIXED_TC mode.
//
// The search evaluates the NNLS loss at grid angles k; every evaluation needs
// f_k = A_k' b (src/lsqnonneg.jl:30-72, the warm-start dual; A_k the basis of
// grid angle k, b the voxel's normalized decay).  All voxels share the K grid
// bases, so the products of a tile of voxels with every grid column form one
// GEMM: F[t, k*n + j] = sum_i A_k(i, j) y_t(i), M = voxels, N = K*n basis
// columns, K-dimension = echoes.
//
// Precision: near-FP64 products are needed (the search compares losses
// between angles, and an FP32-rounded A_k'b moved fitted angles by ~0.05 deg
// at p99), so each operand is split into S = 4 bf16 "slices" of a
// fixed-point value:
//   v = s_0 2^-8 + s_1 2^-16 + s_2 2^-24 + s_3 2^-32 + r,  s_i integers,
//   |s_0| <= 256, |s_1|, |s_2|, |s_3| <= 128, |r| <= 2^-33,
// for v = y / 2^e (e the voxel's exponent: |v| < 1) and for the basis entries
// (0 <= A <= 1).  Every s_i is exactly a bf16.  The slice products are grouped
// by scale: D_d = sum_{s+t=d} sum_i s_s(i) a_t(i), d < S, each an integer
// below 2^24 (m <= 128), so the FP32 accumulation of the tensor cores is
// exact; F = sum_d D_d 2^-8(d+2) is formed exactly as a float pair (hi, lo)
// and carries ~2^-32 relative error from the dropped slice pairs: split-
// precision bf16 with FP32 accumulation, exact up to the truncation.
//
// Layout and flow (one CTA of 4 warps, persistent over 128-voxel tiles):
//   * the CTA gathers its voxels' echo trains from the image, forms e and the
//     slices, and writes them to shared memory in the no-swizzle K-major
//     canonical layout (8 x 16-byte core matrices, K-adjacent ones 128 B
//     apart, 8-row groups mpad*16 B apart);
//   * the basis slices are prepared once per basis key in the same layout,
//     one contiguous block per 64-column tile, and streamed into shared memory
//     by bulk asynchronous copies (double-buffered, mbarrier completion);
//   * one thread issues the S(S+1)/2 * mpad/16 MMAs of a tile
//     (cta_group::1, kind::f16 with bf16 operands, M = 128, N = 64, FP32
//     accumulators D_0..D_{S-1} in TMEM columns [64d, 64d + 64)) and commits
//     them to an mbarrier;
//   * the four warps read their 32 TMEM lanes (one voxel each) with
//     tcgen05.ld, sum the D_d as float pairs and store 64 pairs per voxel.
// Every mbarrier wait is bounded; a CTA that gives up records it in the error
// counter, marks its voxels' rows unusable (the voxel kernel then forms those
// products itself), waits for its own operations still in flight and frees
// its TMEM.
#include <cuda_runtime.h>
#include <cuda_bf16.h>

#include <climits>
#include <cstdint>

#include "decaes_tc.h"
#include "host.h"

namespace dk {
namespace {

constexpr int kS = kTcSlices;

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// Waits for the phase with the given parity to complete; gives up after a
// bounded number of polls (each try_wait itself suspends for a short while).
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity) {
    const uint32_t a = smem_u32(bar);
    #pragma unroll 1
    for (int it = 0; it < (1 << 20); ++it) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor: no swizzle, K-major; start address, the
// K-direction core-matrix stride (LBO) and the 8-row-group stride (SBO), all
// in 16-byte units; bits 46-47 = 1 (descriptor version of this architecture).
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
// Instruction descriptor of kind::f16: FP32 accumulator, bf16 A and B, both
// K-major, N >> 3 at bit 17, M >> 4 at bit 24.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kTcTileN >> 3) << 17) |
                            ((uint32_t)(kTcTileM >> 4) << 24);

__device__ __forceinline__ void mma_bf16(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
        "l"(a), "l"(b), "r"(kIdesc), "r"(acc)
        : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}
// 32 consecutive FP32 columns of this warp's 32 TMEM lanes.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float *v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// s + e = a + b exactly (Knuth's two-sum; the build does not contract).
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// Fixed-point slices of v (|v| <= 1): v = sum_i s_i 2^-8(i+1) (+ r).
__device__ __forceinline__ void slices_of(double v, float *s) {
    double t = v * 256.0;
#pragma unroll
    for (int i = 0; i < kS; ++i) {
        const double a = rint(t);
        s[i] = (float)a;
        t = (t - a) * 256.0;
    }
}

}  // namespace

// Basis slices: one thread per (basis column R = k*n + j, echo i) of the
// padded N x mpad operand; rows past K*n and echoes past m are zero.
__global__ void k_tc_basis_slices(const double *As, int m, int n, int K, int mpad, int ntiles,
                                  unsigned char *out) {
    const long N = (long)ntiles * kTcTileN;
    const long total = N * mpad;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < total; q += (long)gridDim.x * blockDim.x) {
        const int R = (int)(q / mpad), i = (int)(q % mpad);
        double a = 0.0;
        if (R < K * n && i < m) {
            const int k = R / n, j = R % n;
            a = As[(long)k * m * n + i + (long)m * j];
        }
        float s[kS];
        slices_of(a, s);
        const int tile = R / kTcTileN, row = R % kTcTileN;
        unsigned char *base = out + (size_t)tile * kS * tc_slice_bytes(kTcTileN, mpad);
#pragma unroll
        for (int t = 0; t < kS; ++t)
            *reinterpret_cast<__nv_bfloat16 *>(base + (size_t)t * tc_slice_bytes(kTcTileN, mpad) + tc_off(row, i, mpad)) =
                __float2bfloat16_rn(s[t]);
    }
}

__global__ void __launch_bounds__(kTcThreads, 1) k_grid_products(const __grid_constant__ TcParams p) {
    extern __shared__ __align__(1024) unsigned char sm[];
    const int tid = threadIdx.x, warp = tid >> 5;
    const int mpad = p.mpad;
    const unsigned aSlice = tc_slice_bytes(kTcTileM, mpad), bSlice = tc_slice_bytes(kTcTileN, mpad);
    const int nbuf = tc_nbuf(mpad);
    unsigned char *sA = sm;
    unsigned char *sB = sA + kS * aSlice;  // nbuf buffers of kS slices
    uint64_t *bar = reinterpret_cast<uint64_t *>(sB + nbuf * kS * bSlice);  // [0], [1] basis tiles, [2] MMA done
    uint32_t *tslot = reinterpret_cast<uint32_t *>(bar + 4);
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_init(&bar[2], 1);
        fence_mbar_init();
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                     "r"(kTcTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;

    const long nv = (long)*p.nvox < p.t1 ? (long)*p.nvox : p.t1;
    unsigned phB0 = 0, phB1 = 0, phM = 0;  // mbarrier phase parities (uniform over the CTA)
    bool pendB0 = false, pendB1 = false, pendM = false, failed = false;
    const uint32_t lbo = 128, sbo = (uint32_t)mpad * 16;
    const unsigned tileBytes = kS * bSlice;

    #pragma unroll 1
    for (long tile0 = p.t0 + (long)blockIdx.x * kTcTileM; tile0 < nv && !failed; tile0 += (long)gridDim.x * kTcTileM) {
        // ---- the tile's voxels: exponent and slices (one voxel per thread) ----
        {
            const long t = tile0 + tid;
            const bool valid = t < nv;
            long v = valid ? (long)p.vidx[t] : 0;
            double amax = 0.0;
            bool finite = true;
            #pragma unroll 1
            for (int i = 0; i < p.m; ++i) {
                double y = 0.0;
                if (valid) y = p.f32 ? (double)static_cast<const float *>(p.image)[v + p.V * i]
                                     : static_cast<const double *>(p.image)[v + p.V * i];
                finite = finite && isfinite(y);
                amax = fmax(amax, fabs(y));
            }
            const bool ok = valid && finite && amax > 0.0;
            const int e = ok ? ilogb(amax) + 1 : 0;
            const double sc = ok ? ldexp(1.0, -e) : 0.0;
            #pragma unroll 1
            for (int i = 0; i < mpad; ++i) {
                double y = 0.0;
                if (ok && i < p.m)
                    y = p.f32 ? (double)static_cast<const float *>(p.image)[v + p.V * i]
                              : static_cast<const double *>(p.image)[v + p.V * i];
                float s[kS];
                slices_of(y * sc, s);
#pragma unroll
                for (int q = 0; q < kS; ++q)
                    *reinterpret_cast<__nv_bfloat16 *>(sA + q * aSlice + tc_off(tid, i, mpad)) = __float2bfloat16_rn(s[q]);
            }
            if (valid) p.Fexp[t - p.t0] = ok ? e : INT_MIN;
        }
        fence_proxy_async();
        __syncthreads();

        // ---- every 64-column tile of the grid bases ----
        if (tid == 0) {
            mbar_expect_tx(&bar[0], tileBytes);
            bulk_g2s(sB, p.Bsl, tileBytes, &bar[0]);
            pendB0 = true;
        }
        #pragma unroll 1
        for (int nt = 0; nt < p.ntiles; ++nt) {
            const int buf = nbuf == 2 ? (nt & 1) : 0;
            unsigned char *sBb = sB + buf * tileBytes;
            if (tid == 0) {
                if (nbuf == 1 && nt > 0) {  // one buffer: its previous tile's MMAs completed last round
                    mbar_expect_tx(&bar[0], tileBytes);
                    bulk_g2s(sB, p.Bsl + (size_t)nt * tileBytes, tileBytes, &bar[0]);
                    pendB0 = true;
                }
                if (nbuf == 2 && nt + 1 < p.ntiles) {  // the other buffer's MMAs completed in the previous round
                    uint64_t *nb = &bar[buf ^ 1];
                    mbar_expect_tx(nb, tileBytes);
                    bulk_g2s(sB + (buf ^ 1) * tileBytes, p.Bsl + (size_t)(nt + 1) * tileBytes, tileBytes, nb);
                    if (buf ^ 1) pendB1 = true; else pendB0 = true;
                }
                bool ok = buf ? mbar_wait(&bar[1], phB1) : mbar_wait(&bar[0], phB0);
                if (ok) {
                    if (buf) { phB1 ^= 1; pendB1 = false; } else { phB0 ^= 1; pendB0 = false; }
                    tc_fence_after();
                    const uint32_t a0 = smem_u32(sA), b0 = smem_u32(sBb);
                    #pragma unroll 1
                    for (int d = 0; d < kS; ++d) {
                        uint32_t acc = 0;
                        #pragma unroll 1
                        for (int s = 0; s <= d; ++s) {
                            const int t = d - s;
                            #pragma unroll 1
                            for (int kk = 0; kk < mpad / 16; ++kk) {
                                const uint64_t da = sdesc(a0 + s * aSlice + kk * 256, lbo, sbo);
                                const uint64_t db = sdesc(b0 + t * bSlice + kk * 256, lbo, sbo);
                                mma_bf16(tmem + (uint32_t)(d * kTcTileN), da, db, acc);
                                acc = 1;
                            }
                        }
                    }
                    mma_commit(&bar[2]);
                    pendM = true;
                } else {
                    failed = true;
                }
            }
            // the CTA learns whether the issue happened, then waits for the MMAs
            const int issued = __syncthreads_and(tid != 0 || !failed);
            if (!issued) { failed = true; break; }
            const bool okM = mbar_wait(&bar[2], phM);
            if (okM) {
                phM ^= 1;
                if (tid == 0) pendM = false;
            }
            if (!__syncthreads_and(okM)) { failed = true; break; }
            tc_fence_after();
            // ---- epilogue: voxel row tid, columns [nt*64, nt*64 + 64) ----
            const long t = tile0 + tid;
            const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
            #pragma unroll 1
            for (int h = 0; h < 2; ++h) {
                float d[kS][32];
#pragma unroll
                for (int q = 0; q < kS; ++q) tmem_ld32(tmem + lane_base + (uint32_t)(q * kTcTileN + 32 * h), d[q]);
                tmem_wait_ld();
                if (t < nv) {
                    float4 *dst =
                        reinterpret_cast<float4 *>(p.F + (t - p.t0) * p.ldF + 2 * ((long)nt * kTcTileN + 32 * h));
#pragma unroll
                    for (int c2 = 0; c2 < 16; ++c2) {
                        float o[4];
#pragma unroll
                        for (int c = 0; c < 2; ++c) {
                            // sum_d D_d 2^-8(d+2): every term exact in FP32, summed as a float pair
                            const int col = 2 * c2 + c;
                            float s = d[0][col] * 1.52587890625e-05f, e = 0.f, r;  // 2^-16
                            float sc = 1.52587890625e-05f;
#pragma unroll
                            for (int q = 1; q < kS; ++q) {
                                sc *= 0.00390625f;
                                two_sum(s, d[q][col] * sc, s, r);
                                e += r;
                            }
                            const float hi = s + e;
                            o[2 * c] = hi;
                            o[2 * c + 1] = e - (hi - s);
                        }
                        dst[c2] = make_float4(o[0], o[1], o[2], o[3]);
                    }
                }
            }
            tc_fence_before();
            __syncthreads();  // TMEM reads done before the next tile's MMAs overwrite it
        }
        if (failed) {
            // rows of this tile: the voxel kernel forms their products itself
            const long t = tile0 + tid;
            if (t < nv) p.Fexp[t - p.t0] = INT_MIN;
        }
    }
    // ---- teardown: own operations still in flight, then the TMEM ----
    if (tid == 0) {
        if (failed) atomicAdd(p.err, 1u);
        if (pendM && mbar_wait(&bar[2], phM)) pendM = false;
        if (pendB0 && mbar_wait(&bar[0], phB0)) pendB0 = false;
        if (pendB1 && mbar_wait(&bar[1], phB1)) pendB1 = false;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcTmemCols) : "memory");
}

size_t tc_smem_bytes(int mpad) {
    return (size_t)kS * tc_slice_bytes(kTcTileM, mpad) + (size_t)tc_nbuf(mpad) * kS * tc_slice_bytes(kTcTileN, mpad) + 64;
}

cudaError_t tc_make_basis_slices(const double *As, int m, int n, int K, unsigned char *out, cudaStream_t st) {
    const int mpad = tc_mpad(m), ntiles = tc_ntiles(K, n);
    const long total = (long)ntiles * kTcTileN * mpad;
    const int g = (int)((total + 255) / 256);
    k_tc_basis_slices<<<g, 256, 0, st>>>(As, m, n, K, mpad, ntiles, out);
    return cudaGetLastError();
}

cudaError_t tc_grid_products(const TcParams &p, int sms, cudaStream_t st) {
    // at least 100 KB per CTA: at most two CTAs per SM, so their TMEM
    // allocations (kTcTmemCols each) always fit the SM's 512 columns
    size_t smem = tc_smem_bytes(p.mpad);
    if (smem < (size_t)100 << 10) smem = (size_t)100 << 10;
    cudaError_t e = (cudaError_t)dh::raise_smem_limit((const void *)k_grid_products, smem);
    if (e != cudaSuccess) return e;
    k_grid_products<<<2 * sms, kTcThreads, smem, st>>>(p);
    return cudaGetLastError();
}

}  // namespace dk
