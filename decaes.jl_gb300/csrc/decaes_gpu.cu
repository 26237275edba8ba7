// decaes_gpu.cu -- kernels and host orchestration of libdecaes_gpu.so.
//
// Call flow of decaes_t2map_t2part (host buffers):
//   H2D image -> [resident angle-ensemble basis, cached per parameter key]
//   -> NaN-fill outputs -> threshold compaction -> persistent warp-per-voxel
//   solve (flip-angle search, EPG basis, regularized NNLS, save_results! and
//   fused T2part) -> optional FP32 narrowing -> D2H outputs.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "decaes_gpu.h"
#include "decaes_tc.h"
#include "epg.cuh"
#include "host.h"
#include "voxel_kernels.cuh"

namespace dk {

// ---------------------------------------------------------------------------
// Kernels
// ---------------------------------------------------------------------------

// Angle-ensemble basis As[m,n,K] and dAs/dalpha (EPGBasisSetEnsemble +
// ∇epg_decay_basis!, src/T2mapSEcorr.jl:322-371): one curve per thread, the
// value part of a forward-mode dual evaluation.
__global__ void k_ensemble(int m, int n, int K, double TE, double T1, int beta180, double beta, const double *t2,
                           const double *angles, double *As, double *dAs, dx::Dual *work) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * K) return;
    int j = t % n, k = t / n;
    dx::Dual *S = work + (long)t * 3 * m;                    // 3m recursion states
    dx::Dual *out = work + (long)n * K * 3 * m + (long)t * m;  // m curve values
    double *Av = As + ((long)k * n + j) * m, *dAv = dAs + ((long)k * n + j) * m;
    if (beta180) {
        dx::FlatCoef<dx::Dual> q = dx::flat_coef_dual(angles[k], TE, t2[j], T1);
        dx::epg_flat_inplace(m, q, S, 1, out, 1);
    } else {
        dx::VecCoef<dx::Dual> q = dx::vec_coef_dual(angles[k], TE, t2[j], T1, beta);
        dx::epg_vec_inplace(m, q, S, 1, out, 1);
    }
    for (int i = 0; i < m; ++i) { Av[i] = out[i].v; dAv[i] = out[i].d; }
}

// Single basis at a fixed angle (SetFlipAngle), one curve per thread.
__global__ void k_basis_fixed(int m, int n, double alpha, double TE, double T1, int beta180, double beta,
                              const double *t2, double *A, double *work) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    double *S = work + (long)j * 3 * m;
    if (beta180) {
        dx::FlatCoef<double> q = dx::flat_coef(alpha, TE, t2[j], T1);
        dx::epg_flat_inplace(m, q, S, 1, A + (long)j * m, 1);
    } else {
        dx::VecCoef<double> q = dx::vec_coef(alpha, TE, t2[j], T1, beta);
        dx::epg_vec_inplace(m, q, S, 1, A + (long)j * m, 1);
    }
}

// Mixed method, once per basis key: packed Gram matrices G_k = A_k'A_k of
// the K grid bases (upper triangle by columns) and the bases transposed to
// row-major, one block per basis.
__global__ void k_gram_grid(int m, int n, const double *As, double *Gs, double *AsT) {
    const int k = blockIdx.x;
    const double *A = As + (long)k * m * n;
    double *G = Gs + (long)k * (n * (n + 1) / 2);
    double *AT = AsT + (long)k * m * n;
    const int npairs = n * (n + 1) / 2;
    for (int p = threadIdx.x; p < npairs; p += blockDim.x) {
        int j = 0;
        while ((j + 1) * (j + 2) / 2 <= p) ++j;
        int i = p - j * (j + 1) / 2;
        const double *ai = A + (long)i * m, *aj = A + (long)j * m;
        double s = 0.0;
        for (int r = 0; r < m; ++r) s = fma(ai[r], aj[r], s);
        G[p] = s;
    }
    for (int q = threadIdx.x; q < m * n; q += blockDim.x) {
        const int i = q / n, j = q % n;
        AT[q] = A[i + (long)m * j];
    }
}

__global__ void k_fill(double *p, long len, double v) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < len; i += (long)gridDim.x * blockDim.x) p[i] = v;
}

// indices = filter(I -> image[I, 1] > Threshold, CartesianIndices(MatrixSize)),
// src/T2mapSEcorr.jl:177 (order of the compacted list does not matter:
// voxels are independent).
__global__ void k_compact(const void *image, int f32, long V, double thr, int *vidx, int *nvox) {
    for (long v = blockIdx.x * (long)blockDim.x + threadIdx.x; v < V; v += (long)gridDim.x * blockDim.x) {
        double b = f32 ? (double)static_cast<const float *>(image)[v] : static_cast<const double *>(image)[v];
        bool keep = b > thr;
        unsigned msk = __ballot_sync(__activemask(), keep);
        if (keep) {
            int leader = __ffs(msk) - 1, lane = threadIdx.x & 31, base = 0;
            if (lane == leader) base = atomicAdd(nvox, __popc(msk));
            base = __shfl_sync(msk, base, leader);
            vidx[base + __popc(msk & ((1u << lane) - 1))] = (int)v;
        }
    }
}

// The same for the voxel range [v0, v1) of a volume (a chunk of a request in
// the serving loop); voxel indices stay absolute.
__global__ void k_compact_range(const void *image, int f32, long v0, long v1, double thr, int *vidx, int *nvox) {
    for (long v = v0 + blockIdx.x * (long)blockDim.x + threadIdx.x; v < v1; v += (long)gridDim.x * blockDim.x) {
        double b = f32 ? (double)static_cast<const float *>(image)[v] : static_cast<const double *>(image)[v];
        bool keep = b > thr;
        unsigned msk = __ballot_sync(__activemask(), keep);
        if (keep) {
            int leader = __ffs(msk) - 1, lane = threadIdx.x & 31, base = 0;
            if (lane == leader) base = atomicAdd(nvox, __popc(msk));
            base = __shfl_sync(msk, base, leader);
            vidx[base + __popc(msk & ((1u << lane) - 1))] = (int)v;
        }
    }
}

__global__ void __launch_bounds__(128) k_voxels(const __grid_constant__ Params P) { voxels_body(P); }
__global__ void __launch_bounds__(128) k_voxels_batch(const __grid_constant__ BatchParams B) { voxels_batch_body(B); }
// the same kernels with the legacy algorithms (decaes_legacy.cu), and with one
// method each (decaes_plain.cu, decaes_mixed.cu)
__global__ void __launch_bounds__(128) k_voxels_legacy(const __grid_constant__ Params P);
__global__ void __launch_bounds__(128) k_voxels_batch_legacy(const __grid_constant__ BatchParams B);
__global__ void __launch_bounds__(256) k_voxels_plain(const __grid_constant__ Params P);
__global__ void __launch_bounds__(128) k_voxels_mixed(const __grid_constant__ Params P);
__global__ void __launch_bounds__(128) k_voxels_mixed_tc(const __grid_constant__ Params P);
__global__ void __launch_bounds__(128) k_voxels_batch_plain(const __grid_constant__ BatchParams B);
__global__ void __launch_bounds__(128) k_voxels_batch_mixed(const __grid_constant__ BatchParams B);

// The batched kernel for a set of volumes: the legacy one when any volume is
// legacy, else the kernel of the volumes' one method, else the two-method one.
using BatchKern = void (*)(BatchParams);
inline BatchKern batch_kernel(bool legacy, bool any_plain, bool any_mixed) {
    if (legacy) return k_voxels_batch_legacy;
    if (!any_plain) return k_voxels_batch_mixed;
    if (!any_mixed) return k_voxels_batch_plain;
    return k_voxels_batch;
}

// offsets[0] = 0, offsets[v + 1] = offsets[v] + counts[v] (one thread; nvol is small).
__global__ void k_batch_prefix(const int *counts, int nvol, int *offsets) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        int s = 0;
        offsets[0] = 0;
        for (int v = 0; v < nvol; ++v) { s += counts[v]; offsets[v + 1] = s; }
    }
}

// Standalone T2partSEcorr (src/T2partSEcorr.jl:95-138): one thread per voxel.
template <class T>
__global__ void k_t2part(const T *dist, long V, int n, int sp0, int sp1, int mp0, int mp1, const double *logt2,
                         const double *weights, double *sfr, double *sgm, double *mfr, double *mgm) {
    for (long v = blockIdx.x * (long)blockDim.x + threadIdx.x; v < V; v += (long)gridDim.x * blockDim.x) {
        bool anynan = false;
        for (int j = 0; j < n; ++j) anynan |= isnan((double)dist[v + V * j]);
        if (anynan) continue;
        double sd = 0, ssp = 0, smp = 0, dsp = 0, dmp = 0;
        for (int j = 0; j < n; ++j) sd = __dadd_rn(sd, (double)dist[v + V * j]);
        for (int j = sp0; j <= sp1; ++j) {
            double d = dist[v + V * j];
            dsp = __dadd_rn(dsp, __dmul_rn(d, logt2[j]));
            ssp = __dadd_rn(ssp, d);
        }
        for (int j = mp0; j <= mp1; ++j) {
            double d = dist[v + V * j];
            dmp = __dadd_rn(dmp, __dmul_rn(d, logt2[j]));
            smp = __dadd_rn(smp, d);
        }
        if (sd > 0) {
            if (weights) {
                double dw = 0;
                for (int j = 0; j < n; ++j) dw = __dadd_rn(dw, __dmul_rn((double)dist[v + V * j], weights[j]));
                sfr[v] = dw / sd;
            } else {
                sfr[v] = ssp / sd;
            }
            mfr[v] = smp / sd;
        }
        if (ssp > 0) sgm[v] = pm_exp(dsp / ssp);
        if (smp > 0) mgm[v] = pm_exp(dmp / smp);
    }
}

__global__ void k_narrow(const double *src, float *dst, long len) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < len; i += (long)gridDim.x * blockDim.x)
        dst[i] = (float)src[i];
}

}  // namespace dk

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
namespace dh {
// One lock for every change of a kernel's dynamic shared-memory limit in the
// library (the context paths and the no-allocation entry point).  The limit is
// only ever raised: a launch planned for a size below it stays valid whatever
// another thread or context sets in between.
int raise_smem_limit(const void *kern, size_t bytes) {
    static std::mutex mu;
    std::lock_guard<std::mutex> lk(mu);
    cudaFuncAttributes a;
    cudaError_t e = cudaFuncGetAttributes(&a, kern);
    if (e != cudaSuccess) return (int)e;
    if ((size_t)a.maxDynamicSharedSizeBytes >= bytes) return (int)cudaSuccess;
    return (int)cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}
}  // namespace dh

namespace {

struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
};

struct BasisKey {
    int m, n, K, beta180;
    double TE, T1, t2lo, t2hi, minang, beta, fixed;
    bool operator<(const BasisKey &o) const {
        return std::tie(m, n, K, beta180, TE, T1, t2lo, t2hi, minang, beta, fixed) <
               std::tie(o.m, o.n, o.K, o.beta180, o.TE, o.T1, o.t2lo, o.t2hi, o.minang, o.beta, o.fixed);
    }
};
struct Basis {
    double *t2 = nullptr, *logt2 = nullptr, *angles = nullptr, *As = nullptr, *dAs = nullptr, *fixed = nullptr;
    double *Gs = nullptr;   // packed Gram matrices of the grid (or fixed) bases, made on first use by the mixed method
    double *AsT = nullptr;  // the same bases transposed (mixed method)
    unsigned char *Bsl = nullptr;  // the grid bases as bf16 slices for the tensor-core products (DECAES_PREC_MIXED_TC)
    std::vector<double> h_t2, h_angles;
    size_t bytes = 0;
    long last_use = 0;
    int pins = 0;  // prepared batches using this basis (not evicted while > 0)
};

// Autotuning record per problem shape: warps per block of the voxel kernel
// and the measured cost per voxel.
struct TuneKey {
    int m, n, K, reg, mixed, beta180, legacy;
    bool operator<(const TuneKey &o) const {
        return std::tie(m, n, K, reg, mixed, beta180, legacy) < std::tie(o.m, o.n, o.K, o.reg, o.mixed, o.beta180, o.legacy);
    }
};
struct Tune {
    int wpb = 1;
    int bps = 0;  // resident blocks per SM of the persistent grid (0: as many as fit)
    double us_per_voxel = 0;
};

}  // namespace

// Voxel-list positions per tensor-core product launch (its F buffer holds
// this many rows of K*nT2 floats), and the launches whose time is recorded.
constexpr long kTcChunk = 1L << 19;
constexpr int kTcEvents = 16;

struct decaes_ctx {
    int device = 0;
    size_t budget = 0, used = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[8];
    std::string err;
    decaes_stats stats{};
    std::map<std::string, DevBuf> bufs;
    std::map<BasisKey, Basis> bases;
    long tick = 0;
    int sms = 0;
    size_t smem_optin = 0;
    std::map<TuneKey, Tune> tune;
    int force_wpb = 0;  // autotuner trials
    int force_bps = 0;
    int tc_chunks = 0;                 // tensor-core product launches of the last call
    cudaEvent_t tc_ev[2 * kTcEvents];  // their start/end events (the first kTcEvents)
    std::mutex mu;
};

namespace {

int fail(decaes_ctx *c, int code, const std::string &msg) {
    if (c) c->err = msg;
    return code;
}
#define CK(call)                                                                             \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess) return fail(ctx, DECAES_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// Grow-only named device buffers, accounted against the HBM budget.
int buf(decaes_ctx *ctx, const std::string &name, size_t bytes, void **out) {
    DevBuf &b = ctx->bufs[name];
    if (b.bytes < bytes) {
        if (b.p) { cudaFree(b.p); ctx->used -= b.bytes; b.p = nullptr; b.bytes = 0; }
        if (ctx->used + bytes > ctx->budget)
            return fail(ctx, DECAES_ENOMEM, "device allocation of " + std::to_string(bytes) + " bytes for '" + name +
                                                "' exceeds the context's HBM budget");
        cudaError_t e = cudaMalloc(&b.p, bytes);
        if (e != cudaSuccess) return fail(ctx, DECAES_ECUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
        b.bytes = bytes;
        ctx->used += bytes;
    }
    *out = b.p;
    return DECAES_OK;
}

size_t esize(int dtype) { return dtype == DECAES_F32 ? 4 : 8; }

// The mixed method, with the grid products from the CUDA cores or the tensor cores.
bool is_mixed(const decaes_t2map_opts &o) { return o.precision == DECAES_PREC_MIXED || o.precision == DECAES_PREC_MIXED_TC; }

// Resident per-parameter basis: T2 grid, angle grid, As and dAs (or the fixed basis).
int get_basis(decaes_ctx *ctx, const decaes_t2map_opts &o, Basis **out) {
    const bool fixed = !std::isnan(o.SetFlipAngle);
    BasisKey key{o.nTE, o.nT2, fixed ? 1 : o.nRefAngles, o.RefConAngle == 180.0, o.TE, o.T1, o.T2Range[0], o.T2Range[1],
                 fixed ? 0.0 : o.MinRefAngle, o.RefConAngle, fixed ? o.SetFlipAngle : -1.0};
    auto it = ctx->bases.find(key);
    if (it != ctx->bases.end()) {
        it->second.last_use = ++ctx->tick;
        *out = &it->second;
        return DECAES_OK;
    }
    // keep at most 8 keys resident, evicting the least recently used one that
    // no batch holds (a batch may hold more; the HBM budget bounds them)
    auto lru = ctx->bases.end();
    if (ctx->bases.size() >= 8)
        for (auto i = ctx->bases.begin(); i != ctx->bases.end(); ++i)
            if (i->second.pins == 0 && (lru == ctx->bases.end() || i->second.last_use < lru->second.last_use)) lru = i;
    if (lru != ctx->bases.end()) {
        Basis &b = lru->second;
        cudaFree(b.t2); cudaFree(b.logt2); cudaFree(b.angles); cudaFree(b.As); cudaFree(b.dAs); cudaFree(b.fixed);
        cudaFree(b.Gs); cudaFree(b.AsT); cudaFree(b.Bsl);
        ctx->used -= b.bytes;
        ctx->bases.erase(lru);
    }
    const int m = o.nTE, n = o.nT2, K = key.K;
    Basis b;
    b.h_t2 = dh::julia_logrange(o.T2Range[0], o.T2Range[1], n);
    std::vector<double> logt2(n);
    for (int j = 0; j < n; ++j) logt2[j] = std::log(b.h_t2[j]);
    b.h_angles = fixed ? std::vector<double>{o.SetFlipAngle} : dh::julia_range(o.MinRefAngle, 180.0, K);
    size_t mnk = (size_t)m * n * K;
    b.bytes = sizeof(double) * (2 * n + K + (fixed ? (size_t)m * n : 2 * mnk));
    if (ctx->used + b.bytes > ctx->budget) return fail(ctx, DECAES_ENOMEM, "resident basis exceeds the HBM budget");
    CK(cudaMalloc(&b.t2, sizeof(double) * n));
    CK(cudaMalloc(&b.logt2, sizeof(double) * n));
    CK(cudaMalloc(&b.angles, sizeof(double) * K));
    CK(cudaMemcpyAsync(b.t2, b.h_t2.data(), sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(b.logt2, logt2.data(), sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(b.angles, b.h_angles.data(), sizeof(double) * K, cudaMemcpyHostToDevice, ctx->stream));
    const int beta180 = o.RefConAngle == 180.0;
    if (fixed) {
        CK(cudaMalloc(&b.fixed, sizeof(double) * m * n));
        void *work;
        if (int rc = buf(ctx, "epgwork", sizeof(double) * 3 * (size_t)m * n, &work)) return rc;
        dk::k_basis_fixed<<<(n + 63) / 64, 64, 0, ctx->stream>>>(m, n, o.SetFlipAngle, o.TE, o.T1, beta180, o.RefConAngle,
                                                                 b.t2, b.fixed, (double *)work);
    } else {
        CK(cudaMalloc(&b.As, sizeof(double) * mnk));
        CK(cudaMalloc(&b.dAs, sizeof(double) * mnk));
        void *work;
        if (int rc = buf(ctx, "epgwork", sizeof(dx::Dual) * 4 * (size_t)m * n * K, &work)) return rc;
        dk::k_ensemble<<<(n * K + 63) / 64, 64, 0, ctx->stream>>>(m, n, K, o.TE, o.T1, beta180, o.RefConAngle, b.t2,
                                                                  b.angles, b.As, b.dAs, (dx::Dual *)work);
    }
    CK(cudaGetLastError());
    // callers may enqueue the solve on another stream: the basis is complete
    // before any of them can read it
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->used += b.bytes;
    b.last_use = ++ctx->tick;
    auto res = ctx->bases.emplace(key, b);
    *out = &res.first->second;
    return DECAES_OK;
}

struct OutMap {  // device double buffers for each output
    double *dist, *gdn, *ggm, *gva, *fnr, *snr, *alpha, *resnorm, *decaycurve, *mu, *chi2f, *basis;
    double *sfr, *sgm, *mfr, *mgm;
    size_t total;
};

// Core: everything on device pointers; host-buffer entry points wrap it with copies.
// Shape limits and the resident basis of one volume (plus the mixed method's
// Gram matrices, made on first use).
int prepare_basis(decaes_ctx *ctx, const decaes_t2map_opts &o, cudaStream_t st, Basis **out, int *launches) {
    const int m = o.nTE, n = o.nT2;
    if (m > 128) return fail(ctx, DECAES_EINVAL, "nTE > 128 is not supported by libdecaes_gpu");
    if (n > 256) return fail(ctx, DECAES_EINVAL, "nT2 > 256 is not supported by libdecaes_gpu");
    const bool fixed = !std::isnan(o.SetFlipAngle);
    if (!fixed && o.nRefAngles > 256) return fail(ctx, DECAES_EINVAL, "nRefAngles > 256 is not supported by libdecaes_gpu");
    const bool mixed = is_mixed(o);
    if (mixed && n > dk::kGramMaxN)
        return fail(ctx, DECAES_EINVAL, "precision = mixed supports nT2 <= " + std::to_string(dk::kGramMaxN));
    Basis *B;
    if (int rc = get_basis(ctx, o, &B)) return rc;
    if (mixed && !B->Gs) {
        const int K = fixed ? 1 : o.nRefAngles;
        const size_t gb = sizeof(double) * (size_t)K * (n * (n + 1) / 2), tb = sizeof(double) * (size_t)K * m * n;
        if (ctx->used + gb + tb > ctx->budget) return fail(ctx, DECAES_ENOMEM, "Gram matrices exceed the HBM budget");
        CK(cudaMalloc(&B->Gs, gb));
        CK(cudaMalloc(&B->AsT, tb));
        B->bytes += gb + tb;
        ctx->used += gb + tb;
        dk::k_gram_grid<<<K, 256, 0, ctx->stream>>>(m, n, fixed ? B->fixed : B->As, B->Gs, B->AsT);
        ++*launches;
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(ctx->stream));
    }
    if (o.precision == DECAES_PREC_MIXED_TC && !fixed && !B->Bsl) {
        const int K = o.nRefAngles;
        const size_t sb = (size_t)dk::tc_ntiles(K, n) * dk::kTcSlices * dk::tc_slice_bytes(dk::kTcTileN, dk::tc_mpad(m));
        if (ctx->used + sb > ctx->budget) return fail(ctx, DECAES_ENOMEM, "grid-basis slices exceed the HBM budget");
        CK(cudaMalloc(&B->Bsl, sb));
        B->bytes += sb;
        ctx->used += sb;
        CK(dk::tc_make_basis_slices(B->As, m, n, K, B->Bsl, ctx->stream));
        ++*launches;
        CK(cudaStreamSynchronize(ctx->stream));
    }
    *out = B;
    return DECAES_OK;
}

// Voxel-kernel parameters of one volume, except its queue (nvox, vidx,
// counter, stats) and scratch fields; *wsm = its shared-memory doubles per warp.
int make_params(decaes_ctx *ctx, const decaes_t2map_opts &o, const dh::T2partPlan *pp, const double *d_weights,
                const Basis *B, const void *d_image, int dtype, const void *d_b1, const OutMap &out, dk::Params &P,
                long *wsm) {
    const int m = o.nTE, n = o.nT2;
    const long V = (long)o.MatrixSize[0] * o.MatrixSize[1] * o.MatrixSize[2];
    const bool fixed = !std::isnan(o.SetFlipAngle), mixed = is_mixed(o);
    P = dk::Params{};
    P.m = m; P.n = n; P.K = fixed ? 1 : o.nRefAngles; P.M = m + n; P.lda = (m + n) | 1;
    P.reg = o.Reg; P.chi2factor = o.Chi2Factor; P.noiselevel = o.NoiseLevel;
    P.mineval = o.nRefAnglesMin; P.maxeval = o.nRefAngles; P.legacy = o.legacy ? 1 : 0;
    P.angle_mode = d_b1 ? 2 : (fixed ? 1 : 0);
    P.fixed_angle = o.SetFlipAngle;
    P.beta180 = o.RefConAngle == 180.0; P.beta = o.RefConAngle; P.TE = o.TE; P.T1 = o.T1;
    P.V = V;
    P.image = d_image; P.image_f32 = dtype == DECAES_F32; P.b1map = d_b1;
    P.t2 = B->t2; P.logt2 = B->logt2; P.angles = B->angles; P.As = B->As; P.dAs = B->dAs; P.basis_fixed = B->fixed;
    P.dist = out.dist; P.gdn = out.gdn; P.ggm = out.ggm; P.gva = out.gva; P.fnr = out.fnr; P.snr = out.snr;
    P.alpha = out.alpha; P.resnorm = out.resnorm; P.decaycurve = out.decaycurve; P.mu = out.mu; P.chi2f = out.chi2f;
    P.basis_out = out.basis;
    P.need_chi2 = o.SaveRegParam ? 1 : 0;
    if (pp) {
        P.fuse_t2part = 1; P.sp0 = pp->sp0; P.sp1 = pp->sp1; P.mp0 = pp->mp0; P.mp1 = pp->mp1; P.weights = d_weights;
        P.sfr = out.sfr; P.sgm = out.sgm; P.mfr = out.mfr; P.mgm = out.mgm;
    }
    if (mixed) {
        P.mixed = 1;
        P.Gs = B->Gs;
        P.AsT = B->AsT;
        const long rr = dk::mixed_r1_doubles(m, n) + dk::mixed_r2_doubles(m, n, o.Reg == DECAES_REG_GCV);
        P.epg_lanes_f32 = (int)std::max<long>(1, std::min<long>(32, 2 * rr / (3L * m)));
    }
    P.epg_lanes = dk::fp64_epg_lanes(m, n, P.lda);
    P.scr_stride = dk::warp_scratch_doubles(m, n, P.K);
    *wsm = mixed ? dk::warp_smem_doubles_mixed(m, n, o.Reg == DECAES_REG_GCV) : dk::warp_smem_doubles(m, n, P.lda);
    *wsm = (*wsm + 1) & ~1L;  // 16-byte aligned warp workspaces
    if ((size_t)*wsm * sizeof(double) > ctx->smem_optin)
        return fail(ctx, DECAES_EINVAL, "nTE/nT2 too large: the per-voxel workspace (" +
                                            std::to_string(*wsm * sizeof(double)) + " bytes) exceeds shared memory per block");
    return DECAES_OK;
}

// Warps per block of the voxel kernel for a problem shape (autotuned, else 1).
// Warps per block for a launch of these options: forced, else autotuned,
// else 0 (no preference).
int tuned_wpb_or0(decaes_ctx *ctx, const decaes_t2map_opts &o) {
    if (ctx->force_wpb) return ctx->force_wpb;
    const bool fixed = !std::isnan(o.SetFlipAngle);
    TuneKey k{o.nTE, o.nT2, fixed ? 1 : o.nRefAngles, o.Reg, is_mixed(o), o.RefConAngle == 180.0,
              o.legacy != 0};
    auto it = ctx->tune.find(k);
    return it == ctx->tune.end() ? 0 : it->second.wpb;
}
// Resident blocks per SM for a launch of these options: forced, else
// autotuned, else 0 (as many as fit).
int tuned_bps(decaes_ctx *ctx, const decaes_t2map_opts &o) {
    if (ctx->force_bps) return ctx->force_bps;
    const bool fixed = !std::isnan(o.SetFlipAngle);
    TuneKey k{o.nTE, o.nT2, fixed ? 1 : o.nRefAngles, o.Reg, is_mixed(o), o.RefConAngle == 180.0, o.legacy != 0};
    auto it = ctx->tune.find(k);
    return it == ctx->tune.end() ? 0 : it->second.bps;
}
int tuned_wpb(decaes_ctx *ctx, const decaes_t2map_opts &o) {
    const int w = tuned_wpb_or0(ctx, o);
    return w > 0 ? w : 1;
}

// The block size (1..max_wpb warps) that keeps the most warps resident per SM
// for a kernel whose warps each need `stride` doubles of shared memory (each
// block also reserves shared memory of its own, so one large block can hold a
// warp more than single-warp blocks do); ties go to the smaller block.
template <class Kern>
int most_warps_wpb(decaes_ctx *ctx, Kern kern, long stride, int max_wpb) {
    int best = 1, best_warps = 0;
    for (int w = 1; w <= max_wpb; ++w) {
        const size_t smem = (size_t)w * stride * sizeof(double);
        if (smem > ctx->smem_optin) break;
        if (dh::raise_smem_limit((const void *)kern, smem) != (int)cudaSuccess) break;
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * w, smem) != cudaSuccess) break;
        if (per_sm * w > best_warps) { best_warps = per_sm * w; best = w; }
    }
    return best;
}

// Persistent grid for a kernel whose warps each need `stride` doubles of
// shared memory: blocks of wpb warps, as many as fit on every SM at once, or
// at most bps of them per SM when bps > 0.
template <class Kern>
int launch_shape(decaes_ctx *ctx, Kern kern, long stride, int *wpb, int *grid, size_t *smem, int bps = 0) {
    for (; *wpb >= 1; *wpb >>= 1) {
        *smem = (size_t)*wpb * stride * sizeof(double);
        if (*smem > ctx->smem_optin) continue;
        CK((cudaError_t)dh::raise_smem_limit((const void *)kern, *smem));
        int per_sm = 0;
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * *wpb, *smem));
        if (per_sm >= 1) {
            if (bps > 0 && bps < per_sm) per_sm = bps;
            *grid = per_sm * ctx->sms;
            return DECAES_OK;
        }
    }
    return fail(ctx, DECAES_EINVAL, "voxel kernel cannot be resident with this workspace size");
}

// Core: everything on device pointers; host-buffer entry points wrap it with copies.
int run_t2map(decaes_ctx *ctx, const decaes_t2map_opts &o, const decaes_t2part_opts *po, const void *d_image,
              int dtype, const void *d_b1, OutMap &out, cudaStream_t st, int *launches) {
    const long V = (long)o.MatrixSize[0] * o.MatrixSize[1] * o.MatrixSize[2];
    const int n = o.nT2;
    int nl = 0;
    Basis *B;
    if (int rc = prepare_basis(ctx, o, st, &B, &nl)) return rc;
    // T2part plan (fused)
    dh::T2partPlan pp{};
    double *d_weights = nullptr;
    if (po) {
        std::string e = dh::t2part_plan(*po, pp);
        if (!e.empty()) return fail(ctx, DECAES_EINVAL, e);
        if (!pp.weights.empty()) {
            void *w;
            if (int rc = buf(ctx, "weights", sizeof(double) * n, &w)) return rc;
            d_weights = (double *)w;
            CK(cudaMemcpyAsync(d_weights, pp.weights.data(), sizeof(double) * n, cudaMemcpyHostToDevice, st));
        }
    }
    dk::Params P;
    long wsm = 0;
    if (int rc = make_params(ctx, o, po ? &pp : nullptr, d_weights, B, d_image, dtype, d_b1, out, P, &wsm)) return rc;
    // NaN-fill outputs
    {
        int g = std::min<long>(4L * ctx->sms * 8, (long)(out.total + 255) / 256);
        dk::k_fill<<<std::max(g, 1), 256, 0, st>>>(out.dist, (long)out.total, NAN);
        ++nl;
    }
    // compaction
    void *vidx, *cnt;
    if (int rc = buf(ctx, "vidx", sizeof(int) * (size_t)std::max<long>(V, 1), &vidx)) return rc;
    if (int rc = buf(ctx, "counters", 64, &cnt)) return rc;
    CK(cudaMemsetAsync(cnt, 0, 64, st));
    int *d_nvox = (int *)cnt, *d_counter = (int *)cnt + 1;
    unsigned long long *d_stats = (unsigned long long *)((char *)cnt + 16);
    {
        int g = (int)std::min<long>(8L * ctx->sms, (V + 255) / 256);
        dk::k_compact<<<std::max(g, 1), 256, 0, st>>>(d_image, dtype == DECAES_F32, V, o.Threshold, (int *)vidx, d_nvox);
        ++nl;
    }
    // persistent voxel kernel
    P.nvox = d_nvox; P.vidx = (const int *)vidx; P.counter = d_counter; P.stats = d_stats;
    P.smem_stride = wsm;
    int wpb = tuned_wpb(ctx, o), grid = 0;
    size_t smem = 0;
    const bool tc = o.precision == DECAES_PREC_MIXED_TC && P.angle_mode == 0 && !o.legacy;
    auto kern = o.legacy ? dk::k_voxels_legacy
                         : (tc ? dk::k_voxels_mixed_tc : (is_mixed(o) ? dk::k_voxels_mixed : dk::k_voxels_plain));
    // the plain method's large workspace: blocks of up to 8 warps can hold a
    // warp per SM more than single-warp blocks (its kernel allows 256 threads)
    if (kern == dk::k_voxels_plain && tuned_wpb_or0(ctx, o) == 0) wpb = most_warps_wpb(ctx, kern, wsm, 8);
    if (int rc = launch_shape(ctx, kern, wsm, &wpb, &grid, &smem, tuned_bps(ctx, o))) return rc;
    void *scr;
    if (int rc = buf(ctx, "scratch", sizeof(double) * (size_t)P.scr_stride * grid * wpb, &scr)) return rc;
    P.scratch = (double *)scr;
    ctx->tc_chunks = 0;
    if (tc) {
        // The search's grid products on the tensor cores, a chunk of the voxel
        // list at a time (bounded F buffer): products of the chunk, then the
        // chunk's voxel solve.  The host does not know the list's length, so
        // chunks past it launch and return at once.
        const int mpad = dk::tc_mpad(o.nTE), ntiles = dk::tc_ntiles(o.nRefAngles, n);
        const long ldF = 2L * ntiles * dk::kTcTileN;
        const long C = std::max<long>(dk::kTcTileM, std::min<long>(kTcChunk, V));
        void *F, *Fexp;
        if (int rc = buf(ctx, "tc_products", sizeof(float) * (size_t)C * ldF, &F)) return rc;
        if (int rc = buf(ctx, "tc_exponents", sizeof(int) * (size_t)C, &Fexp)) return rc;
        dk::TcParams T{};
        T.image = d_image; T.f32 = dtype == DECAES_F32; T.V = V; T.m = o.nTE; T.mpad = mpad;
        T.vidx = (const int *)vidx; T.nvox = d_nvox; T.Bsl = B->Bsl; T.ntiles = ntiles;
        T.F = (float *)F; T.ldF = ldF; T.Fexp = (int *)Fexp; T.err = (unsigned *)((char *)cnt + 32);
        P.Fk = (const float *)F; P.Fexp = (const int *)Fexp; P.ldF = ldF;
        cudaEventRecord(ctx->ev[2], st);
        for (long c0 = 0; c0 < V; c0 += C) {
            const int q = ctx->tc_chunks < kTcEvents ? ctx->tc_chunks : -1;
            T.t0 = c0; T.t1 = c0 + C;
            if (q >= 0) cudaEventRecord(ctx->tc_ev[2 * q], st);
            CK(dk::tc_grid_products(T, ctx->sms, st));
            if (q >= 0) cudaEventRecord(ctx->tc_ev[2 * q + 1], st);
            if (c0 > 0) CK(cudaMemsetAsync(d_counter, 0, sizeof(int), st));
            P.tq0 = c0; P.tq1 = c0 + C;
            kern<<<grid, 32 * wpb, smem, st>>>(P);
            nl += 2;
            ctx->tc_chunks++;
            CK(cudaGetLastError());
        }
        cudaEventRecord(ctx->ev[3], st);
    } else {
        cudaEventRecord(ctx->ev[2], st);
        kern<<<grid, 32 * wpb, smem, st>>>(P);
        cudaEventRecord(ctx->ev[3], st);
        ++nl;
    }
    CK(cudaGetLastError());
    *launches += nl;
    return DECAES_OK;
}

// FP64 output buffers of one volume carved from d (d = nullptr: size only);
// returns the doubles needed.
size_t layout_outputs(const decaes_t2map_opts &o, bool want_t2part, double *d, OutMap &om) {
    const long V = (long)o.MatrixSize[0] * o.MatrixSize[1] * o.MatrixSize[2];
    const bool fixed = !std::isnan(o.SetFlipAngle);
    size_t tot = 0;
    auto take = [&](size_t len) { size_t off = tot; tot += len; return off; };
    size_t o_dist = take((size_t)V * o.nT2), o_maps = take((size_t)V * 6);
    size_t o_res = o.SaveResidualNorm ? take(V) : SIZE_MAX;
    size_t o_dc = o.SaveDecayCurve ? take((size_t)V * o.nTE) : SIZE_MAX;
    size_t o_mu = o.SaveRegParam ? take(V) : SIZE_MAX, o_chi = o.SaveRegParam ? take(V) : SIZE_MAX;
    size_t o_basis = (o.SaveNNLSBasis && !fixed) ? take((size_t)V * o.nTE * o.nT2) : SIZE_MAX;
    size_t o_part = want_t2part ? take((size_t)V * 4) : SIZE_MAX;
    if (!d) return tot;
    auto at = [&](size_t off) { return off == SIZE_MAX ? nullptr : d + off; };
    om.dist = at(o_dist);
    om.gdn = d + o_maps; om.ggm = om.gdn + V; om.gva = om.ggm + V; om.fnr = om.gva + V; om.snr = om.fnr + V; om.alpha = om.snr + V;
    om.resnorm = at(o_res); om.decaycurve = at(o_dc); om.mu = at(o_mu); om.chi2f = at(o_chi); om.basis = at(o_basis);
    double *pt = at(o_part);
    om.sfr = pt; om.sgm = pt ? pt + V : nullptr; om.mfr = pt ? pt + 2 * V : nullptr; om.mgm = pt ? pt + 3 * V : nullptr;
    om.total = tot;
    return tot;
}

// Statistics of the tensor-core grid products of the last call (its stream
// has completed): device time of the recorded launches, launches, and the
// thread blocks that gave up a bounded wait (counter at byte 32 of cnt).
void fill_tc_stats(decaes_ctx *ctx, const void *cnt) {
    unsigned herr = 0;
    if (ctx->tc_chunks > 0) cudaMemcpy(&herr, (const char *)cnt + 32, sizeof herr, cudaMemcpyDeviceToHost);
    double gp = 0.0;
    for (int q = 0; q < std::min(ctx->tc_chunks, kTcEvents); ++q) {
        float t = 0.f;
        cudaEventElapsedTime(&t, ctx->tc_ev[2 * q], ctx->tc_ev[2 * q + 1]);
        gp += t;
    }
    ctx->stats.ms_grid_products = gp;
    ctx->stats.grid_product_launches = ctx->tc_chunks;
    ctx->stats.grid_product_failures = (int32_t)herr;
}

int out_layout(decaes_ctx *ctx, const decaes_t2map_opts &o, bool want_t2part, OutMap &om) {
    OutMap tmp;
    const size_t tot = layout_outputs(o, want_t2part, nullptr, tmp);
    void *p;
    if (int rc = buf(ctx, "outputs", sizeof(double) * tot, &p)) return rc;
    layout_outputs(o, want_t2part, (double *)p, om);
    return DECAES_OK;
}

// Copy one device double output to a caller host buffer of the call dtype.
int copy_out(decaes_ctx *ctx, const double *src, void *dst, size_t len, int dtype, cudaStream_t st, int *launches) {
    if (!dst || !src || !len) return DECAES_OK;
    if (dtype == DECAES_F64) {
        CK(cudaMemcpyAsync(dst, src, sizeof(double) * len, cudaMemcpyDeviceToHost, st));
    } else {
        void *tmp;
        if (int rc = buf(ctx, "narrow", sizeof(float) * len, &tmp)) return rc;
        int g = (int)std::min<long>(8L * ctx->sms, ((long)len + 255) / 256);
        dk::k_narrow<<<std::max(g, 1), 256, 0, st>>>(src, (float *)tmp, (long)len);
        ++*launches;
        CK(cudaMemcpyAsync(dst, tmp, sizeof(float) * len, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));  // `narrow` is reused by the next output
    }
    return DECAES_OK;
}

int check_both(decaes_ctx *ctx, const decaes_t2map_opts *mo, const decaes_t2part_opts *po, int dtype) {
    if (!ctx) return DECAES_EINVAL;
    if (dtype != DECAES_F32 && dtype != DECAES_F64) return fail(ctx, DECAES_EINVAL, "dtype must be DECAES_F32 or DECAES_F64");
    if (mo) {
        std::string e = dh::check_t2map(*mo);
        if (!e.empty()) return fail(ctx, DECAES_EINVAL, e);
    }
    if (po) {
        std::string e = dh::check_t2part(*po);
        if (!e.empty()) return fail(ctx, DECAES_EINVAL, e);
        if (mo) {
            if (po->nT2 != mo->nT2) return fail(ctx, DECAES_EINVAL, "T2part nT2 must equal T2map nT2");
            for (int d = 0; d < 3; ++d)
                if (po->MatrixSize[d] != mo->MatrixSize[d]) return fail(ctx, DECAES_EINVAL, "T2part MatrixSize must equal T2map MatrixSize");
        }
    }
    return DECAES_OK;
}

void copy_constants(const decaes_t2map_opts &o, const Basis *B, decaes_t2map_out *out, int dtype, decaes_ctx *ctx) {
    auto put = [&](void *dst, const std::vector<double> &v) {
        if (!dst) return;
        for (size_t i = 0; i < v.size(); ++i) {
            if (dtype == DECAES_F32) ((float *)dst)[i] = (float)v[i];
            else ((double *)dst)[i] = v[i];
        }
    };
    std::vector<double> te(o.nTE);
    for (int i = 0; i < o.nTE; ++i) te[i] = o.TE * (i + 1);
    put(out->echotimes, te);
    put(out->t2times, B->h_t2);
    put(out->refangleset, B->h_angles);
    const bool fixed = !std::isnan(o.SetFlipAngle);
    size_t len = (size_t)o.nTE * o.nT2 * (fixed ? 1 : o.nRefAngles);
    void *dsts[2] = {out->decaybasisset, fixed && o.SaveNNLSBasis ? out->decaybasis : nullptr};
    std::vector<double> h;
    for (void *dst : dsts) {
        if (!dst) continue;
        if (h.empty()) {
            h.resize(len);
            cudaMemcpyAsync(h.data(), fixed ? B->fixed : B->As, sizeof(double) * len, cudaMemcpyDeviceToHost, ctx->stream);
            cudaStreamSynchronize(ctx->stream);
        }
        put(dst, h);
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" decaes_ctx *decaes_create(int device, size_t hbm_budget_bytes) {
    auto *c = new decaes_ctx();
    c->device = device;
    c->budget = hbm_budget_bytes ? hbm_budget_bytes : (size_t)160 << 30;
    if (cudaSetDevice(device) != cudaSuccess) { delete c; return nullptr; }
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) { delete c; return nullptr; }
    c->sms = prop.multiProcessorCount;
    c->smem_optin = prop.sharedMemPerBlockOptin;
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) { delete c; return nullptr; }
    for (auto &e : c->ev) cudaEventCreate(&e);
    for (auto &e : c->tc_ev) cudaEventCreate(&e);
    return c;
}

extern "C" void decaes_destroy(decaes_ctx *ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    for (auto &kv : ctx->bufs) cudaFree(kv.second.p);
    for (auto &kv : ctx->bases) {
        Basis &b = kv.second;
        cudaFree(b.t2); cudaFree(b.logt2); cudaFree(b.angles); cudaFree(b.As); cudaFree(b.dAs); cudaFree(b.fixed);
        cudaFree(b.Gs); cudaFree(b.AsT); cudaFree(b.Bsl);
    }
    for (auto &e : ctx->ev) cudaEventDestroy(e);
    for (auto &e : ctx->tc_ev) cudaEventDestroy(e);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
}

extern "C" const char *decaes_last_error(const decaes_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

extern "C" int decaes_get_stats(const decaes_ctx *ctx, decaes_stats *out) {
    if (!ctx || !out) return DECAES_EINVAL;
    *out = ctx->stats;
    return DECAES_OK;
}

static int t2map_host(decaes_ctx *ctx, const decaes_t2map_opts *mo, const decaes_t2part_opts *po, const void *image,
                      int dtype, const void *b1map, decaes_t2map_out *mout, decaes_t2part_out *pout) {
    if (int rc = check_both(ctx, mo, po, dtype)) return rc;
    if (!image || !mout) return fail(ctx, DECAES_EINVAL, "image and out must not be NULL");
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, DECAES_ECUDA, "cudaSetDevice failed");
    const decaes_t2map_opts &o = *mo;
    const long V = (long)o.MatrixSize[0] * o.MatrixSize[1] * o.MatrixSize[2];
    cudaStream_t st = ctx->stream;
    int launches = 0;
    ctx->stats = decaes_stats{};
    void *d_img, *d_b1 = nullptr;
    size_t img_bytes = esize(dtype) * (size_t)V * o.nTE;
    if (int rc = buf(ctx, "image", img_bytes, &d_img)) return rc;
    if (b1map)
        if (int rc = buf(ctx, "b1map", esize(dtype) * (size_t)V, &d_b1)) return rc;
    OutMap om;
    if (int rc = out_layout(ctx, o, pout != nullptr, om)) return rc;
    CK(cudaEventRecord(ctx->ev[0], st));
    CK(cudaMemcpyAsync(d_img, image, img_bytes, cudaMemcpyHostToDevice, st));
    if (b1map) CK(cudaMemcpyAsync(d_b1, b1map, esize(dtype) * (size_t)V, cudaMemcpyHostToDevice, st));
    CK(cudaEventRecord(ctx->ev[1], st));
    if (int rc = run_t2map(ctx, o, pout ? po : nullptr, d_img, dtype, d_b1, om, st, &launches)) return rc;
    CK(cudaEventRecord(ctx->ev[4], st));
    const size_t n = o.nT2, m = o.nTE;
    struct { const double *s; void *d; size_t len; } cp[] = {
        {om.dist, mout->dist, V * n}, {om.gdn, mout->gdn, (size_t)V}, {om.ggm, mout->ggm, (size_t)V},
        {om.gva, mout->gva, (size_t)V}, {om.fnr, mout->fnr, (size_t)V}, {om.snr, mout->snr, (size_t)V},
        {om.alpha, mout->alpha, (size_t)V}, {om.resnorm, mout->resnorm, (size_t)V}, {om.decaycurve, mout->decaycurve, V * m},
        {om.mu, mout->mu, (size_t)V}, {om.chi2f, mout->chi2factor, (size_t)V}, {om.basis, mout->decaybasis, V * m * n},
    };
    for (auto &c : cp)
        if (int rc = copy_out(ctx, c.s, c.d, c.len, dtype, st, &launches)) return rc;
    if (pout) {
        struct { const double *s; void *d; } pc[] = {{om.sfr, pout->sfr}, {om.sgm, pout->sgm}, {om.mfr, pout->mfr}, {om.mgm, pout->mgm}};
        for (auto &c : pc)
            if (int rc = copy_out(ctx, c.s, c.d, (size_t)V, dtype, st, &launches)) return rc;
    }
    CK(cudaEventRecord(ctx->ev[5], st));
    CK(cudaStreamSynchronize(st));
    Basis *B;
    if (int rc = get_basis(ctx, o, &B)) return rc;
    copy_constants(o, B, mout, dtype, ctx);
    unsigned long long hs[2];
    int hn;
    void *cnt;
    buf(ctx, "counters", 64, &cnt);
    CK(cudaMemcpy(&hn, cnt, sizeof(int), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(hs, (char *)cnt + 16, sizeof hs, cudaMemcpyDeviceToHost));
    float t;
    decaes_stats &S = ctx->stats;
    S.voxels = V;
    S.voxels_processed = hn;
    S.nnls_cap_hits = (int64_t)hs[0];
    S.search_limit_hits = (int64_t)hs[1];
    cudaEventElapsedTime(&t, ctx->ev[0], ctx->ev[5]); S.ms_total = t;
    cudaEventElapsedTime(&t, ctx->ev[2], ctx->ev[3]); S.ms_solve = t;
    cudaEventElapsedTime(&t, ctx->ev[0], ctx->ev[1]); S.ms_h2d = t;
    cudaEventElapsedTime(&t, ctx->ev[4], ctx->ev[5]); S.ms_d2h = t;
    S.solve_launches = 1;
    S.kernel_launches = launches;
    fill_tc_stats(ctx, cnt);
    return DECAES_OK;
}

extern "C" int decaes_t2map(decaes_ctx *ctx, const decaes_t2map_opts *opts, const void *image, int dtype,
                            const void *b1map, decaes_t2map_out *out) {
    return t2map_host(ctx, opts, nullptr, image, dtype, b1map, out, nullptr);
}

extern "C" int decaes_t2map_t2part(decaes_ctx *ctx, const decaes_t2map_opts *mopts, const decaes_t2part_opts *popts,
                                   const void *image, int dtype, const void *b1map, decaes_t2map_out *mout,
                                   decaes_t2part_out *pout) {
    if (!popts || !pout) return fail(ctx, DECAES_EINVAL, "T2part options and outputs must not be NULL");
    return t2map_host(ctx, mopts, popts, image, dtype, b1map, mout, pout);
}

extern "C" int decaes_t2map_t2part_device(decaes_ctx *ctx, const decaes_t2map_opts *mopts, const decaes_t2part_opts *popts,
                                          const void *d_image, int dtype, const void *d_b1map, decaes_t2map_out *d_mout,
                                          decaes_t2part_out *d_pout, void *stream) {
    if (int rc = check_both(ctx, mopts, popts, dtype)) return rc;
    if (dtype != DECAES_F64 && dtype != DECAES_F32) return fail(ctx, DECAES_EINVAL, "bad dtype");
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    const decaes_t2map_opts &o = *mopts;
    const long V = (long)o.MatrixSize[0] * o.MatrixSize[1] * o.MatrixSize[2];
    int launches = 0;
    ctx->stats = decaes_stats{};
    OutMap om;
    if (int rc = out_layout(ctx, o, d_pout != nullptr, om)) return rc;
    CK(cudaEventRecord(ctx->ev[0], st));
    if (int rc = run_t2map(ctx, o, d_pout ? popts : nullptr, d_image, dtype, d_b1map, om, st, &launches)) return rc;
    // hand results to the caller's device buffers (double outputs: plain device copies;
    // float outputs: narrowing kernel)
    const size_t n = o.nT2, m = o.nTE;
    struct { const double *s; void *d; size_t len; } cp[] = {
        {om.dist, d_mout->dist, V * n}, {om.gdn, d_mout->gdn, (size_t)V}, {om.ggm, d_mout->ggm, (size_t)V},
        {om.gva, d_mout->gva, (size_t)V}, {om.fnr, d_mout->fnr, (size_t)V}, {om.snr, d_mout->snr, (size_t)V},
        {om.alpha, d_mout->alpha, (size_t)V}, {om.resnorm, d_mout->resnorm, (size_t)V},
        {om.decaycurve, d_mout->decaycurve, V * m}, {om.mu, d_mout->mu, (size_t)V}, {om.chi2f, d_mout->chi2factor, (size_t)V},
        {om.basis, d_mout->decaybasis, V * m * n},
        {om.sfr, d_pout ? d_pout->sfr : nullptr, (size_t)V}, {om.sgm, d_pout ? d_pout->sgm : nullptr, (size_t)V},
        {om.mfr, d_pout ? d_pout->mfr : nullptr, (size_t)V}, {om.mgm, d_pout ? d_pout->mgm : nullptr, (size_t)V},
    };
    // with SetFlipAngle the saved basis is the one nTE x nT2 basis of the volume
    const double *fixed_basis = nullptr;
    if (!std::isnan(o.SetFlipAngle) && o.SaveNNLSBasis && d_mout->decaybasis) {
        Basis *B;
        if (int rc = get_basis(ctx, o, &B)) return rc;
        fixed_basis = B->fixed;
    }
    for (auto &c : cp) {
        if (!c.s || !c.d) continue;
        if (dtype == DECAES_F64) {
            CK(cudaMemcpyAsync(c.d, c.s, sizeof(double) * c.len, cudaMemcpyDeviceToDevice, st));
        } else {
            int g = (int)std::min<long>(8L * ctx->sms, ((long)c.len + 255) / 256);
            dk::k_narrow<<<std::max(g, 1), 256, 0, st>>>(c.s, (float *)c.d, (long)c.len);
            ++launches;
        }
    }
    if (fixed_basis) {
        if (dtype == DECAES_F64) {
            CK(cudaMemcpyAsync(d_mout->decaybasis, fixed_basis, sizeof(double) * m * n, cudaMemcpyDeviceToDevice, st));
        } else {
            dk::k_narrow<<<(int)((m * n + 255) / 256), 256, 0, st>>>(fixed_basis, (float *)d_mout->decaybasis, (long)(m * n));
            ++launches;
        }
    }
    CK(cudaEventRecord(ctx->ev[5], st));
    CK(cudaGetLastError());
    ctx->stats.voxels = V;
    ctx->stats.solve_launches = 1;
    ctx->stats.kernel_launches = launches;
    return DECAES_OK;
}

// Completes the statistics of the last device-pointer call (synchronizes its stream).
extern "C" int decaes_sync_stats(decaes_ctx *ctx, void *stream) {
    if (!ctx) return DECAES_EINVAL;
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    CK(cudaStreamSynchronize(st));
    void *cnt;
    if (int rc = buf(ctx, "counters", 64, &cnt)) return rc;
    int hn;
    unsigned long long hs[2];
    CK(cudaMemcpy(&hn, cnt, sizeof(int), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(hs, (char *)cnt + 16, sizeof hs, cudaMemcpyDeviceToHost));
    float t;
    ctx->stats.voxels_processed = hn;
    ctx->stats.nnls_cap_hits = (int64_t)hs[0];
    ctx->stats.search_limit_hits = (int64_t)hs[1];
    cudaEventElapsedTime(&t, ctx->ev[0], ctx->ev[5]); ctx->stats.ms_total = t;
    cudaEventElapsedTime(&t, ctx->ev[2], ctx->ev[3]); ctx->stats.ms_solve = t;
    fill_tc_stats(ctx, cnt);
    return DECAES_OK;
}

extern "C" int decaes_t2part(decaes_ctx *ctx, const decaes_t2part_opts *opts, const void *dist, int dtype,
                             decaes_t2part_out *out) {
    if (int rc = check_both(ctx, nullptr, opts, dtype)) return rc;
    if (!dist || !out) return fail(ctx, DECAES_EINVAL, "dist and out must not be NULL");
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    const decaes_t2part_opts &o = *opts;
    const long V = (long)o.MatrixSize[0] * o.MatrixSize[1] * o.MatrixSize[2];
    const int n = o.nT2;
    dh::T2partPlan pp{};
    std::string e = dh::t2part_plan(o, pp);
    if (!e.empty()) return fail(ctx, DECAES_EINVAL, e);
    cudaStream_t st = ctx->stream;
    int launches = 0;
    ctx->stats = decaes_stats{};
    void *d_dist, *d_out, *d_lt, *d_w = nullptr;
    if (int rc = buf(ctx, "t2p_dist", esize(dtype) * (size_t)V * n, &d_dist)) return rc;
    if (int rc = buf(ctx, "t2p_out", sizeof(double) * 4 * (size_t)V, &d_out)) return rc;
    if (int rc = buf(ctx, "t2p_logt2", sizeof(double) * n, &d_lt)) return rc;
    if (!pp.weights.empty())
        if (int rc = buf(ctx, "t2p_w", sizeof(double) * n, &d_w)) return rc;
    CK(cudaEventRecord(ctx->ev[0], st));
    CK(cudaMemcpyAsync(d_dist, dist, esize(dtype) * (size_t)V * n, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(d_lt, pp.logt2.data(), sizeof(double) * n, cudaMemcpyHostToDevice, st));
    if (d_w) CK(cudaMemcpyAsync(d_w, pp.weights.data(), sizeof(double) * n, cudaMemcpyHostToDevice, st));
    double *po = (double *)d_out;
    {
        int g = (int)std::min<long>(8L * ctx->sms, (4 * V + 255) / 256);
        dk::k_fill<<<std::max(g, 1), 256, 0, st>>>(po, 4 * V, NAN);
        ++launches;
    }
    int g = (int)std::min<long>(8L * ctx->sms, (V + 127) / 128);
    if (dtype == DECAES_F32)
        dk::k_t2part<float><<<std::max(g, 1), 128, 0, st>>>((const float *)d_dist, V, n, pp.sp0, pp.sp1, pp.mp0, pp.mp1,
                                                             (const double *)d_lt, (const double *)d_w, po, po + V, po + 2 * V, po + 3 * V);
    else
        dk::k_t2part<double><<<std::max(g, 1), 128, 0, st>>>((const double *)d_dist, V, n, pp.sp0, pp.sp1, pp.mp0, pp.mp1,
                                                              (const double *)d_lt, (const double *)d_w, po, po + V, po + 2 * V, po + 3 * V);
    ++launches;
    CK(cudaGetLastError());
    void *dsts[4] = {out->sfr, out->sgm, out->mfr, out->mgm};
    for (int k = 0; k < 4; ++k)
        if (int rc = copy_out(ctx, po + k * V, dsts[k], (size_t)V, dtype, st, &launches)) return rc;
    CK(cudaEventRecord(ctx->ev[5], st));
    CK(cudaStreamSynchronize(st));
    float t;
    cudaEventElapsedTime(&t, ctx->ev[0], ctx->ev[5]);
    ctx->stats.voxels = V;
    ctx->stats.ms_total = t;
    ctx->stats.kernel_launches = launches;
    return DECAES_OK;
}

// ---------------------------------------------------------------------------
// Batched volumes: one persistent launch over many volumes
// ---------------------------------------------------------------------------
namespace {

struct BatchVol {
    decaes_volume v;
    Basis *B = nullptr;
    dh::T2partPlan pp{};
    bool t2part = false;
    long V = 0;
    double cost = 0;
    size_t out_off = 0, out_len = 0, vidx_off = 0, w_off = SIZE_MAX;
    OutMap om{};
    long stride = 0, scr = 0;  // shared-memory doubles per warp (Params copy + workspace), global scratch doubles
    int cls = 0;               // launch class
};

// One persistent launch of a batch: the volumes [first, first + count) of the
// queue, with the workspace of its largest volume.  Volumes are grouped into
// classes by the number of warps an SM can hold for them, so a small volume
// never runs at the occupancy of the batch's largest one.
struct BatchClass {
    int first = 0, count = 0;
    long smem_stride = 0, scr_stride = 0;
    int wpb = 1, grid = 0;
    size_t smem = 0;
    double cost = 0;
    dk::BatchKern kern = nullptr;
};

// Working memory and launch shape of a batch.  The buffers are the context's
// named buffers (one-shot call) or allocations the prepared batch owns.
struct BatchPrep {
    std::vector<BatchVol> vols;  // queue order: most expensive first
    std::vector<Basis *> pinned;  // bases held by this batch
    void unpin() {
        for (Basis *B : pinned) B->pins--;
        pinned.clear();
    }
    size_t n_out = 0, n_vidx = 0, n_w = 0;
    double *outs = nullptr, *weights = nullptr, *scratch = nullptr;
    int *vidx = nullptr, *cnt = nullptr;  // cnt: counts[nvol], offsets[nvol + 1], counter
    unsigned long long *stats = nullptr;  // 2 per volume
    dk::Params *params = nullptr;
    std::vector<BatchClass> classes;  // launched one after another
    long scr_doubles = 0;  // scratch of the largest class (classes run in sequence and share it)
    // cnt: counts[nvol], then per class offsets[count + 1], then per class one queue counter
    size_t cnt_ints() const { return 2 * vols.size() + 2 * classes.size(); }
    size_t cnt_bytes() const { return sizeof(int) * cnt_ints() + 16; }
};

// Relative cost of a voxel: the autotuner's measurement, else a model of the
// methods' measured costs (FP64 GCV ~35x the mixed method, FP64 ~5x mixed).
double voxel_cost(decaes_ctx *ctx, const decaes_t2map_opts &o) {
    const bool fixed = !std::isnan(o.SetFlipAngle), mixed = is_mixed(o);
    TuneKey k{o.nTE, o.nT2, fixed ? 1 : o.nRefAngles, o.Reg, mixed, o.RefConAngle == 180.0, o.legacy != 0};
    auto it = ctx->tune.find(k);
    if (it != ctx->tune.end() && it->second.us_per_voxel > 0) return it->second.us_per_voxel;
    double c = 1e-4 * o.nTE * o.nT2;
    if (o.Reg == DECAES_REG_LCURVE || o.Reg == DECAES_REG_GCV) c *= 3;
    if (!mixed) c *= (o.Reg == DECAES_REG_GCV) ? 35 : 5;
    if (o.legacy && !fixed) c += 0.002 * (180.0 - o.MinRefAngle);  // the sampled spline minimum (~30 us per voxel over 50-180)
    return c;
}

int batch_plan(decaes_ctx *ctx, const decaes_volume *vols, int nvol, cudaStream_t st, BatchPrep &bp, int *launches) {
    if (!vols || nvol < 1) return fail(ctx, DECAES_EINVAL, "a batch needs at least one volume");
    bp.unpin();
    bp.vols.clear();
    for (int i = 0; i < nvol; ++i) {
        const decaes_volume &v = vols[i];
        const decaes_t2part_opts *po = v.has_t2part ? &v.popts : nullptr;
        if (int rc = check_both(ctx, &v.mopts, po, v.dtype)) return rc;
        const decaes_t2map_out &o = v.d_mout;
        if (!v.d_image || !o.dist || !o.gdn || !o.ggm || !o.gva || !o.fnr || !o.snr || !o.alpha)
            return fail(ctx, DECAES_EINVAL, "batch volume " + std::to_string(i) + ": image, dist and the six maps are required");
        if (o.echotimes || o.t2times || o.refangleset || o.decaybasisset)
            return fail(ctx, DECAES_EINVAL, "batch volume " + std::to_string(i) + ": per-call constant outputs must be NULL");
        if (po && (!v.d_pout.sfr || !v.d_pout.sgm || !v.d_pout.mfr || !v.d_pout.mgm))
            return fail(ctx, DECAES_EINVAL, "batch volume " + std::to_string(i) + ": T2part outputs are required");
        BatchVol bv;
        bv.v = v;
        bv.t2part = po != nullptr;
        if (int rc = prepare_basis(ctx, v.mopts, st, &bv.B, launches)) return rc;
        bv.B->pins++;  // held while the batch is planned (and, for a prepared batch, until it is destroyed)
        bp.pinned.push_back(bv.B);
        if (po) {
            std::string e = dh::t2part_plan(*po, bv.pp);
            if (!e.empty()) return fail(ctx, DECAES_EINVAL, e);
        }
        bv.V = (long)v.mopts.MatrixSize[0] * v.mopts.MatrixSize[1] * v.mopts.MatrixSize[2];
        bv.cost = voxel_cost(ctx, v.mopts) * (double)bv.V;
        bp.vols.push_back(bv);
    }
    // workspace of each volume and its occupancy class (warps per SM at its own workspace size)
    for (BatchVol &bv : bp.vols) {
        OutMap tmp;
        layout_outputs(bv.v.mopts, bv.t2part, nullptr, tmp);
        dk::Params P;
        long wsm = 0;
        if (int rc = make_params(ctx, bv.v.mopts, nullptr, nullptr, bv.B, nullptr, bv.v.dtype, nullptr, tmp, P, &wsm)) return rc;
        bv.stride = ((long)dk::kParamsDoubles + wsm + 1) & ~1L;
        bv.scr = P.scr_stride;
        int wpb = 1, grid = 0;
        size_t smem = 0;
        if (int rc = launch_shape(ctx, dk::k_voxels_batch, bv.stride, &wpb, &grid, &smem)) return rc;
        bv.cls = grid / std::max(ctx->sms, 1);  // warps per SM at wpb = 1
    }
    // classes in decreasing occupancy, each volume's queue position by cost
    std::stable_sort(bp.vols.begin(), bp.vols.end(), [](const BatchVol &a, const BatchVol &b) {
        return a.cls != b.cls ? a.cls > b.cls : a.cost > b.cost;
    });
    bp.classes.clear();
    for (int q = 0; q < (int)bp.vols.size(); ++q) {
        if (q == 0 || bp.vols[q].cls != bp.vols[q - 1].cls) {
            BatchClass c;
            c.first = q;
            bp.classes.push_back(c);
        }
        BatchClass &c = bp.classes.back();
        c.count++;
        c.smem_stride = std::max(c.smem_stride, bp.vols[q].stride);
        c.scr_stride = std::max(c.scr_stride, bp.vols[q].scr);
        c.cost += bp.vols[q].cost;
    }
    bp.n_out = bp.n_vidx = bp.n_w = 0;
    for (BatchVol &bv : bp.vols) {
        OutMap tmp;
        bv.out_len = layout_outputs(bv.v.mopts, bv.t2part, nullptr, tmp);
        bv.out_off = bp.n_out;
        bp.n_out += (bv.out_len + 1) & ~size_t(1);
        bv.vidx_off = bp.n_vidx;
        bp.n_vidx += (size_t)std::max<long>(bv.V, 1);
        bv.w_off = SIZE_MAX;
        if (bv.t2part && !bv.pp.weights.empty()) { bv.w_off = bp.n_w; bp.n_w += bv.v.mopts.nT2; }
    }
    bp.scr_doubles = 0;
    for (BatchClass &c : bp.classes) {
        bool legacy = false, any_plain = false, any_mixed = false;
        for (int q = c.first; q < c.first + c.count; ++q) {
            const decaes_t2map_opts &o = bp.vols[q].v.mopts;
            legacy = legacy || o.legacy;
            (is_mixed(o) ? any_mixed : any_plain) = true;
        }
        c.kern = dk::batch_kernel(legacy, any_plain, any_mixed);
        c.wpb = tuned_wpb(ctx, bp.vols[c.first].v.mopts);
        if (int rc = launch_shape(ctx, c.kern, c.smem_stride, &c.wpb, &c.grid, &c.smem, tuned_bps(ctx, bp.vols[c.first].v.mopts)))
            return rc;
        bp.scr_doubles = std::max(bp.scr_doubles, c.scr_stride * c.grid * c.wpb);
    }
    return DECAES_OK;
}

size_t batch_bytes(const BatchPrep &bp, size_t *b_out, size_t *b_vidx, size_t *b_w, size_t *b_par, size_t *b_scr) {
    *b_out = sizeof(double) * std::max<size_t>(bp.n_out, 1);
    *b_vidx = sizeof(int) * std::max<size_t>(bp.n_vidx, 1);
    *b_w = sizeof(double) * std::max<size_t>(bp.n_w, 1);
    *b_par = sizeof(dk::Params) * bp.vols.size() + bp.cnt_bytes() + 16 * bp.vols.size();
    *b_scr = sizeof(double) * (size_t)std::max<long>(bp.scr_doubles, 1);
    return *b_out + *b_vidx + *b_w + *b_par + *b_scr;
}

// Points the batch at its buffers and uploads the per-volume parameters and
// T2part weights (synchronous copies: done once, before any capture).
int batch_bind(decaes_ctx *ctx, BatchPrep &bp, void *outs, void *vidx, void *w, void *par, void *scr) {
    const int nvol = (int)bp.vols.size();
    bp.outs = (double *)outs; bp.vidx = (int *)vidx; bp.weights = (double *)w; bp.scratch = (double *)scr;
    bp.params = (dk::Params *)par;
    char *tail = (char *)par + sizeof(dk::Params) * nvol;
    bp.stats = (unsigned long long *)tail;
    bp.cnt = (int *)(tail + 16 * nvol);
    std::vector<dk::Params> hp(nvol);
    for (int q = 0; q < nvol; ++q) {
        BatchVol &bv = bp.vols[q];
        layout_outputs(bv.v.mopts, bv.t2part, bp.outs + bv.out_off, bv.om);
        const double *wts = nullptr;
        if (bv.w_off != SIZE_MAX) {
            wts = bp.weights + bv.w_off;
            CK(cudaMemcpy((void *)wts, bv.pp.weights.data(), sizeof(double) * bv.v.mopts.nT2, cudaMemcpyHostToDevice));
        }
        long wsm = 0;
        if (int rc = make_params(ctx, bv.v.mopts, bv.t2part ? &bv.pp : nullptr, wts, bv.B, bv.v.d_image, bv.v.dtype,
                                 bv.v.d_b1map, bv.om, hp[q], &wsm))
            return rc;
        hp[q].vidx = bp.vidx + bv.vidx_off;
        hp[q].nvox = bp.cnt + q;
        hp[q].stats = bp.stats + 2 * q;
    }
    CK(cudaMemcpy(bp.params, hp.data(), sizeof(dk::Params) * nvol, cudaMemcpyHostToDevice));
    return DECAES_OK;
}

// The batch's launch sequence on st: memsets, kernels and device copies only,
// so it can be captured into a CUDA graph.
int batch_enqueue(decaes_ctx *ctx, const BatchPrep &bp, cudaStream_t st, int *launches) {
    const int nvol = (int)bp.vols.size(), ncls = (int)bp.classes.size();
    int *counts = bp.cnt, *offsets = bp.cnt + nvol, *counters = offsets + nvol + ncls;
    CK(cudaMemsetAsync(bp.cnt, 0, bp.cnt_bytes(), st));
    CK(cudaMemsetAsync(bp.stats, 0, 16 * nvol, st));
    for (int q = 0; q < nvol; ++q) {
        const BatchVol &bv = bp.vols[q];
        int g = (int)std::min<long>(4L * ctx->sms * 8, (long)(bv.out_len + 255) / 256);
        dk::k_fill<<<std::max(g, 1), 256, 0, st>>>(bp.outs + bv.out_off, (long)bv.out_len, NAN);
        g = (int)std::min<long>(8L * ctx->sms, (bv.V + 255) / 256);
        dk::k_compact<<<std::max(g, 1), 256, 0, st>>>(bv.v.d_image, bv.v.dtype == DECAES_F32, bv.V, bv.v.mopts.Threshold,
                                                      bp.vidx + bv.vidx_off, counts + q);
        *launches += 2;
    }
    // one persistent launch per occupancy class, in sequence (they share the scratch)
    for (int c = 0; c < ncls; ++c) {
        const BatchClass &k = bp.classes[c];
        int *off = offsets + k.first + c;  // this class's count + 1 offsets
        dk::k_batch_prefix<<<1, 32, 0, st>>>(counts + k.first, k.count, off);
        dk::BatchParams B{bp.params + k.first, off, k.count, counters + c, bp.scratch, k.scr_stride, k.smem_stride};
        k.kern<<<k.grid, 32 * k.wpb, k.smem, st>>>(B);
        *launches += 2;
    }
    for (int q = 0; q < nvol; ++q) {
        const BatchVol &bv = bp.vols[q];
        const decaes_t2map_out &d = bv.v.d_mout;
        const OutMap &om = bv.om;
        const size_t V = (size_t)bv.V, n = bv.v.mopts.nT2, m = bv.v.mopts.nTE;
        struct { const double *s; void *d; size_t len; } cp[] = {
            {om.dist, d.dist, V * n}, {om.gdn, d.gdn, V}, {om.ggm, d.ggm, V}, {om.gva, d.gva, V}, {om.fnr, d.fnr, V},
            {om.snr, d.snr, V}, {om.alpha, d.alpha, V}, {om.resnorm, d.resnorm, V}, {om.decaycurve, d.decaycurve, V * m},
            {om.mu, d.mu, V}, {om.chi2f, d.chi2factor, V}, {om.basis, d.decaybasis, V * m * n},
            {om.sfr, bv.t2part ? bv.v.d_pout.sfr : nullptr, V}, {om.sgm, bv.t2part ? bv.v.d_pout.sgm : nullptr, V},
            {om.mfr, bv.t2part ? bv.v.d_pout.mfr : nullptr, V}, {om.mgm, bv.t2part ? bv.v.d_pout.mgm : nullptr, V},
        };
        for (auto &c : cp) {
            if (!c.s || !c.d) continue;
            if (bv.v.dtype == DECAES_F64) {
                CK(cudaMemcpyAsync(c.d, c.s, sizeof(double) * c.len, cudaMemcpyDeviceToDevice, st));
            } else {
                int g = (int)std::min<long>(8L * ctx->sms, ((long)c.len + 255) / 256);
                dk::k_narrow<<<std::max(g, 1), 256, 0, st>>>(c.s, (float *)c.d, (long)c.len);
                ++*launches;
            }
        }
    }
    CK(cudaGetLastError());
    return DECAES_OK;
}

}  // namespace

struct decaes_batch {
    decaes_ctx *ctx = nullptr;
    BatchPrep bp;
    std::vector<void *> owned;
    size_t owned_bytes = 0;
    cudaStream_t cap = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int launches = 0;
};

extern "C" int decaes_t2map_t2part_batch(decaes_ctx *ctx, const decaes_volume *vols, int32_t nvol, void *stream) {
    if (!ctx) return DECAES_EINVAL;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    int launches = 0;
    ctx->stats = decaes_stats{};
    BatchPrep bp;
    struct Unpin { BatchPrep &b; ~Unpin() { b.unpin(); } } unpin{bp};
    if (int rc = batch_plan(ctx, vols, nvol, st, bp, &launches)) return rc;
    size_t b_out, b_vidx, b_w, b_par, b_scr;
    batch_bytes(bp, &b_out, &b_vidx, &b_w, &b_par, &b_scr);
    void *outs, *vidx, *w, *par, *scr;
    if (int rc = buf(ctx, "batch_outputs", b_out, &outs)) return rc;
    if (int rc = buf(ctx, "batch_vidx", b_vidx, &vidx)) return rc;
    if (int rc = buf(ctx, "batch_weights", b_w, &w)) return rc;
    if (int rc = buf(ctx, "batch_params", b_par, &par)) return rc;
    if (int rc = buf(ctx, "scratch", b_scr, &scr)) return rc;
    CK(cudaStreamSynchronize(st));  // the named buffers may still be in use by earlier work on this stream
    if (int rc = batch_bind(ctx, bp, outs, vidx, w, par, scr)) return rc;
    if (int rc = batch_enqueue(ctx, bp, st, &launches)) return rc;
    long V = 0;
    for (auto &bv : bp.vols) V += bv.V;
    ctx->stats.voxels = V;
    ctx->stats.solve_launches = 1;
    ctx->stats.kernel_launches = launches;
    return DECAES_OK;
}

extern "C" decaes_batch *decaes_batch_create(decaes_ctx *ctx, const decaes_volume *vols, int32_t nvol) {
    if (!ctx) return nullptr;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    auto *b = new decaes_batch();
    b->ctx = ctx;
    auto bail = [&](int) {
        if (b->exec) cudaGraphExecDestroy(b->exec);
        if (b->graph) cudaGraphDestroy(b->graph);
        if (b->cap) cudaStreamDestroy(b->cap);
        for (void *p : b->owned) cudaFree(p);
        ctx->used -= b->owned_bytes;
        b->bp.unpin();
        delete b;
        return (decaes_batch *)nullptr;
    };
    int launches = 0;
    if (int rc = batch_plan(ctx, vols, nvol, ctx->stream, b->bp, &launches)) return bail(rc);
    size_t sz[5];
    const size_t total = batch_bytes(b->bp, &sz[0], &sz[1], &sz[2], &sz[3], &sz[4]);
    if (ctx->used + total > ctx->budget) {
        fail(ctx, DECAES_ENOMEM, "the batch's working buffers (" + std::to_string(total) + " bytes) exceed the HBM budget");
        return bail(DECAES_ENOMEM);
    }
    void *p[5];
    for (int i = 0; i < 5; ++i) {
        cudaError_t e = cudaMalloc(&p[i], sz[i]);
        if (e != cudaSuccess) {
            fail(ctx, DECAES_ECUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
            return bail(DECAES_ECUDA);
        }
        b->owned.push_back(p[i]);
        b->owned_bytes += sz[i];
        ctx->used += sz[i];
    }
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) { fail(ctx, DECAES_ECUDA, "basis preparation failed"); return bail(0); }
    if (int rc = batch_bind(ctx, b->bp, p[0], p[1], p[2], p[3], p[4])) return bail(rc);
    if (cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking) != cudaSuccess) {
        fail(ctx, DECAES_ECUDA, "cudaStreamCreate failed");
        return bail(0);
    }
    if (cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        fail(ctx, DECAES_ECUDA, "cudaStreamBeginCapture failed");
        return bail(0);
    }
    int rc = batch_enqueue(ctx, b->bp, b->cap, &b->launches);
    cudaGraph_t g = nullptr;
    cudaError_t ee = cudaStreamEndCapture(b->cap, &g);
    b->graph = g;
    if (rc || ee != cudaSuccess || !g) {
        if (!rc) fail(ctx, DECAES_ECUDA, std::string("stream capture: ") + cudaGetErrorString(ee));
        return bail(0);
    }
    cudaError_t ie = cudaGraphInstantiate(&b->exec, b->graph, 0);
    if (ie != cudaSuccess) {
        fail(ctx, DECAES_ECUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(ie));
        return bail(0);
    }
    return b;
}

extern "C" int decaes_batch_run(decaes_batch *b, void *stream) {
    if (!b) return DECAES_EINVAL;
    decaes_ctx *ctx = b->ctx;
    cudaSetDevice(ctx->device);
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    CK(cudaGraphLaunch(b->exec, st));
    return DECAES_OK;
}

extern "C" void decaes_batch_destroy(decaes_batch *b) {
    if (!b) return;
    decaes_ctx *ctx = b->ctx;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    cudaDeviceSynchronize();
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    if (b->cap) cudaStreamDestroy(b->cap);
    for (void *p : b->owned) cudaFree(p);
    ctx->used -= b->owned_bytes;
    b->bp.unpin();
    delete b;
}

extern "C" int decaes_autotune(decaes_ctx *ctx, const decaes_t2map_opts *opts, decaes_tuning *out) {
    if (int rc = check_both(ctx, opts, nullptr, DECAES_F32)) return rc;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    decaes_t2map_opts o = *opts;
    o.MatrixSize[0] = 96; o.MatrixSize[1] = 96; o.MatrixSize[2] = 1;
    o.Threshold = 0.0;
    o.SaveResidualNorm = o.SaveDecayCurve = o.SaveRegParam = o.SaveNNLSBasis = 0;
    const long V = 96L * 96;
    decaes_mock_opts mo{};
    mo.MatrixSize[0] = 96; mo.MatrixSize[1] = 96; mo.MatrixSize[2] = 1;
    mo.nTE = o.nTE; mo.TE = o.TE; mo.T1 = 1.0;
    mo.FlipAngleRange[0] = 140; mo.FlipAngleRange[1] = 180;
    mo.MyelinT2Range[0] = 15e-3; mo.MyelinT2Range[1] = 25e-3;
    mo.MyelinFracRange[0] = 0.05; mo.MyelinFracRange[1] = 0.25;
    mo.IET2Range[0] = 60e-3; mo.IET2Range[1] = 90e-3;
    mo.CSFT2Range[0] = 1.0; mo.CSFT2Range[1] = 2.0;
    mo.CSFFracRange[0] = 0.0; mo.CSFFracRange[1] = 0.05;
    mo.AmplitudeRange[0] = 500; mo.AmplitudeRange[1] = 2000;
    mo.SNRRange[0] = 50; mo.SNRRange[1] = 200;
    mo.BackgroundFraction = 0.0; mo.BackgroundSigma = 8.0;
    std::vector<float> img((size_t)V * o.nTE);
    dh::mock_image(mo, 7, img.data(), DECAES_F32, 0);
    void *d_img;
    if (int rc = buf(ctx, "tune_image", sizeof(float) * img.size(), &d_img)) return rc;
    CK(cudaMemcpy(d_img, img.data(), sizeof(float) * img.size(), cudaMemcpyHostToDevice));
    OutMap om;
    if (int rc = out_layout(ctx, o, false, om)) return rc;
    // Launch shapes tried: warps per block (voxels in flight per block) 1, 2
    // and 4, each with as many resident blocks per SM as fit and with one and
    // two fewer (fewer warps sharing an SM's FP64 pipes, L1 and L2 share).
    const int cand[3] = {1, 2, 4};
    int best_w = 1, best_b = 0;
    double best_ms = 1e30;
    auto trial = [&](int w, int b, float *ms) -> int {
        ctx->force_wpb = w;
        ctx->force_bps = b;
        float best = 1e30f;
        for (int rep = 0; rep < 2; ++rep) {
            int nl = 0;
            if (int rc = run_t2map(ctx, o, nullptr, d_img, DECAES_F32, nullptr, om, ctx->stream, &nl)) return rc;
            CK(cudaStreamSynchronize(ctx->stream));
            float t = 0;
            cudaEventElapsedTime(&t, ctx->ev[2], ctx->ev[3]);
            if (rep > 0) best = std::min(best, t);  // first run warms the basis and the caches
        }
        *ms = best;
        return DECAES_OK;
    };
    for (int w : cand) {
        float t = 0;
        int rc = trial(w, 0, &t);
        if (rc) { ctx->force_wpb = ctx->force_bps = 0; return rc; }
        if (t < best_ms) { best_ms = t; best_w = w; best_b = 0; }
        // blocks per SM of the full grid of this block size
        Basis *B = nullptr;
        dk::Params P;
        long wsm = 0;
        int wpb = w, grid = 0;
        size_t smem = 0;
        if ((rc = get_basis(ctx, o, &B)) || (rc = make_params(ctx, o, nullptr, nullptr, B, d_img, DECAES_F32, nullptr, om, P, &wsm))) {
            ctx->force_wpb = ctx->force_bps = 0;
            return rc;
        }
        auto kern = o.legacy ? dk::k_voxels_legacy : (is_mixed(o) ? dk::k_voxels_mixed : dk::k_voxels_plain);
        if ((rc = launch_shape(ctx, kern, wsm, &wpb, &grid, &smem))) { ctx->force_wpb = ctx->force_bps = 0; return rc; }
        if (wpb != w) continue;  // this block size does not fit
        const int full = grid / ctx->sms;
        for (int b = full - 1; b >= std::max(1, full - 2); --b) {
            if ((rc = trial(w, b, &t))) { ctx->force_wpb = ctx->force_bps = 0; return rc; }
            if (t < best_ms) { best_ms = t; best_w = w; best_b = b; }
        }
    }
    ctx->force_wpb = ctx->force_bps = 0;
    const bool fixed = !std::isnan(o.SetFlipAngle);
    TuneKey k{o.nTE, o.nT2, fixed ? 1 : o.nRefAngles, o.Reg, is_mixed(o), o.RefConAngle == 180.0,
              o.legacy != 0};
    Tune t;
    t.wpb = best_w;
    t.bps = best_b;
    t.us_per_voxel = best_ms * 1e3 / (double)V;
    ctx->tune[k] = t;
    if (out) { out->warps_per_block = t.wpb; out->us_per_voxel = t.us_per_voxel; out->blocks_per_sm = t.bps; }
    return DECAES_OK;
}

// ---------------------------------------------------------------------------
// Serving loop: continuous batching of host requests
// ---------------------------------------------------------------------------
namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    int64_t id = 0;
    decaes_t2map_opts mo{};
    decaes_t2part_opts po{};
    bool t2part = false;
    const void *image = nullptr;
    int dtype = DECAES_F64;
    decaes_t2map_out mout{};
    decaes_t2part_out pout{};
    long V = 0;
    size_t img_bytes = 0, out_len = 0, footprint = 0;
    void *d_img = nullptr, *d_f32 = nullptr;
    double *d_out = nullptr, *d_w = nullptr;
    OutMap om{};
    Basis *B = nullptr;
    dh::T2partPlan pp{};
    cudaEvent_t h2d = nullptr, d2h = nullptr;
    long next_voxel = 0;  // first voxel not yet handed to a tick
    int inflight = 0;     // chunks in the running tick
    int state = 0;        // 0 queued, 1 admitted, 2 downloading, 3 done, 4 failed
    bool charged = false; // footprint counted against the server's budget
    int status = DECAES_OK;
    Clock::time_point t_submit;
};
using ReqP = std::shared_ptr<Request>;

struct Chunk {
    ReqP r;
    long v0, v1;
    double cost;
};

}  // namespace

struct decaes_server {
    decaes_ctx *ctx = nullptr;
    int64_t tick_voxels = 262144;
    size_t budget = 0, used = 0;
    cudaStream_t copy = nullptr, comp = nullptr;
    cudaEvent_t tick_t0 = nullptr, tick_t1 = nullptr;
    int cap_chunks = 2048;
    dk::Params *d_params = nullptr, *h_params = nullptr;
    int *d_cnt = nullptr, *d_vidx = nullptr;
    unsigned long long *d_stats = nullptr;
    double *d_scratch = nullptr;
    size_t scratch_bytes = 0;
    std::mutex mu;
    std::condition_variable cv, cv_done;
    std::deque<ReqP> queue;
    std::vector<ReqP> active;
    std::map<int64_t, ReqP> all;
    int64_t next_id = 1;
    bool stop = false;
    std::thread th;
    std::vector<double> lat_ms;
    int64_t submitted = 0, completed = 0, failed = 0, voxels = 0, ticks = 0;
    double busy_ms = 0;
    Clock::time_point t0;
};

namespace {

void srv_finish(decaes_server *S, const ReqP &r, int status) {
    // called with S->mu held
    if (r->d_img) cudaFreeAsync(r->d_img, S->copy);
    if (r->d_out) cudaFreeAsync(r->d_out, S->copy);
    if (r->d_f32) cudaFreeAsync(r->d_f32, S->copy);
    if (r->d_w) cudaFreeAsync(r->d_w, S->copy);
    r->d_img = r->d_f32 = nullptr;
    r->d_out = r->d_w = nullptr;
    if (r->h2d) cudaEventDestroy(r->h2d);
    if (r->d2h) cudaEventDestroy(r->d2h);
    r->h2d = r->d2h = nullptr;
    if (r->B) { r->B->pins--; r->B = nullptr; }
    if (r->charged) S->used -= r->footprint;
    r->charged = false;
    r->status = status;
    r->state = status == DECAES_OK ? 3 : 4;
    if (status == DECAES_OK) {
        S->completed++;
        S->voxels += r->V;
        S->lat_ms.push_back(std::chrono::duration<double, std::milli>(Clock::now() - r->t_submit).count());
    } else {
        S->failed++;
    }
    S->active.erase(std::remove(S->active.begin(), S->active.end(), r), S->active.end());
    S->cv_done.notify_all();
}

// Admits queued requests (FIFO) while their footprint fits: device buffers,
// NaN-filled results, image upload on the copy stream.  S->mu held.
void srv_admit(decaes_server *S) {
    decaes_ctx *ctx = S->ctx;
    while (!S->queue.empty()) {
        ReqP r = S->queue.front();
        if (r->footprint > S->budget) {
            S->queue.pop_front();
            S->active.push_back(r);
            srv_finish(S, r, DECAES_ENOMEM);
            continue;
        }
        if (S->used + r->footprint > S->budget) break;
        S->queue.pop_front();
        S->active.push_back(r);
        S->used += r->footprint;
        r->charged = true;
        int nl = 0;
        {
            std::lock_guard<std::mutex> lk(ctx->mu);
            if (prepare_basis(ctx, r->mo, ctx->stream, &r->B, &nl)) { srv_finish(S, r, DECAES_EINVAL); continue; }
            r->B->pins++;
        }
        bool ok = cudaMallocAsync(&r->d_img, r->img_bytes, S->copy) == cudaSuccess &&
                  cudaMallocAsync((void **)&r->d_out, sizeof(double) * r->out_len, S->copy) == cudaSuccess;
        if (ok && r->dtype == DECAES_F32) ok = cudaMallocAsync(&r->d_f32, sizeof(float) * r->out_len, S->copy) == cudaSuccess;
        if (ok && !r->pp.weights.empty()) {
            ok = cudaMallocAsync((void **)&r->d_w, sizeof(double) * r->mo.nT2, S->copy) == cudaSuccess &&
                 cudaMemcpyAsync(r->d_w, r->pp.weights.data(), sizeof(double) * r->mo.nT2, cudaMemcpyHostToDevice,
                                 S->copy) == cudaSuccess;
        }
        if (ok) ok = cudaMemcpyAsync(r->d_img, r->image, r->img_bytes, cudaMemcpyHostToDevice, S->copy) == cudaSuccess;
        if (ok) {
            layout_outputs(r->mo, r->t2part, r->d_out, r->om);
            int g = (int)std::min<long>(4L * ctx->sms * 8, (long)(r->out_len + 255) / 256);
            dk::k_fill<<<std::max(g, 1), 256, 0, S->copy>>>(r->d_out, (long)r->out_len, NAN);
            ok = cudaGetLastError() == cudaSuccess && cudaEventCreateWithFlags(&r->h2d, cudaEventDisableTiming) == cudaSuccess &&
                 cudaEventRecord(r->h2d, S->copy) == cudaSuccess;
        }
        if (!ok) { srv_finish(S, r, DECAES_ECUDA); continue; }
        r->state = 1;
    }
}

// Requests whose results finished downloading.  S->mu held.
void srv_retire(decaes_server *S) {
    std::vector<ReqP> done;
    for (auto &r : S->active)
        if (r->state == 2 && cudaEventQuery(r->d2h) == cudaSuccess) done.push_back(r);
    for (auto &r : done) {
        {
            std::lock_guard<std::mutex> lk(S->ctx->mu);
            copy_constants(r->mo, r->B, &r->mout, r->dtype, S->ctx);
        }
        srv_finish(S, r, DECAES_OK);
    }
}

// Downloads a finished request's results (after the tick that completed it).
void srv_download(decaes_server *S, const ReqP &r) {
    decaes_ctx *ctx = S->ctx;
    cudaStreamWaitEvent(S->copy, S->tick_t1, 0);
    const OutMap &om = r->om;
    const size_t V = (size_t)r->V, n = r->mo.nT2, m = r->mo.nTE;
    struct { const double *s; void *d; size_t len; } cp[] = {
        {om.dist, r->mout.dist, V * n}, {om.gdn, r->mout.gdn, V}, {om.ggm, r->mout.ggm, V}, {om.gva, r->mout.gva, V},
        {om.fnr, r->mout.fnr, V}, {om.snr, r->mout.snr, V}, {om.alpha, r->mout.alpha, V},
        {om.resnorm, r->mout.resnorm, V}, {om.decaycurve, r->mout.decaycurve, V * m}, {om.mu, r->mout.mu, V},
        {om.chi2f, r->mout.chi2factor, V}, {om.basis, r->mout.decaybasis, V * m * n},
        {om.sfr, r->t2part ? r->pout.sfr : nullptr, V}, {om.sgm, r->t2part ? r->pout.sgm : nullptr, V},
        {om.mfr, r->t2part ? r->pout.mfr : nullptr, V}, {om.mgm, r->t2part ? r->pout.mgm : nullptr, V},
    };
    bool ok = true;
    for (auto &c : cp) {
        if (!c.s || !c.d || !ok) continue;
        if (r->dtype == DECAES_F64) {
            ok = cudaMemcpyAsync(c.d, c.s, sizeof(double) * c.len, cudaMemcpyDeviceToHost, S->copy) == cudaSuccess;
        } else {
            float *tmp = (float *)r->d_f32 + (c.s - r->d_out);
            int g = (int)std::min<long>(8L * ctx->sms, ((long)c.len + 255) / 256);
            dk::k_narrow<<<std::max(g, 1), 256, 0, S->copy>>>(c.s, tmp, (long)c.len);
            ok = cudaMemcpyAsync(c.d, tmp, sizeof(float) * c.len, cudaMemcpyDeviceToHost, S->copy) == cudaSuccess;
        }
    }
    if (ok) ok = cudaEventCreateWithFlags(&r->d2h, cudaEventDisableTiming) == cudaSuccess &&
                 cudaEventRecord(r->d2h, S->copy) == cudaSuccess;
    if (!ok) { srv_finish(S, r, DECAES_ECUDA); return; }
    r->state = 2;
}

// Builds and launches one tick (a batched launch over chunks of the admitted
// requests, in arrival order).  Returns the chunks, empty if there was no work.
std::vector<Chunk> srv_launch_tick(decaes_server *S) {
    decaes_ctx *ctx = S->ctx;
    std::vector<Chunk> ch;
    long left = S->tick_voxels;
    std::lock_guard<std::mutex> ctx_lock(ctx->mu);
    // eligible requests (uploaded, voxels left), in arrival order
    std::vector<ReqP> el;
    for (auto &r : S->active) {
        if ((int)el.size() >= S->cap_chunks) break;
        if (r->state != 1 || r->next_voxel >= r->V) continue;
        if (cudaEventQuery(r->h2d) != cudaSuccess) continue;  // still uploading: next tick
        el.push_back(r);
    }
    if (el.empty()) return ch;
    // fair share first (a large request cannot hold back the small ones that
    // arrived after it), then what is left in arrival order; each request
    // still contributes one contiguous chunk
    std::vector<long> take(el.size(), 0);
    const long share = std::max<long>(left / (long)el.size(), 1024);
    for (size_t i = 0; i < el.size() && left > 0; ++i) {
        take[i] = std::min({share, left, el[i]->V - el[i]->next_voxel});
        left -= take[i];
    }
    for (size_t i = 0; i < el.size() && left > 0; ++i) {
        const long more = std::min(left, el[i]->V - el[i]->next_voxel - take[i]);
        take[i] += more;
        left -= more;
    }
    for (size_t i = 0; i < el.size(); ++i) {
        if (take[i] <= 0) continue;
        ReqP &r = el[i];
        ch.push_back(Chunk{r, r->next_voxel, r->next_voxel + take[i], voxel_cost(ctx, r->mo) * (double)take[i]});
        r->next_voxel += take[i];
        r->inflight++;
    }
    if (ch.empty()) return ch;
    // each chunk's workspace and occupancy class (as for batches: one
    // persistent launch per class, so small shapes keep their occupancy)
    const int nq = (int)ch.size();
    std::vector<long> stride(nq), scr(nq);
    std::vector<int> cls(nq);
    bool ok = true;
    for (int q = 0; q < nq && ok; ++q) {
        dk::Params P;
        long wsm = 0;
        ok = make_params(ctx, ch[q].r->mo, nullptr, nullptr, ch[q].r->B, nullptr, ch[q].r->dtype, nullptr, ch[q].r->om, P,
                         &wsm) == DECAES_OK;
        stride[q] = ((long)dk::kParamsDoubles + wsm + 1) & ~1L;
        scr[q] = P.scr_stride;
        int wpb = 1, grid = 0;
        size_t smem = 0;
        ok = ok && launch_shape(ctx, dk::k_voxels_batch, stride[q], &wpb, &grid, &smem) == DECAES_OK;
        cls[q] = grid / std::max(ctx->sms, 1);
    }
    std::vector<int> order(nq);
    for (int q = 0; q < nq; ++q) order[q] = q;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        return cls[a] != cls[b] ? cls[a] > cls[b] : ch[a].cost > ch[b].cost;
    });
    {
        std::vector<Chunk> c2;
        std::vector<long> s2, r2;
        std::vector<int> k2;
        for (int q : order) { c2.push_back(ch[q]); s2.push_back(stride[q]); r2.push_back(scr[q]); k2.push_back(cls[q]); }
        ch.swap(c2); stride.swap(s2); scr.swap(r2); cls.swap(k2);
    }
    std::vector<BatchClass> classes;
    long voff = 0;
    for (int q = 0; q < nq && ok; ++q) {
        const Chunk &c = ch[q];
        long wsm = 0;
        ok = make_params(ctx, c.r->mo, c.r->t2part ? &c.r->pp : nullptr, c.r->d_w, c.r->B, c.r->d_img, c.r->dtype,
                         nullptr, c.r->om, S->h_params[q], &wsm) == DECAES_OK;
        S->h_params[q].vidx = S->d_vidx + voff;
        S->h_params[q].nvox = S->d_cnt + q;
        S->h_params[q].stats = S->d_stats + 2 * q;
        voff += c.v1 - c.v0;
        if (q == 0 || cls[q] != cls[q - 1]) {
            BatchClass k;
            k.first = q;
            classes.push_back(k);
        }
        BatchClass &k = classes.back();
        k.count++;
        k.smem_stride = std::max(k.smem_stride, stride[q]);
        k.scr_stride = std::max(k.scr_stride, scr[q]);
    }
    long scr_doubles = 0;
    for (BatchClass &k : classes) {
        if (!ok) break;
        bool legacy = false, any_plain = false, any_mixed = false;
        for (int q = k.first; q < k.first + k.count; ++q) {
            legacy = legacy || ch[q].r->mo.legacy;
            (is_mixed(ch[q].r->mo) ? any_mixed : any_plain) = true;
        }
        k.kern = dk::batch_kernel(legacy, any_plain, any_mixed);
        k.wpb = tuned_wpb(ctx, ch[k.first].r->mo);
        ok = launch_shape(ctx, k.kern, k.smem_stride, &k.wpb, &k.grid, &k.smem, tuned_bps(ctx, ch[k.first].r->mo)) == DECAES_OK;
        scr_doubles = std::max(scr_doubles, k.scr_stride * k.grid * k.wpb);
    }
    const size_t need = sizeof(double) * (size_t)scr_doubles;
    if (ok && need > S->scratch_bytes) {
        if (S->d_scratch) cudaFreeAsync(S->d_scratch, S->comp);
        S->d_scratch = nullptr;
        ok = cudaMallocAsync((void **)&S->d_scratch, need, S->comp) == cudaSuccess;
        S->scratch_bytes = ok ? need : 0;
    }
    cudaStream_t st = S->comp;
    const int ncls = (int)classes.size();
    int *counts = S->d_cnt, *offsets = S->d_cnt + nq, *counters = offsets + nq + ncls;
    if (ok) ok = cudaMemcpyAsync(S->d_params, S->h_params, sizeof(dk::Params) * nq, cudaMemcpyHostToDevice, st) == cudaSuccess &&
                 cudaMemsetAsync(S->d_cnt, 0, sizeof(int) * (2 * nq + 2 * ncls), st) == cudaSuccess &&
                 cudaMemsetAsync(S->d_stats, 0, 16 * nq, st) == cudaSuccess;
    if (ok) {
        cudaEventRecord(S->tick_t0, st);
        long vo = 0;
        for (int q = 0; q < nq; ++q) {
            const Chunk &c = ch[q];
            cudaStreamWaitEvent(st, c.r->h2d, 0);
            int g = (int)std::min<long>(8L * ctx->sms, (c.v1 - c.v0 + 255) / 256);
            dk::k_compact_range<<<std::max(g, 1), 256, 0, st>>>(c.r->d_img, c.r->dtype == DECAES_F32, c.v0, c.v1,
                                                                c.r->mo.Threshold, S->d_vidx + vo, counts + q);
            vo += c.v1 - c.v0;
        }
        for (int c = 0; c < ncls; ++c) {
            const BatchClass &k = classes[c];
            int *off = offsets + k.first + c;
            dk::k_batch_prefix<<<1, 32, 0, st>>>(counts + k.first, k.count, off);
            dk::BatchParams B{S->d_params + k.first, off, k.count, counters + c, S->d_scratch, k.scr_stride, k.smem_stride};
            k.kern<<<k.grid, 32 * k.wpb, k.smem, st>>>(B);
        }
        ok = cudaGetLastError() == cudaSuccess && cudaEventRecord(S->tick_t1, st) == cudaSuccess;
    }
    if (!ok) {
        cudaStreamSynchronize(S->comp);  // nothing of the failed tick may still read the requests' buffers
        for (auto &c : ch) {
            c.r->inflight--;
            if (c.r->state == 1) srv_finish(S, c.r, DECAES_ECUDA);
        }
        ch.clear();
    }
    return ch;
}

void srv_loop(decaes_server *S) {
    cudaSetDevice(S->ctx->device);
    std::unique_lock<std::mutex> lk(S->mu);
    for (;;) {
        srv_admit(S);
        srv_retire(S);
        std::vector<Chunk> ch = srv_launch_tick(S);
        if (!ch.empty()) {
            S->ticks++;
            // while the tick runs: admit (uploads overlap the solve) and retire downloads
            while (cudaEventQuery(S->tick_t1) == cudaErrorNotReady) {
                srv_admit(S);
                srv_retire(S);
                S->cv.wait_for(lk, std::chrono::microseconds(200));
            }
            float t = 0;
            if (cudaEventElapsedTime(&t, S->tick_t0, S->tick_t1) == cudaSuccess) S->busy_ms += t;
            const bool tick_ok = cudaEventQuery(S->tick_t1) == cudaSuccess;
            for (auto &c : ch) {
                c.r->inflight--;
                if (c.r->state != 1) continue;
                if (!tick_ok) { srv_finish(S, c.r, DECAES_ECUDA); continue; }
                if (c.r->next_voxel >= c.r->V && c.r->inflight == 0) srv_download(S, c.r);
            }
            continue;
        }
        bool downloading = false;
        for (auto &r : S->active) downloading |= r->state == 2;
        if (S->stop && S->queue.empty() && S->active.empty()) break;
        S->cv.wait_for(lk, std::chrono::microseconds(downloading || !S->active.empty() ? 200 : 2000));
    }
}

}  // namespace

extern "C" decaes_server *decaes_server_create(decaes_ctx *ctx, const decaes_server_opts *opts) {
    if (!ctx) return nullptr;
    auto *S = new decaes_server();
    S->ctx = ctx;
    if (opts && opts->tick_voxels > 0) S->tick_voxels = opts->tick_voxels;
    S->budget = (opts && opts->hbm_budget_bytes) ? opts->hbm_budget_bytes : (size_t)160 << 30;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    bool ok = cudaStreamCreateWithFlags(&S->copy, cudaStreamNonBlocking) == cudaSuccess &&
              cudaStreamCreateWithFlags(&S->comp, cudaStreamNonBlocking) == cudaSuccess &&
              cudaEventCreate(&S->tick_t0) == cudaSuccess && cudaEventCreate(&S->tick_t1) == cudaSuccess &&
              cudaMalloc(&S->d_params, sizeof(dk::Params) * S->cap_chunks) == cudaSuccess &&
              cudaMallocHost(&S->h_params, sizeof(dk::Params) * S->cap_chunks) == cudaSuccess &&
              cudaMalloc(&S->d_cnt, sizeof(int) * (4 * S->cap_chunks + 2)) == cudaSuccess &&
              cudaMalloc(&S->d_stats, 16 * S->cap_chunks) == cudaSuccess &&
              cudaMalloc(&S->d_vidx, sizeof(int) * (size_t)S->tick_voxels) == cudaSuccess;
    if (!ok) {
        fail(ctx, DECAES_ECUDA, "server set-up failed");
        if (S->d_params) cudaFree(S->d_params);
        if (S->h_params) cudaFreeHost(S->h_params);
        if (S->d_cnt) cudaFree(S->d_cnt);
        if (S->d_stats) cudaFree(S->d_stats);
        if (S->d_vidx) cudaFree(S->d_vidx);
        if (S->copy) cudaStreamDestroy(S->copy);
        if (S->comp) cudaStreamDestroy(S->comp);
        delete S;
        return nullptr;
    }
    S->t0 = Clock::now();
    S->th = std::thread(srv_loop, S);
    return S;
}

extern "C" int64_t decaes_server_submit(decaes_server *S, const decaes_t2map_opts *mopts, const decaes_t2part_opts *popts,
                                        const void *image, int dtype, decaes_t2map_out *mout, decaes_t2part_out *pout) {
    if (!S || !mopts || !image || !mout) return -DECAES_EINVAL;
    if ((popts == nullptr) != (pout == nullptr)) return -DECAES_EINVAL;
    decaes_ctx *ctx = S->ctx;
    {
        std::lock_guard<std::mutex> lk(ctx->mu);
        if (int rc = check_both(ctx, mopts, popts, dtype)) return -rc;
    }
    auto r = std::make_shared<Request>();
    r->mo = *mopts;
    r->t2part = popts != nullptr;
    if (popts) {
        r->po = *popts;
        std::string e = dh::t2part_plan(*popts, r->pp);
        if (!e.empty()) { std::lock_guard<std::mutex> lk(ctx->mu); fail(ctx, DECAES_EINVAL, e); return -DECAES_EINVAL; }
    }
    r->image = image;
    r->dtype = dtype;
    r->mout = *mout;
    if (pout) r->pout = *pout;
    r->V = (long)mopts->MatrixSize[0] * mopts->MatrixSize[1] * mopts->MatrixSize[2];
    r->img_bytes = esize(dtype) * (size_t)r->V * mopts->nTE;
    OutMap tmp;
    r->out_len = layout_outputs(r->mo, r->t2part, nullptr, tmp);
    r->footprint = r->img_bytes + sizeof(double) * r->out_len + (dtype == DECAES_F32 ? sizeof(float) * r->out_len : 0) +
                   sizeof(double) * mopts->nT2 + 4096;
    r->t_submit = Clock::now();
    std::lock_guard<std::mutex> lk(S->mu);
    r->id = S->next_id++;
    S->all[r->id] = r;
    S->queue.push_back(r);
    S->submitted++;
    S->cv.notify_all();
    return r->id;
}

extern "C" int decaes_server_poll(decaes_server *S, int64_t id) {
    if (!S) return -DECAES_EINVAL;
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->all.find(id);
    if (it == S->all.end()) return -DECAES_EINVAL;
    const Request &r = *it->second;
    if (r.state == 3) return 1;
    if (r.state == 4) return -r.status;
    return 0;
}

extern "C" int decaes_server_wait(decaes_server *S, int64_t id) {
    if (!S) return DECAES_EINVAL;
    std::unique_lock<std::mutex> lk(S->mu);
    auto it = S->all.find(id);
    if (it == S->all.end()) return DECAES_EINVAL;
    ReqP r = it->second;
    S->cv_done.wait(lk, [&] { return r->state >= 3; });
    return r->status;
}

extern "C" int decaes_server_get_stats(decaes_server *S, decaes_server_stats *out) {
    if (!S || !out) return DECAES_EINVAL;
    std::lock_guard<std::mutex> lk(S->mu);
    decaes_server_stats st{};
    st.submitted = S->submitted; st.completed = S->completed; st.failed = S->failed;
    st.voxels = S->voxels; st.ticks = S->ticks; st.busy_ms = S->busy_ms;
    st.wall_ms = std::chrono::duration<double, std::milli>(Clock::now() - S->t0).count();
    if (!S->lat_ms.empty()) {
        std::vector<double> l = S->lat_ms;
        std::sort(l.begin(), l.end());
        auto q = [&](double p) { return l[std::min(l.size() - 1, (size_t)std::floor(p * (l.size() - 1) + 0.5))]; };
        st.p50_ms = q(0.50);
        st.p99_ms = q(0.99);
        st.max_ms = l.back();
        double s = 0;
        for (double v : l) s += v;
        st.mean_ms = s / l.size();
    }
    *out = st;
    return DECAES_OK;
}

extern "C" int decaes_server_reset_stats(decaes_server *S) {
    if (!S) return DECAES_EINVAL;
    std::lock_guard<std::mutex> lk(S->mu);
    S->lat_ms.clear();
    S->submitted = S->completed = S->failed = S->voxels = S->ticks = 0;
    S->busy_ms = 0;
    S->t0 = Clock::now();
    return DECAES_OK;
}

extern "C" void decaes_server_destroy(decaes_server *S) {
    if (!S) return;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
        S->cv.notify_all();
    }
    if (S->th.joinable()) S->th.join();
    cudaSetDevice(S->ctx->device);
    cudaStreamSynchronize(S->copy);
    cudaStreamSynchronize(S->comp);
    if (S->d_scratch) cudaFreeAsync(S->d_scratch, S->comp);
    cudaStreamSynchronize(S->comp);
    cudaFree(S->d_params);
    cudaFreeHost(S->h_params);
    cudaFree(S->d_cnt);
    cudaFree(S->d_stats);
    cudaFree(S->d_vidx);
    cudaEventDestroy(S->tick_t0);
    cudaEventDestroy(S->tick_t1);
    cudaStreamDestroy(S->copy);
    cudaStreamDestroy(S->comp);
    delete S;
}
