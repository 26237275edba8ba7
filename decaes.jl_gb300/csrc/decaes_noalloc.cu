// decaes_noalloc.cu -- decaes_t2map_t2part_noalloc: the fused T2map+T2part
// voxel solve for callers that must not allocate device memory.
//
// Who needs it: hosts that own the device memory themselves and forbid a
// library from taking more (a real-time scanner pipeline with a fixed memory
// plan, a caller inside a region where cudaMalloc is not allowed, an embedding
// runtime whose allocator is the only one permitted).  Such a caller cannot
// use decaes_t2map_t2part_device, whose context grows its own buffers with
// cudaMalloc.  Here the caller passes every input and output buffer, and all
// working memory -- counters, T2/angle grids, the angle-ensemble basis, the
// foreground voxel list and the per-warp solver scratch -- lives in one
// file-scope static device array of kStaticBytes (64 MiB).
//
// The kernels are the ones of the context path (decaes_gpu.cu), given
// addresses inside the static array instead of cudaMalloc'ed buffers, so the
// results are bit-identical to decaes_t2map_t2part_device.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "decaes_gpu.h"
#include "epg.cuh"
#include "host.h"
#include "t2map_params.cuh"

// Kernels defined in decaes_gpu.cu (launched through their host stubs).
namespace dk {
__global__ void k_ensemble(int m, int n, int K, double TE, double T1, int beta180, double beta, const double *t2,
                           const double *angles, double *As, double *dAs, dx::Dual *work);
__global__ void k_basis_fixed(int m, int n, double alpha, double TE, double T1, int beta180, double beta,
                              const double *t2, double *A, double *work);
__global__ void k_fill(double *p, long len, double v);
__global__ void k_compact(const void *image, int f32, long V, double thr, int *vidx, int *nvox);
__global__ void __launch_bounds__(256) k_voxels_plain(const __grid_constant__ Params P);
__global__ void __launch_bounds__(128) k_voxels_legacy(const __grid_constant__ Params P);
}  // namespace dk

namespace {

constexpr size_t kStaticBytes = DECAES_NOALLOC_SCRATCH_BYTES;
constexpr int kMaxDevices = 64;

// The workspace.  Every call on a device shares it and it keeps whatever the
// previous call left; the counters are cleared at the start of each call and
// everything else is fully written before it is read.
static __device__ __align__(256) unsigned char g_workspace[kStaticBytes];

struct DeviceSetup {
    unsigned long long ctx_id = 0;  // context the address was looked up in (0: none cached)
    unsigned char *base = nullptr;
    int sms = 0;
    int smem_optin = 0;
};
std::mutex g_mu;
DeviceSetup g_setup[kMaxDevices];

int fail(char *err, size_t errlen, int code, const std::string &msg) {
    if (err && errlen) {
        size_t k = std::min(errlen - 1, msg.size());
        memcpy(err, msg.data(), k);
        err[k] = 0;
    }
    return code;
}

// Identity of the calling thread's current CUDA context: unique for every
// context the process creates, so it changes when the primary context is
// re-created after cudaDeviceReset and differs between driver-API contexts
// on one device.  0 when there is no current context or the driver does not
// provide the query.  The driver functions are reached through the runtime's
// entry-point lookup, so the library does not link libcuda itself.
unsigned long long current_context_id() {
    using GetCurrent = CUresult (*)(CUcontext *);
    using GetId = CUresult (*)(CUcontext, unsigned long long *);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    static bool looked_up = false;
    if (!looked_up) {  // g_mu is held
        looked_up = true;
        void *p = nullptr, *q = nullptr;
        cudaDriverEntryPointQueryResult r1 = cudaDriverEntryPointSymbolNotFound, r2 = r1;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &r1) == cudaSuccess &&
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &q, 12000, cudaEnableDefault, &r2) == cudaSuccess &&
            r1 == cudaDriverEntryPointSuccess && r2 == cudaDriverEntryPointSuccess) {
            get_current = reinterpret_cast<GetCurrent>(p);
            get_id = reinterpret_cast<GetId>(q);
        }
        cudaGetLastError();  // a failed lookup leaves no sticky error behind
    }
    if (!get_current || !get_id) return 0;
    CUcontext c = nullptr;
    if (get_current(&c) != CUDA_SUCCESS || !c) return 0;
    unsigned long long id = 0;
    if (get_id(c, &id) != CUDA_SUCCESS) return 0;
    return id;
}

// Set-up, with the device current: look up the array's address (the lookup
// also loads this module in the current context, which is when the array is
// reserved) and the device's SM count and shared-memory limit.  The address
// belongs to the context it was looked up in, so it is cached per device
// together with that context's identity and looked up again whenever the
// current context differs (after cudaDeviceReset, or under another
// driver-API context).  Without a context identity nothing is cached and the
// lookup runs on every call.
int setup_device(int dev, DeviceSetup *out, char *err, size_t errlen) {
    if (dev < 0 || dev >= kMaxDevices) return fail(err, errlen, DECAES_EINVAL, "device ordinal out of range");
    std::lock_guard<std::mutex> lk(g_mu);
    DeviceSetup &s = g_setup[dev];
    const unsigned long long id = current_context_id();
    if (id != 0 && s.base && s.ctx_id == id) {
        *out = s;
        return DECAES_OK;
    }
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_workspace);
    if (e != cudaSuccess) return fail(err, errlen, DECAES_ECUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    int sms = 0, optin = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e != cudaSuccess) return fail(err, errlen, DECAES_ECUDA, std::string("cudaDeviceGetAttribute: ") + cudaGetErrorString(e));
    DeviceSetup fresh;
    fresh.base = static_cast<unsigned char *>(p);
    fresh.sms = sms;
    fresh.smem_optin = optin;
    fresh.ctx_id = current_context_id();  // the lookup made the device's context current if none was
    s = fresh.ctx_id ? fresh : DeviceSetup{};
    *out = fresh;
    return DECAES_OK;
}

// Bump carving of the static array, 256-byte aligned.
struct Carve {
    size_t used = 0;
    size_t take(size_t bytes) {
        size_t off = used;
        used += (bytes + 255) & ~size_t(255);
        return off;
    }
};

}  // namespace

#define NA_CK(call)                                                                                      \
    do {                                                                                                 \
        cudaError_t e_ = (call);                                                                         \
        if (e_ != cudaSuccess) return fail(err, errlen, DECAES_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

extern "C" int decaes_t2map_t2part_noalloc(const decaes_t2map_opts *mopts, const decaes_t2part_opts *popts,
                                           const void *d_image, int dtype, const void *d_b1map,
                                           const decaes_t2map_out *d_mout, const decaes_t2part_out *d_pout,
                                           void *stream, char *err, size_t errlen) {
    if (err && errlen) err[0] = 0;
    if (!mopts || !d_image || !d_mout) return fail(err, errlen, DECAES_EINVAL, "options, image and outputs must not be NULL");
    if ((popts == nullptr) != (d_pout == nullptr))
        return fail(err, errlen, DECAES_EINVAL, "T2part options and outputs must be given together");
    if (dtype != DECAES_F32 && dtype != DECAES_F64) return fail(err, errlen, DECAES_EINVAL, "dtype must be DECAES_F32 or DECAES_F64");
    const decaes_t2map_opts &o = *mopts;
    {
        std::string e = dh::check_t2map(o);
        if (!e.empty()) return fail(err, errlen, DECAES_EINVAL, e);
    }
    dh::T2partPlan pp{};
    if (popts) {
        std::string e = dh::check_t2part(*popts);
        if (!e.empty()) return fail(err, errlen, DECAES_EINVAL, e);
        if (popts->nT2 != o.nT2) return fail(err, errlen, DECAES_EINVAL, "T2part nT2 must equal T2map nT2");
        for (int d = 0; d < 3; ++d)
            if (popts->MatrixSize[d] != o.MatrixSize[d])
                return fail(err, errlen, DECAES_EINVAL, "T2part MatrixSize must equal T2map MatrixSize");
        e = dh::t2part_plan(*popts, pp);
        if (!e.empty()) return fail(err, errlen, DECAES_EINVAL, e);
    }
    const decaes_t2map_out &out = *d_mout;
    if (!out.dist || !out.gdn || !out.ggm || !out.gva || !out.fnr || !out.snr || !out.alpha)
        return fail(err, errlen, DECAES_EINVAL, "dist, gdn, ggm, gva, fnr, snr and alpha outputs are required");
    if (out.echotimes || out.t2times || out.refangleset || out.decaybasisset)
        return fail(err, errlen, DECAES_EINVAL,
                    "echotimes, t2times, refangleset and decaybasisset are not written by this entry point; pass NULL");
    if (d_pout && (!d_pout->sfr || !d_pout->sgm || !d_pout->mfr || !d_pout->mgm))
        return fail(err, errlen, DECAES_EINVAL, "sfr, sgm, mfr and mgm outputs are required with T2part options");
    // Optional outputs follow their Save* flags, as the other entry points do;
    // a buffer whose flag is off would never be written, so it is refused.
    if (out.resnorm && !o.SaveResidualNorm)
        return fail(err, errlen, DECAES_EINVAL, "resnorm is written only with SaveResidualNorm; pass NULL or set the flag");
    if (out.decaycurve && !o.SaveDecayCurve)
        return fail(err, errlen, DECAES_EINVAL, "decaycurve is written only with SaveDecayCurve; pass NULL or set the flag");
    if ((out.mu || out.chi2factor) && !o.SaveRegParam)
        return fail(err, errlen, DECAES_EINVAL, "mu and chi2factor are written only with SaveRegParam; pass NULL or set the flag");
    if (out.decaybasis && !o.SaveNNLSBasis)
        return fail(err, errlen, DECAES_EINVAL, "decaybasis is written only with SaveNNLSBasis; pass NULL or set the flag");

    if (o.precision != DECAES_PREC_FP64)
        return fail(err, errlen, DECAES_EINVAL, "this entry point runs the FP64 method only (precision = DECAES_PREC_FP64)");
    const int m = o.nTE, n = o.nT2;
    const bool fixed = !std::isnan(o.SetFlipAngle);
    const int K = fixed ? 1 : o.nRefAngles;
    const long V = (long)o.MatrixSize[0] * o.MatrixSize[1] * o.MatrixSize[2];
    if (m > 128) return fail(err, errlen, DECAES_EINVAL, "nTE > 128 is not supported by libdecaes_gpu");
    if (n > 256) return fail(err, errlen, DECAES_EINVAL, "nT2 > 256 is not supported by libdecaes_gpu");
    if (K > 256) return fail(err, errlen, DECAES_EINVAL, "nRefAngles > 256 is not supported by libdecaes_gpu");

    int dev = 0;
    NA_CK(cudaGetDevice(&dev));
    DeviceSetup ds;
    if (int rc = setup_device(dev, &ds, err, errlen)) return rc;

    // Layout of the static workspace for this call.
    const size_t mnk = (size_t)m * n * K;
    Carve cv;
    const size_t o_cnt = cv.take(256);
    const size_t o_t2 = cv.take(sizeof(double) * n), o_lt2 = cv.take(sizeof(double) * n);
    const size_t o_ang = cv.take(sizeof(double) * K), o_w = cv.take(sizeof(double) * n);
    const size_t o_As = cv.take(sizeof(double) * (fixed ? (size_t)m * n : mnk));
    const size_t o_dAs = fixed ? 0 : cv.take(sizeof(double) * mnk);
    const size_t o_vidx = cv.take(sizeof(int) * (size_t)std::max<long>(V, 1));
    const size_t o_scr = cv.take(0);  // rest: basis build work, then per-warp solver scratch
    const size_t epg_work = fixed ? sizeof(double) * 3 * (size_t)m * n : sizeof(dx::Dual) * 4 * mnk;

    dk::Params P{};
    P.m = m; P.n = n; P.K = K; P.M = m + n; P.lda = (m + n) | 1;
    const size_t smem = sizeof(double) * (size_t)dk::warp_smem_doubles(m, n, P.lda);
    if (smem > (size_t)ds.smem_optin)
        return fail(err, errlen, DECAES_EINVAL, "nTE/nT2 too large: the per-voxel workspace (" + std::to_string(smem) +
                                                    " bytes) exceeds shared memory per block");
    P.scr_stride = dk::warp_scratch_doubles(m, n, K);
    const size_t warp_bytes = sizeof(double) * (size_t)P.scr_stride;
    const size_t need_min = o_scr + std::max(warp_bytes, epg_work);
    if (need_min > kStaticBytes)
        return fail(err, errlen, DECAES_ENOMEM,
                    "problem needs " + std::to_string(need_min) + " bytes of the " + std::to_string(kStaticBytes) +
                        "-byte static workspace (grows with the voxel count, nTE*nT2*nRefAngles and nT2); "
                        "split the image into smaller slabs");
    auto kern = o.legacy ? dk::k_voxels_legacy : dk::k_voxels_plain;
    NA_CK((cudaError_t)dh::raise_smem_limit((const void *)kern, smem));
    int per_sm = 0;
    NA_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32, smem));
    if (per_sm < 1) return fail(err, errlen, DECAES_EINVAL, "voxel kernel cannot be resident with this workspace size");
    const long fit = (long)((kStaticBytes - o_scr) / warp_bytes);
    const int grid = (int)std::max<long>(1, std::min<long>((long)per_sm * ds.sms, fit));

    unsigned char *base = ds.base;
    cudaStream_t st = (cudaStream_t)stream;
    auto dptr = [&](size_t off) { return reinterpret_cast<double *>(base + off); };
    int *d_nvox = reinterpret_cast<int *>(base + o_cnt), *d_counter = d_nvox + 1;
    unsigned long long *d_stats = reinterpret_cast<unsigned long long *>(base + o_cnt + 16);

    // Grids (host-computed with Julia's range semantics) and T2part weights.
    std::vector<double> t2 = dh::julia_logrange(o.T2Range[0], o.T2Range[1], n), lt2(n);
    for (int j = 0; j < n; ++j) lt2[j] = std::log(t2[j]);
    std::vector<double> ang = fixed ? std::vector<double>{o.SetFlipAngle} : dh::julia_range(o.MinRefAngle, 180.0, K);
    NA_CK(cudaMemsetAsync(base + o_cnt, 0, 256, st));
    NA_CK(cudaMemcpyAsync(dptr(o_t2), t2.data(), sizeof(double) * n, cudaMemcpyHostToDevice, st));
    NA_CK(cudaMemcpyAsync(dptr(o_lt2), lt2.data(), sizeof(double) * n, cudaMemcpyHostToDevice, st));
    NA_CK(cudaMemcpyAsync(dptr(o_ang), ang.data(), sizeof(double) * K, cudaMemcpyHostToDevice, st));
    if (!pp.weights.empty())
        NA_CK(cudaMemcpyAsync(dptr(o_w), pp.weights.data(), sizeof(double) * n, cudaMemcpyHostToDevice, st));

    // Basis (into the static array; its build work aliases the solver scratch,
    // which stream order frees before the solve starts).
    const int beta180 = o.RefConAngle == 180.0;
    if (fixed)
        dk::k_basis_fixed<<<(n + 63) / 64, 64, 0, st>>>(m, n, o.SetFlipAngle, o.TE, o.T1, beta180, o.RefConAngle,
                                                         dptr(o_t2), dptr(o_As), dptr(o_scr));
    else
        dk::k_ensemble<<<(n * K + 63) / 64, 64, 0, st>>>(m, n, K, o.TE, o.T1, beta180, o.RefConAngle, dptr(o_t2),
                                                          dptr(o_ang), dptr(o_As), dptr(o_dAs),
                                                          reinterpret_cast<dx::Dual *>(base + o_scr));
    NA_CK(cudaGetLastError());

    // NaN-fill the caller's outputs (unprocessed voxels stay NaN).
    const size_t nm = (size_t)n, mm = (size_t)m;
    struct { void *p; size_t len; } fills[] = {
        {out.dist, V * nm}, {out.gdn, (size_t)V}, {out.ggm, (size_t)V}, {out.gva, (size_t)V}, {out.fnr, (size_t)V},
        {out.snr, (size_t)V}, {out.alpha, (size_t)V}, {out.resnorm, (size_t)V}, {out.decaycurve, V * mm},
        {out.mu, (size_t)V}, {out.chi2factor, (size_t)V},
        {fixed ? nullptr : out.decaybasis, V * mm * nm},
        {d_pout ? d_pout->sfr : nullptr, (size_t)V}, {d_pout ? d_pout->sgm : nullptr, (size_t)V},
        {d_pout ? d_pout->mfr : nullptr, (size_t)V}, {d_pout ? d_pout->mgm : nullptr, (size_t)V},
    };
    for (auto &f : fills) {
        if (!f.p || !f.len) continue;
        int g = (int)std::min<long>(4L * ds.sms * 8, ((long)f.len + 255) / 256);
        dk::k_fill<<<std::max(g, 1), 256, 0, st>>>((double *)f.p, (long)f.len, NAN);
    }
    if (fixed && o.SaveNNLSBasis && out.decaybasis)
        NA_CK(cudaMemcpyAsync(out.decaybasis, dptr(o_As), sizeof(double) * mm * nm, cudaMemcpyDeviceToDevice, st));

    // Threshold compaction into the static voxel list.
    int *vidx = reinterpret_cast<int *>(base + o_vidx);
    {
        int g = (int)std::min<long>(8L * ds.sms, (V + 255) / 256);
        dk::k_compact<<<std::max(g, 1), 256, 0, st>>>(d_image, dtype == DECAES_F32, V, o.Threshold, vidx, d_nvox);
    }

    // Persistent voxel solve.
    P.reg = o.Reg; P.chi2factor = o.Chi2Factor; P.noiselevel = o.NoiseLevel;
    P.mineval = o.nRefAnglesMin; P.maxeval = o.nRefAngles; P.legacy = o.legacy ? 1 : 0;
    P.angle_mode = d_b1map ? 2 : (fixed ? 1 : 0);
    P.fixed_angle = o.SetFlipAngle;
    P.beta180 = beta180; P.beta = o.RefConAngle; P.TE = o.TE; P.T1 = o.T1;
    P.V = V; P.nvox = d_nvox; P.vidx = vidx;
    P.image = d_image; P.image_f32 = dtype == DECAES_F32; P.b1map = d_b1map;
    P.t2 = dptr(o_t2); P.logt2 = dptr(o_lt2); P.angles = dptr(o_ang);
    P.As = fixed ? nullptr : dptr(o_As); P.dAs = fixed ? nullptr : dptr(o_dAs); P.basis_fixed = fixed ? dptr(o_As) : nullptr;
    P.counter = d_counter; P.stats = d_stats;
    P.dist = (double *)out.dist; P.gdn = (double *)out.gdn; P.ggm = (double *)out.ggm; P.gva = (double *)out.gva;
    P.fnr = (double *)out.fnr; P.snr = (double *)out.snr; P.alpha = (double *)out.alpha;
    P.resnorm = (double *)out.resnorm; P.decaycurve = (double *)out.decaycurve; P.mu = (double *)out.mu;
    P.chi2f = (double *)out.chi2factor; P.basis_out = fixed ? nullptr : (double *)out.decaybasis;
    P.need_chi2 = o.SaveRegParam ? 1 : 0;
    if (d_pout) {
        P.fuse_t2part = 1; P.sp0 = pp.sp0; P.sp1 = pp.sp1; P.mp0 = pp.mp0; P.mp1 = pp.mp1;
        P.weights = pp.weights.empty() ? nullptr : dptr(o_w);
        P.sfr = (double *)d_pout->sfr; P.sgm = (double *)d_pout->sgm; P.mfr = (double *)d_pout->mfr; P.mgm = (double *)d_pout->mgm;
    }
    P.epg_lanes = dk::fp64_epg_lanes(m, n, P.lda);
    P.scratch = dptr(o_scr);
    kern<<<grid, 32, smem, st>>>(P);
    NA_CK(cudaGetLastError());
    return DECAES_OK;
}
