/*
 * decaes_gpu.h -- C ABI of libdecaes_gpu.so, the GB300 (sm_103a) implementation
 * of DECAES.jl's voxelwise T2-distribution path.
 *
 * The entry points are what the reference's Julia API would `ccall` for the
 * path: plain pointers and sizes, caller-owned buffers, column-major (Julia)
 * array layout, no Julia or torch types.  All outputs are caller-allocated and
 * NaN-prefilled by the caller as the reference's T2Maps/T2Distributions/T2Parts
 * constructors do; the library writes only processed voxels.
 *
 * Layouts (V = MatrixSize[0]*MatrixSize[1]*MatrixSize[2]):
 *   image        V x nTE     (image[v + V*e]),  DECAES_F32 or DECAES_F64
 *   dist         V x nT2
 *   maps         V
 *   decaycurve   V x nTE
 *   decaybasis   V x nTE x nT2 (or nTE x nT2 when SetFlipAngle is given)
 *
 * Errors: every entry point returns 0 on success and a nonzero DECAES_E* code
 * otherwise; decaes_last_error() returns the message.  Option errors carry the
 * reference's assertion text (src/types.jl).
 */
#ifndef DECAES_GPU_H
#define DECAES_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { DECAES_F32 = 0, DECAES_F64 = 1 };
enum { DECAES_REG_NONE = 0, DECAES_REG_LCURVE = 1, DECAES_REG_GCV = 2, DECAES_REG_CHI2 = 3, DECAES_REG_MDP = 4 };
/* Method of the path.  FP64: the plain method, every step in IEEE binary64,
 * bitwise equal to the FP64 restatement of the reference.  MIXED: the EPG
 * recursion at the fitted angle runs in FP32 and the regularized NNLS solves
 * work on the normal equations (FP64 Gram matrix, LDL' updates, warm-started
 * active sets); root finding, curvature, the spline fit and every solve stay
 * FP64.  MIXED results differ from FP64 by |MWF| <= 1e-3 (measured p99 ~1e-5);
 * it needs nT2 <= 64.  MIXED_TC is MIXED with the flip-angle search's grid
 * products A_k'b (every grid angle, every voxel) computed beforehand as one
 * tensor-core GEMM per chunk of voxels (bf16 fixed-point slices, exact FP32
 * accumulation, ~2^-24 relative error); it applies to the single-volume entry
 * points when the flip angle is searched, and batches and the server run
 * MIXED_TC volumes as MIXED.  No counterpart in the reference (an extension). */
enum { DECAES_PREC_FP64 = 0, DECAES_PREC_MIXED = 1, DECAES_PREC_MIXED_TC = 2 };
enum {
    DECAES_OK = 0,
    DECAES_EINVAL = 1,   /* invalid option or argument (reference AssertionError) */
    DECAES_ECUDA = 2,    /* CUDA runtime error */
    DECAES_ENOMEM = 3,   /* allocation would exceed the context's HBM budget, or the
                            problem does not fit the no-allocation workspace */
    DECAES_ELEGACY = 4,  /* no longer returned (legacy = true is provided); value kept */
};

typedef struct decaes_ctx decaes_ctx;

/* Mirrors T2mapOptions{T} (src/types.jl:19-100).  Optional reference fields
 * (`Union{T,Nothing}`) use NaN for `nothing`. */
typedef struct {
    int32_t MatrixSize[3];
    int32_t nTE;
    double TE;
    int32_t nT2;
    double T2Range[2];
    double T1;
    double Threshold;
    double MinRefAngle;
    int32_t nRefAngles;
    int32_t nRefAnglesMin;
    int32_t Reg;          /* DECAES_REG_* */
    double Chi2Factor;    /* NaN = nothing */
    double NoiseLevel;    /* NaN = nothing */
    double RefConAngle;
    double SetFlipAngle;  /* NaN = nothing */
    int32_t SaveResidualNorm;
    int32_t SaveDecayCurve;
    int32_t SaveRegParam;
    int32_t SaveNNLSBasis;
    int32_t legacy;       /* legacy algorithms: spline-surrogate angle search (spline_opt_legacy),
                             chi2 by mu doubling + spline root (src/T2mapSEcorr.jl:401-403,
                             src/lsqnonneg.jl:595-636) */
    int32_t precision;    /* DECAES_PREC_* (extension; not a reference field) */
} decaes_t2map_opts;

/* Output buffers of T2mapSEcorr (src/T2mapSEcorr.jl:2-19, 64-72), all of the
 * call's dtype.  NULL skips an optional output. */
typedef struct {
    void *dist;
    void *gdn, *ggm, *gva, *fnr, *snr, *alpha;
    void *resnorm, *decaycurve, *mu, *chi2factor, *decaybasis;
    /* per-call constants: echotimes (nTE), t2times (nT2), refangleset
     * (nRefAngles, or 1 with SetFlipAngle), decaybasisset (nTE x nT2 x nRefAngles,
     * or nTE x nT2 with SetFlipAngle) */
    void *echotimes, *t2times, *refangleset, *decaybasisset;
} decaes_t2map_out;

/* Mirrors T2partOptions{T} (src/types.jl:139-172). */
typedef struct {
    int32_t MatrixSize[3];
    int32_t nT2;
    double T2Range[2];
    double SPWin[2];
    double MPWin[2];
    double Sigmoid; /* NaN = nothing */
    int32_t legacy; /* accepted; T2part has no legacy-specific arithmetic */
} decaes_t2part_opts;

typedef struct {
    void *sfr, *sgm, *mfr, *mgm;
} decaes_t2part_out;

/* Per-call statistics of the most recent call on a context. */
typedef struct {
    int64_t voxels;            /* prod(MatrixSize) */
    int64_t voxels_processed;  /* above Threshold */
    int64_t nnls_cap_hits;     /* NNLS solves that reached max_iter = 3n (reference mode = 1) */
    int64_t search_limit_hits; /* flip-angle / L-curve loops stopped by their device iteration caps */
    double ms_total;           /* device time of the whole call (CUDA events, incl. copies) */
    double ms_solve;           /* device time of the voxel-solve kernel */
    double ms_h2d, ms_d2h;     /* device time of the host<->device copies */
    int32_t solve_launches;    /* voxel-solve kernel launches of the call */
    int32_t kernel_launches;   /* all kernels launched by the call */
    double ms_grid_products;   /* DECAES_PREC_MIXED_TC: device time of the tensor-core grid products */
    int32_t grid_product_launches;
    int32_t grid_product_failures; /* their thread blocks that gave up a bounded wait (the voxels
                                      concerned then form their products on the CUDA cores) */
} decaes_stats;

/* ---- context -------------------------------------------------------------
 * One context per device; it owns device buffers, the stream and resident
 * per-parameter bases.  hbm_budget_bytes = 0 means 160 GiB.  Calls on one
 * context are serialized. */
decaes_ctx *decaes_create(int device, size_t hbm_budget_bytes);
void decaes_destroy(decaes_ctx *ctx);
const char *decaes_last_error(const decaes_ctx *ctx);
int decaes_get_stats(const decaes_ctx *ctx, decaes_stats *out);

/* Option validation with the reference's assertion messages; needs no GPU.
 * Replaces the @assert blocks of T2mapOptions (src/types.jl:28-95) and
 * T2partOptions (src/types.jl:148-168). */
int decaes_t2map_check_options(const decaes_t2map_opts *opts, char *msg, size_t msglen);
int decaes_t2part_check_options(const decaes_t2part_opts *opts, char *msg, size_t msglen);

/* T2mapSEcorr!(maps, dist, image, opts) (src/T2mapSEcorr.jl:151-196).
 * Host buffers.  b1map (V values of the call dtype) replaces the flip-angle
 * search by the given angles, as load_B1map! does (src/T2mapSEcorr.jl:56-61).
 * The plain method computes in FP64 whatever the dtype (FP32 input is widened
 * on the device, as the reference CLI does in src/main.jl:612-617); the Julia
 * API of the reference computes a Float32 image in Float32 (src/types.jl:19),
 * so for Float32 input the results here are the FP64 results rounded to
 * Float32, not the reference's single-precision ones. */
int decaes_t2map(decaes_ctx *ctx, const decaes_t2map_opts *opts, const void *image, int dtype,
                 const void *b1map, decaes_t2map_out *out);

/* T2partSEcorr(dist, opts) (src/T2partSEcorr.jl:42-71).  Host buffers. */
int decaes_t2part(decaes_ctx *ctx, const decaes_t2part_opts *opts, const void *dist, int dtype,
                  decaes_t2part_out *out);

/* T2mapSEcorr followed by T2partSEcorr on its distribution, with the T2part
 * window sums fused into the voxel-solve epilogue.  Host buffers. */
int decaes_t2map_t2part(decaes_ctx *ctx, const decaes_t2map_opts *mopts, const decaes_t2part_opts *popts,
                        const void *image, int dtype, const void *b1map, decaes_t2map_out *mout,
                        decaes_t2part_out *pout);

/* Device-pointer variants: all pointers are device addresses on the context's
 * device; `stream` is a cudaStream_t (NULL = the context's stream).  Used for
 * in-HBM throughput measurement and by callers that keep data resident. */
int decaes_t2map_t2part_device(decaes_ctx *ctx, const decaes_t2map_opts *mopts, const decaes_t2part_opts *popts,
                               const void *d_image, int dtype, const void *d_b1map, decaes_t2map_out *d_mout,
                               decaes_t2part_out *d_pout, void *stream);
/* Waits for the last device-pointer call on `stream` and completes its
 * decaes_stats (processed voxels, cap hits, device times). */
int decaes_sync_stats(decaes_ctx *ctx, void *stream);

/* ---- batched volumes -------------------------------------------------------
 * Many volumes, each with its own options (nTE, TE, nT2, regularizer, method,
 * mask), solved by ONE persistent voxel-kernel launch: the compacted voxel
 * lists of all volumes form one work queue, most expensive volume first (cost
 * per voxel from the autotuner when it has seen the shape, else a model), so
 * the end of the launch is made of cheap voxels.  No reference counterpart
 * (the reference runs one volume per call); it serves uneven workloads and the
 * serving loop.  All pointers are device addresses on the context's device;
 * each volume's image and outputs are of its `dtype`; the per-call constant
 * outputs (echotimes ... decaybasisset) must be NULL.  Results are identical
 * to one decaes_t2map_t2part_device call per volume. */
typedef struct {
    decaes_t2map_opts mopts;
    decaes_t2part_opts popts;  /* used when has_t2part != 0 */
    int32_t has_t2part;
    int32_t dtype;             /* DECAES_F32 or DECAES_F64 */
    const void *d_image;
    const void *d_b1map;       /* NULL: flip-angle search */
    decaes_t2map_out d_mout;
    decaes_t2part_out d_pout;
} decaes_volume;

/* Enqueues the batch on `stream` (NULL = the context's stream) and returns;
 * synchronize the stream before reading outputs.  decaes_get_stats reports
 * the number of kernel launches. */
int decaes_t2map_t2part_batch(decaes_ctx *ctx, const decaes_volume *vols, int32_t nvol, void *stream);

/* A batch prepared once and captured as a CUDA graph, for the same volumes
 * (same buffers and options) processed repeatedly: create validates,
 * allocates the batch's own working buffers, makes the bases resident (held
 * until destroy) and captures the launch sequence; run replays it on
 * `stream` (NULL = the context's stream).  create returns NULL on failure
 * (message in decaes_last_error(ctx)).  A prepared batch must be destroyed
 * before its context. */
typedef struct decaes_batch decaes_batch;
decaes_batch *decaes_batch_create(decaes_ctx *ctx, const decaes_volume *vols, int32_t nvol);
int decaes_batch_run(decaes_batch *batch, void *stream);
void decaes_batch_destroy(decaes_batch *batch);

/* Autotuner: times the voxel kernel on a synthetic slab of the given shape
 * and method for a set of launch shapes -- 1, 2 and 4 warps (voxels in
 * flight) per block, each with as many resident blocks per SM as fit and with
 * one and two fewer -- keeps the fastest for that (nTE, nT2, nRefAngles, Reg,
 * precision, control angle) in the context, and reports it.  Later calls,
 * batches and server ticks on the context use the tuned shape; batches also
 * use the measured cost to order their queue. */
typedef struct {
    int32_t warps_per_block;
    double us_per_voxel;       /* device time per above-threshold voxel, whole GPU */
    int32_t blocks_per_sm;     /* resident blocks per SM (0: as many as fit) */
} decaes_tuning;
int decaes_autotune(decaes_ctx *ctx, const decaes_t2map_opts *opts, decaes_tuning *out);

/* ---- serving loop -----------------------------------------------------------
 * A continuous-batching server on one context (the GPU counterpart of the
 * reference's warm-process request loop, api/decaes_server.jl:69-131).
 * decaes_server_submit queues a T2map (+ T2part) request on HOST buffers and
 * returns at once; a scheduler thread admits queued requests while their
 * device footprint fits the server's HBM budget (image, FP64 results, voxel
 * list), uploads them on a copy stream, and runs "ticks": each tick solves up
 * to `tick_voxels` voxels from every admitted request -- an equal share each
 * first, then the remainder in arrival order -- as ONE batched persistent
 * launch, so requests that arrive while the GPU is busy join the next tick
 * (a large volume does not hold back the slices behind it) and their uploads
 * and downloads overlap the solve.
 * Bases stay resident per parameter key.  Each result is identical to the
 * same request run alone.  Pinned host buffers let copies overlap; pageable
 * ones work but serialize the copies with the scheduler. */
typedef struct decaes_server decaes_server;
typedef struct {
    int64_t tick_voxels;       /* voxels per tick (0: 262144) */
    size_t hbm_budget_bytes;   /* admission budget for request buffers (0: 160 GiB) */
} decaes_server_opts;
typedef struct {
    int64_t submitted, completed, failed;
    int64_t voxels;            /* of completed requests */
    int64_t ticks;
    double p50_ms, p99_ms, mean_ms, max_ms;  /* submit-to-result latency of completed requests */
    double busy_ms;            /* device time of the ticks */
    double wall_ms;            /* since the server started */
} decaes_server_stats;
decaes_server *decaes_server_create(decaes_ctx *ctx, const decaes_server_opts *opts);
/* Returns a request id > 0, or -DECAES_E* (options are validated here). */
int64_t decaes_server_submit(decaes_server *srv, const decaes_t2map_opts *mopts, const decaes_t2part_opts *popts,
                             const void *image, int dtype, decaes_t2map_out *mout, decaes_t2part_out *pout);
/* 1 = done, 0 = pending, -DECAES_E* = failed or unknown id. */
int decaes_server_poll(decaes_server *srv, int64_t id);
/* Blocks until the request is done; returns DECAES_OK or its error code. */
int decaes_server_wait(decaes_server *srv, int64_t id);
int decaes_server_get_stats(decaes_server *srv, decaes_server_stats *out);
/* Clears the counters and latency samples (e.g. after warm-up requests); the
 * requests in flight are counted when they finish. */
int decaes_server_reset_stats(decaes_server *srv);
/* Finishes every queued request, then stops the scheduler and frees the server. */
void decaes_server_destroy(decaes_server *srv);

/* Fused T2mapSEcorr + T2partSEcorr that allocates no device memory.  This entry
 * point has no counterpart in the reference; it exists for callers that cannot
 * let a library allocate: a host with a fixed device-memory plan (a real-time
 * reconstruction pipeline, an embedding runtime whose allocator is the only
 * one allowed) or code running where cudaMalloc is not permitted.  It needs no
 * decaes_ctx.
 *
 * All pointers are device addresses on the CURRENT device; `stream` is a
 * cudaStream_t (NULL = the legacy default stream).  `d_image` (and the optional
 * `d_b1map`) are DECAES_F32 or DECAES_F64 per `dtype`; every output is FP64
 * whatever `dtype` is.  dist, gdn, ggm, gva, fnr, snr and alpha are required.
 * The optional outputs follow their Save* flags as in the other entry points:
 * resnorm (SaveResidualNorm), decaycurve (SaveDecayCurve), mu and chi2factor
 * (SaveRegParam), decaybasis (SaveNNLSBasis: V x nTE x nT2, or nTE x nT2 with
 * SetFlipAngle); a non-NULL optional buffer whose flag is off is refused with
 * DECAES_EINVAL, a NULL one whose flag is on is simply not written.
 * echotimes, t2times, refangleset and decaybasisset must be NULL.  T2part is
 * fused when `popts` and `d_pout` are given (both or neither).  The library
 * NaN-fills the outputs before the solve.  Returns before the work finishes:
 * synchronize `stream` before reading the outputs.  Error text goes to
 * `err` (`errlen` bytes, may be NULL).
 *
 * Working memory is one static device array of DECAES_NOALLOC_SCRATCH_BYTES
 * (64 MiB) per device, reserved when the CUDA module holding it is loaded (at
 * the first call under CUDA's default lazy module loading).
 * It holds the counters, grids, angle-ensemble basis (8*nTE*nT2*nRefAngles*2
 * bytes), the foreground voxel list (4 bytes per voxel) and the per-warp solver
 * scratch; a problem whose fixed part leaves no room for one warp's scratch is
 * rejected with DECAES_ENOMEM (split the image into slabs: voxels are
 * independent).  Fewer resident warps fit when the voxel list is large, which
 * lowers throughput but not the results, which are bit-identical to the FP64
 * outputs of decaes_t2map_t2part_device (for a DECAES_F32 call that entry
 * point returns these values rounded to float).
 *
 * The first call on a device does a set-up (symbol lookup of the array in the
 * current context, device attributes), and so does the first call after the
 * device's current context changes (cudaDeviceReset, or another driver-API
 * context made current); make such a call before any stream capture.
 * All calls on a device share the array and it keeps the last call's contents:
 * calls that overlap in time on one device -- from two host threads or on two
 * streams -- race on it and give undefined results.  Serialize them. */
#define DECAES_NOALLOC_SCRATCH_BYTES ((size_t)64 << 20)
int decaes_t2map_t2part_noalloc(const decaes_t2map_opts *mopts, const decaes_t2part_opts *popts,
                                const void *d_image, int dtype, const void *d_b1map,
                                const decaes_t2map_out *d_mout, const decaes_t2part_out *d_pout,
                                void *stream, char *err, size_t errlen);

/* Synthetic multi-echo image, the counterpart of mock_image
 * (src/utils.jl:606-668) with the generator used by this project's benchmarks:
 * per voxel a sum of three EPG decays (myelin, intra/extracellular, CSF) with
 * Rician noise.  Host function (no GPU); deterministic for a given seed and
 * independent of thread count. */
typedef struct {
    int32_t MatrixSize[3];
    int32_t nTE;
    double TE;
    double T1;
    double FlipAngleRange[2];   /* degrees, uniform */
    double MyelinT2Range[2];    /* seconds */
    double MyelinFracRange[2];
    double IET2Range[2];
    double CSFT2Range[2];
    double CSFFracRange[2];
    double AmplitudeRange[2];
    double SNRRange[2];         /* linear SNR; noise sigma = amplitude / SNR */
    double BackgroundFraction;  /* voxels with zero amplitude (noise only) */
    double BackgroundSigma;     /* noise sigma of background voxels */
} decaes_mock_opts;
int decaes_mock_image(const decaes_mock_opts *opts, uint64_t seed, void *image, int dtype, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
