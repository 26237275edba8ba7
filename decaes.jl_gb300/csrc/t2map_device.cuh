// t2map_device.cuh -- per-voxel pipeline of T2mapSEcorr on one warp:
// normalization, flip-angle search, EPG basis, regularized NNLS and the
// save_results!/T2part epilogue (src/T2mapSEcorr.jl:201-238, 409-591;
// src/lsqnonneg.jl; src/splines.jl; src/optimization.jl; src/T2partSEcorr.jl).
#pragma once
#include <climits>
#include "epg.cuh"
#include "nnls_gram.cuh"
#include "legacy.cuh"
#include "nnls_warp.cuh"
#include "t2map_params.cuh"

// The legacy algorithms are compiled only into the kernels of the translation
// unit that defines DECAES_LEGACY_KERNEL=1; elsewhere kLegacyKernel is false
// and the legacy branches fold away.  Likewise DECAES_METHODS selects the
// least-squares methods a translation unit's kernels carry (1 the plain FP64
// method, 2 the mixed method, 3 both, chosen per volume at run time): a kernel
// with one method has half the code, and the voxel pipeline is large enough
// for instruction fetch to show in its stalls.
#ifndef DECAES_LEGACY_KERNEL
#define DECAES_LEGACY_KERNEL 0
#endif
#ifndef DECAES_METHODS
#define DECAES_METHODS 3
#endif
// DECAES_TC_PRODUCTS=1: the kernel reads the flip-angle search's grid
// products from the tensor-core GEMM (DECAES_PREC_MIXED_TC); only its own
// translation unit compiles that path, so the other kernels are unchanged.
#ifndef DECAES_TC_PRODUCTS
#define DECAES_TC_PRODUCTS 0
#endif

namespace dk {

constexpr bool kLegacyKernel = DECAES_LEGACY_KERNEL != 0;
constexpr bool kHasPlain = (DECAES_METHODS & 1) != 0, kHasMixed = (DECAES_METHODS & 2) != 0;
constexpr bool kTcProducts = DECAES_TC_PRODUCTS != 0;

// Helpers with several call sites on the mixed method's hot path are kept out
// of line in its single-method kernel (one copy in the instruction cache
// instead of one per site: the kernel is ~0.5 MB of code and instruction
// fetch is a visible stall); the other kernels inline them as before.
#if DECAES_METHODS == 2
#define DK_OUTLINE __noinline__
#else
#define DK_OUTLINE
#endif

struct Warp {
    const Params *P;
    NnlsWS s;
    double *data;  // normalized decay data (shared), m
    double *xout;  // saved solution (shared), n
    double *A;     // per-voxel basis (global scratch), m x n
    double *scr;   // per-warp global scratch base
    double *sol_key, *sol_x;  // stored Tikhonov solutions: log mu keys, kSolCap x n
    int nsol;
    int lane;
    unsigned nnls_caps, loop_caps;
    // mixed method: normal-equation workspace and the staged basis (shared)
    GramWS g;
    float *As32;   // FP32 basis staged in shared memory, column-major, leading dimension ldA
    int ldA;
    bool mixed;    // the mixed method (Params::mixed)
};
// The warp's method, folded to a constant in single-method kernels.
__device__ __forceinline__ bool use_mixed(const Warp &w) { return kHasMixed && (!kHasPlain || w.mixed); }


__device__ __forceinline__ void note(Warp &w, const NnlsResult &r) { w.nnls_caps += (r.mode != 0); }

// Unregularized (tikh = false) or Tikhonov solve on the voxel's basis w.A:
// the reference's Householder NNLS for the plain method, the normal-equation
// solver on the voxel's prepared Gram matrix for the mixed method.
static __device__ NnlsResult basis_lsq(Warp &w, bool tikh, double mu) {
    const Params &P = *w.P;
    if (use_mixed(w))
        return gram_nnls(w.g, w.s.x, w.s.w, w.s.idx, P.n, tikh ? mu * mu : 0.0, 3 * P.n, &w.g.lastk);
    return warp_lsq(w.s, w.A, P.m, P.n, w.data, tikh, mu);
}

// Keys with Julia's isless order (NaN above everything, -0.0 < +0.0), for
// findmax-style searches on the integer pipes.
__device__ __forceinline__ long long ilkey(double d) {
    long long b = __double_as_longlong(d);
    if ((b & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL) return 0x7fffffffffffffffLL;
    return b >= 0 ? b : (b ^ 0x7fffffffffffffffLL);
}
// isapprox(x, y) with Julia's default rtol = sqrt(eps): x == y, or both
// finite with |x - y| <= rtol * max(|x|, |y|).  Only the difference and the
// tolerance are FP64 arithmetic; the tests and the max of two non-negative
// finite values are bit-pattern comparisons (exact).
__device__ __forceinline__ bool isapprox(double x, double y) {
    const long long bx = __double_as_longlong(x), by = __double_as_longlong(y);
    const long long ax = bx & 0x7fffffffffffffffLL, ay = by & 0x7fffffffffffffffLL;
    if ((bx == by && ax <= 0x7ff0000000000000LL) || (ax | ay) == 0) return true;  // x == y
    if (ax >= 0x7ff0000000000000LL || ay >= 0x7ff0000000000000LL) return false;   // not both finite
    const double tol = 1.4901161193847656e-08 * __longlong_as_double(ax < ay ? ay : ax);
    return (__double_as_longlong(x - y) & 0x7fffffffffffffffLL) <= __double_as_longlong(tol);
}
// First i in [0, len) with isapprox(x, keys[i]), or -1; lanes over entries.
static __device__ int warp_find_approx(const double *keys, int len, double x) {
    const int lane = threadIdx.x & 31;
    #pragma unroll 1
    for (int c = 0; c < len; c += 32) {
        int i = c + lane;
        bool hit = i < len && isapprox(x, keys[i]);
        unsigned msk = __ballot_sync(FULL, hit);
        if (msk) return c + __ffs(msk) - 1;
    }
    return -1;
}
// First i with keys[i] == x exactly (as doubles), or -1.
static __device__ int warp_find_exact(const double *keys, int len, double x) {
    const int lane = threadIdx.x & 31;
    #pragma unroll 1
    for (int c = 0; c < len; c += 32) {
        int i = c + lane;
        bool hit = i < len && keys[i] == x;
        unsigned msk = __ballot_sync(FULL, hit);
        if (msk) return c + __ffs(msk) - 1;
    }
    return -1;
}
// Store the current Tikhonov solution s.x under key log mu.
static __device__ void sol_store(Warp &w, double logmu) {
    if (w.nsol >= kSolCap) return;
    const int n = w.P->n;
    double *dst = w.sol_x + (long)w.nsol * n;
    #pragma unroll 1
    for (int j = w.lane; j < n; j += 32) dst[j] = w.s.x[j];
    if (w.lane == 0) w.sol_key[w.nsol] = logmu;
    __syncwarp();
    w.nsol++;
}
// The solution at mu = exp(logmu): from the store when this exact key was
// solved before (the solve is deterministic), else solved now.  Result in xout.
static __device__ void final_solution(Warp &w, double logmu);

// ----------------------------------------------------------------------------
// Tikhonov helpers (src/lsqnonneg.jl:297-318)
// ----------------------------------------------------------------------------
struct TikhState {
    NnlsResult r;
    double mu;
};
static __device__ TikhState tikh_solve(Warp &w, double mu) {
    TikhState t;
    t.r = basis_lsq(w, true, mu);
    t.mu = mu;
    note(w, t.r);
    return t;
}
// ||A x - b||^2 of a Tikhonov solution from its padded residual and ||x||^2.
static __device__ double tikh_res2_ssq(const TikhState &t, double ssq) {
    return jmax(__dsub_rn(__dmul_rn(t.r.rnorm, t.r.rnorm), __dmul_rn(__dmul_rn(t.mu, t.mu), ssq)), 0.0);
}
static __device__ double tikh_res2(Warp &w, const TikhState &t) {
    return tikh_res2_ssq(t, warp_seminorm_sq(w.s, t.r.nsetp));
}
static __device__ void save_x(Warp &w) {
    #pragma unroll 1
    for (int j = w.lane; j < w.P->n; j += 32) w.xout[j] = w.s.x[j];
    __syncwarp();
}

static __device__ void final_solution(Warp &w, double logmu) {
    int i = warp_find_exact(w.sol_key, w.nsol, logmu);
    if (i >= 0) {
        const double *src = w.sol_x + (long)i * w.P->n;
        #pragma unroll 1
        for (int j = w.lane; j < w.P->n; j += 32) w.xout[j] = src[j];
        __syncwarp();
        return;
    }
    tikh_solve(w, pm_exp(logmu));
    save_x(w);
}

// ----------------------------------------------------------------------------
// Root finding and minimization (src/optimization.jl)
// ----------------------------------------------------------------------------
__device__ __forceinline__ double jsign(double x) { return x < 0 ? -1.0 : (x > 0 ? 1.0 : x); }

// bracket_root_monotonic, src/optimization.jl:191-219
template <class F>
static __device__ void bracket_root_monotonic(F &f, double a, double delta, double dilate, double mono, int maxiters, double &ra,
                                       double &rb, double &rfa, double &rfb) {
    double fa = f(a);
    if (!isfinite(fa)) { ra = rb = a; rfa = rfb = CUDART_NAN; return; }
    if (fa == 0) { ra = rb = a; rfa = rfb = fa; return; }
    double sgn = jsign(mono) * jsign(fa);
    double b = a - sgn * delta;
    double fb = f(b);
    if (!isfinite(fb)) { ra = rb = a; rfa = rfb = fa; return; }
    if (fb == 0) { ra = rb = b; rfa = rfb = fb; return; }
    delta *= dilate;
    int cnt = 0;
    while (fa * fb > 0 && cnt < maxiters) {
        a = b; fa = fb;
        b = a - sgn * delta;
        fb = f(b);
        if (!isfinite(fb)) { ra = rb = a; rfa = rfb = fa; return; }
        if (fb == 0) { ra = rb = b; rfa = rfb = fb; return; }
        delta *= dilate;
        cnt += 1;
    }
    if (a < b) { ra = a; rb = b; rfa = fa; rfb = fb; }
    else { ra = b; rb = a; rfa = fb; rfb = fa; }
}

// brent_root, src/optimization.jl:71-128
template <class F>
static __device__ void brent_root(F &f, double x0, double x1, double fx0, double fx1, double xatol, double xrtol, double ftol,
                           int maxiters, double &xr, double &fxr) {
    if (fx0 == 0) { xr = x0; fxr = fx0; return; }
    if (fx1 == 0) { xr = x1; fxr = fx1; return; }
    double a = x0, b = x1, fa = fx0, fb = fx1;
    if (fabs(fa) < fabs(fb)) { double t = a; a = b; b = t; t = fa; fa = fb; fb = t; }
    double c = x0, d = x0, fc = fx0;
    bool mflag = true;
    #pragma unroll 1
    for (int iter = 1; iter <= maxiters; ++iter) {
        if (fabs(b - a) <= 2 * (xatol + xrtol * fabs(b))) { xr = b; fxr = fb; return; }
        double s = 0;
        s += a * fb * fc / (fa - fb) / (fa - fc);
        s += b * fa * fc / (fb - fa) / (fb - fc);
        s += c * fa * fb / (fc - fa) / (fc - fb);
        if (isnan(s) || isinf(s)) s = a - fa * (b - a) / (fb - fa);
        double u = (3 * a + b) / 4, v = b;
        if (u > v) { double t = u; u = v; v = t; }
        double tol = jmax(xatol, xrtol * jmax(jmax(fabs(b), fabs(c)), fabs(d)));
        if (!(u < s && s < v) || (mflag && fabs(s - b) >= fabs(b - c) / 2) || (!mflag && fabs(s - b) >= fabs(b - c) / 2) ||
            (mflag && fabs(b - c) <= tol) || (!mflag && fabs(c - d) <= tol)) {
            s = (a + b) / 2;
            mflag = true;
        } else {
            mflag = false;
        }
        double fs = f(s);
        if (fs == 0) { xr = s; fxr = fs; return; }
        if (isnan(fs) || isinf(fs)) { xr = b; fxr = fb; return; }
        if (fabs(fs) <= ftol) { xr = s; fxr = fs; return; }
        d = c; c = b; fc = fb;
        if (jsign(fa) * jsign(fs) < 0) { b = s; fb = fs; }
        else { a = s; fa = fs; }
        if (fabs(fa) < fabs(fb)) { double t = a; a = b; b = t; t = fa; fa = fb; fb = t; }
    }
    xr = b;
    fxr = fb;
}

// brent_minimize, src/optimization.jl:319-413
template <class F>
static __device__ void brent_minimize(F &f, double x1, double x2, double xrtol, double xatol, int maxiters, double &xo, double &yo) {
    const double PHI = 1.6180339887498949;
    const double alpha = 2 - PHI;
    double x = x1 + alpha * (x2 - x1);
    double y = f(x);
    double dx_old = 0, dx = 0, x_older = x, x_old = x, y_older = y, y_old = y;
    int iter = 0;
    while (iter < maxiters) {
        double p = 0, q = 0, xm = (x2 + x1) / 2, tolx = xatol + xrtol * fabs(x);
        if (fabs(x - xm) + (x2 - x1) / 2 <= 2 * tolx) break;
        iter += 1;
        if (fabs(dx_old) > tolx) {
            double r = (x - x_old) * (y - y_older);
            q = (x - x_older) * (y - y_old);
            p = (x - x_older) * q - (x - x_old) * r;
            q = 2 * (q - r);
            if (q > 0) p = -p;
            else q = -q;
        }
        if (fabs(p) < fabs(q * dx_old / 2) && p < q * (x2 - x) && p < q * (x - x1)) {
            dx_old = dx;
            dx = p / q;
            double xt = x + dx;
            if ((xt - x1) < 2 * tolx || (x2 - xt) < 2 * tolx) dx = (x < xm) ? tolx : -tolx;
        } else {
            dx_old = (x < xm) ? x2 - x : x1 - x;
            dx = alpha * dx_old;
        }
        double x_new = (fabs(dx) >= tolx) ? x + dx : x + ((dx > 0) ? tolx : -tolx);
        double y_new = f(x_new);
        if (y_new < y) {
            if (x_new < x) x2 = x; else x1 = x;
            x_older = x_old; x_old = x; x = x_new;
            y_older = y_old; y_old = y; y = y_new;
        } else {
            if (x_new < x) x1 = x_new; else x2 = x_new;
            if (y_new <= y_old || x_old == x) {
                x_older = x_old; x_old = x_new;
                y_older = y_old; y_old = y_new;
            } else if (y_new <= y_older || x_older == x || x_older == x_old) {
                x_older = x_new;
                y_older = y_new;
            }
        }
    }
    xo = x;
    yo = y;
}

// ----------------------------------------------------------------------------
// Regularizers (src/lsqnonneg.jl:504-1341)
// ----------------------------------------------------------------------------
struct Chi2F {  // f(logμ) of lsqnonneg_chi2!, src/lsqnonneg.jl:566-569
    Warp *w;
    double target;
    __device__ double operator()(double logmu) {
        TikhState t = tikh_solve(*w, pm_exp(logmu));
        sol_store(*w, logmu);
        return (tikh_res2(*w, t) - target) / target;
    }
};
struct MdpF {  // f(logμ) of lsqnonneg_mdp!, src/lsqnonneg.jl:723-726
    Warp *w;
    double delta2;
    __device__ double operator()(double logmu) {
        TikhState t = tikh_solve(*w, pm_exp(logmu));
        sol_store(*w, logmu);
        return tikh_res2(*w, t) - delta2;
    }
};

// lsqnonneg_chi2! (method :brent), src/lsqnonneg.jl:504-593.  The solution
// that save_results! stores ends up in w.xout.  On the early exit the
// reference saves its smoothing cache's stale slot; x_unreg is stored here.
static __device__ void reg_chi2(Warp &w, double chi2_target, double &mu_out, double &chi2_out) {
    const Params &P = *w.P;
    NnlsResult r0 = basis_lsq(w, false, 0.0);
    note(w, r0);
    double res2_min = __dmul_rn(r0.rnorm, r0.rnorm);
    if (res2_min == 0 || r0.nsetp == 0) {
        save_x(w);
        mu_out = 0; chi2_out = 1;
        return;
    }
    Chi2F f{&w, chi2_target * res2_min};
    double a, b, fa, fb, logmu, relerr;
    bracket_root_monotonic(f, -4.0, 1.0, 1.5, 1.0, 6, a, b, fa, fb);
    if (fa * fb < 0) {
        brent_root(f, a, b, fa, fb, 0.0, 0.0, 1e-3 * (chi2_target - 1), 100, logmu, relerr);
    } else {
        if (!isfinite(fa)) { logmu = b; relerr = fb; }
        else if (!isfinite(fb)) { logmu = a; relerr = fa; }
        else if (fabs(fa) < fabs(fb)) { logmu = a; relerr = fa; }
        else { logmu = b; relerr = fb; }
    }
    double mu, res2;
    if (isfinite(relerr)) {
        mu = pm_exp(logmu);
        res2 = f.target * (1 + relerr);
        final_solution(w, logmu);
    } else {
        mu = 0; res2 = 1;  // saved solution: the last Tikhonov solve
        save_x(w);
    }
    mu_out = mu;
    chi2_out = res2 / res2_min;
}

// The legacy algorithms' workspace: the L-curve cache region of the warp's
// global scratch (the L-curve is not run in the same voxel step).
static_assert(legacy_ws_doubles(kLegacyMaxPts) + 3 <= (long)kCacheCap * 19 &&
                  legacy_ws_doubles(kChi2LegacyMaxDouble + 2) + 2 * (kChi2LegacyMaxDouble + 2) <= (long)kCacheCap * 19,
              "legacy workspace exceeds the L-curve cache region");
__device__ __forceinline__ double *legacy_ws(Warp &w) { return w.scr + (long)w.P->m * w.P->n + 3L * w.P->K; }

// lsqnonneg_chi2!(legacy = true), src/lsqnonneg.jl:504-531, with
// chi2_search_from_minimum(legacy = true), src/lsqnonneg.jl:595-636: mu doubles
// from 1e-3 until res2(mu) >= Chi2Factor * res2_min, then the legacy spline
// root through every (mu, res2) pair including (0, res2_min); the saved
// solution is x_unreg when that root is mu = 0.  The doubling stops after
// kChi2LegacyMaxDouble steps (counted as a loop cap), where the reference
// would keep doubling on data that never reaches the target.
static __device__ __noinline__ void reg_chi2_legacy(Warp &w, double chi2_target, double &mu_out, double &chi2_out) {
    NnlsResult r0 = basis_lsq(w, false, 0.0);
    note(w, r0);
    double res2_min = __dmul_rn(r0.rnorm, r0.rnorm);
    save_x(w);  // x_unreg
    if (res2_min == 0 || r0.nsetp == 0) { mu_out = 0; chi2_out = 1; return; }
    double *mus = legacy_ws(w) + legacy_ws_doubles(kChi2LegacyMaxDouble + 2), *r2s = mus + kChi2LegacyMaxDouble + 2;
    const double target = chi2_target * res2_min;
    if (w.lane == 0) { mus[0] = 0; r2s[0] = res2_min; }
    int cnt = 1;
    double munew = 1e-3;
    #pragma unroll 1
    for (int it = 0;; ++it) {
        TikhState t = tikh_solve(w, munew);
        double res2new = tikh_res2(w, t);
        if (w.lane == 0) { mus[cnt] = munew; r2s[cnt] = res2new; }
        cnt++;
        if (res2new >= target) break;
        if (it == kChi2LegacyMaxDouble) { w.loop_caps++; break; }
        munew *= 2.0;
    }
    __syncwarp();
    const double mu = legacy_scan(mus, r2s, nullptr, cnt, true, target, legacy_ws(w)).x;
    double res2;
    if (mu == 0) {
        res2 = res2_min;
    } else {
        TikhState t = tikh_solve(w, mu);
        res2 = tikh_res2(w, t);
        save_x(w);
    }
    mu_out = mu;
    chi2_out = res2 / res2_min;
}

// lsqnonneg_mdp!, src/lsqnonneg.jl:700-747.  Early exits store the returned
// x (x_unreg or zeros) where the reference saves a stale cache slot.
static __device__ void reg_mdp(Warp &w, double delta, double &mu_out, double &chi2_out) {
    const Params &P = *w.P;
    NnlsResult r0 = basis_lsq(w, false, 0.0);
    note(w, r0);
    double res2_min = __dmul_rn(r0.rnorm, r0.rnorm);
    if (delta <= sqrt(res2_min)) { save_x(w); mu_out = 0; chi2_out = 1; return; }
    double part = 0;
    #pragma unroll 1
    for (int i = w.lane; i < P.m; i += 32) part = __dadd_rn(part, __dmul_rn(w.data[i], w.data[i]));
    double res2_max = wsum(part);
    if (delta >= sqrt(res2_max)) {
        #pragma unroll 1
        for (int j = w.lane; j < P.n; j += 32) w.xout[j] = 0.0;
        __syncwarp();
        mu_out = CUDART_INF; chi2_out = res2_max / res2_min;
        return;
    }
    MdpF f{&w, delta * delta};
    double a, b, fa, fb, logmu, err;
    bracket_root_monotonic(f, -4.0, 1.0, 1.5, 1.0, 6, a, b, fa, fb);
    if (fa * fb < 0) {
        brent_root(f, a, b, fa, fb, 0.0, 0.0, 1e-3 * (delta * delta), 100, logmu, err);
    } else {
        if (!isfinite(fa)) { logmu = b; err = fb; }
        else if (!isfinite(fb)) { logmu = a; err = fa; }
        else if (fabs(fa) < fabs(fb)) { logmu = a; err = fa; }
        else { logmu = b; err = fb; }
    }
    double mu, res2;
    if (isfinite(err)) {
        mu = pm_exp(logmu);
        res2 = delta * delta + err;
        final_solution(w, logmu);
    } else {
        mu = 0; res2 = 1;
        save_x(w);
    }
    mu_out = mu;
    chi2_out = res2 / res2_min;
}

// ---- L-curve corner (src/lsqnonneg.jl:812-972), caches in global scratch ----
struct LCurve {
    Warp *w;
    double *fx, *fP;          // CachedFunction: keys, values (isapprox keys)
    double *px, *pP, *pC;     // point cache
    double *sx, *sP;          // state cache
    int flen, plen, slen;
    bool overflow;
};
// f_lcurve(logμ) = (log ||Ax-b||^2, log ||x||^2) through the isapprox-keyed cache
static __device__ DK_OUTLINE void lc_eval(LCurve &L, double x, double &P0, double &P1) {
    int hit = warp_find_approx(L.fx, L.flen, x);
    if (hit >= 0) { P0 = L.fP[2 * hit]; P1 = L.fP[2 * hit + 1]; return; }
    Warp &w = *L.w;
    TikhState t = tikh_solve(w, pm_exp(x));
    sol_store(w, x);
    double ssq = warp_seminorm_sq(w.s, t.r.nsetp);
    double res2 = tikh_res2_ssq(t, ssq);
    P0 = pm_log(res2);
    P1 = pm_log(ssq);
    if (L.flen < kCacheCap) {
        if (w.lane == 0) { L.fx[L.flen] = x; L.fP[2 * L.flen] = P0; L.fP[2 * L.flen + 1] = P1; }
        __syncwarp();
        L.flen++;
    } else {
        L.overflow = true;
    }
}
static __device__ int pc_find(const LCurve &L, double x) { return warp_find_approx(L.px, L.plen, x); }
static __device__ DK_OUTLINE void pc_set(LCurve &L, double x, double P0, double P1, double C, bool push_only) {
    int i = push_only ? -1 : pc_find(L, x);
    if (i < 0) {
        if (L.plen >= kCacheCap) { L.overflow = true; return; }
        i = L.plen++;
        if (L.w->lane == 0) L.px[i] = x;
    }
    if (L.w->lane == 0) { L.pP[2 * i] = P0; L.pP[2 * i + 1] = P1; L.pC[i] = C; }
    __syncwarp();
}
// mapfindmax over the point cache's curvatures (first maximum under isless)
static __device__ int pc_argmax(const LCurve &L) {
    const int lane = threadIdx.x & 31;
    long long bk = 0;
    int bi = -1;
    #pragma unroll 1
    for (int c = 0; c < L.plen; c += 32) {
        int i = c + lane;
        if (i < L.plen) {
            long long k = ilkey(L.pC[i]);
            if (bi < 0 || k > bk) { bk = k; bi = i; }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        long long ok = __shfl_xor_sync(FULL, bk, o);
        int oi = __shfl_xor_sync(FULL, bi, o);
        if (oi >= 0 && (bi < 0 || ok > bk || (ok == bk && oi < bi))) { bk = ok; bi = oi; }
    }
    return bi;
}
__device__ __forceinline__ double nrm2(double a, double b) { return sqrt(__dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b))); }
// menger(Pj, Pk, Pl), src/lsqnonneg.jl:967-972
static __device__ double menger(double j0, double j1, double k0, double k1, double l0, double l1) {
    double djk0 = j0 - k0, djk1 = j1 - k1, dkl0 = k0 - l0, dkl1 = k1 - l1, dlj0 = l0 - j0, dlj1 = l1 - j1;
    double a = __dadd_rn(__dmul_rn(djk0, djk0), __dmul_rn(djk1, djk1));
    double b = __dadd_rn(__dmul_rn(dkl0, dkl0), __dmul_rn(dkl1, dkl1));
    double c = __dadd_rn(__dmul_rn(dlj0, dlj0), __dmul_rn(dlj1, dlj1));
    double cr = __dsub_rn(__dmul_rn(djk0, dkl1), __dmul_rn(djk1, dkl0));
    return 2 * cr / sqrt(__dmul_rn(__dmul_rn(a, b), c));
}
// The mixed method's forms of the same tests: squared distances against
// squared tolerances, and the curvature with one reciprocal square root (no
// correctly rounded square roots and divisions on its dependency chain).
__device__ __forceinline__ double sq2(double a, double b) { return fma(a, a, b * b); }
static __device__ double menger_fast(double j0, double j1, double k0, double k1, double l0, double l1) {
    double djk0 = j0 - k0, djk1 = j1 - k1, dkl0 = k0 - l0, dkl1 = k1 - l1, dlj0 = l0 - j0, dlj1 = l1 - j1;
    double a = sq2(djk0, djk1), b = sq2(dkl0, dkl1), c = sq2(dlj0, dlj1);
    double cr = fma(djk0, dkl1, -(djk1 * dkl0));
    return 2 * cr * rsqrt(a * b * c);
}
struct LcState {
    double x[4], P[8];
};
// update_curvature!, src/lsqnonneg.jl:948-965.  The nearest cached
// neighbours (largest key below x, smallest above; first index on ties) are
// found lanes-over-entries with integer keys.
static __device__ DK_OUTLINE void lc_update_curvature(LCurve &L, const LcState &s, const double *Ptl, const double *Pbr, double Ctol) {
    const int lane = threadIdx.x & 31;
    #pragma unroll 1
    for (int q = 0; q < 4; ++q) {
        double x = s.x[q], P0 = s.P[2 * q], P1 = s.P[2 * q + 1];
        double C = -CUDART_INF;
        const bool far = use_mixed(*L.w) ? fmin(sq2(P0 - Ptl[0], P1 - Ptl[1]), sq2(P0 - Pbr[0], P1 - Pbr[1])) > Ctol * Ctol
                                    : jmin(nrm2(P0 - Ptl[0], P1 - Ptl[1]), nrm2(P0 - Pbr[0], P1 - Pbr[1])) > Ctol;
        if (far) {
            const long long kx = okey(x);
            long long km = 0, kp = 0;
            int im = -1, ip = -1;
            #pragma unroll 1
            for (int c = 0; c < L.plen; c += 32) {
                int i = c + lane;
                if (i < L.plen) {
                    long long k = okey(L.px[i]);
                    if (k < kx && (im < 0 || k > km)) { km = k; im = i; }
                    if (k > kx && (ip < 0 || k < kp)) { kp = k; ip = i; }
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                long long okm = __shfl_xor_sync(FULL, km, o), okp = __shfl_xor_sync(FULL, kp, o);
                int oim = __shfl_xor_sync(FULL, im, o), oip = __shfl_xor_sync(FULL, ip, o);
                if (oim >= 0 && (im < 0 || okm > km || (okm == km && oim < im))) { km = okm; im = oim; }
                if (oip >= 0 && (ip < 0 || okp < kp || (okp == kp && oip < ip))) { kp = okp; ip = oip; }
            }
            double m0 = P0, m1 = P1, p0 = P0, p1 = P1;
            if (im >= 0) { m0 = L.pP[2 * im]; m1 = L.pP[2 * im + 1]; }
            if (ip >= 0) { p0 = L.pP[2 * ip]; p1 = L.pP[2 * ip + 1]; }
            C = use_mixed(*L.w) ? menger_fast(m0, m1, P0, P1, p0, p1) : menger(m0, m1, P0, P1, p0, p1);
        }
        pc_set(L, x, P0, P1, C, false);
    }
}
// Backtracking scan of the state cache (src/lsqnonneg.jl:895-899): the
// sequential loop adopts state k when it contains the best point and its
// width is <= the width of the state held so far; equivalently, k is adopted
// iff it matches and its width is <= the running minimum over earlier matches
// (and the current width).  Returns the last adopted index, or -1.
static __device__ int lc_backtrack(const LCurve &L, double xb, double w0) {
    const int lane = threadIdx.x & 31;
    long long carry = __double_as_longlong(w0);  // widths are >= +0: bit order == value order
    int last = -1;
    #pragma unroll 1
    for (int c = 0; c < L.slen; c += 32) {
        int k = c + lane;
        bool match = false;
        long long wk = 0x7fffffffffffffffLL;
        if (k < L.slen) {
            const double *sx = L.sx + 4 * k;
            match = (sx[1] == xb || sx[2] == xb);
            if (match) wk = __double_as_longlong(fabs(sx[3] - sx[0]));
        }
        long long incl = wk;  // inclusive prefix minimum of matched widths
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            long long t = __shfl_up_sync(FULL, incl, o);
            if (lane >= o && t < incl) incl = t;
        }
        long long excl = __shfl_up_sync(FULL, incl, 1);
        if (lane == 0) excl = 0x7fffffffffffffffLL;
        long long bound = excl < carry ? excl : carry;
        bool adopted = match && wk <= bound;
        unsigned msk = __ballot_sync(FULL, adopted);
        if (msk) last = c + 31 - __clz(msk);
        long long tot = __shfl_sync(FULL, incl, 31);
        if (tot < carry) carry = tot;
    }
    return last;
}
// lcurve_corner with backtracking, src/lsqnonneg.jl:872-919
static __device__ double lcurve_corner(LCurve &L, double xlow, double xhigh, double xtol, double Ptol, double Ctol) {
    const double PHI = 1.6180339887498949;
    L.flen = L.plen = L.slen = 0;
    L.overflow = false;
    LcState st;
    st.x[0] = xlow;
    st.x[3] = xhigh;
    st.x[1] = (PHI * st.x[0] + st.x[3]) / (PHI + 1);
    st.x[2] = st.x[0] + (st.x[3] - st.x[1]);
    #pragma unroll 1
    for (int i = 0; i < 4; ++i) lc_eval(L, st.x[i], st.P[2 * i], st.P[2 * i + 1]);
    #pragma unroll 1
    for (int i = 0; i < 4; ++i) pc_set(L, st.x[i], st.P[2 * i], st.P[2 * i + 1], -CUDART_INF, true);
    double Ptl[2] = {st.P[0], st.P[1]}, Pbr[2] = {st.P[6], st.P[7]};
    lc_update_curvature(L, st, Ptl, Pbr, Ctol);
    int iter = 0;
    const bool mixed = use_mixed(*L.w);
    while (!(fabs(st.x[3] - st.x[0]) < xtol || (mixed ? sq2(st.P[0] - st.P[6], st.P[1] - st.P[7]) < Ptol * Ptol
                                                      : nrm2(st.P[0] - st.P[6], st.P[1] - st.P[7]) < Ptol))) {
        iter += 1;
        if (iter > kLoopCap || L.overflow) { L.w->loop_caps++; break; }
        double xb = L.px[pc_argmax(L)];
        int kb = lc_backtrack(L, xb, fabs(st.x[3] - st.x[0]));
        if (kb >= 0) {
            #pragma unroll 1
            for (int q = 0; q < 4; ++q) st.x[q] = L.sx[4 * kb + q];
            #pragma unroll 1
            for (int q = 0; q < 8; ++q) st.P[q] = L.sP[8 * kb + q];
        }
        int i2 = pc_find(L, st.x[1]), i3 = pc_find(L, st.x[2]);
        if (i2 < 0 || i3 < 0) { L.w->loop_caps++; break; }
        LcState ns;
        if (L.pC[i2] > L.pC[i3]) {  // move_left
            ns.x[0] = st.x[0]; ns.x[1] = (PHI * st.x[0] + st.x[2]) / (PHI + 1); ns.x[2] = st.x[1]; ns.x[3] = st.x[2];
            ns.P[0] = st.P[0]; ns.P[1] = st.P[1];
            lc_eval(L, ns.x[1], ns.P[2], ns.P[3]);
            ns.P[4] = st.P[2]; ns.P[5] = st.P[3]; ns.P[6] = st.P[4]; ns.P[7] = st.P[5];
        } else {  // move_right
            ns.x[0] = st.x[1]; ns.x[1] = st.x[2]; ns.x[2] = st.x[1] + (st.x[3] - st.x[2]); ns.x[3] = st.x[3];
            ns.P[0] = st.P[2]; ns.P[1] = st.P[3]; ns.P[2] = st.P[4]; ns.P[3] = st.P[5];
            lc_eval(L, ns.x[2], ns.P[4], ns.P[5]);
            ns.P[6] = st.P[6]; ns.P[7] = st.P[7];
        }
        st = ns;
        lc_update_curvature(L, st, Ptl, Pbr, Ctol);
        if (L.slen < kCacheCap) {
            if (L.w->lane == 0) {
                #pragma unroll 1
                for (int q = 0; q < 4; ++q) L.sx[4 * L.slen + q] = st.x[q];
                #pragma unroll 1
                for (int q = 0; q < 8; ++q) L.sP[8 * L.slen + q] = st.P[q];
            }
            __syncwarp();
            L.slen++;
        } else {
            L.overflow = true;
        }
    }
    return L.px[pc_argmax(L)];
}

static __device__ double *lcurve_scratch(Warp &w) { return w.scr + (long)w.P->m * w.P->n + 3L * w.P->K; }

// lsqnonneg_lcurve!, src/lsqnonneg.jl:812-840
static __device__ void reg_lcurve(Warp &w, double &mu_out, double &chi2_out) {
    double *base = lcurve_scratch(w);
    LCurve L;
    L.w = &w;
    L.fx = base; L.fP = L.fx + kCacheCap;
    L.px = L.fP + 2 * kCacheCap; L.pP = L.px + kCacheCap; L.pC = L.pP + 2 * kCacheCap;
    L.sx = L.pC + kCacheCap; L.sP = L.sx + 4 * kCacheCap;
    double logmu = lcurve_corner(L, -8.0, 2.0, 1e-4, 1e-4, 1e-4);
    double mu = pm_exp(logmu);
    double chi2 = CUDART_NAN;
    if (w.P->need_chi2) {
        TikhState t = tikh_solve(w, mu);
        double res2 = tikh_res2(w, t);
        save_x(w);
        NnlsResult r0 = basis_lsq(w, false, 0.0);
        note(w, r0);
        chi2 = res2 / __dmul_rn(r0.rnorm, r0.rnorm);
    } else {
        final_solution(w, logmu);
    }
    mu_out = mu;
    chi2_out = chi2;
}

// ---- GCV (src/lsqnonneg.jl:1136-1341) ----
// Singular values of the m x n basis (stand-in for LAPACK dgesdd job 'N',
// src/utils.jl:67-134): Golub-Kahan Householder bidiagonalization of
// B = A (m >= n) or A' (r x c, r >= c) in shared memory, then bisection on the
// Golub-Kahan tridiagonal (zero diagonal, off-diagonals d0, e0, d1, e1, ...,
// d_{c-1}), whose positive eigenvalues are the singular values, resolved to
// 1e-15 of their Gershgorin bound; written descending to gam.  Every sum runs
// sequentially in one lane (each lane its own columns or rows; the reflector
// norms redundantly on every lane) and the bisection takes one singular value
// per lane, so the oracle repeats it operation for operation.
static __device__ void warp_svdvals(Warp &w, double *gam) {
    const Params &P = *w.P;
    const int m = P.m, n = P.n, lane = w.lane;
    const int r = m >= n ? m : n, c = m >= n ? n : m;
    const int ld = r | 1;
    double *U = w.s.C;  // r x c, ld, fits in the lda x n workspace
    #pragma unroll 1
    for (int j = 0; j < c; ++j)
        #pragma unroll 1
        for (int i = lane; i < r; i += 32) U[i + (long)j * ld] = (m >= n) ? w.A[i + (long)j * m] : w.A[j + (long)i * m];
    __syncwarp();
    double *dv = w.s.zz, *ev = w.s.b;  // bidiagonal: c diagonal, c-1 superdiagonal entries
    #pragma unroll 1
    for (int k = 0; k < c; ++k) {
        const double *uk = U + (long)k * ld;
        // left reflector H = I - tau v v', v = (x0 - alpha, x_{k+1..r-1}), on column k
        double ss = 0.0;
        #pragma unroll 1
        for (int i = k + 1; i < r; ++i) ss = fma(uk[i], uk[i], ss);
        const double x0 = uk[k];
        double alpha = x0, v0 = 0.0, tau = 0.0;
        if (ss != 0.0) {
            const double nrm = sqrt(fma(x0, x0, ss));
            alpha = x0 >= 0.0 ? -nrm : nrm;
            v0 = x0 - alpha;
            tau = 2.0 / fma(v0, v0, ss);
        }
        if (lane == 0) dv[k] = alpha;
        if (tau != 0.0) {
            #pragma unroll 1
            for (int j = k + 1 + lane; j < c; j += 32) {
                double *uj = U + (long)j * ld;
                double sdot = v0 * uj[k];
                #pragma unroll 1
                for (int i = k + 1; i < r; ++i) sdot = fma(uk[i], uj[i], sdot);
                const double f = tau * sdot;
                uj[k] = fma(-f, v0, uj[k]);
                #pragma unroll 1
                for (int i = k + 1; i < r; ++i) uj[i] = fma(-f, uk[i], uj[i]);
            }
        }
        __syncwarp();
        if (k + 2 < c) {
            // right reflector on row k, columns k+1..c-1
            double sr = 0.0;
            #pragma unroll 1
            for (int j = k + 2; j < c; ++j) { const double y = U[k + (long)j * ld]; sr = fma(y, y, sr); }
            const double y0 = U[k + (long)(k + 1) * ld];
            double beta = y0, w0 = 0.0, tau2 = 0.0;
            if (sr != 0.0) {
                const double nrm = sqrt(fma(y0, y0, sr));
                beta = y0 >= 0.0 ? -nrm : nrm;
                w0 = y0 - beta;
                tau2 = 2.0 / fma(w0, w0, sr);
            }
            if (lane == 0) ev[k] = beta;
            if (tau2 != 0.0) {
                #pragma unroll 1
                for (int i = k + 1 + lane; i < r; i += 32) {
                    double sdot = w0 * U[i + (long)(k + 1) * ld];
                    #pragma unroll 1
                    for (int j = k + 2; j < c; ++j) sdot = fma(U[k + (long)j * ld], U[i + (long)j * ld], sdot);
                    const double f = tau2 * sdot;
                    U[i + (long)(k + 1) * ld] = fma(-f, w0, U[i + (long)(k + 1) * ld]);
                    #pragma unroll 1
                    for (int j = k + 2; j < c; ++j) U[i + (long)j * ld] = fma(-f, U[k + (long)j * ld], U[i + (long)j * ld]);
                }
            }
            __syncwarp();
        } else if (k + 1 < c) {
            if (lane == 0) ev[k] = U[k + (long)(k + 1) * ld];
            __syncwarp();
        }
    }
    // Golub-Kahan tridiagonal: squared off-diagonals o2 (2c-1, in U's storage)
    // and the Gershgorin bound
    const int N = 2 * c;
    double *o2 = U;
    double bnd = 0.0;
    #pragma unroll 1
    for (int j = lane; j < N; j += 32) {
        const double oa = j > 0 ? fabs((j - 1) % 2 == 0 ? dv[(j - 1) / 2] : ev[(j - 1) / 2]) : 0.0;
        const double ob = j + 1 < N ? fabs(j % 2 == 0 ? dv[j / 2] : ev[j / 2]) : 0.0;
        bnd = fmax(bnd, oa + ob);
    }
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) bnd = fmax(bnd, __shfl_xor_sync(FULL, bnd, o));
    __syncwarp();
    #pragma unroll 1
    for (int j = lane; j + 1 < N; j += 32) {
        const double o = j % 2 == 0 ? dv[j / 2] : ev[j / 2];
        o2[j] = o * o;
    }
    __syncwarp();
    const double tau0 = 1e-14 * bnd, atol = 1e-15 * bnd;
    // Sturm count: eigenvalues of the tridiagonal below x (zero diagonal)
    auto count_below = [&](double x) {
        double p2 = 1.0, p1 = 0.0 - x;
        bool neg = p1 <= 0;  // a zero takes the sign opposite to its predecessor (p_0 = +1)
        int cnt = neg;
        #pragma unroll 1
        for (int j = 1; j < N; ++j) {
            double p = fma(0.0 - x, p1, -o2[j - 1] * p2);
            bool pneg = p < 0 || (p == 0 && !neg);
            cnt += (pneg != neg);
            neg = pneg;
            p2 = p1;
            p1 = p;
            const int ex = ((__double2hiint(p1) >> 20) & 0x7ff) - 1023;
            if (p1 != 0 && (ex > 400 || ex < -400)) {
                const double sc = __hiloint2double((1023 - ex) << 20, 0);
                p1 *= sc;
                p2 *= sc;
            }
        }
        return cnt;
    };
    const int nres = N - count_below(tau0);  // singular values >= tau0 (the rest are left at zero)
    #pragma unroll 1
    for (int base = 0; base < nres; base += 32) {
        const int t = base + lane;  // t-th largest singular value
        const bool mine = t < nres;
        const int idx = N - 1 - t;  // its index among the eigenvalues in ascending order
        double a = tau0, b = bnd;
        bool done = !mine;
        #pragma unroll 1
        for (int it = 0; it < 80 && __any_sync(FULL, !done); ++it) {
            const double mid = 0.5 * (a + b);
            const int cnt = count_below(mid);
            if (!done) {
                if (cnt > idx) b = mid; else a = mid;
                done = (b - a) <= fmax(atol, 4.0 * 2.220446049250313e-16 * b);
            }
        }
        if (mine && t < c) gam[t] = 0.5 * (a + b);
    }
    #pragma unroll 1
    for (int t = nres + lane; t < c; t += 32) gam[t] = 0.0;
    __syncwarp();
}
struct GcvF {  // log𝒢(logμ), src/lsqnonneg.jl:1150-1154 and gcv!, 1213-1229
    Warp *w;
    const double *gam;
    double low;
    __device__ double operator()(double logmu) {
        const Params &P = *w->P;
        double mu = pm_exp(logmu);
        TikhState t = tikh_solve(*w, mu);
        sol_store(*w, logmu);
        double res2 = tikh_res2(*w, t);
        int k = P.m < P.n ? P.m : P.n;
        double dof = (double)(P.m - P.n > 0 ? P.m - P.n : 0), l2 = mu * mu;
        if (use_mixed(*w)) {  // lanes over singular values
            double part = 0.0;
            #pragma unroll 1
            for (int i = w->lane; i < k; i += 32) { double g2 = gam[i] * gam[i]; part = fma(l2, fast_rcp(g2 + l2), part); }
            dof += wsum(part);
        } else {
            #pragma unroll 1
            for (int i = 0; i < k; ++i) { double g2 = gam[i] * gam[i]; dof += l2 / (g2 + l2); }
        }
        double G = res2 / (dof * dof);
        return pm_log(jmax(G, low));
    }
};
static __device__ void reg_gcv(Warp &w, double &mu_out, double &chi2_out) {
    const Params &P = *w.P;
    double *gam = w.scr + (long)P.m * P.n + 3L * P.K + (long)kCacheCap * 19;
    if (!use_mixed(w)) warp_svdvals(w, gam);  // the mixed method takes them from its Gram matrix (gram_svdvals)
    GcvF f{&w, gam, (2.220446049250313e-16 * 2.220446049250313e-16) / P.m};
    double logmu, logG;
    brent_minimize(f, -8.0, 2.0, 0.0, 1e-4, 20, logmu, logG);
    double mu = pm_exp(logmu);
    double chi2 = CUDART_NAN;
    if (P.need_chi2) {
        TikhState t = tikh_solve(w, mu);
        double res2 = tikh_res2(w, t);
        save_x(w);
        NnlsResult r0 = basis_lsq(w, false, 0.0);
        note(w, r0);
        chi2 = res2 / __dmul_rn(r0.rnorm, r0.rnorm);
    } else {
        final_solution(w, logmu);
    }
    mu_out = mu;
    chi2_out = chi2;
}

// ----------------------------------------------------------------------------
// Flip-angle search (src/T2mapSEcorr.jl:409-423; src/splines.jl:53-110,
// 504-566, 664-850, 975-1051)
// ----------------------------------------------------------------------------
struct Search {
    Warp *w;
    double *u, *du;       // per grid index, global scratch (K each)
    int *sidx;            // sorted evaluated indices, 1-based (K)
    unsigned seen[8];     // bitset over <= 256 grid points (warp-uniform registers)
    int npts, numeval, mineval, maxeval;
#if DECAES_TC_PRODUCTS
    const float *Frow;    // the voxel's tensor-core grid products (float pairs), or null
    double fscale;        // their scale to the normalized decay: 2^e / max
#endif
};
__device__ __forceinline__ bool sseen(const Search &S, int I) { return (S.seen[(I - 1) >> 5] >> ((I - 1) & 31)) & 1u; }

// loss_with_grad!(prob, I), src/splines.jl:1010-1041
static __device__ void fa_update(Search &S, int I) {
    Warp &w = *S.w;
    const Params &P = *w.P;
    const int m = P.m, n = P.n, lane = w.lane;
    const double *A = P.As + (long)(I - 1) * m * n, *dA = P.dAs + (long)(I - 1) * m * n;
    NnlsResult r;
    if (use_mixed(w)) {
        // precomputed Gram matrix of grid basis I; A'b from its transposed copy
        gram_load(w.g, P.Gs + (long)(I - 1) * (n * (n + 1) / 2), n);
#if DECAES_TC_PRODUCTS
        if (S.Frow)  // from the tensor-core grid products
            gram_rhs_f32(w.g, S.Frow + 2L * (I - 1) * n, n, S.fscale, m, w.data);
        else
#endif
            gram_rhs_t(w.g, P.AsT + (long)(I - 1) * m * n, m, n, w.data);
        r = gram_nnls(w.g, w.s.x, w.s.w, w.s.idx, n, 0.0, 3 * n, &w.g.lastk);
    } else {
        r = warp_lsq(w.s, A, m, n, w.data, false, 0.0);
    }
    note(w, r);
    double ell = __dmul_rn(r.rnorm, r.rnorm);
    double part = 0;
    #pragma unroll 1
    for (int i0 = 0; i0 < (kLegacyKernel && P.legacy ? 0 : m); i0 += 32) {  // legacy: loss! only, src/splines.jl:1043-1046
        int i = i0 + lane;
        double ax = 0, dax = 0;
        // the columns with x_j > 0 in increasing order, from one ballot per 32
        // columns instead of a comparison per column
        #pragma unroll 1
        for (int j0 = 0; j0 < n; j0 += 32) {
            unsigned msk = __ballot_sync(FULL, j0 + lane < n && pos_bits(w.s.x[j0 + lane]));
            if (i < m) {
                #pragma unroll 1
                while (msk) {
                    const int j = j0 + __ffs(msk) - 1;
                    msk &= msk - 1;
                    const double xj = w.s.x[j];
                    ax = fma(xj, __ldg(A + i + (long)j * m), ax);
                    dax = fma(xj, __ldg(dA + i + (long)j * m), dax);
                }
            }
        }
        if (i < m) part = fma(dax, ax - w.data[i], part);
    }
    double dt = wsum(part);
    if (lane == 0) {
        S.u[I - 1] = ell;
        S.du[I - 1] = kLegacyKernel && P.legacy ? CUDART_NAN : 2 * dt;
        // insertsorted!(idx, I, npts += 1), src/utils.jl:42-49
        int len = S.npts + 1, val = I;
        #pragma unroll 1
        for (int i = 0; i < len - 1; ++i) {
            int a = S.sidx[i];
            if (val < a) { S.sidx[i] = val; val = a; }
        }
        S.sidx[len - 1] = val;
    }
    __syncwarp();
    S.npts++;
}
// update!(surr, state, I; maxeval), src/splines.jl:736-744
static __device__ DK_OUTLINE bool fa_state_update(Search &S, int I) {
    if (S.numeval >= S.maxeval) return true;
    if (sseen(S, I)) return false;
    fa_update(S, I);
    S.seen[(I - 1) >> 5] |= 1u << ((I - 1) & 31);
    S.numeval += 1;
    return S.numeval >= S.maxeval;
}
__device__ __forceinline__ bool box_done(const Search &S, int lo, int hi) { return (int)sseen(S, lo) + (int)sseen(S, hi) >= 2; }
// evaluate_box!, src/splines.jl:802-815
static __device__ void fa_evaluate_box(Search &S, int lo, int hi, bool have_x, double x) {
    const double *g = S.w->P->angles;
    int c0 = lo, c1 = hi;
    if (have_x) {
        double dlo = (g[lo - 1] - x) * (g[lo - 1] - x), dhi = (g[hi - 1] - x) * (g[hi - 1] - x);
        if (dhi < dlo) { c0 = hi; c1 = lo; }
    }
    if (box_done(S, lo, hi)) return;
    if (fa_state_update(S, c0)) return;
    if (box_done(S, lo, hi)) return;
    fa_state_update(S, c1);
}
// initialize! (recursive breadth-limited bisection), src/splines.jl:716-734,
// run with an explicit depth-first stack.
static __device__ void fa_initialize(Search &S) {
    const int K = S.w->P->K;
    #pragma unroll 1
    for (int depth = 1; depth <= S.mineval; ++depth) {
        // stack of boxes, packed (lo | hi << 9 | depth << 18); 1 <= lo, hi <= 256
        unsigned st[48];
        int sp = 0;
        st[sp++] = 1u | ((unsigned)K << 9) | ((unsigned)depth << 18);
        int guard = 0;
        while (sp > 0 && guard++ < 4096) {
            unsigned e = st[--sp];
            int lo = e & 511, hi = (e >> 9) & 511, d = (int)(e >> 18);
            if (d <= 0) continue;
            fa_evaluate_box(S, lo, hi, false, 0.0);
            if (S.numeval >= S.mineval) continue;
            int mid = (lo + hi) / 2;
            if (sp + 2 > 48) { S.w->loop_caps++; break; }
            st[sp++] = (unsigned)mid | ((unsigned)hi << 9) | ((unsigned)(d - 1) << 18);  // right, after left
            st[sp++] = (unsigned)lo | ((unsigned)mid << 9) | ((unsigned)(d - 1) << 18);
        }
        if (S.numeval >= S.mineval) break;
    }
}
// CubicHermiteInterpolator + minimize, src/splines.jl:62-110
static __device__ void hermite_minimize(double a, double b, double u0, double u1, double m0, double m1, double &xo, double &uo) {
    double r = (b - a) / 2;
    m0 = r * m0; m1 = r * m1;
    double du = u1 - u0, dm = m1 - m0, su = u1 + u0, sm = m1 + m0;
    double c0 = su / 2 - dm / 4, c1 = (3 * du - sm) / 4, c2 = dm / 4, c3 = (sm - du) / 4;
    double xend, uend;
    if (u0 < u1) { xend = a; uend = u0; } else { xend = b; uend = u1; }
    double D = 3 * (u0 - u1), th = D / 2 + (m0 + m1);
    double g = __dsub_rn(__dmul_rn(th, th), __dmul_rn(m0, m1));
    g = g > 0 ? -sqrt(g) : 0.0;
    double p = -(D + (m0 + m1)), q = 2 * g + (m0 - m1);
    if (fabs(p) < fabs(q)) {
        double t = p / q;
        double y = fma(t, fma(t, fma(t, c3, c2), c1), c0);
        if (y < uend) {
            double cc = (a + b) / 2, rr = (b - a) / 2;
            double xx = fma(rr, t, cc);
            xo = xx > b ? b : (xx < a ? a : xx);
            uo = y;
            return;
        }
    }
    xo = xend;
    uo = uend;
}
// suggest_point(::CubicHermiteSplineSurrogate), src/splines.jl:544-566
// suggest_point(::CubicSplineSurrogate) with spline_opt_legacy,
// src/splines.jl:493-500,419-431.  The scan depends only on the evaluated
// points, so an unchanged set reuses it: the last suggestion (points, x, u)
// is kept in the scratch words after the scan's workspace.
static __device__ __noinline__ double2 fa_suggest_legacy(const double *angles, const double *u, const int *sidx, int npts,
                                                  double *ws) {
    double *memo = ws + legacy_ws_doubles(kLegacyMaxPts);
    if (memo[0] != (double)npts) {
        __syncwarp();
        double2 r = legacy_scan(angles, u, sidx, npts, false, 0.0, ws);
        if ((threadIdx.x & 31) == 0) { memo[0] = (double)npts; memo[1] = r.x; memo[2] = r.y; }
        __syncwarp();
        return r;
    }
    return make_double2(memo[1], memo[2]);
}
static __device__ DK_OUTLINE void fa_suggest(Search &S, double &xo, double &uo) {
    const double *g = S.w->P->angles;
    if (kLegacyKernel && S.w->P->legacy) {
        double2 r = fa_suggest_legacy(g, S.u, S.sidx, S.npts, legacy_ws(*S.w));
        xo = r.x;
        uo = r.y;
        return;
    }
    int I0 = S.sidx[0];
    double pl = g[I0 - 1], ul = S.u[I0 - 1], dl = S.du[I0 - 1], p = pl, u = ul;
    #pragma unroll 1
    for (int i = 2; i <= S.npts; ++i) {
        int I = S.sidx[i - 1];
        double pc = g[I - 1], uc = S.u[I - 1], dc = S.du[I - 1], xx, uu;
        hermite_minimize(pl, pc, ul, uc, dl, dc, xx, uu);
        if (uu < u) { p = xx; u = uu; }
        pl = pc; ul = uc; dl = dc;
    }
    xo = p;
    uo = u;
}
// minimal_bounding_box, src/splines.jl:778-800
static __device__ void fa_min_bbox(const Search &S, double x, int &plo, int &phi) {
    const double *g = S.w->P->angles;
    int lo = 1, hi = S.w->P->K;
    #pragma unroll 1
    for (int guard = 0; guard < 64; ++guard) {
        int mid = (lo + hi) / 2;
        if (g[lo - 1] <= x && x <= g[mid - 1]) {
            if (!box_done(S, lo, mid) || !(abs(mid - lo) > 1)) { plo = lo; phi = mid; return; }
            hi = mid;
        } else {
            if (!box_done(S, mid, hi) || !(abs(hi - mid) > 1)) { plo = mid; phi = hi; return; }
            lo = mid;
        }
    }
    plo = lo;
    phi = hi;
}
// optimize_flip_angle!, src/T2mapSEcorr.jl:409-423 + bisection_search, src/splines.jl:750-775
// slot: the voxel's position in this launch's part of the voxel list (its
// row of tensor-core grid products in the kernels that read them)
static __device__ double flip_angle_search(Warp &w, double mx, long slot) {
    const Params &P = *w.P;
    Search S;
    S.w = &w;
#if DECAES_TC_PRODUCTS
    {
        const int e = P.Fexp[slot];
        S.Frow = e != INT_MIN ? P.Fk + slot * P.ldF : nullptr;
        S.fscale = e != INT_MIN ? ldexp(1.0, e) / (mx > 0 ? mx : 1.0) : 0.0;
    }
#endif
    S.u = w.scr + (long)P.m * P.n;
    S.du = S.u + P.K;
    S.sidx = reinterpret_cast<int *>(S.du + P.K);
    #pragma unroll 1
    for (int q = 0; q < 8; ++q) S.seen[q] = 0;
    S.npts = 0; S.numeval = 0; S.mineval = P.mineval; S.maxeval = P.maxeval;
    if (kLegacyKernel && P.legacy && w.lane == 0) legacy_ws(w)[legacy_ws_doubles(kLegacyMaxPts)] = -1.0;  // no suggestion yet
    fa_initialize(S);
    double x, u;
    fa_suggest(S, x, u);
    #pragma unroll 1
    for (int guard = 0; guard <= kLoopCap; ++guard) {
        int lo, hi;
        fa_min_bbox(S, x, lo, hi);
        fa_evaluate_box(S, lo, hi, true, x);
        fa_suggest(S, x, u);
        if (S.numeval >= S.maxeval || abs(hi - lo) <= 1) return x;
    }
    w.loop_caps++;
    return x;
}

// ----------------------------------------------------------------------------
// EPG basis at one angle: lanes over T2 columns, states in shared memory
// (src/T2mapSEcorr.jl:275-283 with the default EPG kernels).
// ----------------------------------------------------------------------------
static __device__ void warp_basis(Warp &w, double alpha, double *out /* m x n, global */) {
    const Params &P = *w.P;
    const int m = P.m, n = P.n, lanes = P.epg_lanes, lane = w.lane;
    double *S = w.s.C;  // 3*m*lanes doubles, lane-contiguous, over the C, b and zz regions
    #pragma unroll 1
    for (int j0 = 0; j0 < n; j0 += lanes) {
        int j = j0 + lane;
        if (lane < lanes && j < n) {
            double *Sl = S + lane;
            if (P.beta180) {
                dx::FlatCoef<double> q = dx::flat_coef(alpha, P.TE, P.t2[j], P.T1);
                dx::epg_flat_inplace(m, q, Sl, lanes, out + (long)j * m, 1);
            } else {
                dx::VecCoef<double> q = dx::vec_coef(alpha, P.TE, P.t2[j], P.T1, P.beta);
                dx::epg_vec_inplace(m, q, Sl, lanes, out + (long)j * m, 1);
            }
        }
        __syncwarp();
    }
    __threadfence_block();
    __syncwarp();
}

// Mixed method: the same curves with the recursion in FP32 (coefficients in
// FP64, rounded once), states in the Gram and factor regions, curves written
// as FP32 to the warp's global scratch, then staged in w.As32 and widened
// (exactly, on the integer pipes) into w.A.  The basis of the voxel is these
// FP32 values, for the Gram matrix and the fitted curve alike, and no FP32 <->
// FP64 conversion occupies the FP64 pipe.
static __device__ void warp_basis_f32(Warp &w, double alpha) {
    const Params &P = *w.P;
    const int m = P.m, n = P.n, lanes = P.epg_lanes_f32, lane = w.lane;
    float *S = reinterpret_cast<float *>(w.g.G);  // 3*m*lanes floats, lane-contiguous
    float *Af = reinterpret_cast<float *>(w.scr + warp_scratch_f32_offset(m, n, P.K));
    #pragma unroll 1
    for (int j0 = 0; j0 < n; j0 += lanes) {
        int j = j0 + lane;
        if (lane < lanes && j < n) {
            float *Sl = S + lane;
            if (P.beta180) {
                dx::FlatCoef<float> q = dx::to_f32(dx::flat_coef(alpha, P.TE, P.t2[j], P.T1));
                dx::epg_flat_inplace(m, q, Sl, lanes, Af + (long)j * m, 1);
            } else {
                dx::VecCoef<float> q = dx::to_f32(dx::vec_coef(alpha, P.TE, P.t2[j], P.T1, P.beta));
                dx::epg_vec_inplace(m, q, Sl, lanes, Af + (long)j * m, 1);
            }
        }
        __syncwarp();
    }
    __threadfence_block();
    __syncwarp();
    #pragma unroll 1
    for (long q = lane; q < (long)m * n; q += 32) {
        const int i = (int)(q % m), j = (int)(q / m);
        const float v = Af[q];
        w.A[q] = widen(v);
        w.As32[i + w.ldA * j] = v;
    }
    __threadfence_block();
    __syncwarp();
}

// ----------------------------------------------------------------------------
// One voxel (src/T2mapSEcorr.jl:201-238, save_results! 512-591, T2part 95-138)
// ----------------------------------------------------------------------------
static __device__ void process_voxel(Warp &w, long v, long slot = 0) {
    const Params &P = *w.P;
    const int m = P.m, n = P.n, lane = w.lane;
    w.nsol = 0;
    // copy + normalize by the maximum echo
    double mx = 0;
    #pragma unroll 1
    for (int i = lane; i < m; i += 32) {
        double bi = P.image_f32 ? (double)static_cast<const float *>(P.image)[v + P.V * i]
                                : static_cast<const double *>(P.image)[v + P.V * i];
        w.data[i] = bi;
        mx = bi > mx ? bi : mx;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        double t = __shfl_xor_sync(FULL, mx, o);
        mx = t > mx ? t : mx;
    }
    __syncwarp();
    if (mx > 0)
        #pragma unroll 1
        for (int i = lane; i < m; i += 32) w.data[i] = w.data[i] / mx;
    __syncwarp();

    double alpha;
    w.g.lastk = 0;  // warm starts never cross voxels (results independent of scheduling)
    if (P.angle_mode == 1) {
        alpha = P.fixed_angle;
        w.A = const_cast<double *>(P.basis_fixed);
    } else {
        w.A = w.scr;
        if (P.angle_mode == 2) {
            alpha = P.image_f32 ? (double)static_cast<const float *>(P.b1map)[v] : static_cast<const double *>(P.b1map)[v];
        } else {
            alpha = flip_angle_search(w, mx, slot);
        }
        if (use_mixed(w)) warp_basis_f32(w, alpha);
        else warp_basis(w, alpha, w.A);
    }
    if (use_mixed(w)) {
        // Gram matrix and right-hand side of the voxel's basis, shared by every
        // solve of the regularizer; GCV's singular values first (their
        // workspace overlaps the staged basis, not the Gram matrix)
        if (P.angle_mode == 1) {
            gram_load(w.g, P.Gs, n);
            gram_rhs_t(w.g, P.AsT, m, n, w.data);
        } else {
            gram_build_f32(w.g, w.As32, w.ldA, m, n, w.data);
        }
        if (P.reg == 2) gram_svdvals(w.g, w.g.L, m, n, w.scr + (long)P.m * P.n + 3L * P.K + (long)kCacheCap * 19);
    }

    double mu = CUDART_NAN, chi2 = CUDART_NAN;
    switch (P.reg) {
    case 0: {  // none
        NnlsResult r = basis_lsq(w, false, 0.0);
        note(w, r);
        save_x(w);
        mu = 0; chi2 = 1;
        break;
    }
    case 1: reg_lcurve(w, mu, chi2); break;
    case 2: reg_gcv(w, mu, chi2); break;
    case 3:
        if (kLegacyKernel && P.legacy) reg_chi2_legacy(w, P.chi2factor, mu, chi2);
        else reg_chi2(w, P.chi2factor, mu, chi2);
        break;
    default: {
        double delta = sqrt((double)m) * (P.noiselevel / mx);
        reg_mdp(w, delta, mu, chi2);
    }
    }

    // save_results!: rescale, fit, residuals and distribution statistics
    double sd = 0, sr2 = 0, sr = 0, dotl = 0;
    #pragma unroll 1
    for (int j = lane; j < n; j += 32) {
        double dj = w.xout[j] * mx;
        w.s.w[j] = dj;  // rescaled distribution (w is free now)
    }
    __syncwarp();
    double res[4] = {0, 0, 0, 0};
#pragma unroll
    for (int t = 0; t < 4; ++t) {
        int i = lane + 32 * t;
        if (i < m) {
            double fit = 0;
            #pragma unroll 1
            for (int j = 0; j < n; ++j) fit = fma(w.A[i + (long)j * m], w.s.w[j], fit);
            double bi = w.data[i] * mx;
            double ri = fit - bi;
            res[t] = ri;
            sr2 = __dadd_rn(sr2, __dmul_rn(ri, ri));
            sr = __dadd_rn(sr, ri);
            if (P.decaycurve) P.decaycurve[v + P.V * i] = fit;
        }
    }
    #pragma unroll 1
    for (int j = lane; j < n; j += 32) {
        double dj = w.s.w[j];
        sd = __dadd_rn(sd, dj);
        dotl = __dadd_rn(dotl, __dmul_rn(dj, P.logt2[j]));
    }
    sd = wsum(sd); sr2 = wsum(sr2); sr = wsum(sr); dotl = wsum(dotl);
    double mean = sr / m, var = 0;
#pragma unroll
    for (int t = 0; t < 4; ++t) {
        int i = lane + 32 * t;
        if (i < m) { double d = res[t] - mean; var = __dadd_rn(var, __dmul_rn(d, d)); }
    }
    var = wsum(var);
    double lggm = dotl / sd, lgva = 0;
    #pragma unroll 1
    for (int j = lane; j < n; j += 32) {
        double d = P.logt2[j] - lggm;
        lgva = __dadd_rn(lgva, __dmul_rn(__dmul_rn(d, d), w.s.w[j]));
    }
    lgva = wsum(lgva) / sd;
    #pragma unroll 1
    for (int j = lane; j < n; j += 32) P.dist[v + P.V * j] = w.s.w[j];
    if (P.basis_out && P.angle_mode != 1)
        #pragma unroll 1
        for (long q = lane; q < (long)m * n; q += 32) P.basis_out[v + P.V * q] = w.A[q];
    if (lane == 0) {
        P.gdn[v] = sd;
        P.ggm[v] = pm_exp(lggm);
        P.gva[v] = pm_expm1(lgva);
        P.fnr[v] = sd / sqrt(sr2 / (m - 1));
        P.snr[v] = mx / sqrt(var / (m - 1));
        P.alpha[v] = alpha;
        if (P.resnorm) P.resnorm[v] = sqrt(sr2);
        if (P.mu) P.mu[v] = mu;
        if (P.chi2f) P.chi2f[v] = chi2;
    }
    // fused T2partSEcorr window sums (src/T2partSEcorr.jl:95-138)
    if (P.fuse_t2part) {
        // Each window sum runs in T2partSEcorr's loop order in a lane of its
        // own (total, SPWin, MPWin, sigmoid weights), so the fused maps equal
        // the standalone T2part of the saved distribution bit for bit.
        const double *dv = w.s.w;
        bool anynan = false;
        #pragma unroll 1
        for (int j = lane; j < n; j += 32) anynan |= isnan(dv[j]);
        anynan = __any_sync(FULL, anynan);
        double a0 = 0, a1 = 0;
        if (lane == 0) {
            #pragma unroll 1
            for (int j = 0; j < n; ++j) a0 = __dadd_rn(a0, dv[j]);
        } else if (lane == 1 || lane == 2) {
            const int j0 = lane == 1 ? P.sp0 : P.mp0, j1 = lane == 1 ? P.sp1 : P.mp1;
            #pragma unroll 1
            for (int j = j0; j <= j1; ++j) { a0 = __dadd_rn(a0, __dmul_rn(dv[j], P.logt2[j])); a1 = __dadd_rn(a1, dv[j]); }
        } else if (lane == 3 && P.weights) {
            #pragma unroll 1
            for (int j = 0; j < n; ++j) a0 = __dadd_rn(a0, __dmul_rn(dv[j], P.weights[j]));
        }
        const double tsd = __shfl_sync(FULL, a0, 0), dsp = __shfl_sync(FULL, a0, 1), ssp = __shfl_sync(FULL, a1, 1);
        const double dmp = __shfl_sync(FULL, a0, 2), smp = __shfl_sync(FULL, a1, 2), dw = __shfl_sync(FULL, a0, 3);
        if (lane == 0 && !anynan) {
            if (tsd > 0) {
                P.sfr[v] = P.weights ? dw / tsd : ssp / tsd;
                P.mfr[v] = smp / tsd;
            }
            if (ssp > 0) P.sgm[v] = pm_exp(dsp / ssp);
            if (smp > 0) P.mgm[v] = pm_exp(dmp / smp);
        }
    }
    __syncwarp();
}

}  // namespace dk
