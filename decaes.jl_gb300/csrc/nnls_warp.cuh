// nnls_warp.cuh -- warp-cooperative Lawson-Hanson NNLS in FP64 (one voxel per warp).
//
// Restates src/NNLS.jl (unsafe_nnls! at 605-825 and its Tikhonov form at
// 827-1061) and the NNLSProblem warm start of src/lsqnonneg.jl:30-164.
//
// GB300 mapping (all control flow is warp-uniform; every lane holds the same
// scalars):
//   * the working matrix lives in shared memory, column-major with an odd
//     leading dimension so both row-parallel and column-parallel accesses are
//     free of bank conflicts;
//   * the reference's physical column swaps are replaced by the idx
//     permutation itself: logical column j lives in physical column
//     idx[j]-1, which is exactly where the reference's swaps would have moved
//     its data, so adds and deletes move no matrix data;
//   * Householder application and dual updates run lanes-over-columns, each
//     lane accumulating its column sequentially in the reference's row order
//     (so those dot products are bitwise the reference's);
//   * Householder construction, the warm-start scalars and residual norms run
//     lanes-over-rows with butterfly reductions (reassociated sums, like the
//     reference's @simd loops).
// Every loop is bounded; the NNLS iteration cap is the reference's 3n.
#pragma once
#include <cuda_runtime.h>
#include <math_constants.h>

namespace dk {

constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ double wsum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = __dadd_rn(v, __shfl_xor_sync(FULL, v, o));
    return v;
}
__device__ __forceinline__ double bcast(double v, int src) { return __shfl_sync(FULL, v, src); }
__device__ __forceinline__ int bcasti(int v, int src) { return __shfl_sync(FULL, v, src); }

// Julia's Base.max / Base.min for Float64 (NaN-propagating, -0.0 < 0.0),
// decided on the integer pipes: tkey orders non-NaN doubles as their values
// with -0.0 below +0.0, which is the order signbit(x - y) gives (x - y is -0.0
// only for x = -0.0, y = +0.0; for equal values, infinities included, x is
// kept).
__device__ __forceinline__ long long tkey(double d) {
    const long long b = __double_as_longlong(d);
    return b >= 0 ? b : (b ^ 0x7fffffffffffffffLL);
}
__device__ __forceinline__ bool isnan_bits(double d);
__device__ __forceinline__ double jmax(double x, double y) {
    if (isnan_bits(x) || isnan_bits(y)) return CUDART_NAN;
    return tkey(x) < tkey(y) ? y : x;
}
__device__ __forceinline__ double jmin(double x, double y) {
    if (isnan_bits(x) || isnan_bits(y)) return CUDART_NAN;
    return tkey(x) < tkey(y) ? x : y;
}

// Order-preserving integer image of a double for comparisons on the integer
// pipes (the FP64 pipe is the kernel's bottleneck): for non-NaN a, b,
// okey(a) < okey(b) iff a < b, with -0.0 and +0.0 mapped to the same key.
__device__ __forceinline__ long long okey(double d) {
    long long b = __double_as_longlong(d);
    if ((b << 1) == 0) return 0;
    return b >= 0 ? b : (b ^ 0x7fffffffffffffffLL);
}
__device__ __forceinline__ bool isnan_bits(double d) {
    return (__double_as_longlong(d) & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL;
}
// d > 0 on the integer pipes (false for zeros and NaN).
__device__ __forceinline__ bool pos_bits(double d) {
    const long long b = __double_as_longlong(d);
    return b > 0 && b <= 0x7ff0000000000000LL;
}
// d > t for a threshold t with its sign bit clear (+0.0 or positive) or NaN,
// on the integer pipes: such doubles order like their bit patterns; negative d
// and NaN d give false, and so does every d against a NaN threshold, as the
// FP64 comparison does.  (t = -0.0 is not covered: +0.0 would compare above
// it.  The solver's thresholds are tol * (sum of squares + mu^2), never -0.0.)
__device__ __forceinline__ bool gt_nonneg_bits(double d, double t) {
    const long long b = __double_as_longlong(d);
    return b > __double_as_longlong(t) && b <= 0x7ff0000000000000LL && !isnan_bits(t);
}
// wsum of two values at once: the first butterfly step exchanges a and b
// between the warp halves, so both sums take five additions instead of ten;
// each sum is added in wsum's order, so the results are wsum's bit for bit.
__device__ __forceinline__ void wsum2(double a, double b, double &sa, double &sb) {
    const bool hi = (threadIdx.x & 16) != 0;
    double v = __dadd_rn(hi ? b : a, __shfl_xor_sync(FULL, hi ? a : b, 16));
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) v = __dadd_rn(v, __shfl_xor_sync(FULL, v, o));
    sa = __shfl_sync(FULL, v, 0);
    sb = __shfl_sync(FULL, v, 16);
}

// Per-warp views of the NNLS workspace (shared memory).
struct NnlsWS {
    double *C;    // lda x n, physical columns
    double *b;    // lda (right-hand side, transformed in place)
    double *zz;   // lda
    double *x;    // n, indexed by original column (0-based)
    double *w;    // n, indexed by logical position (0-based)
    int *idx;     // n, 1-based original column at each logical position
    unsigned char *diag;  // n, indexed by original column
    double *rdiag;        // n, RN(1/diagonal) of each physical column in set P
    int *posof;           // n, 1-based logical position of each physical column (inverse of idx)
    int *zl;              // n, scratch list of physical columns
    int lda;
};

// Physical columns whose logical position is >= jfirst, in increasing
// physical order, written to s.zl; returns their count.  Column-parallel
// loops walk this list so the lanes of a half-warp read distinct bank pairs
// (odd leading dimension), instead of the random physical columns that the
// logical order would give.
__device__ __forceinline__ int warp_active_cols(const NnlsWS &s, int n, int jfirst) {
    const int lane = threadIdx.x & 31;
    int base = 0;
    for (int c = 0; c < n; c += 32) {
        int p = c + lane;
        bool z = p < n && s.posof[p] >= jfirst;
        unsigned msk = __ballot_sync(0xffffffffu, z);
        if (z) s.zl[base + __popc(msk & ((1u << lane) - 1))] = p;
        base += __popc(msk);
    }
    __syncwarp();
    return base;
}

// a / b from r = RN(1/b): q = RN(a r), remainder e = a - b q (exact by fma),
// q' = RN(q + e r).  Markstein's correction (P. Markstein, IBM J. Res. Dev.
// 34(1), 1990) returns the correctly rounded quotient for normal operands, so
// results are bitwise those of a / b at three FP64 operations instead of a
// full division.
__device__ __forceinline__ double mdiv(double a, double b, double r) {
    double q = __dmul_rn(a, r);
    double e = fma(-q, b, a);
    return fma(e, r, q);
}

__device__ __forceinline__ double &Aat(const NnlsWS &s, int i1, int j1) {
    // 1-based row i1 of logical column j1
    return s.C[(i1 - 1) + (size_t)(s.idx[j1 - 1] - 1) * s.lda];
}

// Base.hypot for Float64 (C. F. Borges, "An Improved Algorithm for
// hypot(a,b)", 2019, fma-corrected), used by NNLS.orthogonal_rotmat.
static __device__ double jl_hypot(double x, double y) {
    if (isinf(x) || isinf(y)) return CUDART_INF;
    double ax = fabs(x), ay = fabs(y);
    if (ay > ax) { double t = ax; ax = ay; ay = t; }
    if (ay <= ax * 1.0536712127723509e-08) return ax;
    double scale = 2.220446049250313e-16 * 1.4916681462400413e-154;
    if (ax > 9.480751908109176e+153) {
        ax = ax * scale; ay = ay * scale; scale = 1.0 / scale;
    } else if (ay < 1.4916681462400413e-154) {
        ax = ax / scale; ay = ay / scale;
    } else {
        scale = 1.0;
    }
    double h = sqrt(fma(ax, ax, __dmul_rn(ay, ay)));
    double hsq = __dmul_rn(h, h), axsq = __dmul_rn(ax, ax);
    h -= (fma(-ay, ay, hsq - axsq) + fma(h, h, -hsq) - fma(ax, ax, -axsq)) / (2 * h);
    return h * scale;
}

// construct_apply_householder!(A, b, ip, jp, m), src/NNLS.jl:259-336.
// Writes only the pivot column's physical storage (see header note).
static __device__ double warp_cah(const NnlsWS &s, int ip, int jp, int m) {
    const int lane = threadIdx.x & 31;
    if (ip > m) return 0.0;
    double *col = s.C + (size_t)(s.idx[jp - 1] - 1) * s.lda;  // pivot column (0-based rows)
    double alpha = col[ip - 1];
    double part = 0.0;
    for (int i = ip + lane; i <= m; i += 32) part = fma(col[i - 1], col[i - 1], part);
    double xnorm = sqrt(wsum(part));
    if (xnorm == 0) return -1.0;
    double beta = copysign(xnorm, alpha);
    alpha = alpha + beta;
    const double rbeta = 1.0 / beta;
    double tau = mdiv(alpha, beta, rbeta);
    const double ralpha = 1.0 / alpha;
    // quotients A[i,jp]/alpha, staged in zz (free between solves of the main loop)
    part = 0.0;
    for (int i = ip + 1 + lane; i <= m; i += 32) {
        double qi = mdiv(col[i - 1], alpha, ralpha);
        s.zz[i - 1] = qi;
        part = fma(s.b[i - 1], qi, part);
    }
    double sm = s.b[ip - 1] + wsum(part);
    sm *= -tau;
    double A1 = -beta;
    double b1 = s.b[ip - 1] + sm;
    // b1 / A1 > 0: same nonzero sign and no underflow of the quotient
    bool good;
    if (b1 != 0 && fabs(b1) > 0x1p-900 * fabs(A1)) good = (b1 > 0) == (A1 > 0);
    else good = b1 / A1 > 0;
    if (good) {
        if (ip < m) {
            __syncwarp();
            for (int i = ip + 1 + lane; i <= m; i += 32) {
                double qi = s.zz[i - 1];
                col[i - 1] = qi;
                s.b[i - 1] = fma(sm, qi, s.b[i - 1]);
            }
            const double rA1 = -rbeta;  // 1 / (-beta), exact negation
            if (lane == 0) {
                s.b[ip - 1] = b1;
                col[ip - 1] = A1;
                s.rdiag[s.idx[jp - 1] - 1] = rA1;
            }
            __syncwarp();
        } else {
            tau = 0.0;  // column swap only: done by the caller's idx swap
            const double rd = 1.0 / col[ip - 1];
            if (lane == 0) s.rdiag[s.idx[jp - 1] - 1] = rd;
            __syncwarp();
        }
        return tau;
    }
    return -1.0;
}

// apply_householder_dual!(A, w, b, tau, j1, m1), src/NNLS.jl:379-436.
// Lanes over logical columns j1+1..n.
static __device__ void warp_ahd(const NnlsWS &s, int n, double tau, int j1, int m1) {
    const int lane = threadIdx.x & 31;
    if (j1 >= m1) return;
    const double *u = s.C + (size_t)(s.idx[j1 - 1] - 1) * s.lda;  // u[j1-1] is the diagonal; treated as 1
    const int nz = warp_active_cols(s, n, j1 + 1);
    for (int r0 = 0; r0 < nz; r0 += 32) {
        int r = r0 + lane;
        if (r < nz) {
            const int p = s.zl[r];
            double *a = s.C + (size_t)p * s.lda;
            double sm = fma(a[j1 - 1], 1.0, 0.0);
            for (int i = j1 + 1; i <= m1; ++i) sm = fma(a[i - 1], u[i - 1], sm);
            sm *= -tau;
            double wj = 0.0;
            a[j1 - 1] = a[j1 - 1] + sm;
            for (int i = j1 + 1; i <= m1; ++i) {
                double v = fma(sm, u[i - 1], a[i - 1]);
                wj = fma(v, s.b[i - 1], wj);
                a[i - 1] = v;
            }
            s.w[s.posof[p] - 1] = wj;
        }
    }
    __syncwarp();
}

// compute_dual!(w, A, b, j1, m1), src/NNLS.jl:441-470.  Lanes over columns.
static __device__ void warp_compute_dual(const NnlsWS &s, int n, int j1, int m1) {
    const int lane = threadIdx.x & 31;
    const int nz = warp_active_cols(s, n, j1);
    for (int r0 = 0; r0 < nz; r0 += 32) {
        int r = r0 + lane;
        if (r < nz) {
            const int p = s.zl[r];
            const double *a = s.C + (size_t)p * s.lda;
            double sm = 0.0;
            for (int i = j1; i <= m1; ++i) sm = fma(a[i - 1], s.b[i - 1], sm);
            s.w[s.posof[p] - 1] = sm;
        }
    }
    __syncwarp();
}

// zz[1:n] = b[1:n]; solve_triangular_system!(zz, A, n), src/NNLS.jl:506-523.
// Lanes over rows; the column sweep is sequential as in the reference.
static __device__ void warp_solve_tri(const NnlsWS &s, int n) {
    const int lane = threadIdx.x & 31;
    for (int i = lane; i < n; i += 32) s.zz[i] = s.b[i];
    __syncwarp();
    for (int j = n; j >= 1; --j) {
        const int pj = s.idx[j - 1] - 1;
        const double *a = s.C + (size_t)pj * s.lda;
        double zi = -mdiv(s.zz[j - 1], a[j - 1], s.rdiag[pj]);
        for (int i = 1 + lane; i <= j - 1; i += 32) s.zz[i - 1] = fma(a[i - 1], zi, s.zz[i - 1]);
        __syncwarp();
        if (lane == 0) s.zz[j - 1] = -zi;
        __syncwarp();
    }
}

// Transposed solve (U' z = x) on the first n logical columns, src/NNLS.jl:524-537.
static __device__ void warp_solve_tri_t(const NnlsWS &s, double *z, int n) {
    const int lane = threadIdx.x & 31;
    for (int j = 1; j <= n; ++j) {
        const double *a = s.C + (size_t)(s.idx[j - 1] - 1) * s.lda;
        double part = 0.0;
        for (int l = 1 + lane; l <= j - 1; l += 32) part = fma(-a[l - 1], z[l - 1], part);
        double z1 = z[j - 1] + wsum(part);
        z1 /= a[j - 1];
        __syncwarp();
        if (lane == 0) z[j - 1] = z1;
        __syncwarp();
    }
}

// Largest positive dual over logical positions j1..n (first maximum wins,
// as the reference's `w[j] > wmax` scan from wmax = 0).  Positive doubles
// order like their bit patterns, so the search runs on the integer pipes.
__device__ __forceinline__ void warp_largest_dual(const NnlsWS &s, int n, int j1, double &wmax, int &jmax) {
    const int lane = threadIdx.x & 31;
    long long km = 0;
    int jm = 0;
    for (int j = j1 + lane; j <= n; j += 32) {
        long long k = __double_as_longlong(s.w[j - 1]);
        if (k > 0 && k <= 0x7ff0000000000000LL && k > km) { km = k; jm = j; }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        long long ok = __shfl_xor_sync(FULL, km, o);
        int oj = __shfl_xor_sync(FULL, jm, o);
        if (ok > km || (ok == km && oj != 0 && (jm == 0 || oj < jm))) { km = ok; jm = oj; }
    }
    wmax = __longlong_as_double(km);
    jmax = jm;
}

struct NnlsResult {
    int nsetp;
    int mode;
    double rnorm;
};

// Main + secondary loops of unsafe_nnls! (tikh = false) and of its Tikhonov
// form (tikh = true, rows M = m0 + n with lazily activated padding rows).
static __device__ NnlsResult warp_nnls(const NnlsWS &s, int M, int n, int m0, bool tikh, double lam, int max_iter) {
    const int lane = threadIdx.x & 31;
    int m = tikh ? m0 : M;
    int nsetp = 0, iter = 0, mode = 0;
    bool terminated = false;
    for (;;) {
        if (nsetp >= n || (!tikh && nsetp >= m)) break;
        int jmax = nsetp;
        double tau = 0.0;
        for (;;) {
            double wmax;
            warp_largest_dual(s, n, nsetp + 1, wmax, jmax);
            if (wmax <= 0) { terminated = true; break; }
            if (tikh && !s.diag[s.idx[jmax - 1] - 1]) {
                if (lane == 0) Aat(s, m + 1, jmax) = lam;
                __syncwarp();
            }
            tau = warp_cah(s, nsetp + 1, jmax, tikh ? min(m + 1, M) : m);
            if (tau >= 0) break;
            __syncwarp();
            if (lane == 0) {
                s.w[jmax - 1] = 0.0;
                if (tikh && m < M) Aat(s, m + 1, jmax) = 0.0;
            }
            __syncwarp();
        }
        if (terminated) break;
        if (tikh && !s.diag[s.idx[jmax - 1] - 1]) {
            m = min(m + 1, M);
            __syncwarp();
            if (lane == 0) s.diag[s.idx[jmax - 1] - 1] = 1;
        }
        nsetp += 1;
        __syncwarp();
        if (lane == 0) {
            int t = s.idx[nsetp - 1];
            s.idx[nsetp - 1] = s.idx[jmax - 1];
            s.idx[jmax - 1] = t;
            s.posof[s.idx[nsetp - 1] - 1] = nsetp;
            s.posof[t - 1] = jmax;
        }
        __syncwarp();
        if (nsetp < n) warp_ahd(s, n, tau, nsetp, m);
        {
            double *pc = s.C + (size_t)(s.idx[nsetp - 1] - 1) * s.lda;
            for (int i = nsetp + 1 + lane; i <= m; i += 32) pc[i - 1] = 0.0;
        }
        __syncwarp();
        if (lane == 0) s.w[nsetp - 1] = 0.0;
        __syncwarp();
        warp_solve_tri(s, nsetp);
        bool dual_flag = false;
        for (;;) {
            iter += 1;
            if (iter > max_iter) { mode = 1; terminated = true; break; }
            // feasibility step, src/NNLS.jl:700-727 (first minimum wins)
            int imv = nsetp;
            double alpha = 2.0;
            {
                long long a_key = okey(2.0);
                double a_loc = 2.0;
                int i_loc = 0;
                for (int i = 1 + lane; i <= nsetp; i += 32) {
                    double zi = s.zz[i - 1];
                    if (!isnan_bits(zi) && okey(zi) <= 0) {
                        double xi = s.x[s.idx[i - 1] - 1];
                        double t = -xi / (zi - xi);
                        long long tk = okey(t);
                        if (!isnan_bits(t) && a_key > tk) { a_key = tk; a_loc = t; i_loc = i; }
                    }
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    long long ok = __shfl_xor_sync(FULL, a_key, o);
                    double oa = __shfl_xor_sync(FULL, a_loc, o);
                    int oi = __shfl_xor_sync(FULL, i_loc, o);
                    if (oi != 0 && (i_loc == 0 || ok < a_key || (ok == a_key && oi < i_loc))) { a_key = ok; a_loc = oa; i_loc = oi; }
                }
                if (i_loc != 0) { imv = i_loc; alpha = a_loc; }
            }
            if (alpha == 2.0) break;
            dual_flag = true;
            for (int i = 1 + lane; i <= nsetp; i += 32) {
                int ix = s.idx[i - 1] - 1;
                s.x[ix] = fma(alpha, s.zz[i - 1] - s.x[ix], s.x[ix]);
            }
            __syncwarp();
            // move coefficient imv (and any infeasible ones) from set P to set Z
            for (int guard = 0; guard <= n; ++guard) {
                if (lane == 0) s.x[s.idx[imv - 1] - 1] = 0.0;
                __syncwarp();
                if (imv != nsetp) {
                    for (int i = imv + 1; i <= nsetp; ++i) {
                        double *ci = s.C + (size_t)(s.idx[i - 1] - 1) * s.lda;
                        double a = ci[i - 2], bb = ci[i - 1];
                        double sg = jl_hypot(a, bb);
                        double cc = a / sg, ss = bb / sg;
                        __syncwarp();
                        const int pi = s.idx[i - 1] - 1;
                        for (int pj = lane; pj < n; pj += 32) {
                            if (pj == pi) continue;
                            double *cj = s.C + (size_t)pj * s.lda;
                            double p = cj[i - 2], r = cj[i - 1];
                            cj[i - 2] = fma(cc, p, __dmul_rn(ss, r));
                            cj[i - 1] = fma(-ss, p, __dmul_rn(cc, r));
                        }
                        const double rsg = 1.0 / sg;
                        if (lane == 0) {
                            ci[i - 2] = sg;
                            ci[i - 1] = 0.0;
                            s.rdiag[s.idx[i - 1] - 1] = rsg;
                            double p = s.b[i - 2], r = s.b[i - 1];
                            s.b[i - 2] = fma(cc, p, __dmul_rn(ss, r));
                            s.b[i - 1] = fma(-ss, p, __dmul_rn(cc, r));
                        }
                        __syncwarp();
                    }
                    // move logical column imv to position nsetp (idx rotation; no data moves)
                    if (lane == 0) {
                        int t = s.idx[imv - 1];
                        for (int j = imv; j <= nsetp - 1; ++j) {
                            s.idx[j - 1] = s.idx[j];
                            s.posof[s.idx[j - 1] - 1] = j;
                        }
                        s.idx[nsetp - 1] = t;
                        s.posof[t - 1] = nsetp;
                    }
                    __syncwarp();
                }
                nsetp -= 1;
                // first remaining infeasible coefficient, if any
                int bad = 0;
                for (int ib = 1; ib <= nsetp; ib += 32) {
                    int i = ib + lane;
                    bool neg = (i <= nsetp) && (s.x[s.idx[i - 1] - 1] <= 0);
                    unsigned msk = __ballot_sync(FULL, neg);
                    if (msk) { bad = ib + __ffs(msk) - 1; break; }
                }
                if (bad == 0) break;
                imv = bad;
            }
            warp_solve_tri(s, nsetp);
        }
        if (terminated) break;
        if (dual_flag) warp_compute_dual(s, n, nsetp + 1, m);
        for (int i = 1 + lane; i <= nsetp; i += 32) s.x[s.idx[i - 1] - 1] = s.zz[i - 1];
        __syncwarp();
    }
    // residual norm over the remaining rows (all padded rows for the Tikhonov form)
    const int rows = tikh ? M : m;
    double part = 0.0;
    if (nsetp < rows) {
        for (int i = nsetp + 1 + lane; i <= rows; i += 32) part = fma(s.b[i - 1], s.b[i - 1], part);
    } else {
        for (int j = lane; j < n; j += 32) s.w[j] = 0.0;
    }
    __syncwarp();
    NnlsResult r;
    r.rnorm = sqrt(wsum(part));
    r.nsetp = nsetp;
    r.mode = mode;
    return r;
}

// Warm start of solve!(::NNLSProblem, A, b) (src/lsqnonneg.jl:30-84) and of
// its Tikhonov form (src/lsqnonneg.jl:86-164): copy A (global, m x n) into
// the workspace, seed the dual with column n, then run the NNLS loops.
// `data` is the (shared-memory) right-hand side; it is not modified.
// Not inlined: every caller shares one copy of the NNLS code (instruction
// cache), and the workspace views travel in registers.
static __device__ __noinline__ NnlsResult warp_lsq(const NnlsWS s, const double *A, int m, int n, const double *data,
                                            bool tikh, double mu) {
    const int lane = threadIdx.x & 31;
    const int M = tikh ? m + n : m;
    // C[:, j] = A[:, j] (coalesced), padded rows zeroed
    for (int j = 0; j < n; ++j) {
        const double *aj = A + (size_t)j * m;
        double *cj = s.C + (size_t)j * s.lda;
        for (int i = lane; i < M; i += 32) cj[i] = (i < m) ? aj[i] : 0.0;
    }
    for (int i = lane; i < M; i += 32) s.b[i] = (i < m) ? data[i] : 0.0;
    for (int j = lane; j < n; j += 32) {
        s.x[j] = 0.0;
        s.idx[j] = j + 1;
        s.posof[j] = j + 1;
        s.diag[j] = 0;
    }
    __syncwarp();
    const double *an = s.C + (size_t)(n - 1) * s.lda;
    double part = 0.0;
    for (int i = lane; i < m; i += 32) part = __dadd_rn(part, __dmul_rn(an[i], an[i]));
    double den = wsum(part);
    if (tikh) den = __dadd_rn(den, __dmul_rn(mu, mu));
    const double rden = 1.0 / den;
    part = 0.0;
    for (int i = lane; i < m; i += 32) part = __dadd_rn(part, __dmul_rn(mdiv(an[i], den, rden), data[i]));
    double xj = wsum(part);
    for (int i = lane; i < m; i += 32) s.zz[i] = __dsub_rn(data[i], __dmul_rn(an[i], xj));
    __syncwarp();
    bool pos = false;
    for (int jb = 0; jb < n - 1; jb += 32) {
        int j = jb + lane;
        if (j < n - 1) {
            const double *cj = s.C + (size_t)j * s.lda;
            double wj = 0.0;
            for (int i = 0; i < m; ++i) wj = __dadd_rn(wj, __dmul_rn(cj[i], s.zz[i]));
            s.w[j] = wj;
            pos |= !(wj <= 0);
        }
    }
    bool anypos = __any_sync(FULL, pos);
    if (lane == 0) s.w[n - 1] = anypos ? 0.0 : 1.0;
    __syncwarp();
    return warp_nnls(s, M, n, m, tikh, mu, 3 * n);
}

// sum(abs2, positive_solution): ||x||^2 over the active set in set-P order.
static __device__ double warp_seminorm_sq(const NnlsWS &s, int nsetp) {
    const int lane = threadIdx.x & 31;
    double part = 0.0;
    for (int i = lane; i < nsetp; i += 32) {
        double v = s.x[s.idx[i] - 1];
        part = __dadd_rn(part, __dmul_rn(v, v));
    }
    return wsum(part);
}

}  // namespace dk
