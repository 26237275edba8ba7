// nnls_gram.cuh -- Lawson-Hanson NNLS on the normal equations, one warp per
// problem: the solver of the mixed-precision method (DECAES_PREC_MIXED).
//
// The plain method factors the (m+n) x n Tikhonov-padded basis by Householder
// QR on every solve (src/NNLS.jl).  Here each basis gets its Gram matrix
// G = A'A and right-hand side f = A'b once; a Tikhonov solve at any mu then
// works on H = G + mu^2 I restricted to the passive set P:
//   * the passive set grows and shrinks exactly as in Lawson-Hanson (add the
//     column with the largest positive dual w = f - H x, step back to
//     feasibility when the unconstrained solution on P leaves the orthant);
//   * H_PP is held as an LDL' factorization (unit lower L, pivots D),
//     extended by one bordered row per added column and refactored
//     (right-looking) after a removal or a change of mu;
//   * every solve may start from the previous solve's passive set (the
//     problem is strictly convex for mu > 0, so any start reaches the same
//     minimizer): successive mu's of the regularizer searches share most of
//     their support, which cuts the number of column additions about 7x.
// All arithmetic is FP64 (the Gram matrix squares the basis condition number,
// so single precision is not enough for it); the saving is in operation count:
// per added column O(k) warp instructions on k <= n passive columns instead of
// O((m+n)(n-k)) for a Householder step.
//
// FP64 results take ~64 cycles to come back on this part, so the factorization
// avoids square roots and divisions on its dependency chain: LDL' instead of
// Cholesky, reciprocals seeded in FP32 and finished with one cubic Newton
// step, unit-diagonal substitutions (one shuffle + one FMA per step), and the
// trailing update of the factorization as independent FMAs.
//
// Storage (shared memory, packed to keep more warps resident): G as its upper
// triangle by columns, G(i,j) = Gp[j(j+1)/2 + i] for i <= j; L strictly lower
// by rows, L(r,q) = Lp[r(r-1)/2 + q] for q < r.  Passive rows r live on lanes
// r and r+32 (n <= 64).
#pragma once
#include "nnls_warp.cuh"

namespace dk {

constexpr int kGramMaxN = 64;
constexpr double kGramDepTol = 1e-12;  // reject a column when its pivot <= tol * H_tt

__device__ __forceinline__ int tri(int j) { return (j * (j + 1)) >> 1; }
// packed symmetric G: entry (i, j)
__device__ __forceinline__ int gidx(int i, int j) { return i <= j ? tri(j) + i : tri(i) + j; }

struct GramWS {
    double *G;     // packed upper triangle of the Gram matrix, n(n+1)/2
    double *L;     // packed strictly-lower unit factor of H_PP = L D L'
    double *f;     // A'b
    double *y;     // L^{-1} f_P
    double *dd;    // pivots D (during a factorization: the running diagonal)
    double *dinv;  // 1 / D
    double *xp;    // x on P (xp[r] = x[P[r]])
    int *P;        // passive columns, 0-based, k entries
    int *pos;      // pos[j] = index of column j in P, or -1
    int *lastP;    // passive set left by the previous solve (warm start)
    int lastk;
    double bb;     // b'b
};

// Warp-wide maximum (minimum) of integer keys; ties go to the smaller index.
__device__ __forceinline__ void warp_keymax(long long &key, int &j) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        long long ok = __shfl_xor_sync(FULL, key, o);
        int oj = __shfl_xor_sync(FULL, j, o);
        if (ok > key || (ok == key && oj < j)) { key = ok; j = oj; }
    }
}
__device__ __forceinline__ void warp_keymin(long long &key, int &j) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        long long ok = __shfl_xor_sync(FULL, key, o);
        int oj = __shfl_xor_sync(FULL, j, o);
        if (ok < key || (ok == key && oj < j)) { key = ok; j = oj; }
    }
}

// 1/d for normal d: the hardware's approximate FP64 reciprocal (rcp.approx,
// relative error below 2^-20) refined by one cubic Newton step
// r(1 + e + e^2), e = 1 - d r, whose error e^3 is below FP64 rounding.
__device__ __forceinline__ double fast_rcp(double d) {
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(d));
    const double e = fma(-d, r, 1.0);
    return fma(r, fma(e, e, e), r);
}

__device__ __forceinline__ double lane_pick(double v0, double v1, int i) {
    // value held for row i (rows i < 32 in v0, rows >= 32 in v1) broadcast from its lane
    return __shfl_sync(FULL, i < 32 ? v0 : v1, i & 31);
}

// An FP32 value as FP64 by moving its exponent and mantissa fields (integer
// pipes; exact for zero and normal numbers, the only values an EPG curve takes
// here).
__device__ __forceinline__ double widen(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xffu;
    const unsigned long long sgn = (unsigned long long)(u >> 31) << 63;
    const unsigned long long mag = e == 0 ? 0ull
                                          : ((unsigned long long)(e + (1023 - 127)) << 52) | ((unsigned long long)(u & 0x7fffffu) << 29);
    return __longlong_as_double((long long)(sgn | mag));
}

// b'b.
static __device__ void gram_bb(GramWS &g, int m, const double *b) {
    const int lane = threadIdx.x & 31;
    double part = 0.0;
    #pragma unroll 1
    for (int i = lane; i < m; i += 32) part = fma(b[i], b[i], part);
    g.bb = wsum(part);
}

// f = A'b from a row-major (transposed, m x n) basis in global memory: lanes
// over columns, coalesced over each row.
static __device__ __noinline__ void gram_rhs_t(GramWS &g, const double *AT, int m, int n, const double *b) {
    const int lane = threadIdx.x & 31;
    #pragma unroll 1
    for (int j = lane; j < n; j += 32) {
        double s0 = 0.0, s1 = 0.0;
        int i = 0;
        #pragma unroll 1
        for (; i + 1 < m; i += 2) {
            s0 = fma(__ldg(AT + (long)i * n + j), b[i], s0);
            s1 = fma(__ldg(AT + (long)(i + 1) * n + j), b[i + 1], s1);
        }
        if (i < m) s0 = fma(__ldg(AT + (long)i * n + j), b[i], s0);
        g.f[j] = s0 + s1;
    }
    gram_bb(g, m, b);
    __syncwarp();
}

// f = A'b from a precomputed row of products held as float pairs (hi, lo)
// (the tensor-core grid products of the voxel), times their scale to the
// normalized decay.
static __device__ __noinline__ void gram_rhs_f32(GramWS &g, const float *F, int n, double scale, int m,
                                                 const double *b) {
    const int lane = threadIdx.x & 31;
    #pragma unroll 1
    for (int j = lane; j < n; j += 32) {
        const float2 v = __ldg(reinterpret_cast<const float2 *>(F) + j);
        g.f[j] = (widen(v.x) + widen(v.y)) * scale;
    }
    gram_bb(g, m, b);
    __syncwarp();
}

// f = A'b and G = A'A from a basis staged in shared memory as FP32 values
// (column-major, odd leading dimension lda).  The staged values are the FP32
// EPG curves themselves, so the products are exact in FP64 and G is the Gram
// matrix of the basis to FP64 rounding.  Lanes over columns for f and over the
// n(n+1)/2 upper-triangle entries for G.
static __device__ __noinline__ void gram_build_f32(GramWS &g, const float *As, int lda, int m, int n, const double *b) {
    const int lane = threadIdx.x & 31;
    #pragma unroll 1
    for (int j = lane; j < n; j += 32) {
        const float *aj = As + j * lda;
        double s0 = 0.0, s1 = 0.0;
        int i = 0;
        #pragma unroll 1
        for (; i + 1 < m; i += 2) {
            s0 = fma(widen(aj[i]), b[i], s0);
            s1 = fma(widen(aj[i + 1]), b[i + 1], s1);
        }
        if (i < m) s0 = fma(widen(aj[i]), b[i], s0);
        g.f[j] = s0 + s1;
    }
    gram_bb(g, m, b);
    const int npairs = tri(n);
    #pragma unroll 1
    for (int p = lane; p < npairs; p += 32) {
        int j = (int)((sqrtf(8.0f * (float)p + 1.0f) - 1.0f) * 0.5f);
        while (tri(j) > p) --j;
        while (tri(j + 1) <= p) ++j;
        const int i = p - tri(j);
        const float *ai = As + i * lda, *aj = As + j * lda;
        double s0 = 0.0, s1 = 0.0;
        int r = 0;
        #pragma unroll 1
        for (; r + 1 < m; r += 2) {
            s0 = fma(widen(ai[r]), widen(aj[r]), s0);
            s1 = fma(widen(ai[r + 1]), widen(aj[r + 1]), s1);
        }
        if (r < m) s0 = fma(widen(ai[r]), widen(aj[r]), s0);
        g.G[p] = s0 + s1;
    }
    __syncwarp();
}

// G copied from a precomputed packed Gram matrix in global memory.
static __device__ __noinline__ void gram_load(GramWS &g, const double *Gg, int n) {
    const int lane = threadIdx.x & 31;
    const int np = tri(n);
#pragma unroll 4
    for (int q = lane; q < np; q += 32) g.G[q] = __ldg(Gg + q);
    __syncwarp();
}

// LDL' factorization of H_PP = G_PP + mu2 I from scratch (right-looking),
// with y = L^{-1} f_P carried along as an extra column.  Per pivot: one
// reciprocal, the column scaled by the lanes of its rows, and the trailing
// update -- diagonal included -- spread over lanes by (row, column) pair, so a
// step costs ~(k-j)^2/64 FMA instructions instead of k-j.  Returns false when
// a pivot is not positive relative to its diagonal (numerically dependent set).
static __device__ __noinline__ bool gram_refactor(GramWS g, int k, double mu2) {
    const int lane = threadIdx.x & 31;
    const int r0 = lane, r1 = lane + 32;
    const int p0 = r0 < k ? g.P[r0] : 0, p1 = r1 < k ? g.P[r1] : 0;
    double *L0 = g.L + tri(r0 - 1), *L1 = g.L + tri(r1 - 1);
    double *cu = g.xp;  // unscaled pivot column of the current step
    // strictly lower triangle and diagonal of H_PP, one row per lane, and each
    // row's pivot threshold tol * H_rr
    double th0 = 0.0, th1 = 0.0;
    if (r0 < k) {
        #pragma unroll 1
        for (int c = 0; c < r0; ++c) L0[c] = g.G[gidx(p0, g.P[c])];
        const double h = g.G[tri(p0) + p0] + mu2;
        g.dd[r0] = h;
        th0 = kGramDepTol * h;
    }
    if (r1 < k) {
        #pragma unroll 1
        for (int c = 0; c < r1; ++c) L1[c] = g.G[gidx(p1, g.P[c])];
        const double h = g.G[tri(p1) + p1] + mu2;
        g.dd[r1] = h;
        th1 = kGramDepTol * h;
    }
    double v0 = r0 < k ? g.f[p0] : 0.0, v1 = r1 < k ? g.f[p1] : 0.0;
    __syncwarp();
    #pragma unroll 1
    for (int j = 0; j < k; ++j) {
        const double d = g.dd[j];
        if (!gt_nonneg_bits(d, lane_pick(th0, th1, j))) return false;  // d > tol * H_jj
        const double rd = fast_rcp(d);
        const double yj = lane_pick(v0, v1, j);
        if (r0 > j && r0 < k) {
            const double c0 = L0[j], l0 = c0 * rd;
            L0[j] = l0;
            cu[r0] = c0;
            v0 = fma(-l0, yj, v0);
        }
        if (r1 > j && r1 < k) {
            const double c1 = L1[j], l1 = c1 * rd;
            L1[j] = l1;
            cu[r1] = c1;
            v1 = fma(-l1, yj, v1);
        }
        if (lane == 0) g.dinv[j] = rd;
        __syncwarp();
        // trailing lower entries (r, c), j < c <= r < k, one per lane: the
        // strictly-lower ones in L and the running diagonal (c == r) in dd
        const int t = k - 1 - j, npair = t * (t + 1) / 2;
        #pragma unroll 1
        for (int q = lane; q < npair; q += 32) {
            int a = (int)((sqrtf(8.0f * (float)q + 1.0f) - 1.0f) * 0.5f);
            while (a * (a + 1) / 2 > q) --a;
            while ((a + 1) * (a + 2) / 2 <= q) ++a;
            const int r = j + 1 + a, c = j + 1 + (q - a * (a + 1) / 2);
            double *e = c == r ? g.dd + r : g.L + tri(r - 1) + c;
            *e = fma(-cu[r], g.L[tri(c - 1) + j], *e);
        }
        __syncwarp();
    }
    if (r0 < k) g.y[r0] = v0;
    if (r1 < k) g.y[r1] = v1;
    __syncwarp();
    return true;
}

// Extends the factorization by column t (k -> k+1): u = L^{-1} H[P,t],
// w = D^{-1} u, delta = H_tt - u'w, y_t = f_t - w'y.  Rejects t when delta is
// not positive relative to H_tt or when its coefficient y_t / delta in the
// unconstrained solution on P + {t} is not positive (the guards of the
// reference's Householder step).  Returns true when t was added.
static __device__ __noinline__ bool gram_append(GramWS g, int k, int t, double mu2) {
    const int lane = threadIdx.x & 31;
    const int r0 = lane, r1 = lane + 32;
    const double *L0 = g.L + tri(r0 - 1), *L1 = g.L + tri(r1 - 1);
    double v0 = r0 < k ? g.G[gidx(g.P[r0], t)] : 0.0, v1 = r1 < k ? g.G[gidx(g.P[r1], t)] : 0.0;
    #pragma unroll 1
    for (int i = 0; i < k; ++i) {
        const double ui = lane_pick(v0, v1, i);
        if (r0 > i && r0 < k) v0 = fma(-L0[i], ui, v0);
        if (r1 > i && r1 < k) v1 = fma(-L1[i], ui, v1);
    }
    double w0 = 0.0, w1 = 0.0, pl = 0.0, py = 0.0;
    if (r0 < k) { w0 = v0 * g.dinv[r0]; pl = fma(v0, w0, pl); py = fma(w0, g.y[r0], py); }
    if (r1 < k) { w1 = v1 * g.dinv[r1]; pl = fma(v1, w1, pl); py = fma(w1, g.y[r1], py); }
    double ll, ly;
    wsum2(pl, py, ll, ly);
    const double htt = g.G[tri(t) + t] + mu2;
    const double delta = htt - ll;
    if (!gt_nonneg_bits(delta, kGramDepTol * htt)) return false;
    const double yt = g.f[t] - ly;
    if (!pos_bits(yt)) return false;
    double *Lk = g.L + tri(k - 1);
    if (r0 < k) Lk[r0] = w0;
    if (r1 < k) Lk[r1] = w1;
    if (lane == 0) {
        g.dd[k] = delta;
        g.dinv[k] = fast_rcp(delta);
        g.y[k] = yt;
        g.P[k] = t;
        g.pos[t] = k;
    }
    __syncwarp();
    return true;
}

// z = L^{-T} D^{-1} y (unit upper back substitution, lanes over rows);
// z returned in (z0, z1).
static __device__ __noinline__ double2 gram_back(const GramWS g, int k) {
    const int lane = threadIdx.x & 31;
    const int r0 = lane, r1 = lane + 32;
    double u0 = r0 < k ? g.y[r0] * g.dinv[r0] : 0.0, u1 = r1 < k ? g.y[r1] * g.dinv[r1] : 0.0;
    #pragma unroll 1
    for (int i = k - 1; i >= 0; --i) {
        const double zi = lane_pick(u0, u1, i);
        const double *Li = g.L + tri(i - 1);
        if (r0 < i) u0 = fma(-Li[r0], zi, u0);
        if (r1 < i) u1 = fma(-Li[r1], zi, u1);
    }
    return make_double2(u0, u1);
}

// Singular values of the basis for GCV, as square roots of the eigenvalues of
// its Gram matrix (the mixed method's stand-in for svdvals(A)):
//   1. Householder tridiagonalization of G in a packed lower working copy W
//      (W(r,c) = W[r(r+1)/2 + c], c <= r: the same packing as G's upper
//      triangle by columns, so the copy is a straight one), lanes over rows;
//   2. eigenvalues of the tridiagonal matrix by bisection, one eigenvalue per
//      lane, counting sign changes of the Sturm sequence p_j = (d_j - x)
//      p_{j-1} - e_{j-1}^2 p_{j-2} (no divisions on the chain; rescaled by
//      powers of two when its exponent leaves +-400).
// Only eigenvalues above tau = 1e-14 * (Gershgorin bound) are resolved: GCV's
// mu is at least exp(-8), so smaller ones enter its dof sum as 1 either way
// (error <= tau / mu^2 per eigenvalue).  Eigenvalues are resolved to an
// absolute 1e-15 * bound.  Writes the min(m,n) largest square roots in
// descending order to gam (zeros for the unresolved ones).  Uses y, xp, dd and
// dinv as scratch (free before the first solve) and W (tri(n) doubles).
static __device__ __noinline__ void gram_svdvals(GramWS g, double *W, int m, int n, double *gam) {
    const int lane = threadIdx.x & 31;
    const int np = tri(n);
#pragma unroll 1
    for (int q = lane; q < np; q += 32) W[q] = g.G[q];
    __syncwarp();
    double *d = g.dd, *e = g.dinv, *u = g.y, *qv = g.xp;
    // 1. tridiagonalization (Householder from the left and right, column k)
#pragma unroll 1
    for (int k = 0; k + 2 < n; ++k) {
        double part = 0.0;
#pragma unroll 1
        for (int r = k + 2 + lane; r < n; r += 32) { const double x = W[tri(r) + k]; part = fma(x, x, part); }
        const double sigma = wsum(part);
        const double x1 = W[tri(k + 1) + k];
        if (lane == 0) d[k] = W[tri(k) + k];
        if (!(sigma > 0)) {  // column already reduced
            if (lane == 0) e[k] = x1;
            __syncwarp();
            continue;
        }
        const double nrm = sqrt(fma(x1, x1, sigma));
        const double alpha = x1 >= 0 ? -nrm : nrm;
        const double u1 = x1 - alpha;
        const double beta = 2.0 / fma(u1, u1, sigma);
        if (lane == 0) e[k] = alpha;
#pragma unroll 1
        for (int r = k + 1 + lane; r < n; r += 32) u[r] = (r == k + 1) ? u1 : W[tri(r) + k];
        __syncwarp();
        // p = beta W22 u on rows r > k (W symmetric: W(r,c) from row max(r,c))
        double pk = 0.0;
#pragma unroll 1
        for (int r = k + 1 + lane; r < n; r += 32) {
            const int br = tri(r);
            double s0 = 0.0, s1 = 0.0;
            int c = k + 1;
#pragma unroll 1
            for (; c + 1 < n; c += 2) {
                s0 = fma(W[c <= r ? br + c : tri(c) + r], u[c], s0);
                s1 = fma(W[c + 1 <= r ? br + c + 1 : tri(c + 1) + r], u[c + 1], s1);
            }
            if (c < n) s0 = fma(W[c <= r ? br + c : tri(c) + r], u[c], s0);
            const double pr = beta * (s0 + s1);
            qv[r] = pr;
            pk = fma(u[r], pr, pk);
        }
        const double K = 0.5 * beta * wsum(pk);
        __syncwarp();
#pragma unroll 1
        for (int r = k + 1 + lane; r < n; r += 32) qv[r] = fma(-K, u[r], qv[r]);
        __syncwarp();
        // W22 -= u q' + q u' (lower triangle, row r owned by its lane)
#pragma unroll 1
        for (int r = k + 1 + lane; r < n; r += 32) {
            const int br = tri(r);
            const double ur = u[r], qr = qv[r];
#pragma unroll 1
            for (int c = k + 1; c <= r; ++c) W[br + c] = fma(-ur, qv[c], fma(-qr, u[c], W[br + c]));
        }
        __syncwarp();
    }
    if (lane == 0) {
        if (n >= 2) {
            d[n - 2] = W[tri(n - 2) + n - 2];
            e[n - 2] = W[tri(n - 1) + n - 2];
        }
        d[n - 1] = W[tri(n - 1) + n - 1];
    }
    __syncwarp();
    // squared off-diagonals (reuse W) and the Gershgorin bound
    double bnd = 0.0;
#pragma unroll 1
    for (int j = lane; j < n; j += 32) {
        const double a = j > 0 ? fabs(e[j - 1]) : 0.0, b = j + 1 < n ? fabs(e[j]) : 0.0;
        bnd = fmax(bnd, fabs(d[j]) + a + b);
        if (j + 1 < n) W[j] = e[j] * e[j];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) bnd = fmax(bnd, __shfl_xor_sync(FULL, bnd, o));
    __syncwarp();
    const double *e2 = W;
    const double tau = 1e-14 * bnd, atol = 1e-15 * bnd;
    // Sturm count: eigenvalues of the tridiagonal matrix below x
    auto count_below = [&](double x) {
        double p2 = 1.0, p1 = d[0] - x;
        bool neg = p1 <= 0;  // a zero takes the sign opposite to its predecessor (p_0 = +1)
        int c = neg;
#pragma unroll 1
        for (int j = 1; j < n; ++j) {
            double p = fma(d[j] - x, p1, -e2[j - 1] * p2);
            bool pneg = p < 0 || (p == 0 && !neg);
            c += (pneg != neg);
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
        return c;
    };
    const int nz = count_below(tau);  // eigenvalues below tau: left at zero
    const int kk = m < n ? m : n;
    const int nres = n - nz;  // resolved eigenvalues (the largest)
#pragma unroll 1
    for (int base = 0; base < nres; base += 32) {
        const int t = base + lane;       // t-th largest eigenvalue
        const bool mine = t < nres;
        const int idx = n - 1 - t;       // its index in ascending order
        double a = tau, b = bnd;
        bool done = !mine;
#pragma unroll 1
        for (int it = 0; it < 80 && __any_sync(FULL, !done); ++it) {
            const double mid = 0.5 * (a + b);
            const int c = count_below(mid);
            if (!done) {
                if (c > idx) b = mid; else a = mid;
                done = (b - a) <= fmax(atol, 4.0 * 2.220446049250313e-16 * b);
            }
        }
        if (mine && t < kk) gam[t] = sqrt(0.5 * (a + b));
    }
#pragma unroll 1
    for (int t = nres + lane; t < kk; t += 32) gam[t] = 0.0;
    __syncwarp();
}

// NNLS on H = G + mu2 I with right-hand side f (prepared by gram_rhs_t /
// gram_build_f32 / gram_load, which also set b'b).  On return x (dense, n)
// holds the solution, idx its passive columns (1-based, nsetp entries) and
// rnorm^2 = ||A x - b||^2 + mu2 ||x||^2.  mode = 1 when max_iter was reached
// (the reference's cap 3n).
static __device__ __noinline__ NnlsResult gram_nnls(GramWS g, double *x, double *wv, int *idx, int n, double mu2,
                                             int max_iter, int *lastk_io) {
    const int lane = threadIdx.x & 31;
    const int r0 = lane, r1 = lane + 32;
    #pragma unroll 1
    for (int j = lane; j < n; j += 32) { x[j] = 0.0; g.pos[j] = -1; }
    __syncwarp();
    int k = 0, iters = 0, mode = 0;

    // warm start: the previous passive set, pruned until its unconstrained
    // solution is positive
    const int lastk = *lastk_io;
    if (lastk > 0) {
        #pragma unroll 1
        for (int r = lane; r < lastk; r += 32) { g.P[r] = g.lastP[r]; g.pos[g.lastP[r]] = r; }
        __syncwarp();
        k = lastk;
        #pragma unroll 1
        for (int round = 0; round < kGramMaxN && k > 0; ++round) {
            if (!gram_refactor(g, k, mu2)) {
                #pragma unroll 1
                for (int r = lane; r < k; r += 32) g.pos[g.P[r]] = -1;
                __syncwarp();
                k = 0;
                break;
            }
            const double2 zz = gram_back(g, k);
            const double z0 = zz.x, z1 = zz.y;
            const bool keep0 = r0 < k && pos_bits(z0), keep1 = r1 < k && pos_bits(z1);
            const unsigned m0 = __ballot_sync(FULL, keep0), m1 = __ballot_sync(FULL, keep1);
            const int kk = __popc(m0) + __popc(m1);
            if (kk == k) {
                if (r0 < k) x[g.P[r0]] = z0;
                if (r1 < k) x[g.P[r1]] = z1;
                __syncwarp();
                break;
            }
            // compact P to the positive coefficients
            const int p0 = r0 < k ? g.P[r0] : -1, p1 = r1 < k ? g.P[r1] : -1;
            __syncwarp();
            const unsigned below = (1u << lane) - 1u;
            if (r0 < k) {
                if (keep0) { int d = __popc(m0 & below); g.P[d] = p0; g.pos[p0] = d; }
                else g.pos[p0] = -1;
            }
            if (r1 < k) {
                if (keep1) { int d = __popc(m0) + __popc(m1 & below); g.P[d] = p1; g.pos[p1] = d; }
                else g.pos[p1] = -1;
            }
            __syncwarp();
            k = kk;
        }
    }

    unsigned long long rejected = 0ull;  // columns refused since the last change of P (warp-uniform)
    bool dual_stale = true;
    #pragma unroll 1
    for (int outer = 0;; ++outer) {
        if (outer > 4 * max_iter) { mode = 1; break; }
        // dual w_j = f_j - sum_r G[j, P_r] x_{P_r} on the non-passive columns
        if (dual_stale) {
            #pragma unroll 1
            for (int r = lane; r < k; r += 32) g.xp[r] = x[g.P[r]];
            // the free columns in column order, compacted into idx (free until
            // the outputs), so that up to 32 of them take one round of lanes
            // (only free columns' duals are read)
            const bool fr0 = r0 < n && g.pos[r0] < 0, fr1 = r1 < n && g.pos[r1] < 0;
            const unsigned b0 = __ballot_sync(FULL, fr0), b1 = __ballot_sync(FULL, fr1);
            const unsigned below = (1u << lane) - 1u;
            if (fr0) idx[__popc(b0 & below)] = r0;
            if (fr1) idx[__popc(b0) + __popc(b1 & below)] = r1;
            const int nf = __popc(b0) + __popc(b1);
            __syncwarp();
            #pragma unroll 1
            for (int i = lane; i < nf; i += 32) {
                const int j = idx[i];
                double s = g.f[j], s2 = 0.0;
                int r = 0;
                #pragma unroll 1
                for (; r + 1 < k; r += 2) {
                    s = fma(-g.G[gidx(j, g.P[r])], g.xp[r], s);
                    s2 = fma(-g.G[gidx(j, g.P[r + 1])], g.xp[r + 1], s2);
                }
                if (r < k) s = fma(-g.G[gidx(j, g.P[r])], g.xp[r], s);
                wv[j] = s + s2;
            }
            __syncwarp();
            dual_stale = false;
        }
        if (k >= n) break;
        // entering column: largest positive dual among free, unrefused columns
        long long best = -1;
        int bj = 0x7fffffff;
        #pragma unroll 1
        for (int j = lane; j < n; j += 32) {
            if (g.pos[j] >= 0 || ((rejected >> j) & 1ull)) continue;
            const double wj = wv[j];
            if (!pos_bits(wj)) continue;
            const long long key = okey(wj);
            if (key > best) { best = key; bj = j; }
        }
        warp_keymax(best, bj);
        if (best < 0) break;
        if (!gram_append(g, k, bj, mu2)) {
            rejected |= 1ull << bj;
            continue;
        }
        k += 1;
        rejected = 0ull;
        // inner loop: move toward the unconstrained solution on P
        #pragma unroll 1
        for (;;) {
            const double2 zz = gram_back(g, k);
            const double z0 = zz.x, z1 = zz.y;
            const bool pos0 = !(r0 < k) || pos_bits(z0), pos1 = !(r1 < k) || pos_bits(z1);
            if (__all_sync(FULL, pos0 && pos1)) {
                if (r0 < k) x[g.P[r0]] = z0;
                if (r1 < k) x[g.P[r1]] = z1;
                __syncwarp();
                break;
            }
            if (++iters > max_iter) { mode = 1; break; }
            // alpha = min over z_r <= 0 of x_r / (x_r - z_r)
            double a0 = CUDART_INF, a1 = CUDART_INF;
            const double x0 = r0 < k ? x[g.P[r0]] : 0.0, x1 = r1 < k ? x[g.P[r1]] : 0.0;
            if (r0 < k && !pos_bits(z0)) { const double dz = x0 - z0; a0 = pos_bits(dz) ? x0 * fast_rcp(dz) : 0.0; }
            if (r1 < k && !pos_bits(z1)) { const double dz = x1 - z1; a1 = pos_bits(dz) ? x1 * fast_rcp(dz) : 0.0; }
            const long long ka0 = okey(a0), ka1 = okey(a1);  // a0, a1 are not NaN: min without the FP64 pipe
            long long ka = ka0 <= ka1 ? ka0 : ka1;
            int ia = ka0 <= ka1 ? r0 : r1;
            warp_keymin(ka, ia);
            const double alpha = lane_pick(a0, a1, ia);
            double nx0 = x0, nx1 = x1;
            if (r0 < k) nx0 = fma(alpha, z0 - x0, x0);
            if (r1 < k) nx1 = fma(alpha, z1 - x1, x1);
            if (r0 == ia) nx0 = 0.0;
            if (r1 == ia) nx1 = 0.0;
            const bool keep0 = r0 < k && pos_bits(nx0), keep1 = r1 < k && pos_bits(nx1);
            const unsigned m0 = __ballot_sync(FULL, keep0), m1 = __ballot_sync(FULL, keep1);
            const int p0 = r0 < k ? g.P[r0] : -1, p1 = r1 < k ? g.P[r1] : -1;
            __syncwarp();
            const unsigned below = (1u << lane) - 1u;
            if (r0 < k) {
                x[p0] = keep0 ? nx0 : 0.0;
                if (keep0) { int d = __popc(m0 & below); g.P[d] = p0; g.pos[p0] = d; }
                else g.pos[p0] = -1;
            }
            if (r1 < k) {
                x[p1] = keep1 ? nx1 : 0.0;
                if (keep1) { int d = __popc(m0) + __popc(m1 & below); g.P[d] = p1; g.pos[p1] = d; }
                else g.pos[p1] = -1;
            }
            __syncwarp();
            k = __popc(m0) + __popc(m1);
            if (!gram_refactor(g, k, mu2)) {
                // numerically dependent remainder: restart from the empty set
                #pragma unroll 1
                for (int r = lane; r < k; r += 32) { g.pos[g.P[r]] = -1; x[g.P[r]] = 0.0; }
                __syncwarp();
                k = 0;
            }
        }
        dual_stale = true;
        if (mode) break;
    }

    // outputs: passive list, warm-start set, residual
    #pragma unroll 1
    for (int r = lane; r < k; r += 32) { idx[r] = g.P[r] + 1; g.lastP[r] = g.P[r]; }
    *lastk_io = k;
    __syncwarp();
    #pragma unroll 1
    for (int r = lane; r < k; r += 32) g.xp[r] = x[g.P[r]];
    __syncwarp();
    // ||A x - b||^2 = b'b - f'x - mu^2 ||x||^2 at the solution ((G + mu^2 I)_PP x_P
    // = f_P); the cancellation costs ~eps * b'b, far below the noise floor
    double fx = 0.0, xx = 0.0;
    #pragma unroll 1
    for (int r = lane; r < k; r += 32) {
        const double xr = g.xp[r];
        fx = fma(g.f[g.P[r]], xr, fx);
        xx = fma(xr, xr, xx);
    }
    wsum2(fx, xx, fx, xx);  // the same pairings as wsum, both sums in one butterfly
    const double res = fmax(g.bb - fx - mu2 * xx, 0.0);
    NnlsResult out;
    out.nsetp = k;
    out.mode = mode;
    out.rnorm = sqrt(fma(mu2, xx, res));
    return out;
}

}  // namespace dk
