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
//   * H_PP is held as a Cholesky factor L, extended by one bordered row per
//     added column and refactored after a removal;
//   * every solve may start from the previous solve's passive set (the
//     problem is strictly convex for mu > 0, so any start reaches the same
//     minimizer): successive mu's of the regularizer searches share most of
//     their support, which cuts the number of column additions about 7x.
// All arithmetic is FP64 (the Gram matrix squares the basis condition number,
// so single precision is not enough for it); the saving is in operation count:
// per added column O(k) warp instructions on k <= n passive columns instead of
// O((m+n)(n-k)) for a Householder step.
//
// Lane layout: passive rows r live on lanes r and r+32 (n <= 64); G and L are
// in shared memory with an odd row stride so lanes walking a row or a column
// hit distinct bank pairs.
#pragma once
#include "nnls_warp.cuh"

namespace dk {

constexpr int kGramMaxN = 64;
constexpr double kGramDepTol = 1e-12;  // reject a column when d^2 <= tol * H_tt

struct GramWS {
    double *G;     // n x S symmetric Gram matrix, G[i + S*j]
    double *L;     // Cholesky factor of H_PP, row-major lower: L[r*S + q], q <= r
    double *f;     // A'b
    double *y;     // L^{-1} f_P
    double *rinv;  // 1 / L[r][r]
    double *xp;    // x on P (xp[r] = x[P[r]])
    int *P;        // passive columns, 0-based, k entries
    int *pos;      // pos[j] = index of column j in P, or -1
    int *lastP;    // passive set left by the previous solve (warm start)
    int S, lastk;
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

__device__ __forceinline__ double lane_pick(double v0, double v1, int i) {
    // value held for row i (rows i < 32 in v0, rows >= 32 in v1) broadcast from its lane
    return __shfl_sync(FULL, i < 32 ? v0 : v1, i & 31);
}

// f = A'b (lanes over columns) and b'b; A column-major with leading
// dimension lda (odd, in shared memory, so the lanes' columns fall in
// distinct bank pairs).
__device__ void gram_rhs(GramWS &g, const double *A, int lda, int m, int n, const double *b) {
    const int lane = threadIdx.x & 31;
    for (int j = lane; j < n; j += 32) {
        const double *aj = A + (long)j * lda;
        double s = 0.0;
        for (int i = 0; i < m; ++i) s = fma(aj[i], b[i], s);
        g.f[j] = s;
    }
    double part = 0.0;
    for (int i = lane; i < m; i += 32) part = fma(b[i], b[i], part);
    g.bb = wsum(part);
    __syncwarp();
}

// G = A'A from a basis staged in shared memory (As, column-major with odd
// leading dimension lda): lanes over the n(n+1)/2 upper-triangle entries.
__device__ void gram_build(GramWS &g, const double *As, int lda, int m, int n) {
    const int lane = threadIdx.x & 31, S = g.S;
    const int npairs = n * (n + 1) / 2;
    for (int p = lane; p < npairs; p += 32) {
        // p -> (i, j), i <= j, column-by-column enumeration of the upper triangle
        int j = (int)((sqrtf(8.0f * (float)p + 1.0f) - 1.0f) * 0.5f);
        while (j * (j + 1) / 2 > p) --j;
        while ((j + 1) * (j + 2) / 2 <= p) ++j;
        int i = p - j * (j + 1) / 2;
        const double *ai = As + (long)i * lda, *aj = As + (long)j * lda;
        double s = 0.0;
        for (int r = 0; r < m; ++r) s = fma(ai[r], aj[r], s);
        g.G[i + S * j] = s;
        g.G[j + S * i] = s;
    }
    __syncwarp();
}

// G copied from a precomputed n x n matrix in global memory (column-major).
__device__ void gram_load(GramWS &g, const double *Gg, int n) {
    const int lane = threadIdx.x & 31, S = g.S;
    for (int q = lane; q < n * n; q += 32) {
        int i = q % n, j = q / n;
        g.G[i + S * j] = __ldg(Gg + q);
    }
    __syncwarp();
}

// Cholesky factor of H_PP = G_PP + mu2 I from scratch (left-looking, lanes
// over rows), then y = L^{-1} f_P.  Returns false when a pivot is not
// positive relative to its diagonal (numerically dependent set).
__device__ bool gram_refactor(GramWS &g, int k, double mu2) {
    const int lane = threadIdx.x & 31, S = g.S;
    const int r0 = lane, r1 = lane + 32;
    const int p0 = r0 < k ? g.P[r0] : 0, p1 = r1 < k ? g.P[r1] : 0;
    for (int j = 0; j < k; ++j) {
        const int pj = g.P[j];
        const double *Lj = g.L + (long)j * S;
        double s0 = 0.0, s1 = 0.0;
        if (r0 >= j && r0 < k) {
            s0 = g.G[p0 + S * pj] + (r0 == j ? mu2 : 0.0);
            const double *Lr = g.L + (long)r0 * S;
            for (int q = 0; q < j; ++q) s0 = fma(-Lr[q], Lj[q], s0);
        }
        if (r1 >= j && r1 < k) {
            s1 = g.G[p1 + S * pj] + (r1 == j ? mu2 : 0.0);
            const double *Lr = g.L + (long)r1 * S;
            for (int q = 0; q < j; ++q) s1 = fma(-Lr[q], Lj[q], s1);
        }
        const double d2 = lane_pick(s0, s1, j);
        const double hjj = g.G[pj + S * pj] + mu2;
        if (!(d2 > kGramDepTol * hjj)) return false;
        const double d = sqrt(d2), rd = 1.0 / d;
        if (r0 > j && r0 < k) g.L[(long)r0 * S + j] = s0 * rd;
        if (r1 > j && r1 < k) g.L[(long)r1 * S + j] = s1 * rd;
        if (lane == 0) { g.L[(long)j * S + j] = d; g.rinv[j] = rd; }
        __syncwarp();
    }
    // y = L^{-1} f_P, column-oriented forward substitution
    double v0 = r0 < k ? g.f[p0] : 0.0, v1 = r1 < k ? g.f[p1] : 0.0;
    for (int i = 0; i < k; ++i) {
        const double yi = lane_pick(v0, v1, i) * g.rinv[i];
        if (r0 == i) v0 = yi;
        if (r1 == i) v1 = yi;
        if (r0 > i && r0 < k) v0 = fma(-g.L[(long)r0 * S + i], yi, v0);
        if (r1 > i && r1 < k) v1 = fma(-g.L[(long)r1 * S + i], yi, v1);
    }
    if (r0 < k) g.y[r0] = v0;
    if (r1 < k) g.y[r1] = v1;
    __syncwarp();
    return true;
}

// Extends the factor by column t (k -> k+1).  Rejects t when its Schur
// complement is not positive relative to H_tt or when its coefficient in the
// unconstrained solution on P + {t} is not positive (the guards of the
// reference's Householder step).  Returns true when t was added.
__device__ bool gram_append(GramWS &g, int k, int t, double mu2) {
    const int lane = threadIdx.x & 31, S = g.S;
    const int r0 = lane, r1 = lane + 32;
    double v0 = r0 < k ? g.G[g.P[r0] + S * t] : 0.0, v1 = r1 < k ? g.G[g.P[r1] + S * t] : 0.0;
    for (int i = 0; i < k; ++i) {
        const double li = lane_pick(v0, v1, i) * g.rinv[i];
        if (r0 == i) v0 = li;
        if (r1 == i) v1 = li;
        if (r0 > i && r0 < k) v0 = fma(-g.L[(long)r0 * S + i], li, v0);
        if (r1 > i && r1 < k) v1 = fma(-g.L[(long)r1 * S + i], li, v1);
    }
    double pl = 0.0, py = 0.0;
    if (r0 < k) { pl = fma(v0, v0, pl); py = fma(v0, g.y[r0], py); }
    if (r1 < k) { pl = fma(v1, v1, pl); py = fma(v1, g.y[r1], py); }
    const double ll = wsum(pl), ly = wsum(py);
    const double htt = g.G[t + S * t] + mu2;
    const double d2 = htt - ll;
    if (!(d2 > kGramDepTol * htt)) return false;
    const double d = sqrt(d2);
    const double yt = (g.f[t] - ly) / d;
    if (!(yt > 0)) return false;
    if (r0 < k) g.L[(long)k * S + r0] = v0;
    if (r1 < k) g.L[(long)k * S + r1] = v1;
    if (lane == 0) {
        g.L[(long)k * S + k] = d;
        g.rinv[k] = 1.0 / d;
        g.y[k] = yt;
        g.P[k] = t;
        g.pos[t] = k;
    }
    __syncwarp();
    return true;
}

// z = L^{-T} y (back substitution, lanes over rows); z returned in (z0, z1).
__device__ void gram_back(const GramWS &g, int k, double &z0, double &z1) {
    const int lane = threadIdx.x & 31, S = g.S;
    const int r0 = lane, r1 = lane + 32;
    double u0 = r0 < k ? g.y[r0] : 0.0, u1 = r1 < k ? g.y[r1] : 0.0;
    for (int i = k - 1; i >= 0; --i) {
        const double zi = lane_pick(u0, u1, i) * g.rinv[i];
        if (r0 == i) u0 = zi;
        if (r1 == i) u1 = zi;
        if (r0 < i) u0 = fma(-g.L[(long)i * S + r0], zi, u0);
        if (r1 < i) u1 = fma(-g.L[(long)i * S + r1], zi, u1);
    }
    z0 = u0;
    z1 = u1;
}

// NNLS on H = G + mu2 I with right-hand side f (prepared by gram_rhs and
// gram_build / gram_load).  On return x (dense, n) holds the solution, idx
// its passive columns (1-based, nsetp entries) and rnorm^2 = ||A x - b||^2 +
// mu2 ||x||^2 with the residual formed explicitly from A (column-major m x n,
// global or shared).  mode = 1 when max_iter was reached (the reference's
// iteration cap 3n).
__device__ __noinline__ NnlsResult gram_nnls(GramWS g, double *x, double *wv, int *idx, const double *A, int m, int n,
                                             const double *b, double mu2, int max_iter, int *lastk_io) {
    const int lane = threadIdx.x & 31;
    const int r0 = lane, r1 = lane + 32;
    for (int j = lane; j < n; j += 32) { x[j] = 0.0; g.pos[j] = -1; }
    __syncwarp();
    int k = 0, iters = 0, mode = 0;

    // warm start: the previous passive set, pruned until its unconstrained
    // solution is positive
    const int lastk = *lastk_io;
    if (lastk > 0) {
        for (int r = lane; r < lastk; r += 32) { g.P[r] = g.lastP[r]; g.pos[g.lastP[r]] = r; }
        __syncwarp();
        k = lastk;
        for (int round = 0; round < kGramMaxN && k > 0; ++round) {
            if (!gram_refactor(g, k, mu2)) {
                for (int r = lane; r < k; r += 32) g.pos[g.P[r]] = -1;
                __syncwarp();
                k = 0;
                break;
            }
            double z0, z1;
            gram_back(g, k, z0, z1);
            const bool keep0 = r0 < k && z0 > 0, keep1 = r1 < k && z1 > 0;
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
    for (int outer = 0;; ++outer) {
        if (outer > 4 * max_iter) { mode = 1; break; }
        // dual w_j = f_j - sum_r G[j, P_r] x_{P_r} on the non-passive columns
        if (dual_stale) {
            for (int r = lane; r < k; r += 32) g.xp[r] = x[g.P[r]];
            __syncwarp();
            for (int j = lane; j < n; j += 32) {
                double s = g.f[j];
                if (g.pos[j] < 0)
                    for (int r = 0; r < k; ++r) s = fma(-g.G[j + g.S * g.P[r]], g.xp[r], s);
                wv[j] = s;
            }
            __syncwarp();
            dual_stale = false;
        }
        if (k >= n) break;
        // entering column: largest positive dual among free, unrefused columns
        long long best = -1;
        int bj = 0x7fffffff;
        for (int j = lane; j < n; j += 32) {
            if (g.pos[j] >= 0 || ((rejected >> j) & 1ull)) continue;
            const double wj = wv[j];
            if (!(wj > 0)) continue;
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
        for (;;) {
            double z0, z1;
            gram_back(g, k, z0, z1);
            const bool pos0 = !(r0 < k) || z0 > 0, pos1 = !(r1 < k) || z1 > 0;
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
            if (r0 < k && !(z0 > 0)) a0 = (x0 - z0 > 0) ? x0 / (x0 - z0) : 0.0;
            if (r1 < k && !(z1 > 0)) a1 = (x1 - z1 > 0) ? x1 / (x1 - z1) : 0.0;
            long long ka = okey(a0 <= a1 ? a0 : a1);
            int ia = a0 <= a1 ? r0 : r1;
            warp_keymin(ka, ia);
            const double alpha = lane_pick(a0, a1, ia);
            double nx0 = x0, nx1 = x1;
            if (r0 < k) nx0 = fma(alpha, z0 - x0, x0);
            if (r1 < k) nx1 = fma(alpha, z1 - x1, x1);
            if (r0 == ia) nx0 = 0.0;
            if (r1 == ia) nx1 = 0.0;
            const bool keep0 = r0 < k && nx0 > 0, keep1 = r1 < k && nx1 > 0;
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
                for (int r = lane; r < k; r += 32) { g.pos[g.P[r]] = -1; x[g.P[r]] = 0.0; }
                __syncwarp();
                k = 0;
            }
        }
        dual_stale = true;
        if (mode) break;
    }

    // outputs: passive list, warm-start set, residual
    for (int r = lane; r < k; r += 32) { idx[r] = g.P[r] + 1; g.lastP[r] = g.P[r]; }
    *lastk_io = k;
    __syncwarp();
    for (int r = lane; r < k; r += 32) g.xp[r] = x[g.P[r]];
    __syncwarp();
    double res = 0.0, xx = 0.0;
    for (int i = lane; i < m; i += 32) {
        double ri = b[i];
        for (int r = 0; r < k; ++r) ri = fma(-A[i + (long)m * g.P[r]], g.xp[r], ri);
        res = fma(ri, ri, res);
    }
    for (int r = lane; r < k; r += 32) xx = fma(g.xp[r], g.xp[r], xx);
    res = wsum(res);
    xx = wsum(xx);
    NnlsResult out;
    out.nsetp = k;
    out.mode = mode;
    out.rnorm = sqrt(fma(mu2, xx, res));
    return out;
}

}  // namespace dk
