// legacy.cuh -- the legacy algorithms (T2mapOptions.legacy = true) on one warp:
//   * Julia's start:step:stop for Float64 (Base twiceprecision.jl, Julia 1.9):
//     a StepRangeLen with a TwicePrecision reference and step, element i
//     computed as the range's getindex computes it;
//   * Dierckx.Spline1D(x, y; k, bc = "extrapolate", s = 0)
//     (src/splines.jl:312-315), i.e. netlib FITPACK curfit/fpcurf with s = 0
//     (interpolating spline; Givens QR of the banded collocation matrix,
//     fpgivs/fprota/fpback) and splev/fpbspl (de Boor-Cox B-spline values);
//   * spline_opt_legacy / spline_root_legacy (src/splines.jl:417-446): the
//     spline sampled on knots[1]:0.001:knots[end], first strict minimum of the
//     spline (or of |spline - value|).
// The fit is a short serial recurrence (lane 0); the sampling (~10^5 points
// for a 50..180 degree search) is spread over the lanes, each lane walking its
// points in increasing order with its knot interval and interval constants in
// registers.  Every operation is the restated FITPACK / Julia operation, in
// the same order, so results equal the CPU restatement bit for bit.
#pragma once

namespace dk {

constexpr int kLegacyMaxPts = 256;     // points a legacy spline is fitted to (nRefAngles <= 256)
constexpr int kChi2LegacyMaxDouble = 20;  // mu doublings of the legacy chi2 search (mu <= 1e-3 * 2^20)

// ---- Julia float ranges -----------------------------------------------------
struct JlRange {
    double ref_hi, ref_lo, step_hi, step_lo;
    long long offset, len;
};
__device__ __forceinline__ void lg_add12(double x, double y, double &h, double &l) {
    if (fabs(y) > fabs(x)) { double t = x; x = y; y = t; }
    h = __dadd_rn(x, y);
    l = __dadd_rn(__dsub_rn(x, h), y);
}
__device__ __forceinline__ double lg_truncbits(double x, int nb) {
    unsigned long long u = (unsigned long long)__double_as_longlong(x);
    u &= (~0ULL) << nb;
    return __longlong_as_double((long long)u);
}
__device__ inline int lg_nbitslen(long long len, long long offset) {
    if (len < 2) return 0;
    long long k = (offset - 1 > len - offset) ? offset - 1 : len - offset;
    long long v = k - 1;
    int b = 0;
    while (v > 0) { b++; v >>= 1; }
    b += 1;
    return b < 27 ? b : 27;  // min(cld(precision(Float64), 2), ...)
}
// Base.rat: continued-fraction rational approximation
__device__ inline void lg_rat(double x, long long &num, long long &den) {
    double y = x;
    long long a = 1, d = 1, b = 0, c = 0;
    const double m = 16777216.0;  // maxintfloat(Float32, Int)
    #pragma unroll 1
    for (int guard = 0; fabs(y) <= m && guard < 128; ++guard) {
        long long f = (long long)trunc(y);
        y = __dsub_rn(y, (double)f);
        long long an = f * a + c, bn = f * b + d;
        c = a; d = b; a = an; b = bn;
        if (llabs(a) > (long long)m || llabs(b) > (long long)m) { num = c; den = d; return; }
        if (__ddiv_rn((double)a, (double)b) == x) break;
        y = __ddiv_rn(1.0, y);
    }
    num = a; den = b;
}
// TwicePrecision{Float64}((num, den)): TwicePrecision(num) / den (Base.mul12, canonicalize2)
__device__ inline void lg_tp_ratio(long long num, long long den, double &hi, double &lo) {
    double xh = (double)num, yh = (double)den;
    double h = __ddiv_rn(xh, yh);
    double p = __dmul_rn(h, yh), uh, ul;
    if (p == 0 || !isfinite(p)) { uh = p; ul = p; }
    else {
        double e = fma(h, yh, -p);
        uh = __dadd_rn(p, e);
        ul = __dadd_rn(__dsub_rn(p, uh), e);
    }
    double l = __ddiv_rn(__dsub_rn(__dadd_rn(__dsub_rn(__dsub_rn(xh, uh), ul), 0.0), __dmul_rn(h, 0.0)), yh);
    if (xh == 0 || !isfinite(h)) { hi = h; lo = h; return; }
    double s = __dadd_rn(h, l);
    hi = s;
    lo = __dadd_rn(__dsub_rn(h, s), l);
}
__device__ __forceinline__ bool lg_between(double a, double x, double b) { return (a <= x && x <= b) || (b <= x && x <= a); }
__device__ inline long long lg_gcd(long long a, long long b) {
    a = llabs(a); b = llabs(b);
    #pragma unroll 1
    while (b) { long long t = a % b; a = b; b = t; }
    return a;
}
// (:)(start::Float64, step::Float64, stop::Float64)
__device__ inline JlRange jl_colon(double start, double step, double stop) {
    JlRange r;
    long long step_n, step_d;
    lg_rat(step, step_n, step_d);
    if (step_d != 0 && __ddiv_rn((double)step_n, (double)step_d) == step) {
        long long start_n, start_d, stop_n, stop_d;
        lg_rat(start, start_n, start_d);
        lg_rat(stop, stop_n, stop_d);
        if (start_d != 0 && stop_d != 0 && __ddiv_rn((double)start_n, (double)start_d) == start &&
            __ddiv_rn((double)stop_n, (double)stop_d) == stop) {
            long long g = lg_gcd(start_d, step_d);
            long long den = g == 0 ? 0 : llabs(start_d / g * step_d);
            const double m = 9007199254740992.0;  // maxintfloat(Float64, Int)
            if (den != 0 && fabs(__dmul_rn(start, (double)den)) <= m && fabs(__dmul_rn(step, (double)den)) <= m &&
                den % start_d == 0 && den % step_d == 0) {
                long long sn = (long long)rint(__dmul_rn(start, (double)den));
                long long tn = (long long)rint(__dmul_rn(step, (double)den));
                long long q = (den * stop_n - stop_d * sn + tn * stop_d) / (tn * stop_d);
                long long len = q > 0 ? q : 0;
                if (lg_between(start, __dadd_rn(start, __dmul_rn((double)(len - 1), step)), __dadd_rn(stop, __ddiv_rn(step, 2.0))) &&
                    !lg_between(start, __dadd_rn(start, __dmul_rn((double)len, step)), stop)) {
                    // floatrange(Float64, sn, tn, len, den)
                    long long imin, ref_n;
                    int nb;
                    if (len < 2 || tn == 0) { imin = 1; ref_n = sn; nb = 0; }
                    else {
                        double t = rint(__dadd_rn(__ddiv_rn(-(double)sn, (double)tn), 1.0));
                        imin = t < 1 ? 1 : (t > (double)len ? len : (long long)t);
                        ref_n = sn + (imin - 1) * tn;
                        nb = lg_nbitslen(len, imin);
                    }
                    lg_tp_ratio(ref_n, den, r.ref_hi, r.ref_lo);
                    double sh, sl;
                    lg_tp_ratio(tn, den, sh, sl);
                    r.step_hi = lg_truncbits(sh, nb);
                    r.step_lo = __dadd_rn(__dsub_rn(sh, r.step_hi), sl);
                    r.offset = imin;
                    r.len = len;
                    return r;
                }
            }
        }
    }
    // fallback: start and step taken literally
    double lf = __ddiv_rn(__dsub_rn(stop, start), step);
    long long len;
    if (lf < 0) len = 0;
    else if (lf == 0) len = 1;
    else {
        len = (long long)rint(lf) + 1;
        double stop2 = __dadd_rn(start, __dmul_rn((double)(len - 1), step));
        len -= (start < stop && stop < stop2) + (start > stop && stop > stop2);
    }
    r.ref_hi = start; r.ref_lo = 0;
    r.step_hi = step; r.step_lo = 0;
    r.offset = 1;
    r.len = len;
    return r;
}
// unsafe_getindex(::StepRangeLen{Float64, TwicePrecision, TwicePrecision}, i), 1-based
__device__ __forceinline__ double jl_at(const JlRange &r, long long i) {
    double u = (double)(i - r.offset);
    double sh = __dmul_rn(u, r.step_hi), sl = __dmul_rn(u, r.step_lo), xh, xl;
    lg_add12(r.ref_hi, sh, xh, xl);
    return __dadd_rn(xh, __dadd_rn(xl, __dadd_rn(sl, r.ref_lo)));
}

// ---- FITPACK (1-based arrays) ------------------------------------------------
__device__ __forceinline__ void fp_givs(double piv, double &ww, double &c, double &s) {
    double store = fabs(piv), dd;
    if (store >= ww) { double q = __ddiv_rn(ww, piv); dd = __dmul_rn(store, __dsqrt_rn(__dadd_rn(1.0, __dmul_rn(q, q)))); }
    else { double q = __ddiv_rn(piv, ww); dd = __dmul_rn(ww, __dsqrt_rn(__dadd_rn(1.0, __dmul_rn(q, q)))); }
    c = __ddiv_rn(ww, dd);
    s = __ddiv_rn(piv, dd);
    ww = dd;
}
__device__ __forceinline__ void fp_rota(double c, double s, double &a, double &b) {
    double s1 = a, s2 = b;
    b = __dadd_rn(__dmul_rn(c, s2), __dmul_rn(s, s1));
    a = __dsub_rn(__dmul_rn(c, s1), __dmul_rn(s, s2));
}
// fpbspl with the knots given explicitly: the k+1 B-splines of degree k at x
// in the knot interval [t(l), t(l+1)); h is 1-based (h[1..k+1]).
__device__ inline void fp_bspl(const double *t, int k, double x, int l, double *h) {
    double hh[4];
    h[1] = 1.0;
    #pragma unroll 1
    for (int j = 1; j <= k; ++j) {
        #pragma unroll 1
        for (int i = 1; i <= j; ++i) hh[i] = h[i];
        h[1] = 0.0;
        #pragma unroll 1
        for (int i = 1; i <= j; ++i) {
            int li = l + i, lj = li - j;
            if (t[li] == t[lj]) { h[i + 1] = 0.0; continue; }
            double f = __ddiv_rn(hh[i], __dsub_rn(t[li], t[lj]));
            h[i] = __dadd_rn(h[i], __dmul_rn(f, __dsub_rn(t[li], x)));
            h[i + 1] = __dmul_rn(f, __dsub_rn(x, t[lj]));
        }
    }
}
// curfit(iopt = 0, s = 0, w = 1), lane 0: the interpolating spline of degree k
// through (X(i), Y(i)), i = 1..m, X increasing, m > k.  X(i) = gx[sidx[i-1]-1]
// when sidx is given (the search's sorted evaluated indices), else gx[i-1].
// Writes the n = m + k + 1 knots t(1..n) and the m coefficients c(1..m);
// a ((m+1) x (k+2)) and z (m+1) are workspaces.  Returns n.
__device__ inline int fp_curfit0(const double *gx, const double *gy, const int *sidx, int m, int k,
                                 double *t, double *c, double *a, double *z) {
    const int k1 = k + 1, k2 = k1 + 1, n = m + k1, nk1 = n - k1;
    auto X = [&](int i) { return sidx ? gx[sidx[i - 1] - 1] : gx[i - 1]; };
    auto Y = [&](int i) { return sidx ? gy[sidx[i - 1] - 1] : gy[i - 1]; };
    const int mk1 = m - k1;
    if (mk1 > 0) {
        int k3 = k / 2, i = k2, j = k3 + 2;
        if (k3 * 2 != k) {
            #pragma unroll 1
            for (int l = 1; l <= mk1; ++l, ++i, ++j) t[i] = X(j);
        } else {
            #pragma unroll 1
            for (int l = 1; l <= mk1; ++l, ++i, ++j) t[i] = __dmul_rn(__dadd_rn(X(j), X(j - 1)), 0.5);
        }
    }
    const double xb = X(1), xe = X(m);
    #pragma unroll 1
    for (int j = 1, i = n; j <= k1; ++j, --i) { t[j] = xb; t[i] = xe; }
#define FA(i, j) a[(i) * (k2) + (j)]
    #pragma unroll 1
    for (int i = 1; i <= nk1; ++i) {
        z[i] = 0;
        #pragma unroll 1
        for (int j = 1; j <= k1; ++j) FA(i, j) = 0;
    }
    int l = k1;
    double h[5];
    #pragma unroll 1
    for (int it = 1; it <= m; ++it) {
        double xi = X(it), yi = Y(it);
        #pragma unroll 1
        while (!(xi < t[l + 1] || l == nk1)) l++;
        fp_bspl(t, k, xi, l, h);
        int j = l - k1;
        #pragma unroll 1
        for (int i = 1; i <= k1; ++i) {
            j++;
            double piv = h[i];
            if (piv == 0) continue;
            double cs, sn;
            fp_givs(piv, FA(j, 1), cs, sn);
            fp_rota(cs, sn, yi, z[j]);
            if (i == k1) break;
            #pragma unroll 1
            for (int i1 = i + 1, i2 = 1; i1 <= k1; ++i1) {
                i2++;
                fp_rota(cs, sn, h[i1], FA(j, i2));
            }
        }
    }
    // fpback: back substitution, bandwidth k1
    c[nk1] = __ddiv_rn(z[nk1], FA(nk1, 1));
    int i = nk1 - 1;
    #pragma unroll 1
    for (int j = 2; j <= nk1 && i >= 1; ++j, --i) {
        double store = z[i];
        int i1 = (j <= k) ? j - 1 : k, mm = i;
        #pragma unroll 1
        for (int q = 1; q <= i1; ++q) { mm++; store = __dsub_rn(store, __dmul_rn(c[mm], FA(i, q + 1))); }
        c[i] = __ddiv_rn(store, FA(i, 1));
    }
#undef FA
    return n;
}
// Doubles of workspace legacy_scan needs for npts points.
__host__ __device__ constexpr long legacy_ws_doubles(int npts) {
    return 2L * (npts + 5) + (long)(npts + 1) * 5 + (npts + 1);
}

// spline_opt_legacy (root = false) or spline_root_legacy (root = true, the
// minimum of |spline - value|) through the npts points (X, Y) described as in
// fp_curfit0.  ws holds legacy_ws_doubles(npts) doubles of this warp's global
// scratch.  All lanes return the same (x, y): x = the sampled point, y = the
// minimized quantity there.  (Arguments and result by value: the callers'
// state stays in registers.)
static __device__ __noinline__ double2 legacy_scan(const double *gx, const double *gy, const int *sidx, int npts, bool root,
                                            double value, double *ws) {
    const int lane = threadIdx.x & 31;
    const int k = npts - 1 < 3 ? npts - 1 : 3, k1 = k + 1;
    double *t = ws, *c = t + (npts + 5), *a = c + (npts + 5), *z = a + (long)(npts + 1) * 5;
    int n = 0;
    if (lane == 0) n = fp_curfit0(gx, gy, sidx, npts, k, t, c, a, z);
    n = __shfl_sync(0xffffffffu, n, 0);
    __syncwarp();
    const int nk1 = n - k1;
    const JlRange r = jl_colon(t[k1], 0.001, t[n - k]);  // get_knots(spl): t[k+1 .. n-k]
    // each lane: its points in increasing order, knot interval and its
    // constants (knots t(l-k+1..l+k), denominators, coefficients) in registers
    int l = -1;
    double tk[7], den[7], cc[4];
    double bv = 0, bx = 0;
    long long bi = -1;
    double v1 = 0;  // value at the first point (lane 0), for the NaN rule
    #pragma unroll 1
    for (long long i = 1 + lane; i <= r.len; i += 32) {
        const double x = jl_at(r, i);
        int ln = l < 0 ? k1 : l;
        #pragma unroll 1
        while (!(x < t[ln + 1] || ln == nk1)) ln++;
        #pragma unroll 1
        while (ln > k1 && x < t[ln]) ln--;
        if (ln != l) {
            l = ln;
            #pragma unroll
            for (int q = 0; q < 7; ++q) {
                int idx = l - k + 1 + q;  // t(l-k+1) .. t(l+k)
                tk[q] = (q < 2 * k) ? t[idx] : 0.0;
            }
            // den index (j, i) -> j(j-1)/2 + i - 1: t(l+i) - t(l+i-j)
            #pragma unroll
            for (int j = 1; j <= 3; ++j)
                #pragma unroll
                for (int ii = 1; ii <= 3; ++ii)
                    if (ii <= j && j <= k) den[j * (j - 1) / 2 + ii - 1] = __dsub_rn(tk[k - 1 + ii], tk[k - 1 + ii - j]);
            #pragma unroll
            for (int q = 0; q < 4; ++q) cc[q] = (q <= k) ? c[l - k1 + 1 + q] : 0.0;
        }
        // fpbspl on the register copies (t(m) = tk[m - (l-k+1)])
        double h[5], hh[4];
        h[1] = 1.0;
        #pragma unroll
        for (int j = 1; j <= 3; ++j) {
            if (j > k) break;
            #pragma unroll
            for (int ii = 1; ii <= 3; ++ii) if (ii <= j) hh[ii] = h[ii];
            h[1] = 0.0;
            #pragma unroll
            for (int ii = 1; ii <= 3; ++ii) {
                if (ii > j) break;
                const double dn = den[j * (j - 1) / 2 + ii - 1];
                const double tli = tk[k - 1 + ii], tlj = tk[k - 1 + ii - j];
                if (dn == 0) { h[ii + 1] = 0.0; continue; }
                double f = __ddiv_rn(hh[ii], dn);
                h[ii] = __dadd_rn(h[ii], __dmul_rn(f, __dsub_rn(tli, x)));
                h[ii + 1] = __dmul_rn(f, __dsub_rn(x, tlj));
            }
        }
        double sp = 0;
        #pragma unroll
        for (int q = 0; q < 4; ++q) if (q <= k) sp = __dadd_rn(sp, __dmul_rn(cc[q], h[q + 1]));
        const double y = root ? fabs(__dsub_rn(sp, value)) : sp;
        if (i == 1) v1 = y;
        if (!isnan(y) && (bi < 0 || y < bv)) { bv = y; bx = x; bi = i; }
    }
    // first strict minimum in index order: smallest value, ties to the lowest
    // index (-0.0 == 0.0 ties as in the sequential `<` scan)
    #pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        double ov = __shfl_xor_sync(0xffffffffu, bv, off), ox = __shfl_xor_sync(0xffffffffu, bx, off);
        long long oi = __shfl_xor_sync(0xffffffffu, bi, off);
        bool take = oi >= 0 && (bi < 0 || ov < bv || (ov == bv && oi < bi));
        if (take) { bv = ov; bx = ox; bi = oi; }
    }
    v1 = __shfl_sync(0xffffffffu, v1, 0);
    if (isnan(v1) || bi < 0) return make_double2(jl_at(r, 1), v1);  // the scan starts at the first point; NaN never compares less
    return make_double2(bx, bv);
}

}  // namespace dk
