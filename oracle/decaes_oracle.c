/*
 * decaes_oracle.c -- CPU oracle: plain-C FP64 restatement of DECAES.jl v0.6.1's
 * voxelwise T2 path (T2mapSEcorr + T2partSEcorr).
 *
 * TEST INFRASTRUCTURE ONLY (the checker).  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg use it; the GPU product never does.
 *
 * Parity: the reference is Julia (not runnable here) and ships no golden
 * vectors.  Components are pinned against the known answers of the reference's
 * own tests; whole-pipeline parity against the Julia reference is unpinned.
 *
 * Floating-point conventions of the restatement:
 *   - every `muladd`, and every `a*b + c` inside NNLS.jl's `@muladd` block,
 *     is an explicit fma() here (Julia lowers muladd to a fused FMA on FMA
 *     hardware); all other expressions keep Julia's evaluation order unfused.
 *     The file is compiled with -ffp-contract=off so x86 and Arm agree.
 *   - `@simd` reductions (which Julia may reassociate) are sequential here.
 *   - 1-based index macros keep the loops line-for-line comparable with the
 *     reference.
 */
#include "decaes_oracle.h"
#include "orc_pmath.h"

#include <complex.h>
#undef I /* the grid index below is named I, as in the reference */
#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------- */
/* FP64 operation counters (per thread, per stage)                            */
/* ------------------------------------------------------------------------- */
static __thread double g_fl[ORC_NSTAGES];
static __thread int g_st;
#define FL(k) (g_fl[g_st] += (double)(k))

/* The GPU path reduces across a 32-lane warp: element i of a loop starting at
 * `start` accumulates into lane (i - start) mod 32, then a butterfly adds
 * lane partials (p[l] + p[l^16], then ^8, ^4, ^2, ^1).  Julia's @simd permits
 * exactly this kind of reassociation; the oracle uses the same order so the
 * two agree bit for bit. */
typedef struct { double p[32]; } lacc;
static inline double lacc_tree(lacc *L) {
    double t[32];
    for (int o = 16; o > 0; o >>= 1) {
        for (int l = 0; l < 32; ++l) t[l] = L->p[l] + L->p[l ^ o];
        memcpy(L->p, t, sizeof t);
    }
    return L->p[0];
}

/* ------------------------------------------------------------------------- */
/* Julia scalar semantics                                                     */
/* ------------------------------------------------------------------------- */
static const double PHI = 1.6180339887498948482045868343656381; /* Base.MathConstants.φ */
static const double D2R = 0.017453292519943295;                  /* Float64(π)/180 (deg2rad factor) */
static const double EPS64 = 2.220446049250313e-16;
static const double SQRT_EPS64 = 1.4901161193847656e-08;

/* Base.max/min for Float64: NaN-propagating, -0.0 < 0.0 */
static inline double jmax(double x, double y) {
    if (isnan(x) || isnan(y)) return NAN;
    double d = x - y;
    return signbit(d) ? y : x;
}
static inline double jmin(double x, double y) {
    if (isnan(x) || isnan(y)) return NAN;
    double d = x - y;
    return signbit(d) ? x : y;
}
static inline double jsign(double x) { return x < 0 ? -1.0 : (x > 0 ? 1.0 : x); }
static inline double jclamp(double x, double lo, double hi) { return x > hi ? hi : (x < lo ? lo : x); }
static inline double strictsign(double x) { return signbit(x) ? -1.0 : 1.0; }
static inline int jisfinite(double x) { return isfinite(x); }
/* isapprox(x, y) with default rtol = sqrt(eps), atol = 0 */
static inline int isapprox(double x, double y) {
    if (x == y) return 1;
    if (!(isfinite(x) && isfinite(y))) return 0;
    return fabs(x - y) <= jmax(0.0, SQRT_EPS64 * jmax(fabs(x), fabs(y)));
}
/* isless for findmax: NaN is larger than everything, -0.0 < 0.0 */
static inline int jisless(double a, double b) {
    if (isnan(a)) return 0;
    if (isnan(b)) return 1;
    if (a == b) return signbit(a) && !signbit(b);
    return a < b;
}

/* ------------------------------------------------------------------------- */
/* Grids: Julia's range(a, b; length) for Float64 and logrange                */
/* (src/utils.jl:7, src/types.jl:108-110)                                     */
/* ------------------------------------------------------------------------- */
static void add12(double x, double y, double *h, double *l) {
    if (fabs(y) > fabs(x)) { double t = x; x = y; y = t; }
    *h = x + y;
    *l = (x - *h) + y;
}
static double truncbits(double x, int nb) {
    uint64_t u;
    memcpy(&u, &x, 8);
    u &= (~(uint64_t)0) << nb;
    memcpy(&x, &u, 8);
    return x;
}
static int top_set_bit(long v) {
    int b = 0;
    while (v > 0) { b++; v >>= 1; }
    return b;
}
static int nbitslen(int len, int offset) {
    if (len < 2) return 0;
    int k = (offset - 1 > len - offset) ? offset - 1 : len - offset;
    int nb = top_set_bit(k - 1) + 1;
    return nb < 27 ? nb : 27; /* min(cld(precision(Float64), 2), ...) */
}
/* Base.rat: continued-fraction rational approximation (twiceprecision.jl) */
static void jl_rat(double x, long *num, long *den) {
    double y = x;
    long a = 1, d = 1, b = 0, c = 0;
    const double m = 16777216.0; /* maxintfloat(Float32, Int) */
    while (fabs(y) <= m) {
        long f = (long)trunc(y);
        y -= (double)f;
        long an = f * a + c, bn = f * b + d;
        c = a; d = b; a = an; b = bn;
        if (labs(a) > (long)m || labs(b) > (long)m) { *num = c; *den = d; return; }
        if ((double)a / (double)b == x) break;
        y = 1.0 / y;
    }
    *num = a; *den = b;
}
static long lgcd(long a, long b) {
    a = labs(a); b = labs(b);
    while (b) { long t = a % b; a = b; b = t; }
    return a;
}
/* collect(range(a, b; length=len)) for Float64 endpoints */
void orc_linrange(double start, double stop, int len, double *out) {
    if (len == 1) { out[0] = start; return; }
    if (start == stop) { for (int i = 0; i < len; ++i) out[i] = start; return; }
    long sn, sd, en, ed;
    jl_rat(start, &sn, &sd);
    jl_rat(stop, &en, &ed);
    if (sd != 0 && ed != 0) {
        long den = labs(sd / lgcd(sd, ed) * ed);
        double m = 9007199254740992.0; /* maxintfloat(Float64, Int) */
        if (den != 0 && fabs((double)den * start) <= m && fabs((double)den * stop) <= m) {
            long s_n = (long)rint((double)den * start), e_n = (long)rint((double)den * stop);
            if ((double)s_n / (double)den == start && (double)e_n / (double)den == stop) {
                /* exact rational path: element = correctly rounded ((len-i) s_n + (i-1) e_n) / ((len-1) den) */
                for (int i = 1; i <= len; ++i) {
                    long double numv = (long double)(len - i) * s_n + (long double)(i - 1) * e_n;
                    double num = (double)numv; /* exact: |num| < 2^53 for the grids used here */
                    out[i - 1] = num / ((double)(len - 1) * (double)den);
                }
                return;
            }
        }
    }
    /* _linspace(start, stop, len) floating path */
    double D = stop - start;
    double tmin = -(start / D) / 1.0;
    long imin = lrint(tmin * (double)(len - 1) + 1.0);
    double ref, step;
    if (1 < imin && imin < len) {
        double t = (double)(imin - 1) / (double)(len - 1);
        ref = (1 - t) * start + t * stop;
        step = (imin - 1 < len - imin) ? (ref - start) / (double)(imin - 1) : (stop - ref) / (double)(len - imin);
    } else if (imin <= 1) {
        imin = 1; ref = start; step = (D / (double)(len - 1)) * 1.0;
    } else {
        imin = len; ref = stop; step = (D / (double)(len - 1)) * 1.0;
    }
    int nb = nbitslen(len, (int)imin);
    double step_hi = truncbits(step, nb);
    double x1h, x1l, x2h, x2l;
    add12((double)(1 - imin) * step_hi, ref, &x1h, &x1l);
    add12((double)(len - imin) * step_hi, ref, &x2h, &x2l);
    double a = (start - x1h) - x1l, b = (stop - x2h) - x2l;
    double step_lo = (b - a) / (double)(len - 1);
    double ref_lo = a - (double)(1 - imin) * step_lo;
    for (int i = 1; i <= len; ++i) {
        double u = (double)(i - imin);
        double sh = u * step_hi, sl = u * step_lo, xh, xl;
        add12(ref, sh, &xh, &xl);
        out[i - 1] = xh + (xl + (sl + ref_lo));
    }
}
/* logrange(a, b, len): exp.(range(log(a), log(b); length=len)) with exact endpoints (src/utils.jl:7) */
void orc_logrange(double a, double b, int len, double *out) {
    orc_linrange(log(a), log(b), len, out);
    for (int i = 0; i < len; ++i) out[i] = exp(out[i]);
    out[0] = a;
    out[len - 1] = b;
}

/* sind: argument reduction in degrees as in Base.sind, then sin/cos of a
 * double-double radian argument (sin(h + l) ~ sin h + l cos h). */
static const double D2R_LO = 2.9486522708701687e-19; /* pi/180 - D2R */
static double sin_dd(double y) {
    double h = y * D2R, l = fma(y, D2R, -h) + y * D2R_LO, sh, ch;
    pm_sincos(h, &sh, &ch);
    return sh + l * ch;
}
static double cos_dd(double y) {
    double h = y * D2R, l = fma(y, D2R, -h) + y * D2R_LO, sh, ch;
    pm_sincos(h, &sh, &ch);
    return ch - l * sh;
}
double orc_sind(double x) {
    if (isnan(x) || isinf(x)) return NAN;
    double rx = copysign(fmod(x, 360.0), x), arx = fabs(rx);
    if (rx == 0) return rx;
    if (arx < 45) return sin_dd(rx);
    if (arx <= 135) return copysign(cos_dd(90 - arx), rx);
    if (arx == 180) return copysign(0.0, rx);
    if (arx < 225) return sin_dd((180 - arx) * jsign(rx));
    if (arx <= 315) return -copysign(cos_dd(270 - arx), rx);
    return sin_dd(rx - copysign(360.0, rx));
}

/* erfinv (SpecialFunctions.erfinv, used only for the sigmoid weights of
 * src/T2partSEcorr.jl:155-164): Giles' single-precision-style initial guess
 * (M. Giles, "Approximating the erfinv function", GPU Computing Gems, 2011)
 * refined by three Newton steps on erf(). */
double orc_erfinv(double x) {
    if (x <= -1) return x == -1 ? -INFINITY : NAN;
    if (x >= 1) return x == 1 ? INFINITY : NAN;
    double w = -log((1.0 - x) * (1.0 + x)), p;
    if (w < 5.0) {
        w = w - 2.5;
        p = 2.81022636e-08; p = 3.43273939e-07 + p * w; p = -3.5233877e-06 + p * w;
        p = -4.39150654e-06 + p * w; p = 0.00021858087 + p * w; p = -0.00125372503 + p * w;
        p = -0.00417768164 + p * w; p = 0.246640727 + p * w; p = 1.50140941 + p * w;
    } else {
        w = sqrt(w) - 3.0;
        p = -0.000200214257; p = 0.000100950558 + p * w; p = 0.00134934322 + p * w;
        p = -0.00367342844 + p * w; p = 0.00573950773 + p * w; p = -0.0076224613 + p * w;
        p = 0.00943887047 + p * w; p = 1.00167406 + p * w; p = 2.83297682 + p * w;
    }
    double y = p * x;
    for (int it = 0; it < 3; ++it) {
        double err = erf(y) - x;
        y -= err / (1.1283791670955126 * exp(-y * y));
    }
    return y;
}

/* ------------------------------------------------------------------------- */
/* EPG decay curves (src/EPGdecaycurve.jl)                                    */
/* ------------------------------------------------------------------------- */

/* EPGWork_ReIm_DualFlat_Split_Dynamic, epg_decay_curve! + epg_impulse_response!
 * for EPGConstantFlipAngleOptions (refocusing control angle 180),
 * src/EPGdecaycurve.jl:936-1028. */
static void epg_flat(int ETL, double alpha_deg, double TE, double T2, double T1, double *dc, double *work) {
    double *M1 = work, *M2 = work + 3 * ETL, *t;
    memset(work, 0, sizeof(double) * 6 * ETL);
    double al = alpha_deg * D2R;
    double E1 = pm_exp(-(TE / 2) / T1), E2 = pm_exp(-(TE / 2) / T2);
    double sa, ca;
    pm_sincos(al, &sa, &ca);
    double E22h = (E2 * E2) / 2, E1E2 = E1 * E2, E11 = E1 * E1;
    double a = E22h, b = E22h * ca, c = E1E2 * sa, d = E11 * ca, cp = -c / 2;
    const int Dy = ETL, Dz = 2 * ETL;
#define M1_(k) M1[(k) - 1]
#define M2_(k) M2[(k) - 1]
    FL(8);
    dc[0] = a - b;
    M1_(1) = a - b; M1_(1 + Dy) = 0; M1_(1 + Dz) = cp;
    M1_(2) = a + b; M1_(2 + Dy) = 0; M1_(2 + Dz) = 0;
    t = M1; M1 = M2; M2 = t;
    for (int i = 2; i <= ETL / 2; ++i) {
        double F = M2_(1), Fb = M2_(1 + Dy), Z = M2_(1 + Dz);
        double C = F + Fb, S = F - Fb, Cp = a * C, Sp = b * S;
        dc[i - 1] = M1_(1) = fma(-c, Z, Cp - Sp);
        M1_(2) = fma(c, Z, Cp + Sp);
        M1_(1 + Dz) = fma(cp, S, d * Z);
        for (int k = 2; k <= i - 1; ++k) {
            F = M2_(k); Fb = M2_(k + Dy); Z = M2_(k + Dz);
            C = F + Fb; S = F - Fb; Cp = a * C; Sp = b * S;
            M1_(k + 1) = fma(c, Z, Cp + Sp);
            M1_(k - 1 + Dy) = fma(-c, Z, Cp - Sp);
            M1_(k + Dz) = fma(cp, S, d * Z);
        }
        F = M2_(i); Fb = M2_(i + Dy); Z = M2_(i + Dz);
        C = F + Fb; S = F - Fb; Cp = a * C; Sp = b * S;
        M1_(i + 1) = fma(c, Z, Cp + Sp);
        M1_(i - 1 + Dy) = fma(-c, Z, Cp - Sp);
        M1_(i + Dz) = fma(cp, S, d * Z);
        M1_(i + Dy) = 0; M1_(i + 1 + Dy) = 0; M1_(i + 1 + Dz) = 0;
        FL(14 * i);
        t = M1; M1 = M2; M2 = t;
    }
    for (int i = ETL / 2 + 1; i <= ETL - 1; ++i) {
        double F = M2_(1), Fb = M2_(1 + Dy), Z = M2_(1 + Dz);
        double C = F + Fb, S = F - Fb, Cp = a * C, Sp = b * S;
        dc[i - 1] = M1_(1) = fma(-c, Z, Cp - Sp);
        M1_(2) = fma(c, Z, Cp + Sp);
        M1_(1 + Dz) = fma(cp, S, d * Z);
        for (int k = 2; k <= ETL - i + 1; ++k) {
            F = M2_(k); Fb = M2_(k + Dy); Z = M2_(k + Dz);
            C = F + Fb; S = F - Fb; Cp = a * C; Sp = b * S;
            M1_(k + 1) = fma(c, Z, Cp + Sp);
            M1_(k - 1 + Dy) = fma(-c, Z, Cp - Sp);
            M1_(k + Dz) = fma(cp, S, d * Z);
        }
        FL(14 * (ETL - i + 1));
        t = M1; M1 = M2; M2 = t;
    }
    {
        double F = M2_(1), Fb = M2_(1 + Dy), Z = M2_(1 + Dz);
        double C = F + Fb, S = F - Fb;
        dc[ETL - 1] = fma(-c, Z, fma(a, C, -b * S));
    }
#undef M1_
#undef M2_
    double m0 = orc_sind(alpha_deg / 2);
    for (int i = 0; i < ETL; ++i) dc[i] = fabs(m0 * dc[i]);
    FL(2 * ETL + 8);
}

/* EPGWork_ReIm_DualVector_Split_Dynamic, epg_decay_curve! for EPGOptions
 * (refocusing control angle beta != 180), src/EPGdecaycurve.jl:722-818. */
typedef struct { double x, y, z; } v3;
static inline double dot3(v3 a, v3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
static void epg_vec(int ETL, double alpha_deg, double TE, double T2, double T1, double beta, double *dc, v3 *work) {
    v3 *M1 = work, *M2 = work + ETL, *t;
    memset(work, 0, sizeof(v3) * 2 * ETL);
    double A = alpha_deg / 180;
    double a1r = (A * 180) * D2R, air = (A * beta) * D2R;
    double E1 = pm_exp(-(TE / 2) / T1), E2 = pm_exp(-(TE / 2) / T2);
    double sh, ch, sai, cai;
    pm_sincos(a1r / 2, &sh, &ch);
    pm_sincos(air, &sai, &cai);
    double sh2 = sh * sh, ch2 = ch * ch;
    double sa1 = 2 * sh * ch;
    double chi2 = (1 + cai) / 2, shi2 = 1 - chi2;
    double a1 = (E2 * E2) * ch2, b1 = (E2 * E2) * sh2, c1 = (E1 * E2) * sa1;
    double ai = (E2 * E2) * chi2, bi = (E2 * E2) * shi2, ci = (E1 * E2) * sai, di = (E1 * E1) * cai;
    v3 F = {ai, bi, ci}, Fb = {bi, ai, -ci}, Z = {-ci / 2, ci / 2, di};
    FL(40);
    double m0 = sh;
    v3 M0 = {b1 * m0, 0, ((-c1) * m0) / 2};
    M1[0] = M0;
    M1[1] = (v3){a1 * m0, 0, 0};
    dc[0] = fabs(M0.x);
    t = M1; M1 = M2; M2 = t;
    {
        v3 m0v = M2[0], m1v = M2[1];
        double FM0 = dot3(F, m0v), FbM0 = dot3(Fb, m0v), ZM0 = dot3(Z, m0v);
        double FM1 = dot3(F, m1v), FbM1 = dot3(Fb, m1v), ZM1 = dot3(Z, m1v);
        M1[0] = (v3){FbM0, FbM1, ZM0};
        M1[1] = (v3){FM0, 0, ZM1};
        M1[2] = (v3){FM1, 0, 0};
        dc[1] = fabs(FbM0);
        t = M1; M1 = M2; M2 = t;
        FL(30);
    }
    for (int i = 3; i <= ETL / 2; ++i) {
        v3 m0v = M2[0], m1v = M2[1], m2v = M2[2];
        double FM0 = dot3(F, m0v), FbM0 = dot3(Fb, m0v), ZM0 = dot3(Z, m0v);
        double FM1 = dot3(F, m1v), FbM1 = dot3(Fb, m1v), ZM1 = dot3(Z, m1v);
        double FM2 = dot3(F, m2v), FbM2 = dot3(Fb, m2v), ZM2 = dot3(Z, m2v);
        M1[0] = (v3){FbM0, FbM1, ZM0};
        M1[1] = (v3){FM0, FbM2, ZM1};
        for (int j = 3; j <= i - 1; ++j) {
            FM0 = FM1; FM1 = FM2; ZM1 = ZM2;
            m2v = M2[j];
            FM2 = dot3(F, m2v); FbM2 = dot3(Fb, m2v); ZM2 = dot3(Z, m2v);
            M1[j - 1] = (v3){FM0, FbM2, ZM1};
        }
        M1[i - 1] = (v3){FM1, 0, ZM2};
        M1[i] = (v3){FM2, 0, 0};
        dc[i - 1] = fabs(FbM0);
        FL(15 * (i + 1));
        t = M1; M1 = M2; M2 = t;
    }
    for (int i = ETL / 2 + 1; i <= ETL - 1; ++i) {
        v3 m0v = M2[0], m1v = M2[1], m2v = M2[2];
        double FM0 = dot3(F, m0v), FbM0 = dot3(Fb, m0v), ZM0 = dot3(Z, m0v);
        double FM1 = dot3(F, m1v), FbM1 = dot3(Fb, m1v), ZM1 = dot3(Z, m1v);
        double FM2 = dot3(F, m2v), FbM2 = dot3(Fb, m2v), ZM2 = dot3(Z, m2v);
        M1[0] = (v3){FbM0, FbM1, ZM0};
        M1[1] = (v3){FM0, FbM2, ZM1};
        for (int j = 3; j <= ETL - i; ++j) {
            FM0 = FM1; FM1 = FM2; ZM1 = ZM2;
            m2v = M2[j];
            FM2 = dot3(F, m2v); FbM2 = dot3(Fb, m2v); ZM2 = dot3(Z, m2v);
            M1[j - 1] = (v3){FM0, FbM2, ZM1};
        }
        dc[i - 1] = fabs(FbM0);
        FL(15 * (ETL - i + 1));
        t = M1; M1 = M2; M2 = t;
    }
    dc[ETL - 1] = fabs(dot3(Fb, M2[0]));
}

/* Dual numbers (value, d/dalpha) following ForwardDiff's primal arithmetic, so
 * the value part equals the plain evaluation (the basis `As` of the angle
 * ensemble is the primal of the dual evaluation, src/T2mapSEcorr.jl:362-371). */
typedef struct { double v, d; } dual;
static inline dual dc_(double v) { return (dual){v, 0}; }
static inline dual dadd(dual a, dual b) { return (dual){a.v + b.v, a.d + b.d}; }
static inline dual dsub(dual a, dual b) { return (dual){a.v - b.v, a.d - b.d}; }
static inline dual dneg(dual a) { return (dual){-a.v, -a.d}; }
static inline dual dmul(dual a, dual b) { return (dual){a.v * b.v, a.d * b.v + b.d * a.v}; }
static inline dual dmuls(dual a, double s) { return (dual){a.v * s, a.d * s}; }
static inline dual ddivs(dual a, double s) { return (dual){a.v / s, a.d / s}; }
static inline dual dfma(dual a, dual b, dual c) { return (dual){fma(a.v, b.v, c.v), (a.d * b.v + b.d * a.v) + c.d}; }
static inline dual dabs(dual a) { return signbit(a.v) ? dneg(a) : a; }

static void epg_flat_dual(int ETL, double alpha_deg, double TE, double T2, double T1, double *dcv, double *dcd, dual *work) {
    dual *M1 = work, *M2 = work + 3 * ETL, *t;
    for (int i = 0; i < 6 * ETL; ++i) work[i] = dc_(0);
    dual al = {alpha_deg * D2R, D2R};
    double E1 = pm_exp(-(TE / 2) / T1), E2 = pm_exp(-(TE / 2) / T2);
    double s, co;
    pm_sincos(al.v, &s, &co);
    dual sa = {s, co * al.d}, ca = {co, -s * al.d};
    double E22h = (E2 * E2) / 2, E1E2 = E1 * E2, E11 = E1 * E1;
    dual a = dc_(E22h), b = dmuls(ca, E22h), c = dmuls(sa, E1E2), d = dmuls(ca, E11), cp = ddivs(dneg(c), 2);
    const int Dy = ETL, Dz = 2 * ETL;
#define M1_(k) M1[(k) - 1]
#define M2_(k) M2[(k) - 1]
    dual *dc = (dual *)alloca(sizeof(dual) * ETL);
    FL(16);
    dc[0] = dsub(a, b);
    M1_(1) = dsub(a, b); M1_(1 + Dy) = dc_(0); M1_(1 + Dz) = cp;
    M1_(2) = dadd(a, b); M1_(2 + Dy) = dc_(0); M1_(2 + Dz) = dc_(0);
    t = M1; M1 = M2; M2 = t;
#define EPG_STEP(kk, writeF, writeFb, writeZ)                                      \
    {                                                                              \
        dual F = M2_(kk), Fb = M2_((kk) + Dy), Z = M2_((kk) + Dz);                 \
        dual C = dadd(F, Fb), S = dsub(F, Fb), Cp = dmul(a, C), Sp = dmul(b, S);   \
        writeF = dfma(c, Z, dadd(Cp, Sp));                                         \
        writeFb = dfma(dneg(c), Z, dsub(Cp, Sp));                                  \
        writeZ = dfma(cp, S, dmul(d, Z));                                          \
    }
    for (int i = 2; i <= ETL / 2; ++i) {
        dual Fb1;
        EPG_STEP(1, M1_(2), Fb1, M1_(1 + Dz));
        dc[i - 1] = M1_(1) = Fb1;
        for (int k = 2; k <= i - 1; ++k) EPG_STEP(k, M1_(k + 1), M1_(k - 1 + Dy), M1_(k + Dz));
        EPG_STEP(i, M1_(i + 1), M1_(i - 1 + Dy), M1_(i + Dz));
        M1_(i + Dy) = dc_(0); M1_(i + 1 + Dy) = dc_(0); M1_(i + 1 + Dz) = dc_(0);
        FL(30 * i);
        t = M1; M1 = M2; M2 = t;
    }
    for (int i = ETL / 2 + 1; i <= ETL - 1; ++i) {
        dual Fb1;
        EPG_STEP(1, M1_(2), Fb1, M1_(1 + Dz));
        dc[i - 1] = M1_(1) = Fb1;
        for (int k = 2; k <= ETL - i + 1; ++k) EPG_STEP(k, M1_(k + 1), M1_(k - 1 + Dy), M1_(k + Dz));
        FL(30 * (ETL - i + 1));
        t = M1; M1 = M2; M2 = t;
    }
#undef EPG_STEP
    {
        dual F = M2_(1), Fb = M2_(1 + Dy), Z = M2_(1 + Dz);
        dual C = dadd(F, Fb), S = dsub(F, Fb);
        dc[ETL - 1] = dfma(dneg(c), Z, dfma(a, C, dmul(dneg(b), S)));
    }
#undef M1_
#undef M2_
    /* m0 = sind(alpha/2); d/dalpha = (pi/180) cosd(alpha/2) / 2 */
    dual m0 = {orc_sind(alpha_deg / 2), D2R * pm_cos((alpha_deg / 2) * D2R) * 0.5};
    for (int i = 0; i < ETL; ++i) {
        dual r = dabs(dmul(m0, dc[i]));
        dcv[i] = r.v;
        dcd[i] = r.d;
    }
    FL(4 * ETL + 10);
}

typedef struct { dual x, y, z; } dv3;
static inline dual ddot3(dv3 a, dv3 b) { return dadd(dadd(dmul(a.x, b.x), dmul(a.y, b.y)), dmul(a.z, b.z)); }
static void epg_vec_dual(int ETL, double alpha_deg, double TE, double T2, double T1, double beta, double *dcv, double *dcd, dv3 *work) {
    dv3 *M1 = work, *M2 = work + ETL, *t;
    for (int i = 0; i < 2 * ETL; ++i) work[i] = (dv3){dc_(0), dc_(0), dc_(0)};
    dual alpha = {alpha_deg, 1.0};
    dual A = ddivs(alpha, 180);
    dual a1r = dmuls(dmuls(A, 180), D2R), air = dmuls(dmuls(A, beta), D2R);
    double E1 = pm_exp(-(TE / 2) / T1), E2 = pm_exp(-(TE / 2) / T2);
    dual h = ddivs(a1r, 2);
    double shv, chv, saiv, caiv;
    pm_sincos(h.v, &shv, &chv);
    pm_sincos(air.v, &saiv, &caiv);
    dual sh = {shv, chv * h.d}, ch = {chv, -shv * h.d};
    dual sh2 = dmul(sh, sh), ch2 = dmul(ch, ch);
    dual sa1 = dmul(dmuls(sh, 2), ch);
    dual sai = {saiv, caiv * air.d}, cai = {caiv, -saiv * air.d};
    dual chi2 = ddivs(dadd(dc_(1), cai), 2), shi2 = dsub(dc_(1), chi2);
    dual a1 = dmuls(ch2, E2 * E2), b1 = dmuls(sh2, E2 * E2), c1 = dmuls(sa1, E1 * E2);
    dual ai = dmuls(chi2, E2 * E2), bi = dmuls(shi2, E2 * E2), ci = dmuls(sai, E1 * E2), di = dmuls(cai, E1 * E1);
    dv3 F = {ai, bi, ci}, Fb = {bi, ai, dneg(ci)}, Z = {ddivs(dneg(ci), 2), ddivs(ci, 2), di};
    dual *dc = (dual *)alloca(sizeof(dual) * ETL);
    FL(80);
    dual m0 = sh;
    dv3 M0 = {dmul(b1, m0), dc_(0), ddivs(dmul(dneg(c1), m0), 2)};
    M1[0] = M0;
    M1[1] = (dv3){dmul(a1, m0), dc_(0), dc_(0)};
    dc[0] = dabs(M0.x);
    t = M1; M1 = M2; M2 = t;
    {
        dv3 m0v = M2[0], m1v = M2[1];
        dual FM0 = ddot3(F, m0v), FbM0 = ddot3(Fb, m0v), ZM0 = ddot3(Z, m0v);
        dual FM1 = ddot3(F, m1v), FbM1 = ddot3(Fb, m1v), ZM1 = ddot3(Z, m1v);
        M1[0] = (dv3){FbM0, FbM1, ZM0};
        M1[1] = (dv3){FM0, dc_(0), ZM1};
        M1[2] = (dv3){FM1, dc_(0), dc_(0)};
        dc[1] = dabs(FbM0);
        t = M1; M1 = M2; M2 = t;
    }
    for (int i = 3; i <= ETL / 2; ++i) {
        dv3 m0v = M2[0], m1v = M2[1], m2v = M2[2];
        dual FM0 = ddot3(F, m0v), FbM0 = ddot3(Fb, m0v), ZM0 = ddot3(Z, m0v);
        dual FM1 = ddot3(F, m1v), FbM1 = ddot3(Fb, m1v), ZM1 = ddot3(Z, m1v);
        dual FM2 = ddot3(F, m2v), FbM2 = ddot3(Fb, m2v), ZM2 = ddot3(Z, m2v);
        M1[0] = (dv3){FbM0, FbM1, ZM0};
        M1[1] = (dv3){FM0, FbM2, ZM1};
        for (int j = 3; j <= i - 1; ++j) {
            FM0 = FM1; FM1 = FM2; ZM1 = ZM2;
            m2v = M2[j];
            FM2 = ddot3(F, m2v); FbM2 = ddot3(Fb, m2v); ZM2 = ddot3(Z, m2v);
            M1[j - 1] = (dv3){FM0, FbM2, ZM1};
        }
        M1[i - 1] = (dv3){FM1, dc_(0), ZM2};
        M1[i] = (dv3){FM2, dc_(0), dc_(0)};
        dc[i - 1] = dabs(FbM0);
        FL(30 * (i + 1));
        t = M1; M1 = M2; M2 = t;
    }
    for (int i = ETL / 2 + 1; i <= ETL - 1; ++i) {
        dv3 m0v = M2[0], m1v = M2[1], m2v = M2[2];
        dual FM0 = ddot3(F, m0v), FbM0 = ddot3(Fb, m0v), ZM0 = ddot3(Z, m0v);
        dual FM1 = ddot3(F, m1v), FbM1 = ddot3(Fb, m1v), ZM1 = ddot3(Z, m1v);
        dual FM2 = ddot3(F, m2v), FbM2 = ddot3(Fb, m2v), ZM2 = ddot3(Z, m2v);
        M1[0] = (dv3){FbM0, FbM1, ZM0};
        M1[1] = (dv3){FM0, FbM2, ZM1};
        for (int j = 3; j <= ETL - i; ++j) {
            FM0 = FM1; FM1 = FM2; ZM1 = ZM2;
            m2v = M2[j];
            FM2 = ddot3(F, m2v); FbM2 = ddot3(Fb, m2v); ZM2 = ddot3(Z, m2v);
            M1[j - 1] = (dv3){FM0, FbM2, ZM1};
        }
        dc[i - 1] = dabs(FbM0);
        FL(30 * (ETL - i + 1));
        t = M1; M1 = M2; M2 = t;
    }
    dc[ETL - 1] = dabs(ddot3(Fb, M2[0]));
    for (int i = 0; i < ETL; ++i) { dcv[i] = dc[i].v; dcd[i] = dc[i].d; }
}

void orc_epg_decay_curve(int ETL, double alpha, double TE, double T2, double T1, double beta, double *dc) {
    if (beta == 180) {
        double *w = (double *)malloc(sizeof(double) * 6 * ETL);
        epg_flat(ETL, alpha, TE, T2, T1, dc, w);
        free(w);
    } else {
        v3 *w = (v3 *)malloc(sizeof(v3) * 2 * ETL);
        epg_vec(ETL, alpha, TE, T2, T1, beta, dc, w);
        free(w);
    }
}
void orc_epg_decay_curve_dual(int ETL, double alpha, double TE, double T2, double T1, double beta, double *dc, double *ddc) {
    if (beta == 180) {
        dual *w = (dual *)malloc(sizeof(dual) * 6 * ETL);
        epg_flat_dual(ETL, alpha, TE, T2, T1, dc, ddc, w);
        free(w);
    } else {
        dv3 *w = (dv3 *)malloc(sizeof(dv3) * 2 * ETL);
        epg_vec_dual(ETL, alpha, TE, T2, T1, beta, dc, ddc, w);
        free(w);
    }
}

/* EPGWork_Basic_Cplx for EPGOptions: the readable specification,
 * src/EPGdecaycurve.jl:271-322 (used only by the oracle's own tests). */
void orc_epg_decay_curve_basic(int ETL, double alpha, double TE, double T2, double T1, double beta, double *dc) {
    double complex *M = (double complex *)calloc(3 * ETL, sizeof(double complex));
    double A = alpha / 180, aex = A * 90, a1 = A * 180, ai = A * beta;
    double E1 = exp(-(TE / 2) / T1), E2 = exp(-(TE / 2) / T2), E[3] = {E2, E2, E1};
    double complex R1[9], Ri[9];
    double *angs[2] = {&a1, &ai};
    double complex *Rs[2] = {R1, Ri};
    for (int r = 0; r < 2; ++r) {
        double a = *angs[r];
        double c2 = orc_sind(90 - a / 2), s2 = orc_sind(a / 2), sa = orc_sind(a), ca = orc_sind(90 - a);
        double complex *R = Rs[r];
        R[0] = c2 * c2; R[1] = s2 * s2; R[2] = -_Complex_I * sa;
        R[3] = s2 * s2; R[4] = c2 * c2; R[5] = _Complex_I * sa;
        R[6] = -_Complex_I * sa / 2; R[7] = _Complex_I * sa / 2; R[8] = ca;
    }
    M[0] = orc_sind(aex);
    for (int i = 1; i <= ETL; ++i) {
        double complex *R = (i == 1) ? R1 : Ri;
        for (int j = 0; j < ETL; ++j) {
            double complex v[3] = {E[0] * M[3 * j], E[1] * M[3 * j + 1], E[2] * M[3 * j + 2]};
            for (int r = 0; r < 3; ++r) M[3 * j + r] = R[3 * r] * v[0] + R[3 * r + 1] * v[1] + R[3 * r + 2] * v[2];
        }
        double complex Mi[3], Mn[3], Mp[3];
        memcpy(Mi, &M[0], sizeof Mi);
        memcpy(Mn, &M[3], sizeof Mn);
        M[0] = Mi[1]; M[1] = Mn[1]; M[2] = Mi[2];
        for (int j = 2; j <= ETL - 1; ++j) {
            memcpy(Mp, Mi, sizeof Mp);
            memcpy(Mi, Mn, sizeof Mi);
            memcpy(Mn, &M[3 * j], sizeof Mn);
            M[3 * (j - 1)] = Mp[0]; M[3 * (j - 1) + 1] = Mn[1]; M[3 * (j - 1) + 2] = Mi[2];
        }
        memcpy(Mp, Mi, sizeof Mp);
        memcpy(Mi, Mn, sizeof Mi);
        M[3 * (ETL - 1)] = Mp[0]; M[3 * (ETL - 1) + 1] = 0; M[3 * (ETL - 1) + 2] = Mi[2];
        for (int j = 0; j < ETL; ++j)
            for (int r = 0; r < 3; ++r) M[3 * j + r] *= E[r];
        dc[i - 1] = cabs(M[0]);
    }
    free(M);
}

/* ------------------------------------------------------------------------- */
/* Lawson-Hanson NNLS (src/NNLS.jl)                                           */
/* ------------------------------------------------------------------------- */
typedef struct {
    int M, N; /* rows (incl. Tikhonov padding), columns */
    double *A, *b, *x, *w, *zz;
    int *idx, *invidx;
    unsigned char *diag;
    double rnorm;
    int mode, nsetp;
} nnls_ws;

#define Aij(i, j) A[((i) - 1) + (size_t)((j) - 1) * lda]
#define V1(v, i) (v)[(i) - 1]

static void nnls_ws_alloc(nnls_ws *ws, int M, int N) {
    ws->M = M; ws->N = N;
    ws->A = (double *)calloc((size_t)M * N, sizeof(double));
    ws->b = (double *)calloc(M, sizeof(double));
    ws->x = (double *)calloc(N, sizeof(double));
    ws->w = (double *)calloc(N, sizeof(double));
    ws->zz = (double *)calloc(M, sizeof(double));
    ws->idx = (int *)calloc(N, sizeof(int));
    ws->invidx = (int *)calloc(N, sizeof(int));
    ws->diag = (unsigned char *)calloc(N, 1);
    ws->rnorm = 0; ws->mode = 0; ws->nsetp = 0;
}
static void nnls_ws_free(nnls_ws *ws) {
    free(ws->A); free(ws->b); free(ws->x); free(ws->w); free(ws->zz);
    free(ws->idx); free(ws->invidx); free(ws->diag);
}

/* construct_apply_householder!, src/NNLS.jl:259-336 */
static double cah(double *A, int lda, double *b, int ip, int jp, int m) {
    if (ip > m) return 0;
    double alpha = Aij(ip, jp);
    lacc La = {{0}};
    for (int i = ip; i <= m; ++i) La.p[(i - ip) & 31] = fma(Aij(i, jp), Aij(i, jp), La.p[(i - ip) & 31]);
    double xnorm = sqrt(lacc_tree(&La));
    FL(2 * (m - ip + 1) + 1);
    if (xnorm == 0) return -1;
    double beta = copysign(xnorm, alpha);
    alpha = alpha + beta;
    double tau = alpha / beta;
    lacc Lb = {{0}};
    for (int i = ip + 1; i <= m; ++i) Lb.p[(i - ip - 1) & 31] = fma(V1(b, i), Aij(i, jp) / alpha, Lb.p[(i - ip - 1) & 31]);
    double sm = V1(b, ip) + lacc_tree(&Lb);
    sm *= -tau;
    double A1 = -beta;
    double b1 = V1(b, ip) + sm;
    FL(3 * (m - ip) + 6);
    if (b1 / A1 > 0) {
        if (ip < m) {
            if (ip != jp) {
                for (int i = 1; i <= ip - 1; ++i) { double t = Aij(i, ip); Aij(i, ip) = Aij(i, jp); Aij(i, jp) = t; }
                V1(b, ip) = b1;
                { double t = Aij(ip, ip); Aij(ip, ip) = A1; Aij(ip, jp) = t; }
                for (int i = ip + 1; i <= m; ++i) {
                    double a = Aij(i, jp) / alpha;
                    double t = Aij(i, ip);
                    Aij(i, ip) = a; Aij(i, jp) = t;
                    V1(b, i) = fma(sm, a, V1(b, i));
                }
            } else {
                V1(b, ip) = b1;
                Aij(ip, ip) = A1;
                for (int i = ip + 1; i <= m; ++i) {
                    double a = Aij(i, ip) / alpha;
                    Aij(i, ip) = a;
                    V1(b, i) = fma(sm, a, V1(b, i));
                }
            }
            FL(3 * (m - ip));
        } else {
            tau = 0;
            if (ip != jp)
                for (int i = 1; i <= m; ++i) { double t = Aij(i, ip); Aij(i, ip) = Aij(i, jp); Aij(i, jp) = t; }
        }
        return tau;
    }
    return -1;
}

/* apply_householder_dual!, src/NNLS.jl:379-436 (the 4-column unrolling of the
 * reference only interleaves independent columns; per-column arithmetic is
 * identical to its remainder loop). */
static void ahd(double *A, int lda, int n, double *w, const double *b, double tau, int j1, int m1) {
    if (j1 >= m1) return;
    double aii = Aij(j1, j1);
    Aij(j1, j1) = 1;
    for (int j = j1 + 1; j <= n; ++j) {
        double sm = 0;
        for (int i = j1; i <= m1; ++i) sm = fma(Aij(i, j), Aij(i, j1), sm);
        sm *= -tau;
        double wj = 0;
        Aij(j1, j) = Aij(j1, j) + sm;
        for (int i = j1 + 1; i <= m1; ++i) {
            double a = fma(sm, Aij(i, j1), Aij(i, j));
            wj = fma(a, V1(b, i), wj);
            Aij(i, j) = a;
        }
        V1(w, j) = wj;
    }
    Aij(j1, j1) = aii;
    FL((double)(n - j1) * (6.0 * (m1 - j1) + 4));
}

/* compute_dual!, src/NNLS.jl:441-470 */
static void compute_dual(double *w, const double *A, int lda, int n, const double *b, int j1, int m1) {
    for (int j = j1; j <= n; ++j) {
        double sm = 0;
        for (int i = j1; i <= m1; ++i) sm = fma(Aij(i, j), V1(b, i), sm);
        V1(w, j) = sm;
    }
    FL((double)(n - j1 + 1) * 2.0 * (m1 - j1 + 1));
}

/* Base.hypot for Float64 (the algorithm NNLS.orthogonal_rotmat calls):
 * C. F. Borges, "An Improved Algorithm for hypot(a,b)", 2019, with the
 * fma correction step. */
static double jl_hypot(double x, double y) {
    if (isinf(x) || isinf(y)) return INFINITY;
    double ax = fabs(x), ay = fabs(y);
    if (ay > ax) { double t = ax; ax = ay; ay = t; }
    if (ay <= ax * 1.0536712127723509e-08) return ax; /* sqrt(eps/2) */
    double scale = EPS64 * 1.4916681462400413e-154;   /* eps * sqrt(floatmin) */
    if (ax > 9.480751908109176e+153) {                 /* sqrt(floatmax/2) */
        ax = ax * scale; ay = ay * scale; scale = 1.0 / scale;
    } else if (ay < 1.4916681462400413e-154) {         /* sqrt(floatmin) */
        ax = ax / scale; ay = ay / scale;
    } else {
        scale = 1.0;
    }
    double h = sqrt(fma(ax, ax, ay * ay));
    double hsq = h * h, axsq = ax * ax;
    h -= (fma(-ay, ay, hsq - axsq) + fma(h, h, -hsq) - fma(ax, ax, -axsq)) / (2 * h);
    return h * scale;
}
static inline void rotmat(double a, double b, double *c, double *s, double *sig) {
    double sg = jl_hypot(a, b);
    *c = a / sg; *s = b / sg; *sig = sg;
}
static inline void rotvec(double c, double s, double *a, double *b) {
    double x = fma(c, *a, s * *b), y = fma(-s, *a, c * *b);
    *a = x; *b = y;
}

/* solve_triangular_system!, src/NNLS.jl:506-539 */
static void solve_tri(double *z, const double *A, int lda, int n, int transp) {
    if (!transp) {
        for (int j = n; j >= 1; --j) {
            double zi = -V1(z, j) / Aij(j, j);
            for (int i = 1; i <= j - 1; ++i) V1(z, i) = fma(Aij(i, j), zi, V1(z, i));
            V1(z, j) = -zi;
        }
    } else {
        for (int j = 1; j <= n; ++j) {
            double z1 = V1(z, j);
            for (int l = 1; l <= j - 1; ++l) z1 = fma(-Aij(l, j), V1(z, l), z1);
            z1 /= Aij(j, j);
            V1(z, j) = z1;
        }
    }
    FL((double)n * n + n);
}

/* largest_positive_dual, src/NNLS.jl:541-554 */
static int largest_positive_dual(const double *w, int n, int j1, double *wmax) {
    double wm = 0;
    int jm = 0;
    for (int j = j1; j <= n; ++j)
        if (V1(w, j) > wm) { wm = V1(w, j); jm = j; }
    *wmax = wm;
    return jm;
}

/* Deletion of column `imv` from the active set with Givens rotations
 * (shared by both NNLS variants), src/NNLS.jl:731-779 / 967-1015. */
static void nnls_delete(double *A, int lda, int n, int m, double *b, double *x, int *idx, int *pnsetp, int imv) {
    int nsetp = *pnsetp;
    for (;;) {
        V1(x, V1(idx, imv)) = 0;
        if (imv != nsetp) {
            for (int i = imv + 1; i <= nsetp; ++i) {
                double cc, ss, rr;
                rotmat(Aij(i - 1, i), Aij(i, i), &cc, &ss, &rr);
                Aij(i - 1, i) = rr;
                Aij(i, i) = 0;
                for (int j = 1; j <= i - 1; ++j) rotvec(cc, ss, &Aij(i - 1, j), &Aij(i, j));
                for (int j = i + 1; j <= n; ++j) rotvec(cc, ss, &Aij(i - 1, j), &Aij(i, j));
                rotvec(cc, ss, &V1(b, i - 1), &V1(b, i));
                FL(6.0 * n + 20);
            }
            for (int j = imv; j <= nsetp - 1; ++j) {
                for (int i = 1; i <= m; ++i) { double t = Aij(i, j + 1); Aij(i, j + 1) = Aij(i, j); Aij(i, j) = t; }
                int t = V1(idx, j); V1(idx, j) = V1(idx, j + 1); V1(idx, j + 1) = t;
            }
        }
        nsetp -= 1;
        int allfeasible = 1;
        for (int i = 1; i <= nsetp; ++i)
            if (V1(x, V1(idx, i)) <= 0) { allfeasible = 0; imv = i; break; }
        if (allfeasible) break;
    }
    *pnsetp = nsetp;
}

/* One pass of the secondary loop's feasibility step; returns 1 when all new
 * coefficients are feasible.  src/NNLS.jl:700-727 */
static int nnls_feasible_step(double *x, const double *zz, const int *idx, int nsetp, int *imv_out, double *alpha_out) {
    int imv = nsetp;
    double alpha = 2;
    for (int i = 1; i <= nsetp; ++i) {
        if (V1(zz, i) <= 0) {
            double xi = V1(x, V1(idx, i));
            double t = -xi / (V1(zz, i) - xi);
            if (alpha > t) { imv = i; alpha = t; }
        }
    }
    FL(2 * nsetp);
    *imv_out = imv;
    *alpha_out = alpha;
    if (alpha == 2) return 1;
    for (int i = 1; i <= nsetp; ++i) {
        int ix = V1(idx, i);
        V1(x, ix) = fma(alpha, V1(zz, i) - V1(x, ix), V1(x, ix));
    }
    FL(3 * nsetp);
    return 0;
}

/* unsafe_nnls!(work; init_dual, max_iter), src/NNLS.jl:605-825 */
static void nnls_unsafe(nnls_ws *ws, int init_dual, int max_iter) {
    double *A = ws->A, *b = ws->b, *x = ws->x, *w = ws->w, *zz = ws->zz;
    int *idx = ws->idx;
    const int m = ws->M, n = ws->N, lda = ws->M;
    if (init_dual) {
        memset(w, 0, sizeof(double) * n);
        compute_dual(w, A, lda, n, b, 1, m);
    }
    int nsetp = 0, iter = 0, terminated = 0;
    ws->mode = 0;
    for (;;) {
        if (nsetp >= n || nsetp >= m) { terminated = 1; break; }
        int jmax = nsetp;
        double tau = 0;
        for (;;) {
            double wmax;
            jmax = largest_positive_dual(w, n, nsetp + 1, &wmax);
            if (wmax <= 0) { terminated = 1; break; }
            tau = cah(A, lda, b, nsetp + 1, jmax, m);
            if (tau >= 0) break;
            V1(w, jmax) = 0;
        }
        if (terminated) break;
        nsetp += 1;
        { int t = V1(idx, nsetp); V1(idx, nsetp) = V1(idx, jmax); V1(idx, jmax) = t; }
        if (nsetp < n) ahd(A, lda, n, w, b, tau, nsetp, m);
        for (int i = nsetp + 1; i <= m; ++i) Aij(i, nsetp) = 0;
        V1(w, nsetp) = 0;
        for (int i = 1; i <= nsetp; ++i) V1(zz, i) = V1(b, i);
        solve_tri(zz, A, lda, nsetp, 0);
        int dual_flag = 0;
        for (;;) {
            iter += 1;
            if (iter > max_iter) { ws->mode = 1; terminated = 1; break; }
            int imv;
            double alpha;
            if (nnls_feasible_step(x, zz, idx, nsetp, &imv, &alpha)) break;
            dual_flag = 1;
            nnls_delete(A, lda, n, m, b, x, idx, &nsetp, imv);
            for (int i = 1; i <= nsetp; ++i) V1(zz, i) = V1(b, i);
            solve_tri(zz, A, lda, nsetp, 0);
        }
        if (terminated) break;
        if (dual_flag) compute_dual(w, A, lda, n, b, nsetp + 1, m);
        for (int i = 1; i <= nsetp; ++i) V1(x, V1(idx, i)) = V1(zz, i);
    }
    for (int i = 1; i <= n; ++i) ws->invidx[V1(idx, i) - 1] = i;
    lacc Lr = {{0}};
    if (nsetp < m) {
        for (int i = nsetp + 1; i <= m; ++i) {
            double bi = V1(b, i);
            V1(zz, i) = bi;
            Lr.p[(i - nsetp - 1) & 31] = fma(bi, bi, Lr.p[(i - nsetp - 1) & 31]);
        }
        FL(2 * (m - nsetp));
    } else {
        memset(w, 0, sizeof(double) * n);
    }
    ws->rnorm = sqrt(lacc_tree(&Lr));
    ws->nsetp = nsetp;
}

/* unsafe_nnls!(work, λ; ...): Tikhonov form [A; λI] with lazily activated
 * padding rows, src/NNLS.jl:827-1061 */
static void nnls_unsafe_tikh(nnls_ws *ws, double lambda, int init_dual, int max_iter) {
    double *A = ws->A, *b = ws->b, *x = ws->x, *w = ws->w, *zz = ws->zz;
    int *idx = ws->idx;
    unsigned char *diag = ws->diag;
    const int M = ws->M, N = ws->N, lda = ws->M, n = N;
    int m = M - N;
    if (init_dual) {
        memset(w, 0, sizeof(double) * N);
        compute_dual(w, A, lda, n, b, 1, m);
    }
    int nsetp = 0, iter = 0, terminated = 0;
    ws->mode = 0;
    for (;;) {
        if (nsetp >= n) { terminated = 1; break; }
        int jmax = nsetp;
        double tau = 0;
        for (;;) {
            double wmax;
            jmax = largest_positive_dual(w, n, nsetp + 1, &wmax);
            if (wmax <= 0) { terminated = 1; break; }
            if (!diag[V1(idx, jmax) - 1]) Aij(m + 1, jmax) = lambda;
            tau = cah(A, lda, b, nsetp + 1, jmax, (m + 1 < M ? m + 1 : M));
            if (tau >= 0) break;
            V1(w, jmax) = 0;
            if (m < M) Aij(m + 1, jmax) = 0;
        }
        if (terminated) break;
        if (!diag[V1(idx, jmax) - 1]) {
            m = (m + 1 < M ? m + 1 : M);
            diag[V1(idx, jmax) - 1] = 1;
        }
        nsetp += 1;
        { int t = V1(idx, nsetp); V1(idx, nsetp) = V1(idx, jmax); V1(idx, jmax) = t; }
        if (nsetp < N) ahd(A, lda, n, w, b, tau, nsetp, m);
        for (int i = nsetp + 1; i <= m; ++i) Aij(i, nsetp) = 0;
        V1(w, nsetp) = 0;
        for (int i = 1; i <= nsetp; ++i) V1(zz, i) = V1(b, i);
        solve_tri(zz, A, lda, nsetp, 0);
        int dual_flag = 0;
        for (;;) {
            iter += 1;
            if (iter > max_iter) { ws->mode = 1; terminated = 1; break; }
            int imv;
            double alpha;
            if (nnls_feasible_step(x, zz, idx, nsetp, &imv, &alpha)) break;
            dual_flag = 1;
            nnls_delete(A, lda, n, m, b, x, idx, &nsetp, imv);
            for (int i = 1; i <= nsetp; ++i) V1(zz, i) = V1(b, i);
            solve_tri(zz, A, lda, nsetp, 0);
        }
        if (terminated) break;
        if (dual_flag) compute_dual(w, A, lda, n, b, nsetp + 1, m);
        for (int i = 1; i <= nsetp; ++i) V1(x, V1(idx, i)) = V1(zz, i);
    }
    for (int i = 1; i <= n; ++i) ws->invidx[V1(idx, i) - 1] = i;
    lacc Lr = {{0}};
    if (nsetp < M) {
        for (int i = nsetp + 1; i <= M; ++i) {
            double bi = V1(b, i);
            V1(zz, i) = bi;
            Lr.p[(i - nsetp - 1) & 31] = fma(bi, bi, Lr.p[(i - nsetp - 1) & 31]);
        }
        FL(2 * (M - nsetp));
    } else {
        memset(w, 0, sizeof(double) * N);
    }
    ws->rnorm = sqrt(lacc_tree(&Lr));
    ws->nsetp = nsetp;
}
#undef Aij

/* ------------------------------------------------------------------------- */
/* NNLSProblem warm start (src/lsqnonneg.jl:30-164)                           */
/* ------------------------------------------------------------------------- */
/* solve!(::NNLSProblem, A, b): seed with column n, src/lsqnonneg.jl:30-84 */
static void nnlsprob_solve(nnls_ws *ws, const double *A, int m, int n, const double *b) {
    double *C = ws->A, *f = ws->b, *x = ws->x, *w = ws->w, *z = ws->zz;
    const double *An = A + (size_t)(n - 1) * m;
    lacc Ld = {{0}}, Lx = {{0}};
    for (int i = 0; i < m; ++i) Ld.p[i & 31] = Ld.p[i & 31] + An[i] * An[i];
    double den = lacc_tree(&Ld);
    for (int i = 0; i < m; ++i) Lx.p[i & 31] = Lx.p[i & 31] + (An[i] / den) * b[i];
    double xj = lacc_tree(&Lx);
    for (int i = 0; i < m; ++i) z[i] = b[i] - An[i] * xj;
    for (int j = 0; j < n - 1; ++j) {
        double wj = 0;
        const double *Aj = A + (size_t)j * m;
        double *Cj = C + (size_t)j * m;
        for (int i = 0; i < m; ++i) { double a = Aj[i]; wj += a * z[i]; Cj[i] = a; }
        w[j] = wj;
    }
    w[n - 1] = 0;
    int allle = 1;
    for (int j = 0; j < n; ++j) if (!(w[j] <= 0)) { allle = 0; break; }
    w[n - 1] = allle ? 1.0 : 0.0;
    for (int i = 0; i < m; ++i) { f[i] = b[i]; C[i + (size_t)(n - 1) * m] = An[i]; }
    for (int j = 0; j < n; ++j) { x[j] = 0; ws->idx[j] = j + 1; }
    FL(5.0 * m + 2.0 * m * (n - 1));
    nnls_unsafe(ws, 0, 3 * n);
}
/* solve!(::NNLSProblem, A, b, μ) on the padded [A; μI], src/lsqnonneg.jl:86-164 */
static void nnlsprob_solve_tikh(nnls_ws *ws, const double *A, int m, int n, const double *b, double mu) {
    const int M = m + n;
    double *C = ws->A, *f = ws->b, *x = ws->x, *w = ws->w, *z = ws->zz;
    const double *An = A + (size_t)(n - 1) * m;
    lacc Ld = {{0}}, Lx = {{0}};
    for (int i = 0; i < m; ++i) Ld.p[i & 31] = Ld.p[i & 31] + An[i] * An[i];
    double den = lacc_tree(&Ld);
    den = den + mu * mu;
    for (int i = 0; i < m; ++i) Lx.p[i & 31] = Lx.p[i & 31] + (An[i] / den) * b[i];
    double xj = lacc_tree(&Lx);
    for (int i = 0; i < m; ++i) z[i] = b[i] - An[i] * xj;
    for (int j = 0; j < n - 1; ++j) {
        double wj = 0;
        const double *Aj = A + (size_t)j * m;
        double *Cj = C + (size_t)j * M;
        for (int i = 0; i < m; ++i) { double a = Aj[i]; wj += a * z[i]; Cj[i] = a; }
        w[j] = wj;
    }
    w[n - 1] = 0;
    int allle = 1;
    for (int j = 0; j < n; ++j) if (!(w[j] <= 0)) { allle = 0; break; }
    w[n - 1] = allle ? 1.0 : 0.0;
    for (int i = 0; i < m; ++i) { f[i] = b[i]; C[i + (size_t)(n - 1) * M] = An[i]; }
    for (int j = 0; j < n; ++j)
        for (int i = m; i < M; ++i) C[i + (size_t)j * M] = 0;
    for (int j = 0; j < n; ++j) { x[j] = 0; f[m + j] = 0; ws->idx[j] = j + 1; ws->diag[j] = 0; }
    FL(5.0 * m + 2.0 * m * (n - 1) + 2);
    nnls_unsafe_tikh(ws, mu, 0, 3 * n);
}

/* Tikhonov quantities, src/lsqnonneg.jl:307-318 */
static inline double tikh_loss(const nnls_ws *ws) { return ws->rnorm * ws->rnorm; }
static double tikh_seminorm_sq(const nnls_ws *ws) {
    lacc L = {{0}};
    for (int i = 0; i < ws->nsetp; ++i) { double v = ws->x[ws->idx[i] - 1]; L.p[i & 31] = L.p[i & 31] + v * v; }
    FL(2 * ws->nsetp);
    return lacc_tree(&L);
}
static double tikh_resnorm_sq(const nnls_ws *ws, double mu) {
    double reg = (mu * mu) * tikh_seminorm_sq(ws);
    return jmax(tikh_loss(ws) - reg, 0.0);
}

/* ------------------------------------------------------------------------- */
/* Root finding / minimization (src/optimization.jl)                          */
/* ------------------------------------------------------------------------- */
/* bracket_root_monotonic, src/optimization.jl:191-219 */
static void bracket_root_monotonic(orc_fn f, void *ctx, double a, double delta, double dilate, double mono, int maxiters,
                                   double *ra, double *rb, double *rfa, double *rfb) {
    double fa = f(a, ctx);
    if (!jisfinite(fa)) { *ra = a; *rb = a; *rfa = NAN; *rfb = NAN; return; }
    if (fa == 0) { *ra = a; *rb = a; *rfa = fa; *rfb = fa; return; }
    double sgn = jsign(mono) * jsign(fa);
    double b = a - sgn * delta;
    double fb = f(b, ctx);
    if (!jisfinite(fb)) { *ra = a; *rb = a; *rfa = fa; *rfb = fa; return; }
    if (fb == 0) { *ra = b; *rb = b; *rfa = fb; *rfb = fb; return; }
    delta *= dilate;
    int cnt = 0;
    while (fa * fb > 0 && cnt < maxiters) {
        a = b; fa = fb;
        b = a - sgn * delta;
        fb = f(b, ctx);
        if (!jisfinite(fb)) { *ra = a; *rb = a; *rfa = fa; *rfb = fa; return; }
        if (fb == 0) { *ra = b; *rb = b; *rfa = fb; *rfb = fb; return; }
        delta *= dilate;
        cnt += 1;
    }
    if (a < b) { *ra = a; *rb = b; *rfa = fa; *rfb = fb; }
    else { *ra = b; *rb = a; *rfa = fb; *rfb = fa; }
}

/* brent_root, src/optimization.jl:71-128 */
static void brent_root(orc_fn f, void *ctx, double x0, double x1, double fx0, double fx1, double xatol, double xrtol,
                       double ftol, int maxiters, double *xr, double *fxr) {
    if (fx0 == 0) { *xr = x0; *fxr = fx0; return; }
    if (fx1 == 0) { *xr = x1; *fxr = fx1; return; }
    /* the reference asserts fx0*fx1 < 0 here */
    double a = x0, b = x1, fa = fx0, fb = fx1;
    if (fabs(fa) < fabs(fb)) { double t = a; a = b; b = t; t = fa; fa = fb; fb = t; }
    double c = x0, d = x0, fc = fx0;
    int mflag = 1;
    for (int iter = 1; iter <= maxiters; ++iter) {
        if (fabs(b - a) <= 2 * (xatol + xrtol * fabs(b))) { *xr = b; *fxr = fb; return; }
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
            mflag = 1;
        } else {
            mflag = 0;
        }
        double fs = f(s, ctx);
        if (fs == 0) { *xr = s; *fxr = fs; return; }
        if (isnan(fs) || isinf(fs)) { *xr = b; *fxr = fb; return; }
        if (fabs(fs) <= ftol) { *xr = s; *fxr = fs; return; }
        d = c; c = b; fc = fb;
        if (jsign(fa) * jsign(fs) < 0) { b = s; fb = fs; }
        else { a = s; fa = fs; }
        if (fabs(fa) < fabs(fb)) { double t = a; a = b; b = t; t = fa; fa = fb; fb = t; }
    }
    *xr = b; *fxr = fb;
}
void orc_brent_root(orc_fn f, void *ctx, double a, double b, double xatol, double xrtol, double ftol, int maxiters,
                    double *x, double *fx) {
    double fa = f(a, ctx), fb = f(b, ctx);
    brent_root(f, ctx, a, b, fa, fb, xatol, xrtol, ftol, maxiters, x, fx);
}

/* bisect_root, src/optimization.jl:31-67 */
void orc_bisect_root(orc_fn f, void *ctx, double a, double b, double xatol, double xrtol, double ftol, int maxiters,
                     double *xo, double *fo) {
    double x1 = a, x2 = b, y1 = f(x1, ctx), y2 = f(x2, ctx);
    if (x1 == x2 || y1 * y2 >= 0) {
        if (fabs(y1) <= fabs(y2)) { *xo = x1; *fo = y1; } else { *xo = x2; *fo = y2; }
        return;
    }
    if (y2 < 0) { double t = x1; x1 = x2; x2 = t; t = y1; y1 = y2; y2 = t; }
    double xm = (x1 + x2) / 2, ym = f(xm, ctx);
    for (int iter = 1; iter <= maxiters; ++iter) {
        if (fabs(ym) <= ftol || 2 * jmin(fabs(xm - x1), fabs(x2 - xm)) <= xatol + xrtol * fabs(xm)) break;
        if (ym < 0) { x1 = xm; y1 = ym; } else { x2 = xm; y2 = ym; }
        xm = (x1 + x2) / 2;
        ym = f(xm, ctx);
        if (!jisfinite(ym)) {
            if (fabs(y1) <= fabs(y2)) { xm = x1; ym = y1; } else { xm = x2; ym = y2; }
            break;
        }
    }
    *xo = xm; *fo = ym;
}

/* brent_minimize, src/optimization.jl:319-413 */
static void brent_minimize(orc_fn f, void *ctx, double x1, double x2, double xrtol, double xatol, int maxiters,
                           double *xo, double *yo) {
    const double alpha = 2 - PHI;
    double x = x1 + alpha * (x2 - x1);
    double y = f(x, ctx);
    double dx_old = 0, dx = 0;
    double x_older = x, x_old = x, y_older = y, y_old = y;
    int iter = 0;
    while (iter < maxiters) {
        double p = 0, q = 0;
        double xm = (x2 + x1) / 2;
        double tolx = xatol + xrtol * fabs(x);
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
        double y_new = f(x_new, ctx);
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
    *xo = x; *yo = y;
}
void orc_brent_minimize(orc_fn f, void *ctx, double a, double b, double xatol, double xrtol, int maxiters, double *x, double *fx) {
    brent_minimize(f, ctx, a, b, xrtol, xatol, maxiters, x, fx);
}

/* ------------------------------------------------------------------------- */
/* Singular values (stand-in for LAPACK dgesdd job='N', src/utils.jl:67-134)  */
/* Householder bidiagonalization + bisection on the Golub-Kahan tridiagonal.  */
/* ------------------------------------------------------------------------- */
/* Golub-Kahan Householder bidiagonalization of B = A (m >= n) or A' (r x c,
 * r >= c), then bisection on the Golub-Kahan tridiagonal (zero diagonal,
 * off-diagonals d0, e0, d1, e1, ..., d_{c-1}) whose positive eigenvalues are
 * the singular values, resolved to 1e-15 of their Gershgorin bound; sorted
 * descending.  The GPU path (warp_svdvals) performs the same operations in the
 * same order: sequential sums, FMAs and IEEE square roots and divisions. */
static int sturm_count_gk(const double *o2, int N, double x) {
    double p2 = 1.0, p1 = 0.0 - x;
    int neg = p1 <= 0;
    int cnt = neg;
    for (int j = 1; j < N; ++j) {
        double p = fma(0.0 - x, p1, -o2[j - 1] * p2);
        int pneg = p < 0 || (p == 0 && !neg);
        cnt += (pneg != neg);
        neg = pneg;
        p2 = p1;
        p1 = p;
        uint64_t u;
        memcpy(&u, &p1, 8);
        const int ex = (int)((u >> 52) & 0x7ff) - 1023;
        if (p1 != 0 && (ex > 400 || ex < -400)) {
            const uint64_t su = (uint64_t)(uint32_t)((1023 - ex) << 20) << 32;
            double sc;
            memcpy(&sc, &su, 8);
            p1 *= sc;
            p2 *= sc;
        }
    }
    return cnt;
}
static void bidiag_svdvals(const double *A, int m, int n, double *s, double *U) {
    const int r = m >= n ? m : n, c = m >= n ? n : m; /* U is r x c with c <= r */
    for (int j = 0; j < c; ++j)
        for (int i = 0; i < r; ++i) U[i + (size_t)j * r] = (m >= n) ? A[i + (size_t)j * m] : A[j + (size_t)i * m];
    double *dv = (double *)malloc(sizeof(double) * (2 * (size_t)c + 1)), *ev = dv + c;
    for (int k = 0; k < c; ++k) {
        const double *uk = U + (size_t)k * r;
        double ss = 0.0;
        for (int i = k + 1; i < r; ++i) ss = fma(uk[i], uk[i], ss);
        const double x0 = uk[k];
        double alpha = x0, v0 = 0.0, tau = 0.0;
        if (ss != 0.0) {
            const double nrm = sqrt(fma(x0, x0, ss));
            alpha = x0 >= 0.0 ? -nrm : nrm;
            v0 = x0 - alpha;
            tau = 2.0 / fma(v0, v0, ss);
        }
        dv[k] = alpha;
        if (tau != 0.0) {
            for (int j = k + 1; j < c; ++j) {
                double *uj = U + (size_t)j * r;
                double sdot = v0 * uj[k];
                for (int i = k + 1; i < r; ++i) sdot = fma(uk[i], uj[i], sdot);
                const double f = tau * sdot;
                uj[k] = fma(-f, v0, uj[k]);
                for (int i = k + 1; i < r; ++i) uj[i] = fma(-f, uk[i], uj[i]);
            }
            FL(4.0 * (r - k) * (c - k - 1));
        }
        if (k + 2 < c) {
            double sr = 0.0;
            for (int j = k + 2; j < c; ++j) { const double y = U[k + (size_t)j * r]; sr = fma(y, y, sr); }
            const double y0 = U[k + (size_t)(k + 1) * r];
            double beta = y0, w0 = 0.0, tau2 = 0.0;
            if (sr != 0.0) {
                const double nrm = sqrt(fma(y0, y0, sr));
                beta = y0 >= 0.0 ? -nrm : nrm;
                w0 = y0 - beta;
                tau2 = 2.0 / fma(w0, w0, sr);
            }
            ev[k] = beta;
            if (tau2 != 0.0) {
                for (int i = k + 1; i < r; ++i) {
                    double sdot = w0 * U[i + (size_t)(k + 1) * r];
                    for (int j = k + 2; j < c; ++j) sdot = fma(U[k + (size_t)j * r], U[i + (size_t)j * r], sdot);
                    const double f = tau2 * sdot;
                    U[i + (size_t)(k + 1) * r] = fma(-f, w0, U[i + (size_t)(k + 1) * r]);
                    for (int j = k + 2; j < c; ++j) U[i + (size_t)j * r] = fma(-f, U[k + (size_t)j * r], U[i + (size_t)j * r]);
                }
                FL(4.0 * (r - k - 1) * (c - k - 1));
            }
        } else if (k + 1 < c) {
            ev[k] = U[k + (size_t)(k + 1) * r];
        }
    }
    const int N = 2 * c;
    double bnd = 0.0;
    for (int j = 0; j < N; ++j) {
        const double oa = j > 0 ? fabs((j - 1) % 2 == 0 ? dv[(j - 1) / 2] : ev[(j - 1) / 2]) : 0.0;
        const double ob = j + 1 < N ? fabs(j % 2 == 0 ? dv[j / 2] : ev[j / 2]) : 0.0;
        bnd = fmax(bnd, oa + ob);
    }
    double *o2 = U;
    for (int j = 0; j + 1 < N; ++j) {
        const double o = j % 2 == 0 ? dv[j / 2] : ev[j / 2];
        o2[j] = o * o;
    }
    const double tau0 = 1e-14 * bnd, atol = 1e-15 * bnd;
    const int nres = N - sturm_count_gk(o2, N, tau0);
    for (int t = 0; t < c; ++t) {
        if (t >= nres) { s[t] = 0.0; continue; }
        const int idx = N - 1 - t;
        double a = tau0, b = bnd;
        int done = 0;
        for (int it = 0; it < 80 && !done; ++it) {
            const double mid = 0.5 * (a + b);
            const int cnt = sturm_count_gk(o2, N, mid);
            if (cnt > idx) b = mid; else a = mid;
            done = (b - a) <= fmax(atol, 4.0 * 2.220446049250313e-16 * b);
            FL(3.0 * N);
        }
        s[t] = 0.5 * (a + b);
    }
    free(dv);
}
int orc_svdvals(const double *A, int m, int n, double *s) {
    int r = m >= n ? m : n, c = m >= n ? n : m;
    double *U = (double *)malloc(sizeof(double) * (size_t)r * c);
    bidiag_svdvals(A, m, n, s, U);
    free(U);
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Regularized problems on one (A, b)                                         */
/* ------------------------------------------------------------------------- */
typedef struct {
    int m, n;
    const double *A, *b;
    nnls_ws un;  /* NNLSProblem (m x n) */
    nnls_ws tk;  /* NNLSTikhonovRegProblem ((m+n) x n) */
    double tk_mu; /* μ of the current Tikhonov solution (the cache's current slot) */
    /* lcurve caches (GrowableCache with isapprox keys, src/utils.jl:140-232) */
    int fc_len, fc_cap; double *fc_x; double *fc_P;        /* CachedFunction */
    int pc_len, pc_cap; double *pc_x; double *pc_P; double *pc_C; /* point cache */
    int sc_len, sc_cap; double *sc_x; double *sc_P;        /* state cache: 4 x's, 4x2 P's */
    double *gamma; double *svdU; /* gcv */
    double res2_target, delta2;  /* chi2 / mdp targets */
} reg_ws;

static void reg_ws_init(reg_ws *r, int m, int n) {
    memset(r, 0, sizeof(*r));
    r->m = m; r->n = n;
    nnls_ws_alloc(&r->un, m, n);
    nnls_ws_alloc(&r->tk, m + n, n);
    r->tk_mu = NAN;
    r->fc_cap = r->pc_cap = r->sc_cap = 64;
    r->fc_x = (double *)malloc(sizeof(double) * 64); r->fc_P = (double *)malloc(sizeof(double) * 128);
    r->pc_x = (double *)malloc(sizeof(double) * 64); r->pc_P = (double *)malloc(sizeof(double) * 128);
    r->pc_C = (double *)malloc(sizeof(double) * 64);
    r->sc_x = (double *)malloc(sizeof(double) * 256); r->sc_P = (double *)malloc(sizeof(double) * 512);
    int mn = m < n ? m : n, mx = m > n ? m : n;
    r->gamma = (double *)malloc(sizeof(double) * mn);
    r->svdU = (double *)malloc(sizeof(double) * (size_t)mn * mx);
}
static void reg_ws_free(reg_ws *r) {
    nnls_ws_free(&r->un); nnls_ws_free(&r->tk);
    free(r->fc_x); free(r->fc_P); free(r->pc_x); free(r->pc_P); free(r->pc_C);
    free(r->sc_x); free(r->sc_P); free(r->gamma); free(r->svdU);
}
static void reg_solve_unreg(reg_ws *r) { nnlsprob_solve(&r->un, r->A, r->m, r->n, r->b); }
static void reg_solve_tikh(reg_ws *r, double mu) {
    nnlsprob_solve_tikh(&r->tk, r->A, r->m, r->n, r->b, mu);
    r->tk_mu = mu;
}
static inline double unreg_res2(const reg_ws *r) { return r->un.rnorm * r->un.rnorm; }
static inline double tikh_res2(const reg_ws *r) { return tikh_resnorm_sq(&r->tk, r->tk_mu); }

static void spline_root_legacy_pts(const double *X, const double *Y, int npts, double value, double *x);
/* lsqnonneg_chi2!(method=:brent), src/lsqnonneg.jl:504-593 */
static double chi2_f(double logmu, void *ctx) {
    reg_ws *r = (reg_ws *)ctx;
    int st = g_st; g_st = ORC_ST_REG_NNLS;
    reg_solve_tikh(r, pm_exp(logmu));
    g_st = st;
    double res2 = tikh_res2(r);
    FL(3);
    return (res2 - r->res2_target) / r->res2_target;
}
/* Returns the solution that save_results! stores.  Deviation: on the early
 * exit (exact or empty unregularized fit) the reference saves the smoothing
 * cache's stale current slot; the restatement uses x_unreg (the returned x). */
static const double *reg_chi2(reg_ws *r, double chi2_target, double *mu_out, double *chi2_out) {
    g_st = ORC_ST_REG_NNLS;
    reg_solve_unreg(r);
    g_st = ORC_ST_REG_OTHER;
    double res2_min = unreg_res2(r);
    if (res2_min == 0 || r->un.nsetp == 0) { *mu_out = 0; *chi2_out = 1; return r->un.x; }
    r->res2_target = chi2_target * res2_min;
    double a, b, fa, fb, logmu, relerr;
    bracket_root_monotonic(chi2_f, r, -4.0, 1.0, 1.5, 1.0, 6, &a, &b, &fa, &fb);
    if (fa * fb < 0) {
        brent_root(chi2_f, r, a, b, fa, fb, 0.0, 0.0, 1e-3 * (chi2_target - 1), 100, &logmu, &relerr);
    } else {
        if (!jisfinite(fa)) { logmu = b; relerr = fb; }
        else if (!jisfinite(fb)) { logmu = a; relerr = fa; }
        else if (fabs(fa) < fabs(fb)) { logmu = a; relerr = fa; }
        else { logmu = b; relerr = fb; }
    }
    double mu, res2;
    if (jisfinite(relerr)) {
        mu = pm_exp(logmu);
        res2 = r->res2_target * (1 + relerr);
        g_st = ORC_ST_REG_NNLS;
        reg_solve_tikh(r, mu);
        g_st = ORC_ST_REG_OTHER;
    } else {
        /* saved solution: the current Tikhonov slot (last solve) */
        mu = 0;
        res2 = 1;
    }
    *mu_out = mu;
    *chi2_out = res2 / res2_min;
    return r->tk.x;
}

/* lsqnonneg_chi2!(legacy = true), src/lsqnonneg.jl:504-531, with
 * chi2_search_from_minimum(legacy = true), src/lsqnonneg.jl:595-636: double mu
 * from 1e-3 until res2(mu) >= Chi2Factor * res2_min, then the legacy spline
 * root through all (mu, res2) pairs including (0, res2_min).  Deviation: the
 * doubling stops after CHI2_LEGACY_MAXDOUBLE steps (mu = 1e-3 * 2^20), where the
 * reference would keep doubling without bound on data that never reaches the
 * target. */
#define CHI2_LEGACY_MAXDOUBLE 20
static const double *reg_chi2_legacy(reg_ws *r, double chi2_target, double *mu_out, double *chi2_out) {
    g_st = ORC_ST_REG_NNLS;
    reg_solve_unreg(r);
    g_st = ORC_ST_REG_OTHER;
    double res2_min = unreg_res2(r);
    if (res2_min == 0 || r->un.nsetp == 0) { *mu_out = 0; *chi2_out = 1; return r->un.x; }
    double mus[CHI2_LEGACY_MAXDOUBLE + 2], r2s[CHI2_LEGACY_MAXDOUBLE + 2];
    int cnt = 0;
    mus[cnt] = 0; r2s[cnt++] = res2_min;
    double munew = 1e-3;
    for (int it = 0;; ++it) {
        g_st = ORC_ST_REG_NNLS;
        reg_solve_tikh(r, munew);
        g_st = ORC_ST_REG_OTHER;
        double res2new = tikh_res2(r);
        mus[cnt] = munew; r2s[cnt++] = res2new;
        if (res2new >= chi2_target * res2_min || it == CHI2_LEGACY_MAXDOUBLE) break;
        munew *= 2.0;
    }
    double mu, res2;
    spline_root_legacy_pts(mus, r2s, cnt, chi2_target * res2_min, &mu);
    if (mu == 0) res2 = res2_min;
    else {
        g_st = ORC_ST_REG_NNLS;
        reg_solve_tikh(r, mu);
        g_st = ORC_ST_REG_OTHER;
        res2 = tikh_res2(r);
    }
    *mu_out = mu;
    *chi2_out = res2 / res2_min;
    return mu == 0 ? r->un.x : r->tk.x;
}

/* lsqnonneg_mdp!, src/lsqnonneg.jl:700-747 */
static double mdp_f(double logmu, void *ctx) {
    reg_ws *r = (reg_ws *)ctx;
    int st = g_st; g_st = ORC_ST_REG_NNLS;
    reg_solve_tikh(r, pm_exp(logmu));
    g_st = st;
    return tikh_res2(r) - r->delta2;
}
/* Deviation: on the two early exits the reference saves the smoothing cache's
 * stale current slot; the restatement saves the returned x (x_unreg, or the
 * zero vector for δ >= ||b||). */
static const double *reg_mdp(reg_ws *r, double delta, double *mu_out, double *chi2_out, double *zero_n) {
    g_st = ORC_ST_REG_NNLS;
    reg_solve_unreg(r);
    g_st = ORC_ST_REG_OTHER;
    double res2_min = unreg_res2(r);
    if (delta <= sqrt(res2_min)) { *mu_out = 0; *chi2_out = 1; return r->un.x; }
    /* sum(abs2, work.nnls_prob.b): the problem's (unmodified) data vector */
    lacc Lm = {{0}};
    for (int i = 0; i < r->m; ++i) Lm.p[i & 31] = Lm.p[i & 31] + r->b[i] * r->b[i];
    double res2_max = lacc_tree(&Lm);
    if (delta >= sqrt(res2_max)) {
        memset(zero_n, 0, sizeof(double) * r->n);
        *mu_out = INFINITY; *chi2_out = res2_max / res2_min;
        return zero_n;
    }
    r->delta2 = delta * delta;
    double a, b, fa, fb, logmu, err;
    bracket_root_monotonic(mdp_f, r, -4.0, 1.0, 1.5, 1.0, 6, &a, &b, &fa, &fb);
    if (fa * fb < 0) {
        brent_root(mdp_f, r, a, b, fa, fb, 0.0, 0.0, 1e-3 * (delta * delta), 100, &logmu, &err);
    } else {
        if (!jisfinite(fa)) { logmu = b; err = fb; }
        else if (!jisfinite(fb)) { logmu = a; err = fa; }
        else if (fabs(fa) < fabs(fb)) { logmu = a; err = fa; }
        else { logmu = b; err = fb; }
    }
    double mu, res2;
    if (jisfinite(err)) {
        mu = pm_exp(logmu);
        res2 = delta * delta + err;
        g_st = ORC_ST_REG_NNLS;
        reg_solve_tikh(r, mu);
        g_st = ORC_ST_REG_OTHER;
    } else {
        mu = 0; res2 = 1;
    }
    *mu_out = mu;
    *chi2_out = res2 / res2_min;
    return r->tk.x;
}

/* ---- L-curve (src/lsqnonneg.jl:812-972) ---- */
typedef struct {
    orc_fn2 f; void *ctx; /* the L-curve point function (ξ(logμ), η(logμ)) */
    reg_ws *r;            /* caches live here */
} lc_ctx;

/* f_lcurve(logμ) through the isapprox-keyed CachedFunction */
static void lc_eval(lc_ctx *c, double x, double *P) {
    reg_ws *r = c->r;
    for (int i = 0; i < r->fc_len; ++i)
        if (isapprox(x, r->fc_x[i])) { P[0] = r->fc_P[2 * i]; P[1] = r->fc_P[2 * i + 1]; return; }
    c->f(x, P, c->ctx);
    if (r->fc_len >= r->fc_cap) {
        r->fc_cap *= 2;
        r->fc_x = (double *)realloc(r->fc_x, sizeof(double) * r->fc_cap);
        r->fc_P = (double *)realloc(r->fc_P, sizeof(double) * 2 * r->fc_cap);
    }
    r->fc_x[r->fc_len] = x;
    r->fc_P[2 * r->fc_len] = P[0];
    r->fc_P[2 * r->fc_len + 1] = P[1];
    r->fc_len++;
}
static int pc_find(const reg_ws *r, double x) {
    for (int i = 0; i < r->pc_len; ++i) if (isapprox(x, r->pc_x[i])) return i;
    return -1;
}
static void pc_push(reg_ws *r, double x, const double *P, double C) {
    if (r->pc_len >= r->pc_cap) {
        r->pc_cap *= 2;
        r->pc_x = (double *)realloc(r->pc_x, sizeof(double) * r->pc_cap);
        r->pc_P = (double *)realloc(r->pc_P, sizeof(double) * 2 * r->pc_cap);
        r->pc_C = (double *)realloc(r->pc_C, sizeof(double) * r->pc_cap);
    }
    r->pc_x[r->pc_len] = x;
    r->pc_P[2 * r->pc_len] = P[0];
    r->pc_P[2 * r->pc_len + 1] = P[1];
    r->pc_C[r->pc_len] = C;
    r->pc_len++;
}
static void pc_set(reg_ws *r, double x, const double *P, double C) {
    int i = pc_find(r, x);
    if (i < 0) { pc_push(r, x, P, C); return; }
    r->pc_P[2 * i] = P[0]; r->pc_P[2 * i + 1] = P[1]; r->pc_C[i] = C;
}
/* mapfindmax over the point cache: first maximal C under isless */
static int pc_argmax(const reg_ws *r) {
    int im = 0;
    for (int i = 1; i < r->pc_len; ++i) if (jisless(r->pc_C[im], r->pc_C[i])) im = i;
    return im;
}
typedef struct { double x[4]; double P[8]; } lc_state;
static void sc_push(reg_ws *r, const lc_state *s) {
    if (r->sc_len >= r->sc_cap) {
        r->sc_cap *= 2;
        r->sc_x = (double *)realloc(r->sc_x, sizeof(double) * 4 * r->sc_cap);
        r->sc_P = (double *)realloc(r->sc_P, sizeof(double) * 8 * r->sc_cap);
    }
    memcpy(r->sc_x + 4 * r->sc_len, s->x, sizeof(double) * 4);
    memcpy(r->sc_P + 8 * r->sc_len, s->P, sizeof(double) * 8);
    r->sc_len++;
}
static inline double norm2(double a, double b) { return sqrt(a * a + b * b); }
/* menger(Pj, Pk, Pl), src/lsqnonneg.jl:967-972 */
static double menger(const double *Pj, const double *Pk, const double *Pl) {
    double djk0 = Pj[0] - Pk[0], djk1 = Pj[1] - Pk[1];
    double dkl0 = Pk[0] - Pl[0], dkl1 = Pk[1] - Pl[1];
    double dlj0 = Pl[0] - Pj[0], dlj1 = Pl[1] - Pj[1];
    double PjPk = djk0 * djk0 + djk1 * djk1, PkPl = dkl0 * dkl0 + dkl1 * dkl1, PlPj = dlj0 * dlj0 + dlj1 * dlj1;
    FL(20);
    return 2 * (djk0 * dkl1 - djk1 * dkl0) / sqrt(PjPk * PkPl * PlPj);
}
/* update_curvature!, src/lsqnonneg.jl:948-965 */
static void lc_update_curvature(reg_ws *r, const lc_state *s, const double *Ptl, const double *Pbr, double Ctol) {
    for (int i = 0; i < 4; ++i) {
        double x = s->x[i];
        const double *P = s->P + 2 * i;
        double C = -INFINITY;
        double dtl = norm2(P[0] - Ptl[0], P[1] - Ptl[1]), dbr = norm2(P[0] - Pbr[0], P[1] - Pbr[1]);
        if (jmin(dtl, dbr) > Ctol) {
            double xm = -INFINITY, xp = INFINITY;
            const double *Pm = P, *Pp = P;
            for (int k = 0; k < r->pc_len; ++k) {
                double xk = r->pc_x[k];
                if (xm < xk && xk < x) { xm = xk; Pm = r->pc_P + 2 * k; }
                if (x < xk && xk < xp) { xp = xk; Pp = r->pc_P + 2 * k; }
            }
            double Pmc[2] = {Pm[0], Pm[1]}, Ppc[2] = {Pp[0], Pp[1]};
            C = menger(Pmc, P, Ppc);
        }
        double Pc[2] = {P[0], P[1]};
        pc_set(r, x, Pc, C);
    }
}
/* lcurve_corner, src/lsqnonneg.jl:872-919 (backtracking = true) */
static double lcurve_corner_impl(lc_ctx *c, double xlow, double xhigh, double xtol, double Ptol, double Ctol, int *iters_out) {
    reg_ws *r = c->r;
    r->fc_len = r->pc_len = r->sc_len = 0;
    lc_state st;
    /* initial_state, src/lsqnonneg.jl:921-929 */
    double x1 = xlow, x4 = xhigh;
    double x2 = (PHI * x1 + x4) / (PHI + 1);
    double x3 = x1 + (x4 - x2);
    st.x[0] = x1; st.x[1] = x2; st.x[2] = x3; st.x[3] = x4;
    for (int i = 0; i < 4; ++i) lc_eval(c, st.x[i], st.P + 2 * i);
    for (int i = 0; i < 4; ++i) pc_push(r, st.x[i], st.P + 2 * i, -INFINITY);
    double Ptl[2] = {st.P[0], st.P[1]}, Pbr[2] = {st.P[6], st.P[7]};
    lc_update_curvature(r, &st, Ptl, Pbr, Ctol);
    int iter = 0;
    while (!(fabs(st.x[3] - st.x[0]) < xtol || norm2(st.P[0] - st.P[6], st.P[1] - st.P[7]) < Ptol)) {
        iter += 1;
        if (iter > 1000) break; /* unreachable guard: the widths shrink by 1/φ per step */
        /* backtracking */
        double xb = r->pc_x[pc_argmax(r)];
        for (int k = 0; k < r->sc_len; ++k) {
            const double *sx = r->sc_x + 4 * k;
            if ((sx[1] == xb || sx[2] == xb) && fabs(sx[3] - sx[0]) <= fabs(st.x[3] - st.x[0])) {
                memcpy(st.x, sx, sizeof(double) * 4);
                memcpy(st.P, r->sc_P + 8 * k, sizeof(double) * 8);
            }
        }
        int i2 = pc_find(r, st.x[1]), i3 = pc_find(r, st.x[2]);
        if (i2 < 0 || i3 < 0) break; /* unreachable: state points are always cached */
        if (r->pc_C[i2] > r->pc_C[i3]) {
            /* move_left, src/lsqnonneg.jl:933-939 */
            lc_state ns;
            ns.x[0] = st.x[0]; ns.x[1] = (PHI * st.x[0] + st.x[2]) / (PHI + 1); ns.x[2] = st.x[1]; ns.x[3] = st.x[2];
            memcpy(ns.P, st.P, sizeof(double) * 2);
            lc_eval(c, ns.x[1], ns.P + 2);
            memcpy(ns.P + 4, st.P + 2, sizeof(double) * 2);
            memcpy(ns.P + 6, st.P + 4, sizeof(double) * 2);
            st = ns;
        } else {
            /* move_right, src/lsqnonneg.jl:941-946 */
            lc_state ns;
            ns.x[0] = st.x[1]; ns.x[1] = st.x[2]; ns.x[2] = st.x[1] + (st.x[3] - st.x[2]); ns.x[3] = st.x[3];
            memcpy(ns.P, st.P + 2, sizeof(double) * 2);
            memcpy(ns.P + 2, st.P + 4, sizeof(double) * 2);
            lc_eval(c, ns.x[2], ns.P + 4);
            memcpy(ns.P + 6, st.P + 6, sizeof(double) * 2);
            st = ns;
        }
        lc_update_curvature(r, &st, Ptl, Pbr, Ctol);
        sc_push(r, &st);
    }
    if (iters_out) *iters_out = iter;
    return r->pc_x[pc_argmax(r)];
}

/* f_lcurve(logμ) = (log ||Ax-b||², log ||x||²), src/lsqnonneg.jl:819-824 */
static void lcurve_point(double logmu, double *P, void *ctx) {
    reg_ws *r = (reg_ws *)ctx;
    int st = g_st; g_st = ORC_ST_REG_NNLS;
    reg_solve_tikh(r, pm_exp(logmu));
    g_st = st;
    P[0] = pm_log(tikh_res2(r));
    P[1] = pm_log(tikh_seminorm_sq(&r->tk));
}
static const double *reg_lcurve(reg_ws *r, double *mu_out, double *chi2_out, int need_chi2) {
    g_st = ORC_ST_REG_OTHER;
    lc_ctx c = {lcurve_point, r, r};
    double logmu = lcurve_corner_impl(&c, -8.0, 2.0, 1e-4, 1e-4, 1e-4, NULL);
    double mu = pm_exp(logmu);
    g_st = ORC_ST_REG_NNLS;
    reg_solve_tikh(r, mu);
    double chi2 = NAN;
    if (need_chi2) {
        reg_solve_unreg(r);
        chi2 = tikh_res2(r) / unreg_res2(r);
    }
    g_st = ORC_ST_REG_OTHER;
    *mu_out = mu;
    *chi2_out = chi2;
    return r->tk.x;
}

/* ---- GCV (src/lsqnonneg.jl:1136-1341) ---- */
static double gcv_dof(int m, int n, const double *g, double lam) {
    double dof = (double)(m - n > 0 ? m - n : 0);
    double l2 = lam * lam;
    int k = m < n ? m : n;
    for (int i = 0; i < k; ++i) { double g2 = g[i] * g[i]; dof += l2 / (g2 + l2); }
    FL(4 * k + 1);
    return dof;
}
static double gcv_logf(double logmu, void *ctx) {
    reg_ws *r = (reg_ws *)ctx;
    double mu = pm_exp(logmu);
    int st = g_st; g_st = ORC_ST_REG_NNLS;
    reg_solve_tikh(r, mu);
    g_st = st;
    double res2 = tikh_res2(r);
    double dof = gcv_dof(r->m, r->n, r->gamma, mu);
    double G = res2 / (dof * dof);
    double low = (EPS64 * EPS64) / r->m;
    FL(4);
    return pm_log(jmax(G, low));
}
static const double *reg_gcv(reg_ws *r, double *mu_out, double *chi2_out, int need_chi2) {
    g_st = ORC_ST_SVD;
    bidiag_svdvals(r->A, r->m, r->n, r->gamma, r->svdU);
    g_st = ORC_ST_REG_OTHER;
    double logmu, logG;
    brent_minimize(gcv_logf, r, -8.0, 2.0, 0.0, 1e-4, 20, &logmu, &logG);
    double mu = pm_exp(logmu);
    g_st = ORC_ST_REG_NNLS;
    reg_solve_tikh(r, mu);
    double chi2 = NAN;
    if (need_chi2) {
        reg_solve_unreg(r);
        chi2 = tikh_res2(r) / unreg_res2(r);
    }
    g_st = ORC_ST_REG_OTHER;
    *mu_out = mu;
    *chi2_out = chi2;
    return r->tk.x;
}

#define LEGACY_MAXPTS 256
/* ------------------------------------------------------------------------- */
/* Legacy algorithms (T2mapOptions.legacy = true)                             */
/*   - Julia's start:step:stop for Float64 (Base twiceprecision.jl, the       */
/*     Julia 1.9 the reference targets): a StepRangeLen with a TwicePrecision */
/*     reference and step;                                                    */
/*   - Dierckx.Spline1D(x, y; k, bc = "extrapolate", s = 0) (src/splines.jl:  */
/*     312-315), which calls netlib FITPACK: curfit/fpcurf with s = 0 (the    */
/*     interpolating spline: Givens QR of the banded B-spline collocation     */
/*     matrix, fpgivs/fprota/fpback) and splev/fpbspl (de Boor-Cox values);   */
/*   - spline_opt_legacy / spline_root_legacy (src/splines.jl:417-446):       */
/*     brute force over knots[1]:0.001:knots[end];                            */
/*   - chi2_search_from_minimum(legacy = true) (src/lsqnonneg.jl:595-636).    */
/* ------------------------------------------------------------------------- */
typedef struct { double ref_hi, ref_lo, step_hi, step_lo; long offset, len; } jl_range;

/* Base.mul12 and Base.canonicalize2 */
static void jl_mul12(double x, double y, double *h, double *l) {
    double p = x * y;
    if (p == 0 || !isfinite(p)) { *h = p; *l = p; return; }
    double e = fma(x, y, -p);
    double s = p + e;
    *h = s; *l = (p - s) + e;
}
/* TwicePrecision{Float64}((num, den)) = TwicePrecision(num) / den, for |num|, |den| < 2^53 */
static void tp_ratio(long num, long den, double *hi, double *lo) {
    double xh = (double)num, yh = (double)den;
    double h = xh / yh, uh, ul;
    jl_mul12(h, yh, &uh, &ul);
    double l = ((((xh - uh) - ul) + 0.0) - h * 0.0) / yh;
    if (xh == 0 || !isfinite(h)) { *hi = h; *lo = h; return; }
    double s = h + l;
    *hi = s; *lo = (h - s) + l;
}
static int isbetween(double a, double x, double b) { return (a <= x && x <= b) || (b <= x && x <= a); }
static long lgcd_pos(long a, long b) { a = labs(a); b = labs(b); while (b) { long t = a % b; a = b; b = t; } return a; }

/* (:)(start::Float64, step::Float64, stop::Float64) */
static void jl_colon(double start, double step, double stop, jl_range *r) {
    long step_n, step_d;
    jl_rat(step, &step_n, &step_d);
    if (step_d != 0 && (double)step_n / (double)step_d == step) {
        long start_n, start_d, stop_n, stop_d;
        jl_rat(start, &start_n, &start_d);
        jl_rat(stop, &stop_n, &stop_d);
        if (start_d != 0 && stop_d != 0 && (double)start_n / (double)start_d == start &&
            (double)stop_n / (double)stop_d == stop) {
            long g = lgcd_pos(start_d, step_d);
            long den = g == 0 ? 0 : labs(start_d / g * step_d);
            const double m = 9007199254740992.0; /* maxintfloat(Float64, Int) */
            if (den != 0 && fabs(start * (double)den) <= m && fabs(step * (double)den) <= m &&
                den % start_d == 0 && den % step_d == 0) {
                long sn = (long)rint(start * (double)den), tn = (long)rint(step * (double)den);
                long q = (den * stop_n - stop_d * sn + tn * stop_d) / (tn * stop_d); /* div truncates */
                long len = q > 0 ? q : 0;
                if (isbetween(start, start + (double)(len - 1) * step, stop + step / 2) &&
                    !isbetween(start, start + (double)len * step, stop)) {
                    /* floatrange(Float64, sn, tn, len, den) */
                    long imin, ref_n;
                    int nb;
                    if (len < 2 || tn == 0) { imin = 1; ref_n = sn; nb = 0; }
                    else {
                        double t = rint(-(double)sn / (double)tn + 1);
                        imin = t < 1 ? 1 : (t > (double)len ? len : (long)t);
                        ref_n = sn + (imin - 1) * tn;
                        nb = nbitslen((int)len, (int)imin);
                    }
                    tp_ratio(ref_n, den, &r->ref_hi, &r->ref_lo);
                    double sh, sl;
                    tp_ratio(tn, den, &sh, &sl);
                    r->step_hi = truncbits(sh, nb);
                    r->step_lo = (sh - r->step_hi) + sl;
                    r->offset = imin;
                    r->len = len;
                    return;
                }
            }
        }
    }
    /* fallback: start and step taken literally */
    double lf = (stop - start) / step;
    long len;
    if (lf < 0) len = 0;
    else if (lf == 0) len = 1;
    else {
        len = (long)rint(lf) + 1;
        double stop2 = start + (double)(len - 1) * step;
        len -= (start < stop && stop < stop2) + (start > stop && stop > stop2);
    }
    r->ref_hi = start; r->ref_lo = 0;
    r->step_hi = step; r->step_lo = 0;
    r->offset = 1;
    r->len = len;
}
/* unsafe_getindex(::StepRangeLen{Float64, TwicePrecision, TwicePrecision}, i), 1-based */
static inline double jl_range_at(const jl_range *r, long i) {
    double u = (double)(i - r->offset);
    double sh = u * r->step_hi, sl = u * r->step_lo, xh, xl;
    add12(r->ref_hi, sh, &xh, &xl);
    return xh + (xl + (sl + r->ref_lo));
}
int orc_jl_colon(double start, double step, double stop, double *out, long maxlen, long *len) {
    jl_range r;
    jl_colon(start, step, stop, &r);
    *len = r.len;
    for (long i = 1; i <= r.len && i <= maxlen; ++i) out[i - 1] = jl_range_at(&r, i);
    return 0;
}

/* FITPACK fpbspl: the k+1 non-zero B-splines of degree k at t(l) <= x < t(l+1)
 * (t and h 1-based). */
static void fp_bspl(const double *t, int k, double x, int l, double *h) {
    double hh[4];
    h[1] = 1.0;
    for (int j = 1; j <= k; ++j) {
        for (int i = 1; i <= j; ++i) hh[i] = h[i];
        h[1] = 0.0;
        for (int i = 1; i <= j; ++i) {
            int li = l + i, lj = li - j;
            if (t[li] == t[lj]) { h[i + 1] = 0.0; continue; }
            double f = hh[i] / (t[li] - t[lj]);
            h[i] = h[i] + f * (t[li] - x);
            h[i + 1] = f * (x - t[lj]);
        }
    }
}
/* FITPACK fpgivs / fprota */
static void fp_givs(double piv, double *ww, double *c, double *s) {
    double store = fabs(piv), dd;
    if (store >= *ww) { double q = *ww / piv; dd = store * sqrt(1.0 + q * q); }
    else { double q = piv / *ww; dd = *ww * sqrt(1.0 + q * q); }
    *c = *ww / dd;
    *s = piv / dd;
    *ww = dd;
}
static inline void fp_rota(double c, double s, double *a, double *b) {
    double s1 = *a, s2 = *b;
    *b = c * s2 + s * s1;
    *a = c * s1 - s * s2;
}
/* curfit(iopt = 0, s = 0, w = 1): the interpolating spline of degree k through
 * (x(i), y(i)), i = 1..m (x increasing, m > k).  Writes the n = m + k + 1 knots
 * t(1..n) and the m coefficients c(1..m) (1-based arrays of n + 1 entries);
 * a and z are workspaces of (m + 1) * (k + 2) and m + 1 entries.  Returns n. */
static int fp_curfit0(const double *x, const double *y, int m, int k, double *t, double *c, double *a, double *z) {
    const int k1 = k + 1, k2 = k1 + 1, n = m + k1, nk1 = n - k1;
    /* interior knots of the interpolating spline */
    int mk1 = m - k1;
    if (mk1 > 0) {
        int k3 = k / 2, i = k2, j = k3 + 2;
        if (k3 * 2 != k) for (int l = 1; l <= mk1; ++l, ++i, ++j) t[i] = x[j];
        else for (int l = 1; l <= mk1; ++l, ++i, ++j) t[i] = (x[j] + x[j - 1]) * 0.5;
    }
    for (int j = 1, i = n; j <= k1; ++j, --i) { t[j] = x[1]; t[i] = x[m]; }
    /* observation matrix reduced to upper triangular form by Givens rotations */
#define FA(i, j) a[(i) * (k2) + (j)]
    for (int i = 1; i <= nk1; ++i) { z[i] = 0; for (int j = 1; j <= k1; ++j) FA(i, j) = 0; }
    int l = k1;
    double h[5];
    for (int it = 1; it <= m; ++it) {
        double xi = x[it], yi = y[it];
        while (!(xi < t[l + 1] || l == nk1)) l++;
        fp_bspl(t, k, xi, l, h);
        int j = l - k1;
        for (int i = 1; i <= k1; ++i) {
            j++;
            double piv = h[i];
            if (piv == 0) continue;
            double cs, sn;
            fp_givs(piv, &FA(j, 1), &cs, &sn);
            fp_rota(cs, sn, &yi, &z[j]);
            if (i == k1) break;
            for (int i1 = i + 1, i2 = 1; i1 <= k1; ++i1) {
                i2++;
                fp_rota(cs, sn, &h[i1], &FA(j, i2));
            }
        }
    }
    /* fpback(a, z, nk1, k1, c): back substitution, bandwidth k1 */
    c[nk1] = z[nk1] / FA(nk1, 1);
    int i = nk1 - 1;
    for (int j = 2; j <= nk1 && i >= 1; ++j, --i) {
        double store = z[i];
        int i1 = (j <= k) ? j - 1 : k, mm = i;
        for (int q = 1; q <= i1; ++q) { mm++; store = store - c[mm] * FA(i, q + 1); }
        c[i] = store / FA(i, 1);
    }
#undef FA
    return n;
}
/* splev for one point, bc = "extrapolate" (e = 0) */
static double fp_splev1(const double *t, int n, const double *c, int k, double arg) {
    const int k1 = k + 1, nk1 = n - k1;
    int l = k1;
    while (!(arg < t[l + 1] || l == nk1)) l++;
    double h[5];
    fp_bspl(t, k, arg, l, h);
    double sp = 0;
    for (int j = 1, ll = l - k1; j <= k1; ++j) { ll++; sp = sp + c[ll] * h[j]; }
    return sp;
}
int orc_fitpack_curfit0(const double *x, const double *y, int m, int k, double *t, double *c) {
    if (m <= k || k < 1 || k > 3) return 1;
    double *xs = (double *)calloc((size_t)(m + 1) * 2, sizeof(double)), *ys = xs + m + 1;
    double *tt = (double *)calloc((size_t)(m + k + 2) * 2, sizeof(double)), *cc = tt + m + k + 2;
    double *a = (double *)calloc((size_t)(m + 1) * (k + 2), sizeof(double)), *z = (double *)calloc(m + 1, sizeof(double));
    for (int i = 0; i < m; ++i) { xs[i + 1] = x[i]; ys[i + 1] = y[i]; }
    int n = fp_curfit0(xs, ys, m, k, tt, cc, a, z);
    for (int i = 0; i < n; ++i) t[i] = tt[i + 1];
    for (int i = 0; i < m; ++i) c[i] = cc[i + 1];
    free(xs); free(tt); free(a); free(z);
    return 0;
}
int orc_fitpack_splev(const double *t, int n, const double *c, int k, const double *x, int npts, double *y) {
    double *tt = (double *)malloc(sizeof(double) * (n + 1) * 2), *cc = tt + n + 1;
    for (int i = 0; i < n; ++i) { tt[i + 1] = t[i]; cc[i + 1] = i < n - k - 1 ? c[i] : 0; }
    for (int i = 0; i < npts; ++i) y[i] = fp_splev1(tt, n, cc, k, x[i]);
    free(tt);
    return 0;
}

/* Shared core of spline_opt_legacy (value = NaN: minimize the spline) and
 * spline_root_legacy (minimize |spline - value|): fit with
 * deg_spline = min(3, npts - 1), then scan knots[1]:0.001:knots[end] keeping
 * the first strict minimum.  X, Y are 0-based of length npts.  */
static void spline_scan_legacy(const double *X, const double *Y, int npts, int root, double value, double *xo, double *yo) {
    int k = npts - 1 < 3 ? npts - 1 : 3;
    double xs[LEGACY_MAXPTS + 1], ys[LEGACY_MAXPTS + 1], t[LEGACY_MAXPTS + 5], c[LEGACY_MAXPTS + 5];
    double a[(LEGACY_MAXPTS + 1) * 5], z[LEGACY_MAXPTS + 1];
    for (int i = 0; i < npts; ++i) { xs[i + 1] = X[i]; ys[i + 1] = Y[i]; }
    int n = fp_curfit0(xs, ys, npts, k, t, c, a, z);
    jl_range r;
    jl_colon(t[k + 1], 0.001, t[n - k], &r);  /* get_knots: t[k+1 .. n-k] */
    double bx = jl_range_at(&r, 1), by = fp_splev1(t, n, c, k, bx);
    if (root) by = fabs(by - value);
    for (long i = 2; i <= r.len; ++i) {
        double xi = jl_range_at(&r, i), yi = fp_splev1(t, n, c, k, xi);
        if (root) yi = fabs(yi - value);
        if (yi < by) { bx = xi; by = yi; }
    }
    *xo = bx;
    *yo = by;
}
int orc_spline_opt_legacy(const double *X, const double *Y, int npts, double *x, double *y) {
    if (npts < 2 || npts > LEGACY_MAXPTS) return 1;
    spline_scan_legacy(X, Y, npts, 0, 0.0, x, y);
    return 0;
}
static void spline_root_legacy_pts(const double *X, const double *Y, int npts, double value, double *x) {
    double y;
    spline_scan_legacy(X, Y, npts, 1, value, x, &y);
}
int orc_spline_root_legacy(const double *X, const double *Y, int npts, double value, double *x) {
    if (npts < 2 || npts > LEGACY_MAXPTS) return 1;
    double y;
    spline_scan_legacy(X, Y, npts, 1, value, x, &y);
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Flip-angle search (src/splines.jl, src/T2mapSEcorr.jl:409-423)             */
/* ------------------------------------------------------------------------- */
static inline double evalpoly4(double t, const double *c) { return fma(t, fma(t, fma(t, c[3], c[2]), c[1]), c[0]); }

/* CubicHermiteInterpolator + minimize, src/splines.jl:62-110 */
static void hermite_minimize(double a, double b, double u0, double u1, double m0, double m1, double *xo, double *uo) {
    double r = (b - a) / 2;
    m0 = r * m0; m1 = r * m1;
    double du = u1 - u0, dm = m1 - m0, su = u1 + u0, sm = m1 + m0;
    double c[4] = {su / 2 - dm / 4, (3 * du - sm) / 4, dm / 4, (sm - du) / 4};
    double xend, uend;
    if (u0 < u1) { xend = a; uend = u0; } else { xend = b; uend = u1; }
    double D = 3 * (u0 - u1);
    double th = D / 2 + (m0 + m1);
    double g = th * th - m0 * m1;
    g = g > 0 ? -sqrt(g) : 0.0;
    double p = -(D + (m0 + m1));
    double q = 2 * g + (m0 - m1);
    FL(40);
    if (fabs(p) < fabs(q)) {
        double t = p / q;
        double y = evalpoly4(t, c);
        if (y < uend) {
            double cc = (a + b) / 2, rr = (b - a) / 2;
            *xo = jclamp(fma(rr, t, cc), a, b);
            *uo = y;
            return;
        }
    }
    *xo = xend; *uo = uend;
}
void orc_cubic_hermite_minimize(double a, double b, double u0, double u1, double m0, double m1, double *x, double *u) {
    hermite_minimize(a, b, u0, u1, m0, m1, x, u);
}

typedef struct {
    int K, m, n;
    const double *grid;             /* flip angles */
    const double *As, *dAs;         /* m x n x K, basis and d/dα */
    const double *b;                /* normalized decay data */
    nnls_ws *un;
    double *Axb, *dAx;              /* m */
    unsigned char seen[256];
    double u[256], du[256];
    int idx[256], npts, numeval, maxeval, mineval;
    int legacy;                     /* CubicSplineSurrogate(legacy = true): loss only, brute-force spline minimum */
    int sugg_npts;                  /* points behind the last legacy suggestion (-1: none) */
    double sugg_x, sugg_u;
} fa_search;

/* loss_with_grad!, src/splines.jl:1010-1041 */
static void fa_update(fa_search *s, int I) {
    if (s->seen[I - 1]) return; /* the surrogate's own `seen` (src/splines.jl:526-534) */
    const int m = s->m, n = s->n;
    const double *A = s->As + (size_t)(I - 1) * m * n, *dA = s->dAs + (size_t)(I - 1) * m * n;
    g_st = ORC_ST_SEARCH_NNLS;
    nnlsprob_solve(s->un, A, m, n, s->b);
    g_st = ORC_ST_SEARCH_OTHER;
    double ell = s->un->rnorm * s->un->rnorm;
    const double *x = s->un->x;
    if (s->legacy) { s->du[I - 1] = NAN; goto store; } /* loss! only, src/splines.jl:1043-1046 */
    for (int i = 0; i < m; ++i) s->Axb[i] = 0;
    for (int j = 0; j < n; ++j)
        if (x[j] > 0) { for (int i = 0; i < m; ++i) s->Axb[i] = fma(x[j], A[i + (size_t)j * m], s->Axb[i]); FL(2 * m); }
    for (int i = 0; i < m; ++i) s->Axb[i] -= s->b[i];
    for (int i = 0; i < m; ++i) s->dAx[i] = 0;
    for (int j = 0; j < n; ++j)
        if (x[j] > 0) { for (int i = 0; i < m; ++i) s->dAx[i] = fma(x[j], dA[i + (size_t)j * m], s->dAx[i]); FL(2 * m); }
    lacc Lg = {{0}};
    for (int i = 0; i < m; ++i) Lg.p[i & 31] = fma(s->dAx[i], s->Axb[i], Lg.p[i & 31]);
    double dt = lacc_tree(&Lg);
    FL(3 * m + 2);
    s->du[I - 1] = 2 * dt;
store:
    s->seen[I - 1] = 1;
    s->u[I - 1] = ell;
    /* insertsorted!(idx, I, npts += 1), src/utils.jl:42-49 */
    int len = ++s->npts, val = I;
    for (int i = 0; i < len - 1; ++i) {
        int a = s->idx[i];
        if (val < a) { s->idx[i] = val; val = a; }
    }
    s->idx[len - 1] = val;
}
/* update!(surr, state, I; maxeval), src/splines.jl:736-744 */
static int fa_state_update(fa_search *s, int I, unsigned char *sseen) {
    if (s->numeval >= s->maxeval) return 1;
    if (sseen[I - 1]) return 0;
    fa_update(s, I);
    sseen[I - 1] = 1;
    s->numeval += 1;
    return s->numeval >= s->maxeval;
}
static inline int box_evaluated(const unsigned char *sseen, int lo, int hi) { return (sseen[lo - 1] + sseen[hi - 1]) >= 2; }
/* evaluate_box!, src/splines.jl:802-815 */
static void fa_evaluate_box(fa_search *s, unsigned char *sseen, int lo, int hi, int have_x, double x) {
    int cs[2] = {lo, hi};
    if (have_x) {
        double dlo = (s->grid[lo - 1] - x) * (s->grid[lo - 1] - x);
        double dhi = (s->grid[hi - 1] - x) * (s->grid[hi - 1] - x);
        if (dhi < dlo) { cs[0] = hi; cs[1] = lo; }
    }
    for (int k = 0; k < 2; ++k) {
        if (box_evaluated(sseen, lo, hi)) break;
        if (fa_state_update(s, cs[k], sseen)) break;
    }
}
/* initialize!(surr, state, box, depth), src/splines.jl:726-734 */
static void fa_init_rec(fa_search *s, unsigned char *sseen, int lo, int hi, int depth) {
    if (depth <= 0) return;
    fa_evaluate_box(s, sseen, lo, hi, 0, 0);
    if (s->numeval >= s->mineval) return;
    int mid = (lo + hi) / 2;
    fa_init_rec(s, sseen, lo, mid, depth - 1);
    fa_init_rec(s, sseen, mid, hi, depth - 1);
}
/* suggest_point(::CubicHermiteSplineSurrogate), src/splines.jl:544-566 */
static void fa_suggest(fa_search *s, double *xo, double *uo) {
    if (s->legacy) {
        /* suggest_point(::CubicSplineSurrogate) with spline_opt_legacy, src/splines.jl:493-500,419-431.
         * The scan depends only on the evaluated points, so an unchanged set reuses it. */
        if (s->sugg_npts != s->npts) {
            double ps[256], us[256];
            for (int i = 0; i < s->npts; ++i) { ps[i] = s->grid[s->idx[i] - 1]; us[i] = s->u[s->idx[i] - 1]; }
            spline_scan_legacy(ps, us, s->npts, 0, 0.0, &s->sugg_x, &s->sugg_u);
            s->sugg_npts = s->npts;
        }
        *xo = s->sugg_x; *uo = s->sugg_u;
        return;
    }
    int I0 = s->idx[0];
    double pl = s->grid[I0 - 1], ul = s->u[I0 - 1], dl = s->du[I0 - 1];
    double p = pl, u = ul;
    for (int i = 2; i <= s->npts; ++i) {
        int I = s->idx[i - 1];
        double pc = s->grid[I - 1], uc = s->u[I - 1], dcur = s->du[I - 1];
        double xx, uu;
        hermite_minimize(pl, pc, ul, uc, dl, dcur, &xx, &uu);
        if (uu < u) { p = xx; u = uu; }
        pl = pc; ul = uc; dl = dcur;
    }
    *xo = p; *uo = u;
}
/* minimal_bounding_box, src/splines.jl:778-800 */
static void min_bbox(int K, const double *grid, const unsigned char *sseen, double x, int *plo, int *phi) {
    int lo = 1, hi = K;
    for (;;) {
        int mid = (lo + hi) / 2;
        if (grid[lo - 1] <= x && x <= grid[mid - 1]) {
            if (!box_evaluated(sseen, lo, mid) || !(abs(mid - lo) > 1)) { *plo = lo; *phi = mid; return; }
            hi = mid;
        } else {
            if (!box_evaluated(sseen, mid, hi) || !(abs(hi - mid) > 1)) { *plo = mid; *phi = hi; return; }
            lo = mid;
        }
    }
}
int orc_minimal_bounding_box(int K, const double *grid, const unsigned char *seen, double x, int *lo, int *hi) {
    min_bbox(K, grid, seen, x, lo, hi);
    return 0;
}
/* optimize_flip_angle!, src/T2mapSEcorr.jl:409-423 with bisection_search, src/splines.jl:750-775 */
static double fa_optimize(fa_search *s, int mineval, int maxeval) {
    unsigned char sseen[256];
    memset(sseen, 0, sizeof sseen);
    memset(s->seen, 0, sizeof s->seen);
    s->npts = 0; s->numeval = 0; s->mineval = mineval; s->maxeval = maxeval; s->sugg_npts = -1;
    for (int depth = 1; depth <= mineval; ++depth) {
        fa_init_rec(s, sseen, 1, s->K, depth);
        if (s->numeval >= mineval) break;
    }
    double x, u;
    fa_suggest(s, &x, &u);
    for (;;) {
        int lo, hi;
        min_bbox(s->K, s->grid, sseen, x, &lo, &hi);
        fa_evaluate_box(s, sseen, lo, hi, 1, x);
        fa_suggest(s, &x, &u);
        if (s->numeval >= maxeval || abs(hi - lo) <= 1) return x;
    }
}

/* ------------------------------------------------------------------------- */
/* Per-voxel pipeline (src/T2mapSEcorr.jl:201-238, 512-591)                  */
/* ------------------------------------------------------------------------- */
typedef struct {
    orc_t2map_opts o;
    int m, n, K, fixed_angle;
    double *t2, *logt2, *angles;
    double *As, *dAs;        /* ensemble basis, m x n x K */
    double *basis_fixed;     /* SetFlipAngle basis */
    double beta;
} t2map_plan;

typedef struct {
    double *A, *b, *fit, *res, *epgw, *zero_n;
    nnls_ws search_un;
    reg_ws reg;
    fa_search fa;
} vox_ws;

static void basis_at(const t2map_plan *p, double alpha, double *A, double *w) {
    for (int j = 0; j < p->n; ++j) {
        if (p->beta == 180) epg_flat(p->m, alpha, p->o.TE, p->t2[j], p->o.T1, A + (size_t)j * p->m, w);
        else epg_vec(p->m, alpha, p->o.TE, p->t2[j], p->o.T1, p->beta, A + (size_t)j * p->m, (v3 *)w);
    }
}

static void vox_ws_init(vox_ws *w, const t2map_plan *p) {
    int m = p->m, n = p->n;
    w->A = (double *)calloc((size_t)m * n, sizeof(double));
    w->b = (double *)calloc(m, sizeof(double));
    w->fit = (double *)calloc(m, sizeof(double));
    w->res = (double *)calloc(m, sizeof(double));
    w->epgw = (double *)calloc(6 * (size_t)m + 8, sizeof(double));
    w->zero_n = (double *)calloc(n, sizeof(double));
    nnls_ws_alloc(&w->search_un, m, n);
    reg_ws_init(&w->reg, m, n);
    w->reg.A = w->A; w->reg.b = w->b;
    memset(&w->fa, 0, sizeof(w->fa));
    w->fa.K = p->K; w->fa.m = m; w->fa.n = n;
    w->fa.grid = p->angles; w->fa.As = p->As; w->fa.dAs = p->dAs; w->fa.b = w->b;
    w->fa.un = &w->search_un;
    w->fa.legacy = p->o.legacy;
    w->fa.Axb = (double *)calloc(m, sizeof(double));
    w->fa.dAx = (double *)calloc(m, sizeof(double));
}
static void vox_ws_free(vox_ws *w) {
    free(w->A); free(w->b); free(w->fit); free(w->res); free(w->epgw); free(w->zero_n);
    nnls_ws_free(&w->search_un); reg_ws_free(&w->reg);
    free(w->fa.Axb); free(w->fa.dAx);
}

static void voxel(const t2map_plan *p, vox_ws *w, const double *image, long V, long v, const double *b1map, orc_t2map_out *out) {
    const int m = p->m, n = p->n;
    const orc_t2map_opts *o = &p->o;
    /* normalize by the maximum echo, src/T2mapSEcorr.jl:205-218 */
    double mx = 0;
    for (int i = 0; i < m; ++i) { double bi = image[v + V * i]; mx = bi > mx ? bi : mx; w->b[i] = bi; }
    if (mx > 0) for (int i = 0; i < m; ++i) w->b[i] /= mx;
    double alpha;
    if (b1map) {
        alpha = b1map[v];
        g_st = ORC_ST_BASIS;
        basis_at(p, alpha, w->A, w->epgw);
    } else if (p->fixed_angle) {
        alpha = o->SetFlipAngle;
        memcpy(w->A, p->basis_fixed, sizeof(double) * m * n);
    } else {
        alpha = fa_optimize(&w->fa, o->nRefAnglesMin, o->nRefAngles);
        g_st = ORC_ST_BASIS;
        basis_at(p, alpha, w->A, w->epgw);
    }
    /* T2_distribution!, src/T2mapSEcorr.jl:475-505 */
    double mu = NAN, chi2f = NAN;
    const double *x;
    int need_chi2 = out->chi2factor != NULL;
    switch (o->Reg) {
    case ORC_REG_NONE:
        g_st = ORC_ST_REG_NNLS;
        reg_solve_unreg(&w->reg);
        x = w->reg.un.x; mu = 0; chi2f = 1;
        break;
    case ORC_REG_LCURVE: x = reg_lcurve(&w->reg, &mu, &chi2f, need_chi2); break;
    case ORC_REG_GCV: x = reg_gcv(&w->reg, &mu, &chi2f, need_chi2); break;
    case ORC_REG_CHI2:
        x = o->legacy ? reg_chi2_legacy(&w->reg, o->Chi2Factor, &mu, &chi2f) : reg_chi2(&w->reg, o->Chi2Factor, &mu, &chi2f);
        break;
    default: {
        double sigma = o->NoiseLevel / mx;
        double delta = sqrt((double)m) * sigma;
        x = reg_mdp(&w->reg, delta, &mu, &chi2f, w->zero_n);
    }
    }
    /* save_results!, src/T2mapSEcorr.jl:512-591 */
    g_st = ORC_ST_SAVE;
    double *dist = (double *)alloca(sizeof(double) * n);
    for (int i = 0; i < m; ++i) w->b[i] *= mx;
    for (int j = 0; j < n; ++j) dist[j] = x[j] * mx;
    for (int i = 0; i < m; ++i) w->fit[i] = 0;
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < m; ++i) w->fit[i] = fma(w->A[i + (size_t)j * m], dist[j], w->fit[i]);
    for (int i = 0; i < m; ++i) w->res[i] = w->fit[i] - w->b[i];
    lacc Lsd = {{0}}, Lr2 = {{0}}, Lsr = {{0}}, Ldl = {{0}}, Lv = {{0}}, Lg = {{0}};
    for (int j = 0; j < n; ++j) Lsd.p[j & 31] = Lsd.p[j & 31] + dist[j];
    for (int i = 0; i < m; ++i) Lr2.p[i & 31] = Lr2.p[i & 31] + w->res[i] * w->res[i];
    for (int i = 0; i < m; ++i) Lsr.p[i & 31] = Lsr.p[i & 31] + w->res[i];
    for (int j = 0; j < n; ++j) Ldl.p[j & 31] = Ldl.p[j & 31] + dist[j] * p->logt2[j];
    double sd = lacc_tree(&Lsd), sr2 = lacc_tree(&Lr2), sr = lacc_tree(&Lsr), dotl = lacc_tree(&Ldl);
    double mean = sr / m;
    for (int i = 0; i < m; ++i) { double d = w->res[i] - mean; Lv.p[i & 31] = Lv.p[i & 31] + d * d; }
    double var = lacc_tree(&Lv);
    double sigres = sqrt(var / (m - 1));
    double lggm = dotl / sd;
    for (int j = 0; j < n; ++j) { double d = p->logt2[j] - lggm; Lg.p[j & 31] = Lg.p[j & 31] + (d * d) * dist[j]; }
    double lgva = lacc_tree(&Lg) / sd;
    FL(4.0 * m * n + 12.0 * m + 8.0 * n + 20);
    if (out->gdn) out->gdn[v] = sd;
    if (out->ggm) out->ggm[v] = pm_exp(lggm);
    if (out->gva) out->gva[v] = pm_expm1(lgva);
    if (out->fnr) out->fnr[v] = sd / sqrt(sr2 / (m - 1));
    if (out->snr) out->snr[v] = mx / sigres;
    if (out->alpha) out->alpha[v] = alpha;
    if (out->dist) for (int j = 0; j < n; ++j) out->dist[v + V * j] = dist[j];
    if (out->mu) out->mu[v] = mu;
    if (out->chi2factor) out->chi2factor[v] = chi2f;
    if (out->resnorm) out->resnorm[v] = sqrt(sr2);
    if (out->decaycurve) for (int i = 0; i < m; ++i) out->decaycurve[v + V * i] = w->fit[i];
}

typedef struct {
    const t2map_plan *p;
    const double *image, *b1map;
    long V, nidx;
    const long *vidx;
    orc_t2map_out *out;
    atomic_long next;
    double flops[ORC_NSTAGES];
    pthread_mutex_t mu;
} t2map_job;

static void *t2map_worker(void *arg) {
    t2map_job *J = (t2map_job *)arg;
    vox_ws w;
    vox_ws_init(&w, J->p);
    memset(g_fl, 0, sizeof g_fl);
    for (;;) {
        long c = atomic_fetch_add(&J->next, 64);
        if (c >= J->nidx) break;
        long e = c + 64 < J->nidx ? c + 64 : J->nidx;
        for (long k = c; k < e; ++k) voxel(J->p, &w, J->image, J->V, J->vidx[k], J->b1map, J->out);
    }
    pthread_mutex_lock(&J->mu);
    for (int s = 0; s < ORC_NSTAGES; ++s) J->flops[s] += g_fl[s];
    pthread_mutex_unlock(&J->mu);
    vox_ws_free(&w);
    return NULL;
}

/* T2mapSEcorr(image, opts) with the outputs preallocated by the caller
 * (NaN-filled as T2Maps/T2Distributions do), src/T2mapSEcorr.jl:151-196. */
int orc_t2map(const orc_t2map_opts *o, const double *image, long V, const double *b1map, orc_t2map_out *out, int nthreads,
              double *flops) {
    t2map_plan p;
    memset(&p, 0, sizeof p);
    p.o = *o;
    p.m = o->nTE; p.n = o->nT2;
    p.fixed_angle = !isnan(o->SetFlipAngle);
    p.K = p.fixed_angle ? 1 : o->nRefAngles;
    p.beta = o->RefConAngle;
    if (p.K > 256) return -1;
    p.t2 = (double *)malloc(sizeof(double) * p.n);
    p.logt2 = (double *)malloc(sizeof(double) * p.n);
    p.angles = (double *)malloc(sizeof(double) * p.K);
    orc_logrange(o->T2Range[0], o->T2Range[1], p.n, p.t2);
    for (int j = 0; j < p.n; ++j) p.logt2[j] = log(p.t2[j]);
    double *wk = (double *)malloc(sizeof(dual) * 6 * (size_t)p.m + 64);
    memset(g_fl, 0, sizeof g_fl);
    g_st = ORC_ST_ENSEMBLE;
    if (p.fixed_angle) {
        p.angles[0] = o->SetFlipAngle;
        p.basis_fixed = (double *)malloc(sizeof(double) * p.m * p.n);
        basis_at(&p, o->SetFlipAngle, p.basis_fixed, wk);
    } else {
        orc_linrange(o->MinRefAngle, 180.0, p.K, p.angles);
        p.As = (double *)malloc(sizeof(double) * (size_t)p.m * p.n * p.K);
        p.dAs = (double *)malloc(sizeof(double) * (size_t)p.m * p.n * p.K);
        for (int k = 0; k < p.K; ++k)
            for (int j = 0; j < p.n; ++j) {
                double *Av = p.As + ((size_t)k * p.n + j) * p.m, *dAv = p.dAs + ((size_t)k * p.n + j) * p.m;
                if (p.beta == 180) epg_flat_dual(p.m, p.angles[k], o->TE, p.t2[j], o->T1, Av, dAv, (dual *)wk);
                else epg_vec_dual(p.m, p.angles[k], o->TE, p.t2[j], o->T1, p.beta, Av, dAv, (dv3 *)wk);
            }
    }
    double ens_fl = g_fl[ORC_ST_ENSEMBLE];
    free(wk);
    /* threshold filter, src/T2mapSEcorr.jl:177 */
    long *vidx = (long *)malloc(sizeof(long) * (V > 0 ? V : 1));
    long nidx = 0;
    for (long v = 0; v < V; ++v) if (image[v] > o->Threshold) vidx[nidx++] = v;
    t2map_job J;
    J.p = &p; J.image = image; J.b1map = b1map; J.V = V; J.nidx = nidx; J.vidx = vidx; J.out = out;
    atomic_init(&J.next, 0);
    memset(J.flops, 0, sizeof J.flops);
    pthread_mutex_init(&J.mu, NULL);
    if (nthreads < 1) nthreads = 1;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nthreads);
    for (int t = 0; t < nthreads; ++t) pthread_create(&th[t], NULL, t2map_worker, &J);
    for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
    free(th);
    pthread_mutex_destroy(&J.mu);
    if (flops) {
        for (int s = 0; s < ORC_NSTAGES; ++s) flops[s] = J.flops[s];
        flops[ORC_ST_ENSEMBLE] += ens_fl;
    }
    free(vidx); free(p.t2); free(p.logt2); free(p.angles); free(p.As); free(p.dAs); free(p.basis_fixed);
    return 0;
}

/* ------------------------------------------------------------------------- */
/* T2partSEcorr (src/T2partSEcorr.jl:42-164)                                  */
/* ------------------------------------------------------------------------- */
int orc_t2part(const orc_t2part_opts *o, const double *dist, long V, orc_t2part_out *out, int nthreads) {
    (void)nthreads;
    const int n = o->nT2;
    double *t2 = (double *)malloc(sizeof(double) * n), *lt2 = (double *)malloc(sizeof(double) * n);
    double *wts = NULL;
    orc_logrange(o->T2Range[0], o->T2Range[1], n, t2);
    for (int j = 0; j < n; ++j) lt2[j] = log(t2[j]);
    int sp0 = -1, sp1 = -2, mp0 = -1, mp1 = -2;
    for (int j = 0; j < n; ++j) if (t2[j] >= o->SPWin[0]) { sp0 = j; break; }
    for (int j = n - 1; j >= 0; --j) if (t2[j] <= o->SPWin[1]) { sp1 = j; break; }
    for (int j = 0; j < n; ++j) if (t2[j] >= o->MPWin[0]) { mp0 = j; break; }
    for (int j = n - 1; j >= 0; --j) if (t2[j] <= o->MPWin[1]) { mp1 = j; break; }
    if (sp0 < 0 || sp1 < 0 || mp0 < 0 || mp1 < 0) { free(t2); free(lt2); return -1; } /* Julia: findfirst -> nothing */
    if (!isnan(o->Sigmoid)) {
        wts = (double *)malloc(sizeof(double) * n);
        double k = 0.1, sigma = fabs(o->Sigmoid / (sqrt(2.0) * orc_erfinv(2 * k - 1)));
        for (int j = 0; j < n; ++j) {
            double x = (t2[j] - o->SPWin[1]) / sigma;
            double wv = erfc(x / sqrt(2.0)) / 2;
            wts[j] = wv <= EPS64 ? 0.0 : wv;
        }
    }
    g_st = ORC_ST_T2PART;
    for (long v = 0; v < V; ++v) {
        int hasnan = 0;
        for (int j = 0; j < n; ++j) if (isnan(dist[v + V * j])) { hasnan = 1; break; }
        if (hasnan) continue;
        double sd = 0, ssp = 0, smp = 0, dsp = 0, dmp = 0;
        for (int j = 0; j < n; ++j) sd += dist[v + V * j];
        for (int j = sp0; j <= sp1; ++j) { double d = dist[v + V * j]; dsp += d * lt2[j]; ssp += d; }
        for (int j = mp0; j <= mp1; ++j) { double d = dist[v + V * j]; dmp += d * lt2[j]; smp += d; }
        if (sd > 0) {
            if (wts) {
                double dw = 0;
                for (int j = 0; j < n; ++j) dw += dist[v + V * j] * wts[j];
                out->sfr[v] = dw / sd;
            } else {
                out->sfr[v] = ssp / sd;
            }
            out->mfr[v] = smp / sd;
        }
        if (ssp > 0) out->sgm[v] = pm_exp(dsp / ssp);
        if (smp > 0) out->mgm[v] = pm_exp(dmp / smp);
        FL(4.0 * n + 8);
    }
    free(t2); free(lt2); free(wts);
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Component entry points for the tests                                       */
/* ------------------------------------------------------------------------- */
int orc_nnls(const double *A, int m, int n, const double *b, double *x, double *rnorm, int *nsetp, int *mode) {
    nnls_ws ws;
    nnls_ws_alloc(&ws, m, n);
    memcpy(ws.A, A, sizeof(double) * m * n);
    memcpy(ws.b, b, sizeof(double) * m);
    for (int j = 0; j < n; ++j) { ws.x[j] = 0; ws.idx[j] = j + 1; ws.invidx[j] = j + 1; }
    nnls_unsafe(&ws, 1, 3 * n);
    memcpy(x, ws.x, sizeof(double) * n);
    *rnorm = ws.rnorm; *nsetp = ws.nsetp; *mode = ws.mode;
    nnls_ws_free(&ws);
    return 0;
}
int orc_lsqnonneg(const double *A, int m, int n, const double *b, double *x, double *rnorm, int *nsetp) {
    nnls_ws ws;
    nnls_ws_alloc(&ws, m, n);
    nnlsprob_solve(&ws, A, m, n, b);
    memcpy(x, ws.x, sizeof(double) * n);
    *rnorm = ws.rnorm; *nsetp = ws.nsetp;
    nnls_ws_free(&ws);
    return 0;
}
int orc_lsqnonneg_tikh(const double *A, int m, int n, const double *b, double mu, double *x, double *loss, double *ssq,
                       double *rsq, int *nsetp) {
    nnls_ws ws;
    nnls_ws_alloc(&ws, m + n, n);
    nnlsprob_solve_tikh(&ws, A, m, n, b, mu);
    memcpy(x, ws.x, sizeof(double) * n);
    *loss = tikh_loss(&ws);
    *ssq = tikh_seminorm_sq(&ws);
    *rsq = tikh_resnorm_sq(&ws, mu);
    *nsetp = ws.nsetp;
    nnls_ws_free(&ws);
    return 0;
}
#define REG_ENTRY(body)                                          \
    reg_ws r;                                                    \
    reg_ws_init(&r, m, n);                                       \
    r.A = A; r.b = b;                                            \
    double *zero_n = (double *)calloc(n, sizeof(double));        \
    const double *xs = body;                                     \
    memcpy(x, xs, sizeof(double) * n);                           \
    free(zero_n);                                                \
    reg_ws_free(&r);                                             \
    return 0;
int orc_lsqnonneg_chi2(const double *A, int m, int n, const double *b, double chi2_target, double *x, double *mu, double *chi2) {
    REG_ENTRY(reg_chi2(&r, chi2_target, mu, chi2))
}
int orc_lsqnonneg_chi2_legacy(const double *A, int m, int n, const double *b, double chi2_target, double *x, double *mu, double *chi2) {
    REG_ENTRY(reg_chi2_legacy(&r, chi2_target, mu, chi2))
}
int orc_lsqnonneg_mdp(const double *A, int m, int n, const double *b, double delta, double *x, double *mu, double *chi2) {
    REG_ENTRY(reg_mdp(&r, delta, mu, chi2, zero_n))
}
int orc_lsqnonneg_lcurve(const double *A, int m, int n, const double *b, double *x, double *mu, double *chi2) {
    REG_ENTRY(reg_lcurve(&r, mu, chi2, 1))
}
int orc_lsqnonneg_gcv(const double *A, int m, int n, const double *b, double *x, double *mu, double *chi2) {
    REG_ENTRY(reg_gcv(&r, mu, chi2, 1))
}
double orc_lcurve_corner(orc_fn2 f, void *ctx, double xlow, double xhigh, double xtol, double Ptol, double Ctol) {
    reg_ws r;
    memset(&r, 0, sizeof r);
    r.fc_cap = r.pc_cap = r.sc_cap = 64;
    r.fc_x = (double *)malloc(sizeof(double) * 64); r.fc_P = (double *)malloc(sizeof(double) * 128);
    r.pc_x = (double *)malloc(sizeof(double) * 64); r.pc_P = (double *)malloc(sizeof(double) * 128);
    r.pc_C = (double *)malloc(sizeof(double) * 64);
    r.sc_x = (double *)malloc(sizeof(double) * 256); r.sc_P = (double *)malloc(sizeof(double) * 512);
    lc_ctx c = {f, ctx, &r};
    double x = lcurve_corner_impl(&c, xlow, xhigh, xtol, Ptol, Ctol, NULL);
    free(r.fc_x); free(r.fc_P); free(r.pc_x); free(r.pc_P); free(r.pc_C); free(r.sc_x); free(r.sc_P);
    return x;
}


/* ==========================================================================
 * Synthetic multi-echo image (test and benchmark input, not part of the
 * reference path): per voxel three constant-flip EPG decays (myelin,
 * intra/extracellular, CSF) at one refocusing angle, mixed, scaled and given
 * Rician noise.  The reference's own generator (mock_image,
 * src/utils.jl:606-668) draws bi-exponential decays; this one is the
 * generator of the benchmark configurations and produces exactly the bytes
 * of libdecaes_gpu's decaes_mock_image, so the CPU baseline can make its
 * input without loading the GPU library.  Counter-based: voxel v draws from
 * a xoshiro256** stream seeded by splitmix64 from (seed, v), so any slab of
 * the volume can be generated on its own and thread count does not matter.
 * ========================================================================== */
typedef struct { uint64_t s[4]; } orc_rng;
static uint64_t orc_splitmix(uint64_t *x) {
    uint64_t z = (*x += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
static void orc_rng_init(orc_rng *g, uint64_t seed, uint64_t stream) {
    uint64_t x = seed ^ (stream * 0xd1b54a32d192ed03ull);
    for (int i = 0; i < 4; ++i) g->s[i] = orc_splitmix(&x);
}
static uint64_t orc_rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
static uint64_t orc_rng_next(orc_rng *g) {
    uint64_t *s = g->s;
    uint64_t r = orc_rotl(s[1] * 5, 7) * 9, t = s[1] << 17;
    s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3]; s[2] ^= t; s[3] = orc_rotl(s[3], 45);
    return r;
}
static double orc_unif(orc_rng *g) { return (double)(orc_rng_next(g) >> 11) * 0x1.0p-53; }
static double orc_unif_in(orc_rng *g, const double *r) { return r[0] + (r[1] - r[0]) * orc_unif(g); }
static double orc_normal(orc_rng *g) { /* Box-Muller */
    double u1 = orc_unif(g), u2 = orc_unif(g);
    if (u1 < 1e-300) u1 = 1e-300;
    return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

typedef struct {
    const orc_mock_opts *o;
    uint64_t seed;
    long V, v0, v1;
    void *image;
    int f32;
} mock_job;

static void *mock_worker(void *arg) {
    const mock_job *J = (const mock_job *)arg;
    const orc_mock_opts *o = J->o;
    const int m = o->nTE;
    double *d1 = (double *)malloc(sizeof(double) * 3 * (size_t)m), *d2 = d1 + m, *d3 = d2 + m;
    for (long v = J->v0; v < J->v1; ++v) {
        orc_rng g;
        orc_rng_init(&g, J->seed, (uint64_t)v);
        double alpha = orc_unif_in(&g, o->FlipAngleRange);
        double wmy = orc_unif_in(&g, o->MyelinFracRange), t2my = orc_unif_in(&g, o->MyelinT2Range);
        double t2ie = orc_unif_in(&g, o->IET2Range);
        double wcsf = orc_unif_in(&g, o->CSFFracRange), t2csf = orc_unif_in(&g, o->CSFT2Range);
        double amp = orc_unif_in(&g, o->AmplitudeRange), snr = orc_unif_in(&g, o->SNRRange);
        int bg = orc_unif(&g) < o->BackgroundFraction;
        double wie = 1.0 - wmy - wcsf;
        orc_epg_decay_curve(m, alpha, o->TE, t2my, o->T1, 180.0, d1);
        orc_epg_decay_curve(m, alpha, o->TE, t2ie, o->T1, 180.0, d2);
        orc_epg_decay_curve(m, alpha, o->TE, t2csf, o->T1, 180.0, d3);
        double sigma = bg ? o->BackgroundSigma : amp / snr;
        for (int e = 0; e < m; ++e) {
            double sig = bg ? 0.0 : amp * (wmy * d1[e] + wie * d2[e] + wcsf * d3[e]);
            double zr = orc_normal(&g), zi = orc_normal(&g);
            double val = sqrt((sig + sigma * zr) * (sig + sigma * zr) + (sigma * zi) * (sigma * zi));
            if (J->f32) ((float *)J->image)[v + J->V * e] = (float)val;
            else ((double *)J->image)[v + J->V * e] = val;
        }
    }
    free(d1);
    return NULL;
}

int orc_mock_image(const orc_mock_opts *o, uint64_t seed, long V, void *image, int f32, int nthreads) {
    if (!o || !image || V <= 0 || o->nTE < 1) return 1;
    if (nthreads < 1) nthreads = 1;
    mock_job *jobs = (mock_job *)malloc(sizeof(mock_job) * nthreads);
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nthreads);
    long chunk = (V + nthreads - 1) / nthreads;
    int nt = 0;
    for (int t = 0; t < nthreads; ++t) {
        long a = t * chunk, b = a + chunk < V ? a + chunk : V;
        if (a >= b) break;
        mock_job J = {o, seed, V, a, b, image, f32};
        jobs[nt] = J;
        pthread_create(&th[nt], NULL, mock_worker, &jobs[nt]);
        ++nt;
    }
    for (int t = 0; t < nt; ++t) pthread_join(th[t], NULL);
    free(jobs);
    free(th);
    return 0;
}
