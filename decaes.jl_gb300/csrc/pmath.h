// pmath.h -- portable exp / expm1 / log / sin / cos, host + device.
//
// The voxel pipeline makes discrete decisions (L-curve curvature comparisons,
// spline minima, root-finder branches) that amplify last-bit differences.  To
// make the GPU path reproduce the CPU oracle bit for bit, every
// transcendental that feeds a decision is evaluated with these functions,
// which use only IEEE-exact operations (+ - * / fma, bit manipulation) and
// so give identical results on x86, Arm and sm_103a.
//
// Methods (standard, from the mathematics):
//   exp:   Cody-Waite reduction x = k ln2 + r (ln2 split in two words,
//          fma-applied), |r| <= ln2/2, degree-13 Taylor polynomial, 2^k by
//          exponent construction.
//   expm1: Taylor series (degree 16) for |x| < 0.35, exp(x) - 1 otherwise.
//   log:   x = 2^e f with f in [sqrt(2)/2, sqrt(2)), log f = 2 atanh(s),
//          s = (f-1)/(f+1), odd series to s^23, plus e ln2 in two words.
//   sin/cos: reduction by pi/2 in three words (fma), Taylor polynomials of
//          degree 17 / 18 on |r| <= pi/4, quadrant selection.
// Accuracy is within a few ulps of the correctly rounded result on the
// argument ranges used here (checked against libm in the tests).
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define PM_FN __host__ __device__ __forceinline__
#else
#define PM_FN static inline
#endif

#if defined(__CUDA_ARCH__)
#define PM_BITS(d) ((uint64_t)__double_as_longlong(d))
#define PM_DBL(u) __longlong_as_double((long long)(u))
#else
#include <math.h>
#include <string.h>
PM_FN uint64_t pm_bits_(double d) { uint64_t u; memcpy(&u, &d, 8); return u; }
PM_FN double pm_dbl_(uint64_t u) { double d; memcpy(&d, &u, 8); return d; }
#define PM_BITS(d) pm_bits_(d)
#define PM_DBL(u) pm_dbl_(u)
#endif

#define PM_LN2_HI 0.6931471805599453
#define PM_LN2_LO 2.3190468138462996e-17
#define PM_INV_LN2 1.4426950408889634
#define PM_PIO2_1 1.5707963267948966
#define PM_PIO2_2 6.123233995736766e-17
#define PM_PIO2_3 -1.4973849048591698e-33
#define PM_2_OVER_PI 0.6366197723675814
#define PM_SQRT2 1.4142135623730951

PM_FN double pm_pow2i(int k) { return PM_DBL((uint64_t)(k + 1023) << 52); }  // -1022 <= k <= 1023

// The argument tests below compare bit patterns (integer operations, exact):
// on the GPU they keep the FP64 pipe, the kernels' bottleneck, for arithmetic.
#define PM_ABS_BITS 0x7fffffffffffffffULL
#define PM_INF_BITS 0x7ff0000000000000ULL

PM_FN double pm_exp(double x) {
    const uint64_t ub = PM_BITS(x);
    if ((ub & PM_ABS_BITS) > PM_INF_BITS) return x;                           // NaN
    if (!(ub >> 63) && ub > 0x40862e42fefa39efULL) return 1.0 / 0.0;         // x > 709.782712893384
    if ((ub >> 63) && (ub & PM_ABS_BITS) > 0x40874910d52d3052ULL) return 0.0;  // x < -745.1332191019412
    double kd = rint(x * PM_INV_LN2);
    int k = (int)kd;
    double r = fma(-kd, PM_LN2_HI, x);
    r = fma(-kd, PM_LN2_LO, r);
    double p = 1.6059043836821613e-10;
    p = fma(p, r, 2.08767569878681e-09);
    p = fma(p, r, 2.505210838544172e-08);
    p = fma(p, r, 2.755731922398589e-07);
    p = fma(p, r, 2.7557319223985893e-06);
    p = fma(p, r, 2.48015873015873e-05);
    p = fma(p, r, 0.0001984126984126984);
    p = fma(p, r, 0.001388888888888889);
    p = fma(p, r, 0.008333333333333333);
    p = fma(p, r, 0.041666666666666664);
    p = fma(p, r, 0.16666666666666666);
    p = fma(p, r, 0.5);
    p = fma(p, r, 1.0);
    p = fma(p, r, 1.0);
    if (k > 1023) return (p * 2.0) * pm_pow2i(k - 1);
    if (k < -1022) return (p * pm_pow2i(k + 600)) * pm_pow2i(-600);
    return p * pm_pow2i(k);
}

PM_FN double pm_expm1(double x) {
    if (x != x) return x;
    if (x > -0.35 && x < 0.35) {
        double p = 4.779477332387385e-14;
        p = fma(p, x, 7.647163731819816e-13);
        p = fma(p, x, 1.1470745597729725e-11);
        p = fma(p, x, 1.6059043836821613e-10);
        p = fma(p, x, 2.08767569878681e-09);
        p = fma(p, x, 2.505210838544172e-08);
        p = fma(p, x, 2.755731922398589e-07);
        p = fma(p, x, 2.7557319223985893e-06);
        p = fma(p, x, 2.48015873015873e-05);
        p = fma(p, x, 0.0001984126984126984);
        p = fma(p, x, 0.001388888888888889);
        p = fma(p, x, 0.008333333333333333);
        p = fma(p, x, 0.041666666666666664);
        p = fma(p, x, 0.16666666666666666);
        p = fma(p, x, 0.5);
        return fma(p * x, x, x);
    }
    return pm_exp(x) - 1.0;
}

PM_FN double pm_log(double x) {
    uint64_t u = PM_BITS(x);
    if ((u & PM_ABS_BITS) > PM_INF_BITS) return x;  // NaN
    if ((u & PM_ABS_BITS) == 0) return -1.0 / 0.0;  // +-0
    if (u >> 63) return 0.0 / 0.0;                  // x < 0
    if (u == PM_INF_BITS) return x;                 // +Inf
    int e = (int)((u >> 52) & 0x7ff);
    if (e == 0) {  // subnormal: scale by 2^54
        x = x * 18014398509481984.0;
        u = PM_BITS(x);
        e = (int)((u >> 52) & 0x7ff) - 54;
    }
    e -= 1023;
    double f = PM_DBL((u & 0x000fffffffffffffULL) | 0x3ff0000000000000ULL);
    if (PM_BITS(f) > 0x3ff6a09e667f3bcdULL) {  // f > sqrt(2), f in [1, 2)
        f = f * 0.5;
        e += 1;
    }
    double s = (f - 1.0) / (f + 1.0);
    double z = s * s;
    double p = 0.043478260869565216;
    p = fma(p, z, 0.047619047619047616);
    p = fma(p, z, 0.05263157894736842);
    p = fma(p, z, 0.058823529411764705);
    p = fma(p, z, 0.06666666666666667);
    p = fma(p, z, 0.07692307692307693);
    p = fma(p, z, 0.09090909090909091);
    p = fma(p, z, 0.1111111111111111);
    p = fma(p, z, 0.14285714285714285);
    p = fma(p, z, 0.2);
    p = fma(p, z, 0.3333333333333333);
    double t = 2.0 * s;
    double lf = fma(t * z, p, t);
    double ed = (double)e;
    return fma(ed, PM_LN2_HI, fma(ed, PM_LN2_LO, lf));
}

PM_FN void pm_sincos(double x, double *sp, double *cp) {
    if (x != x || x == 1.0 / 0.0 || x == -1.0 / 0.0) { *sp = *cp = 0.0 / 0.0; return; }
    double qd = rint(x * PM_2_OVER_PI);
    int q = (int)qd;
    double r = fma(-qd, PM_PIO2_1, x);
    r = fma(-qd, PM_PIO2_2, r);
    r = fma(-qd, PM_PIO2_3, r);
    double z = r * r;
    double ps = 2.8114572543455206e-15;
    ps = fma(ps, z, -7.647163731819816e-13);
    ps = fma(ps, z, 1.6059043836821613e-10);
    ps = fma(ps, z, -2.505210838544172e-08);
    ps = fma(ps, z, 2.7557319223985893e-06);
    ps = fma(ps, z, -0.0001984126984126984);
    ps = fma(ps, z, 0.008333333333333333);
    ps = fma(ps, z, -0.16666666666666666);
    double sr = fma(r * z, ps, r);
    double pc = -1.5619206968586225e-16;
    pc = fma(pc, z, 4.779477332387385e-14);
    pc = fma(pc, z, -1.1470745597729725e-11);
    pc = fma(pc, z, 2.08767569878681e-09);
    pc = fma(pc, z, -2.755731922398589e-07);
    pc = fma(pc, z, 2.48015873015873e-05);
    pc = fma(pc, z, -0.001388888888888889);
    pc = fma(pc, z, 0.041666666666666664);
    pc = fma(pc, z, -0.5);
    double cr = fma(z, pc, 1.0);
    switch (q & 3) {
    case 0: *sp = sr; *cp = cr; break;
    case 1: *sp = cr; *cp = -sr; break;
    case 2: *sp = -sr; *cp = -cr; break;
    default: *sp = -cr; *cp = sr; break;
    }
}
PM_FN double pm_sin(double x) { double s, c; pm_sincos(x, &s, &c); return s; }
PM_FN double pm_cos(double x) { double s, c; pm_sincos(x, &s, &c); return c; }
