// epg.cuh -- stimulated-echo EPG decay curves, host + device.
//
// Restates the reference's default kernels (src/EPGdecaycurve.jl):
//   * EPGWork_ReIm_DualFlat_Split_Dynamic for EPGConstantFlipAngleOptions
//     (refocusing control angle 180), lines 936-1028;
//   * EPGWork_ReIm_DualVector_Split_Dynamic for EPGOptions (control angle
//     beta != 180), lines 722-818.
// The reference ping-pongs two state buffers; here each step updates one
// buffer in place, walking states in ascending order and holding the one
// not-yet-consumed old value in a register.  Every state a step reads is the
// previous step's value in both forms, so the curves are the same bits.
//
// State storage is strided so a warp can keep one curve per lane in shared
// memory with lane-contiguous layout: F(k) = S[(k-1)*st], Fbar(k) =
// S[(ETL+k-1)*st], Z(k) = S[(2*ETL+k-1)*st].
#pragma once
#include <cmath>

#include "pmath.h"

#ifdef __CUDACC__
#define DX_HD __host__ __device__ __forceinline__
#else
#define DX_HD inline
#endif

namespace dx {

#ifndef __CUDA_ARCH__
using std::cos;
using std::exp;
using std::fabs;
using std::fma;
using std::fmod;
using std::isinf;
using std::isnan;
using std::signbit;
using std::sin;
#endif

// deg2rad factor Float64(pi)/180 and the low word of pi/180 (double-double)
constexpr double kD2R = 0.017453292519943295;
constexpr double kD2RLo = 2.9486522708701687e-19;

DX_HD double fmad(double a, double b, double c) { return fma(a, b, c); }

// Dual number (value, d/dalpha) with ForwardDiff's primal arithmetic: the
// value part is bitwise the plain evaluation.
struct Dual {
    double v, d;
};
DX_HD Dual mkd(double v, double d = 0.0) { return Dual{v, d}; }
DX_HD Dual operator+(Dual a, Dual b) { return Dual{a.v + b.v, a.d + b.d}; }
DX_HD Dual operator-(Dual a, Dual b) { return Dual{a.v - b.v, a.d - b.d}; }
DX_HD Dual operator-(Dual a) { return Dual{-a.v, -a.d}; }
DX_HD Dual operator*(Dual a, Dual b) { return Dual{a.v * b.v, a.d * b.v + b.d * a.v}; }
DX_HD Dual operator*(Dual a, double s) { return Dual{a.v * s, a.d * s}; }
DX_HD Dual operator/(Dual a, double s) { return Dual{a.v / s, a.d / s}; }
DX_HD Dual fmad(Dual a, Dual b, Dual c) { return Dual{fma(a.v, b.v, c.v), (a.d * b.v + b.d * a.v) + c.d}; }
DX_HD Dual absd(Dual a) { return signbit(a.v) ? -a : a; }
DX_HD double absd(double a) { return fabs(a); }
DX_HD double zero_of(double) { return 0.0; }
DX_HD Dual zero_of(Dual) { return Dual{0.0, 0.0}; }
// single-precision recursion of the mixed method
DX_HD float fmad(float a, float b, float c) { return fmaf(a, b, c); }
DX_HD float absd(float a) { return fabsf(a); }
DX_HD float zero_of(float) { return 0.0f; }

// sind: the degree reduction of Base.sind with a double-double radian
// argument (sin(h + l) = sin h + l cos h to first order).
DX_HD double sin_dd(double y) {
    double h = y * kD2R, l = fma(y, kD2R, -h) + y * kD2RLo, sh, ch;
    pm_sincos(h, &sh, &ch);
    return sh + l * ch;
}
DX_HD double cos_dd(double y) {
    double h = y * kD2R, l = fma(y, kD2R, -h) + y * kD2RLo, sh, ch;
    pm_sincos(h, &sh, &ch);
    return ch - l * sh;
}
DX_HD double sgn(double x) { return x < 0 ? -1.0 : (x > 0 ? 1.0 : x); }
DX_HD double sind(double x) {
    if (isnan(x) || isinf(x)) return NAN;
    double rx = copysign(fmod(x, 360.0), x), arx = fabs(rx);
    if (rx == 0) return rx;
    if (arx < 45) return sin_dd(rx);
    if (arx <= 135) return copysign(cos_dd(90 - arx), rx);
    if (arx == 180) return copysign(0.0, rx);
    if (arx < 225) return sin_dd((180 - arx) * sgn(rx));
    if (arx <= 315) return -copysign(cos_dd(270 - arx), rx);
    return sin_dd(rx - copysign(360.0, rx));
}

// Coefficients of the constant-flip recursion, src/EPGdecaycurve.jl:955-962.
template <class T>
struct FlatCoef {
    T a, b, c, d, cp, m0;
};
DX_HD FlatCoef<double> flat_coef(double alpha_deg, double TE, double T2, double T1) {
    double al = alpha_deg * kD2R;
    double E1 = pm_exp(-(TE / 2) / T1), E2 = pm_exp(-(TE / 2) / T2);
    double sa, ca;
    pm_sincos(al, &sa, &ca);
    double E22h = (E2 * E2) / 2, E1E2 = E1 * E2, E11 = E1 * E1;
    FlatCoef<double> k;
    k.a = E22h;
    k.b = E22h * ca;
    k.c = E1E2 * sa;
    k.d = E11 * ca;
    k.cp = -k.c / 2;
    k.m0 = sind(alpha_deg / 2);
    return k;
}
DX_HD FlatCoef<Dual> flat_coef_dual(double alpha_deg, double TE, double T2, double T1) {
    Dual al{alpha_deg * kD2R, kD2R};
    double E1 = pm_exp(-(TE / 2) / T1), E2 = pm_exp(-(TE / 2) / T2);
    double s, co;
    pm_sincos(al.v, &s, &co);
    Dual sa{s, co * al.d}, ca{co, -s * al.d};
    double E22h = (E2 * E2) / 2, E1E2 = E1 * E2, E11 = E1 * E1;
    FlatCoef<Dual> k;
    k.a = mkd(E22h);
    k.b = ca * E22h;
    k.c = sa * E1E2;
    k.d = ca * E11;
    k.cp = (-k.c) / 2;
    k.m0 = Dual{sind(alpha_deg / 2), kD2R * pm_cos((alpha_deg / 2) * kD2R) * 0.5};
    return k;
}

// Coefficients rounded to single precision (mixed method; the coefficients
// themselves are evaluated in FP64).
DX_HD FlatCoef<float> to_f32(const FlatCoef<double> &k) {
    return FlatCoef<float>{(float)k.a, (float)k.b, (float)k.c, (float)k.d, (float)k.cp, (float)k.m0};
}

// One state of the constant-flip step: outputs (F of state k+1, Fbar of
// state k-1, Z of state k) from (F, Fbar, Z) of state k.
template <class T>
DX_HD void flat_state(const FlatCoef<T> &q, T F, T Fb, T Z, T &oF, T &oFb, T &oZ) {
    T C = F + Fb, S = F - Fb, Cp = q.a * C, Sp = q.b * S;
    oF = fmad(q.c, Z, Cp + Sp);
    oFb = fmad(-q.c, Z, Cp - Sp);
    oZ = fmad(q.cp, S, q.d * Z);
}

// epg_decay_curve! for the constant-flip kernel: impulse response, then
// dc[i] = |m0 * dc[i]|.  S holds 3*ETL strided values (st apart).
template <class T, class O>
DX_HD void epg_flat_inplace(int ETL, const FlatCoef<T> &q, T *S, int st, O *dc, int dst) {
#define EF(k) S[((k)-1) * st]
#define EFb(k) S[(ETL + (k)-1) * st]
#define EZ(k) S[(2 * ETL + (k)-1) * st]
    const T z0 = zero_of(q.a);
    dc[0] = q.a - q.b;
    EF(1) = q.a - q.b; EFb(1) = z0; EZ(1) = q.cp;
    EF(2) = q.a + q.b; EFb(2) = z0; EZ(2) = z0;
    for (int i = 2; i <= ETL - 1; ++i) {
        const int kend = (i <= ETL / 2) ? i : ETL - i + 1;
        T Fo = EF(1);
        for (int k = 1; k <= kend; ++k) {
            T Fk = Fo, Fbk = EFb(k), Zk = EZ(k);
            Fo = EF(k + 1);
            T oF, oFb, oZ;
            flat_state(q, Fk, Fbk, Zk, oF, oFb, oZ);
            if (k == 1) {
                EF(1) = oFb;
                dc[(i - 1) * dst] = oFb;
            } else {
                EFb(k - 1) = oFb;
            }
            EF(k + 1) = oF;
            EZ(k) = oZ;
        }
        if (i <= ETL / 2) {
            EFb(i) = z0;
            EFb(i + 1) = z0;
            EZ(i + 1) = z0;
        }
    }
    {
        T F = EF(1), Fb = EFb(1), Z = EZ(1);
        T C = F + Fb, S2 = F - Fb;
        dc[(ETL - 1) * dst] = fmad(-q.c, Z, fmad(q.a, C, (-q.b) * S2));
    }
    for (int i = 0; i < ETL; ++i) dc[i * dst] = absd(q.m0 * dc[i * dst]);
#undef EF
#undef EFb
#undef EZ
}

// Coefficients of the general-control-angle recursion, src/EPGdecaycurve.jl:729-746.
template <class T>
struct VecCoef {
    T F[3], Fb[3], Z[3];
    T a1, b1, c1, m0;
};
template <class T>
DX_HD T dot3(const T *a, T x, T y, T z) {
    return (a[0] * x + a[1] * y) + a[2] * z;
}
DX_HD VecCoef<double> vec_coef(double alpha_deg, double TE, double T2, double T1, double beta) {
    double A = alpha_deg / 180;
    double a1r = (A * 180) * kD2R, air = (A * beta) * kD2R;
    double E1 = pm_exp(-(TE / 2) / T1), E2 = pm_exp(-(TE / 2) / T2);
    double sh, ch, sai, cai;
    pm_sincos(a1r / 2, &sh, &ch);
    pm_sincos(air, &sai, &cai);
    double sh2 = sh * sh, ch2 = ch * ch, sa1 = 2 * sh * ch;
    double chi2 = (1 + cai) / 2, shi2 = 1 - chi2;
    VecCoef<double> k;
    k.a1 = (E2 * E2) * ch2; k.b1 = (E2 * E2) * sh2; k.c1 = (E1 * E2) * sa1;
    double ai = (E2 * E2) * chi2, bi = (E2 * E2) * shi2, ci = (E1 * E2) * sai, di = (E1 * E1) * cai;
    k.F[0] = ai; k.F[1] = bi; k.F[2] = ci;
    k.Fb[0] = bi; k.Fb[1] = ai; k.Fb[2] = -ci;
    k.Z[0] = -ci / 2; k.Z[1] = ci / 2; k.Z[2] = di;
    k.m0 = sh;
    return k;
}
DX_HD VecCoef<Dual> vec_coef_dual(double alpha_deg, double TE, double T2, double T1, double beta) {
    Dual alpha{alpha_deg, 1.0};
    Dual A = alpha / 180;
    Dual a1r = (A * 180.0) * kD2R, air = (A * beta) * kD2R;
    double E1 = pm_exp(-(TE / 2) / T1), E2 = pm_exp(-(TE / 2) / T2);
    Dual h = a1r / 2;
    double shv, chv, saiv, caiv;
    pm_sincos(h.v, &shv, &chv);
    pm_sincos(air.v, &saiv, &caiv);
    Dual sh{shv, chv * h.d}, ch{chv, -shv * h.d};
    Dual sh2 = sh * sh, ch2 = ch * ch, sa1 = (sh * 2.0) * ch;
    Dual sai{saiv, caiv * air.d}, cai{caiv, -saiv * air.d};
    Dual chi2 = (mkd(1.0) + cai) / 2, shi2 = mkd(1.0) - chi2;
    VecCoef<Dual> k;
    k.a1 = ch2 * (E2 * E2); k.b1 = sh2 * (E2 * E2); k.c1 = sa1 * (E1 * E2);
    Dual ai = chi2 * (E2 * E2), bi = shi2 * (E2 * E2), ci = sai * (E1 * E2), di = cai * (E1 * E1);
    k.F[0] = ai; k.F[1] = bi; k.F[2] = ci;
    k.Fb[0] = bi; k.Fb[1] = ai; k.Fb[2] = -ci;
    k.Z[0] = (-ci) / 2; k.Z[1] = ci / 2; k.Z[2] = di;
    k.m0 = sh;
    return k;
}

DX_HD VecCoef<float> to_f32(const VecCoef<double> &k) {
    VecCoef<float> o;
    for (int c = 0; c < 3; ++c) { o.F[c] = (float)k.F[c]; o.Fb[c] = (float)k.Fb[c]; o.Z[c] = (float)k.Z[c]; }
    o.a1 = (float)k.a1; o.b1 = (float)k.b1; o.c1 = (float)k.c1; o.m0 = (float)k.m0;
    return o;
}

// epg_decay_curve! for EPGOptions (DualVector_Split_Dynamic), in place.
// S holds 3*ETL strided values: state k's (x,y,z) at S[(3(k-1)+c)*st].
template <class T, class O>
DX_HD void epg_vec_inplace(int ETL, const VecCoef<T> &q, T *S, int st, O *dc, int dst) {
#define SX(k, c) S[(3 * ((k)-1) + (c)) * st]
    const T z0 = zero_of(q.m0);
    T M0x = q.b1 * q.m0, M0z = ((-q.c1) * q.m0) / 2;
    SX(1, 0) = M0x; SX(1, 1) = z0; SX(1, 2) = M0z;
    SX(2, 0) = q.a1 * q.m0; SX(2, 1) = z0; SX(2, 2) = z0;
    dc[0] = absd(M0x);
    {
        T m0x = SX(1, 0), m0y = SX(1, 1), m0z = SX(1, 2), m1x = SX(2, 0), m1y = SX(2, 1), m1z = SX(2, 2);
        T FM0 = dot3(q.F, m0x, m0y, m0z), FbM0 = dot3(q.Fb, m0x, m0y, m0z), ZM0 = dot3(q.Z, m0x, m0y, m0z);
        T FM1 = dot3(q.F, m1x, m1y, m1z), FbM1 = dot3(q.Fb, m1x, m1y, m1z), ZM1 = dot3(q.Z, m1x, m1y, m1z);
        SX(1, 0) = FbM0; SX(1, 1) = FbM1; SX(1, 2) = ZM0;
        SX(2, 0) = FM0; SX(2, 1) = z0; SX(2, 2) = ZM1;
        SX(3, 0) = FM1; SX(3, 1) = z0; SX(3, 2) = z0;
        dc[1 * dst] = absd(FbM0);
    }
    for (int i = 3; i <= ETL - 1; ++i) {
        const bool first = (i <= ETL / 2);
        const int jend = first ? i - 1 : ETL - i;
        T m0x = SX(1, 0), m0y = SX(1, 1), m0z = SX(1, 2);
        T m1x = SX(2, 0), m1y = SX(2, 1), m1z = SX(2, 2);
        T m2x = SX(3, 0), m2y = SX(3, 1), m2z = SX(3, 2);
        T FM0 = dot3(q.F, m0x, m0y, m0z), FbM0 = dot3(q.Fb, m0x, m0y, m0z), ZM0 = dot3(q.Z, m0x, m0y, m0z);
        T FM1 = dot3(q.F, m1x, m1y, m1z), FbM1 = dot3(q.Fb, m1x, m1y, m1z), ZM1 = dot3(q.Z, m1x, m1y, m1z);
        T FM2 = dot3(q.F, m2x, m2y, m2z), FbM2 = dot3(q.Fb, m2x, m2y, m2z), ZM2 = dot3(q.Z, m2x, m2y, m2z);
        SX(1, 0) = FbM0; SX(1, 1) = FbM1; SX(1, 2) = ZM0;
        SX(2, 0) = FM0; SX(2, 1) = FbM2; SX(2, 2) = ZM1;
        for (int j = 3; j <= jend; ++j) {
            FM0 = FM1; FM1 = FM2; ZM1 = ZM2;
            T x = SX(j + 1, 0), y = SX(j + 1, 1), z = SX(j + 1, 2);
            FM2 = dot3(q.F, x, y, z); FbM2 = dot3(q.Fb, x, y, z); ZM2 = dot3(q.Z, x, y, z);
            SX(j, 0) = FM0; SX(j, 1) = FbM2; SX(j, 2) = ZM1;
        }
        if (first) {
            SX(i, 0) = FM1; SX(i, 1) = z0; SX(i, 2) = ZM2;
            SX(i + 1, 0) = FM2; SX(i + 1, 1) = z0; SX(i + 1, 2) = z0;
        }
        dc[(i - 1) * dst] = absd(FbM0);
    }
    dc[(ETL - 1) * dst] = absd(dot3(q.Fb, SX(1, 0), SX(1, 1), SX(1, 2)));
#undef SX
}

}  // namespace dx
