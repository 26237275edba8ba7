// host.cpp -- host-side pieces of libdecaes_gpu.so: parameter grids, option
// validation with the reference's assertion messages, and the synthetic
// image generator.  No GPU is needed for anything in this file.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "decaes_gpu.h"
#include "epg.cuh"
#include "host.h"

namespace dh {

// ---------------------------------------------------------------------------
// Julia's range(a, b; length) for Float64 endpoints (Base twiceprecision.jl):
// an exact rational path when both endpoints are small rationals, otherwise
// the split (hi, lo) reference/step evaluation.  Used for the flip-angle grid
// (src/types.jl:109) and, through logrange, the T2 grid (src/utils.jl:7).
// ---------------------------------------------------------------------------
static void add12(double x, double y, double &h, double &l) {
    if (std::fabs(y) > std::fabs(x)) std::swap(x, y);
    h = x + y;
    l = (x - h) + y;
}
static double truncbits(double x, int nb) {
    uint64_t u;
    std::memcpy(&u, &x, 8);
    u &= (~uint64_t(0)) << nb;
    std::memcpy(&x, &u, 8);
    return x;
}
static int nbitslen(long len, long offset) {
    if (len < 2) return 0;
    long k = std::max(offset - 1, len - offset) - 1;
    int b = 0;
    while (k > 0) { ++b; k >>= 1; }
    return std::min(27, b + 1);
}
static void rat(double x, long &num, long &den) {
    double y = x;
    long a = 1, d = 1, b = 0, c = 0;
    const double m = 16777216.0;
    while (std::fabs(y) <= m) {
        long f = (long)std::trunc(y);
        y -= (double)f;
        long an = f * a + c, bn = f * b + d;
        c = a; d = b; a = an; b = bn;
        if (std::labs(a) > (long)m || std::labs(b) > (long)m) { num = c; den = d; return; }
        if ((double)a / (double)b == x) break;
        y = 1.0 / y;
    }
    num = a;
    den = b;
}
static long gcdl(long a, long b) {
    a = std::labs(a); b = std::labs(b);
    while (b) { long t = a % b; a = b; b = t; }
    return a;
}

std::vector<double> julia_range(double start, double stop, int len) {
    std::vector<double> out(len);
    if (len == 1) { out[0] = start; return out; }
    if (start == stop) { for (auto &v : out) v = start; return out; }
    long sn, sd, en, ed;
    rat(start, sn, sd);
    rat(stop, en, ed);
    if (sd != 0 && ed != 0) {
        long den = std::labs(sd / gcdl(sd, ed) * ed);
        const double m = 9007199254740992.0;
        if (den != 0 && std::fabs((double)den * start) <= m && std::fabs((double)den * stop) <= m) {
            long s_n = (long)std::rint((double)den * start), e_n = (long)std::rint((double)den * stop);
            if ((double)s_n / (double)den == start && (double)e_n / (double)den == stop) {
                for (int i = 1; i <= len; ++i) {
                    long double numv = (long double)(len - i) * s_n + (long double)(i - 1) * e_n;
                    out[i - 1] = (double)numv / ((double)(len - 1) * (double)den);
                }
                return out;
            }
        }
    }
    double D = stop - start;
    double tmin = -(start / D) / 1.0;
    long imin = std::lrint(tmin * (double)(len - 1) + 1.0);
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
    int nb = nbitslen(len, imin);
    double step_hi = truncbits(step, nb);
    double x1h, x1l, x2h, x2l;
    add12((double)(1 - imin) * step_hi, ref, x1h, x1l);
    add12((double)(len - imin) * step_hi, ref, x2h, x2l);
    double a = (start - x1h) - x1l, b = (stop - x2h) - x2l;
    double step_lo = (b - a) / (double)(len - 1);
    double ref_lo = a - (double)(1 - imin) * step_lo;
    for (int i = 1; i <= len; ++i) {
        double u = (double)(i - imin);
        double sh = u * step_hi, sl = u * step_lo, xh, xl;
        add12(ref, sh, xh, xl);
        out[i - 1] = xh + (xl + (sl + ref_lo));
    }
    return out;
}

std::vector<double> julia_logrange(double a, double b, int len) {
    std::vector<double> r = julia_range(std::log(a), std::log(b), len);
    for (auto &v : r) v = std::exp(v);
    r[0] = a;
    r[len - 1] = b;
    return r;
}

// erfinv for the sigmoid width (SpecialFunctions.erfinv in
// src/T2partSEcorr.jl:159): M. Giles' approximation ("Approximating the
// erfinv function", GPU Computing Gems, 2011) refined by Newton steps on erf.
double erfinv(double x) {
    if (x <= -1) return x == -1 ? -INFINITY : NAN;
    if (x >= 1) return x == 1 ? INFINITY : NAN;
    double w = -std::log((1.0 - x) * (1.0 + x)), p;
    if (w < 5.0) {
        w -= 2.5;
        p = 2.81022636e-08; p = 3.43273939e-07 + p * w; p = -3.5233877e-06 + p * w;
        p = -4.39150654e-06 + p * w; p = 0.00021858087 + p * w; p = -0.00125372503 + p * w;
        p = -0.00417768164 + p * w; p = 0.246640727 + p * w; p = 1.50140941 + p * w;
    } else {
        w = std::sqrt(w) - 3.0;
        p = -0.000200214257; p = 0.000100950558 + p * w; p = 0.00134934322 + p * w;
        p = -0.00367342844 + p * w; p = 0.00573950773 + p * w; p = -0.0076224613 + p * w;
        p = 0.00943887047 + p * w; p = 1.00167406 + p * w; p = 2.83297682 + p * w;
    }
    double y = p * x;
    for (int it = 0; it < 3; ++it) y -= (std::erf(y) - x) / (1.1283791670955126 * std::exp(-y * y));
    return y;
}

// ---------------------------------------------------------------------------
// Option validation (src/types.jl:28-95, 148-168), messages as Julia prints them.
// ---------------------------------------------------------------------------
std::string jlfmt(double v) {
    if (std::isnan(v)) return "NaN";
    if (std::isinf(v)) return v > 0 ? "Inf" : "-Inf";
    if (v == 0) return std::signbit(v) ? "-0.0" : "0.0";
    // shortest round-trip digits, then Julia's layout: plain decimal for
    // 1e-4 <= |v| < 1e6, otherwise d.ddd e<exp> (e.g. 190.0, 0.01, 1.0e-5, 1.0e6)
    char buf[64];
    int p = 1;
    for (; p <= 17; ++p) {
        std::snprintf(buf, sizeof buf, "%.*e", p - 1, v);
        if (std::strtod(buf, nullptr) == v) break;
    }
    std::string s(buf);
    size_t epos = s.find('e');
    int E = std::atoi(s.c_str() + epos + 1);
    std::string mant = s.substr(0, epos);
    bool neg = mant[0] == '-';
    if (neg) mant = mant.substr(1);
    std::string digits;
    for (char ch : mant) if (ch != '.') digits += ch;
    std::string out;
    if (E >= -4 && E < 6) {
        if (E >= 0) {
            std::string ip = digits.substr(0, std::min<size_t>(digits.size(), E + 1));
            while ((int)ip.size() < E + 1) ip += '0';
            std::string fp = (int)digits.size() > E + 1 ? digits.substr(E + 1) : "0";
            out = ip + "." + fp;
        } else {
            out = "0." + std::string(-E - 1, '0') + digits;
        }
    } else {
        out = digits.substr(0, 1) + "." + (digits.size() > 1 ? digits.substr(1) : "0") + "e" + std::to_string(E);
    }
    return neg ? "-" + out : out;
}
static std::string nothing_or(double v) { return std::isnan(v) ? "nothing" : jlfmt(v); }

std::string check_t2map(const decaes_t2map_opts &o) {
    char b[512];
    if (o.MatrixSize[0] < 1 || o.MatrixSize[1] < 1 || o.MatrixSize[2] < 1) {
        std::snprintf(b, sizeof b, "MatrixSize must be a tuple of 3 positive integers, but MatrixSize = (%d, %d, %d).",
                      o.MatrixSize[0], o.MatrixSize[1], o.MatrixSize[2]);
        return b;
    }
    if (!(o.nTE >= 4)) { std::snprintf(b, sizeof b, "At least four echoes are required for T2 mapping, but nTE = %d.", o.nTE); return b; }
    if (!(o.TE > 0.0)) return "Echo spacing must be positive, but TE = " + jlfmt(o.TE) + ".";
    if (!(o.nT2 >= 2)) { std::snprintf(b, sizeof b, "At least two T2 components are required for T2 mapping, but nT2 = %d.", o.nT2); return b; }
    if (!(0.0 < o.T2Range[0] && o.T2Range[0] < o.T2Range[1]))
        return "T2Range must a sorted 2-tuple of positive values, but T2Range = (" + jlfmt(o.T2Range[0]) + ", " + jlfmt(o.T2Range[1]) + ").";
    if (!(o.T1 > 0.0)) return "T1 must be positive, but T1 = " + jlfmt(o.T1) + ".";
    if (!(o.Threshold >= 0.0 || o.Threshold == -INFINITY))
        return "First echo signal threshold must be non-negative or -Inf to force processing of every voxel, but Threshold = " + jlfmt(o.Threshold) + ".";
    if (!(0.0 <= o.MinRefAngle && o.MinRefAngle <= 180.0))
        return "Minimum refocusing angle must be in the range [0, 180], but MinRefAngle = " + jlfmt(o.MinRefAngle) + ".";
    if (!(o.nRefAngles >= 2)) {
        std::snprintf(b, sizeof b, "Maximum number of angles to check during flip angle optimization must be at least 2, but nRefAngles = %d.", o.nRefAngles);
        return b;
    }
    if (!(2 <= o.nRefAnglesMin && o.nRefAnglesMin <= o.nRefAngles)) {
        std::snprintf(b, sizeof b, "Minimum number of angles to check during flip angle optimization must be in the range [2, nRefAngles], but nRefAngles = %d and nRefAnglesMin = %d.", o.nRefAngles, o.nRefAnglesMin);
        return b;
    }
    if (o.Reg < DECAES_REG_NONE || o.Reg > DECAES_REG_MDP) return "Reg ∈ (\"none\", \"lcurve\", \"gcv\", \"chi2\", \"mdp\")";
    if (o.Reg == DECAES_REG_CHI2 && !(!std::isnan(o.Chi2Factor) && o.Chi2Factor > 1.0))
        return "Chi2Factor must be greater than 1.0, but Chi2Factor = " + nothing_or(o.Chi2Factor) + ".";
    if (o.Reg == DECAES_REG_MDP && !(!std::isnan(o.NoiseLevel) && o.NoiseLevel > 0.0))
        return "Noise level must be positive, but NoiseLevel = " + nothing_or(o.NoiseLevel) + ".";
    if (!(0.0 <= o.RefConAngle && o.RefConAngle <= 180.0))
        return "Refocusing control angle must be in the range [0, 180], but RefConAngle = " + jlfmt(o.RefConAngle) + ".";
    if (!std::isnan(o.SetFlipAngle) && !(0.0 <= o.SetFlipAngle && o.SetFlipAngle <= 180.0))
        return "Fixed flip angle must be in the range [0, 180], but SetFlipAngle = " + jlfmt(o.SetFlipAngle) + ".";
    if (o.precision != DECAES_PREC_FP64 && o.precision != DECAES_PREC_MIXED && o.precision != DECAES_PREC_MIXED_TC)
        return "precision must be DECAES_PREC_FP64, DECAES_PREC_MIXED or DECAES_PREC_MIXED_TC.";
    return "";
}

std::string check_t2part(const decaes_t2part_opts &o) {
    if (o.MatrixSize[0] < 1 || o.MatrixSize[1] < 1 || o.MatrixSize[2] < 1) return "all(MatrixSize .>= 1)";
    if (!(o.nT2 >= 2)) return "nT2 >= 2";
    if (!(0.0 < o.T2Range[0] && o.T2Range[0] < o.T2Range[1])) return "0.0 < T2Range[1] < T2Range[2]";
    if (!(o.SPWin[0] < o.SPWin[1])) return "SPWin[1] < SPWin[2]";
    if (!(o.MPWin[0] < o.MPWin[1])) return "MPWin[1] < MPWin[2]";
    if (!(std::isnan(o.Sigmoid) || o.Sigmoid > 0)) return "Sigmoid === nothing || Sigmoid > 0";
    return "";
}

// T2part window index ranges and sigmoid weights (src/T2partSEcorr.jl:143-164).
std::string t2part_plan(const decaes_t2part_opts &o, T2partPlan &p) {
    const int n = o.nT2;
    p.t2 = julia_logrange(o.T2Range[0], o.T2Range[1], n);
    p.logt2.resize(n);
    for (int j = 0; j < n; ++j) p.logt2[j] = std::log(p.t2[j]);
    p.sp0 = p.sp1 = p.mp0 = p.mp1 = -1;
    for (int j = 0; j < n; ++j) if (p.t2[j] >= o.SPWin[0]) { p.sp0 = j; break; }
    for (int j = n - 1; j >= 0; --j) if (p.t2[j] <= o.SPWin[1]) { p.sp1 = j; break; }
    for (int j = 0; j < n; ++j) if (p.t2[j] >= o.MPWin[0]) { p.mp0 = j; break; }
    for (int j = n - 1; j >= 0; --j) if (p.t2[j] <= o.MPWin[1]) { p.mp1 = j; break; }
    if (p.sp0 < 0 || p.sp1 < 0) return "SPWin does not overlap the T2 grid (findfirst/findlast returned nothing).";
    if (p.mp0 < 0 || p.mp1 < 0) return "MPWin does not overlap the T2 grid (findfirst/findlast returned nothing).";
    p.weights.clear();
    if (!std::isnan(o.Sigmoid)) {
        double k = 0.1, sigma = std::fabs(o.Sigmoid / (std::sqrt(2.0) * erfinv(2 * k - 1)));
        p.weights.resize(n);
        for (int j = 0; j < n; ++j) {
            double wv = std::erfc(((p.t2[j] - o.SPWin[1]) / sigma) / std::sqrt(2.0)) / 2;
            p.weights[j] = wv <= 2.220446049250313e-16 ? 0.0 : wv;
        }
    }
    return "";
}

// ---------------------------------------------------------------------------
// Synthetic image: per voxel a sum of three EPG decays with Rician noise, the
// generator of this project's benchmark workloads (the reference's own
// mock_image, src/utils.jl:623-658, draws a bi-exponential instead).
// Counter-based: voxel v's stream is seeded from (seed, v), so the image does
// not depend on the thread count.
// ---------------------------------------------------------------------------
struct Rng {
    uint64_t s[4];
    static uint64_t splitmix(uint64_t &x) {
        uint64_t z = (x += 0x9e3779b97f4a7c15ull);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        return z ^ (z >> 31);
    }
    Rng(uint64_t seed, uint64_t stream) {
        uint64_t x = seed ^ (stream * 0xd1b54a32d192ed03ull);
        for (auto &v : s) v = splitmix(x);
    }
    static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    uint64_t next() {  // xoshiro256** (Blackman & Vigna)
        uint64_t r = rotl(s[1] * 5, 7) * 9, t = s[1] << 17;
        s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3]; s[2] ^= t; s[3] = rotl(s[3], 45);
        return r;
    }
    double unif() { return (double)(next() >> 11) * 0x1.0p-53; }
    double unif(const double *r) { return r[0] + (r[1] - r[0]) * unif(); }
    double normal() {  // Box-Muller
        double u1 = unif(), u2 = unif();
        if (u1 < 1e-300) u1 = 1e-300;
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    }
};

int mock_image(const decaes_mock_opts &o, uint64_t seed, void *image, int dtype, int nthreads) {
    const long V = (long)o.MatrixSize[0] * o.MatrixSize[1] * o.MatrixSize[2];
    const int m = o.nTE;
    if (V <= 0 || m < 1) return DECAES_EINVAL;
    if (nthreads <= 0) nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
    auto work = [&](long v0, long v1) {
        std::vector<double> S(3 * (size_t)m), d1(m), d2(m), d3(m);
        for (long v = v0; v < v1; ++v) {
            Rng g(seed, (uint64_t)v);
            double alpha = g.unif(o.FlipAngleRange);
            double wmy = g.unif(o.MyelinFracRange), t2my = g.unif(o.MyelinT2Range);
            double t2ie = g.unif(o.IET2Range);
            double wcsf = g.unif(o.CSFFracRange), t2csf = g.unif(o.CSFT2Range);
            double amp = g.unif(o.AmplitudeRange), snr = g.unif(o.SNRRange);
            bool bg = g.unif() < o.BackgroundFraction;
            double wie = 1.0 - wmy - wcsf;
            auto q1 = dx::flat_coef(alpha, o.TE, t2my, o.T1);
            auto q2 = dx::flat_coef(alpha, o.TE, t2ie, o.T1);
            auto q3 = dx::flat_coef(alpha, o.TE, t2csf, o.T1);
            dx::epg_flat_inplace(m, q1, S.data(), 1, d1.data(), 1);
            dx::epg_flat_inplace(m, q2, S.data(), 1, d2.data(), 1);
            dx::epg_flat_inplace(m, q3, S.data(), 1, d3.data(), 1);
            double sigma = bg ? o.BackgroundSigma : amp / snr;
            for (int e = 0; e < m; ++e) {
                double s = bg ? 0.0 : amp * (wmy * d1[e] + wie * d2[e] + wcsf * d3[e]);
                double zr = g.normal(), zi = g.normal();
                double val = std::sqrt((s + sigma * zr) * (s + sigma * zr) + (sigma * zi) * (sigma * zi));
                if (dtype == DECAES_F32) ((float *)image)[v + V * e] = (float)val;
                else ((double *)image)[v + V * e] = val;
            }
        }
    };
    std::vector<std::thread> th;
    long chunk = (V + nthreads - 1) / nthreads;
    for (int t = 0; t < nthreads; ++t) {
        long a = t * chunk, b = std::min(V, a + chunk);
        if (a < b) th.emplace_back(work, a, b);
    }
    for (auto &t : th) t.join();
    return DECAES_OK;
}

}  // namespace dh

extern "C" int decaes_mock_image(const decaes_mock_opts *opts, uint64_t seed, void *image, int dtype, int nthreads) {
    if (!opts || !image || (dtype != DECAES_F32 && dtype != DECAES_F64)) return DECAES_EINVAL;
    return dh::mock_image(*opts, seed, image, dtype, nthreads);
}

extern "C" int decaes_t2map_check_options(const decaes_t2map_opts *opts, char *msg, size_t msglen) {
    std::string e = opts ? dh::check_t2map(*opts) : std::string("opts is NULL");
    if (msg && msglen) { std::strncpy(msg, e.c_str(), msglen - 1); msg[msglen - 1] = 0; }
    return e.empty() ? DECAES_OK : DECAES_EINVAL;
}

extern "C" int decaes_t2part_check_options(const decaes_t2part_opts *opts, char *msg, size_t msglen) {
    std::string e = opts ? dh::check_t2part(*opts) : std::string("opts is NULL");
    if (msg && msglen) { std::strncpy(msg, e.c_str(), msglen - 1); msg[msglen - 1] = 0; }
    return e.empty() ? DECAES_OK : DECAES_EINVAL;
}
