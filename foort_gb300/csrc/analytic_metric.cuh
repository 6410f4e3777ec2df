// Analytic metric plugins (host + device), templated on the arithmetic type.
//
// Each plugin evaluates, at (r, theta), the derivatives d_r g_ij and d_theta g_ij of
// the five non-zero covariant components, the contravariant components g^ij and g_rr
// (gen_christoffel.inc, generated from the reference's Metric.cpp formulas). The
// mixed-precision kernel runs them in FP32 (and in FP64 near the horizon when asked);
// the host runs them in FP64 for foort_metric_christoffel().
#pragma once

#include <math.h>

#include <cmath>

#include "gen_christoffel.inc"
#include "metric_fp64.cuh"

namespace foort {

template <typename T>
struct G5T {
    T tt, tp, rr, hh, pp;
};

// Reciprocal for the generated bodies, which multiply by reciprocals of their
// denominators' factors instead of dividing. On the device: the hardware's approximate
// reciprocal r0 refined by one Newton-Raphson step, r1 = r0 + r0 (1 - x r0), which
// squares r0's relative error (~2^-23) away and leaves the final FMA's rounding: within
// one ulp, in three instructions and without the branches of a correctly rounded
// reciprocal (which sit on the critical path of every right-hand side). For x = 0 it
// gives NaN where 1/x is infinite, and so for any |x| below FLT_MIN, which the .ftz
// forms flush to 0: the factors are r - r_+, r - r_-, sin(theta), Sigma, r and the like,
// below 1.2e-38 only within that distance of a horizon, a pole or the origin, where the
// state turns non-finite with either value. Passing the infinity through cost 1.2 % on
// GB300 in the Kerr a = 0.99 adaptive run (509² grid, 26,547 geodesics).
FOORT_HD float rcp(float x) {
#ifdef __CUDA_ARCH__
    float r0;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r0) : "f"(x));
    return __fmaf_rn(r0, __fmaf_rn(-x, r0, 1.0f), r0);
#else
    return 1.0f / x;
#endif
}
FOORT_HD double rcp(double x) { return 1.0 / x; }

// sin and cos of a float-float angle theta = th_hi + th_lo, to FP32 relative accuracy
// also where the result is tiny (sin near theta = 0 and pi, cos near pi/2). A float theta
// cannot give that: its rounding error (up to 1.2e-7 near pi) exceeds the distance to
// the pole of rays that pass it closely, and cos(float(pi/2)) = -4.4e-8 pulls rays out of
// the equatorial plane. The angle is reduced against pi/2 split into three floats (the
// true pi: the metric's poles are at the true 0 and pi), d = theta - k pi/2, |d| <= pi/4;
// sin d and cos d are their Taylor series (coefficients 1/n!) to the terms d^9 and d^10,
// whose truncation error at pi/4 is below 3e-9 relative.
FOORT_HD void ff_sincos(float th_hi, float th_lo, float& s, float& c) {
    constexpr float kPiO2Hi = 0x1.921fb6p+0f;    // pi/2 = hi + mid + lo to 2^-76
    constexpr float kPiO2Mid = -0x1.777a5cp-25f;
    constexpr float kPiO2Lo = -0x1.ee59dap-50f;
    const float k = rintf(th_hi * 0.636619772f);
    // th_hi - k hi is exact for |k| <= 2 (Sterbenz) and rounded once beyond; when it is 0
    // the fma leaves d with one rounding relative to itself.
    float d = fmaf(-k, kPiO2Hi, th_hi) + fmaf(-k, kPiO2Mid, th_lo);
    d = fmaf(-k, kPiO2Lo, d);
    const float d2 = d * d;
    float sp = fmaf(d2, 2.75573192e-6f, -1.98412698e-4f);  // 1/9!, -1/7!
    sp = fmaf(d2, sp, 8.33333333e-3f);                      // 1/5!
    sp = fmaf(d2, sp, -1.66666667e-1f);                     // -1/3!
    const float sd = fmaf(d * d2, sp, d);
    float cp = fmaf(d2, -2.75573192e-7f, 2.48015873e-5f);   // -1/10!, 1/8!
    cp = fmaf(d2, cp, -1.38888889e-3f);                     // -1/6!
    cp = fmaf(d2, cp, 4.16666667e-2f);                      // 1/4!
    cp = fmaf(d2, cp, -0.5f);                               // -1/2!
    const float cd = fmaf(d2, cp, 1.0f);
    const int q = static_cast<int>(k) & 3;
    s = (q == 0) ? sd : (q == 1) ? cd : (q == 2) ? -sd : -cd;
    c = (q == 0) ? cd : (q == 1) ? -sd : (q == 2) ? -cd : sd;
}

template <int MID>
struct MixedMetric {
    static constexpr bool kAvailable = false;
    static constexpr bool kInline = true;
};

// kInline: inline the body into each RK4 stage, or call it. Calling keeps large bodies
// (Johannsen, ~300 temporaries) out of the register allocation of the stepping loop.
// Kerr is inlined: with branch-free reciprocals its four copies fit the instruction
// cache, and the five rounds of the Kerr a = 0.99 adaptive run (509² grid, 26,547 geodesics)
// take 695 ms inlined against 786 ms called on GB300.
#define FOORT_DEFINE_MIXED_METRIC(ID, BODY, INL)                                                   \
    template <>                                                                                    \
    struct MixedMetric<ID> {                                                                       \
        static constexpr bool kAvailable = true;                                                   \
        static constexpr bool kInline = INL;                                                       \
        template <typename T>                                                                      \
        static FOORT_HD void eval(const T* q, T r, T dp, T dm, T s, T c, G5T<T>& dr, G5T<T>& dh,   \
                                  G5T<T>& gu, T& grr) {                                            \
            (void)q; (void)dp; (void)dm;                                                           \
            BODY                                                                                   \
        }                                                                                          \
    };

FOORT_DEFINE_MIXED_METRIC(kKerr, FOORT_MIXED_BODY_KERR, true)
FOORT_DEFINE_MIXED_METRIC(kJohannsen, FOORT_MIXED_BODY_JOHANNSEN, false)
FOORT_DEFINE_MIXED_METRIC(kFlat, FOORT_MIXED_BODY_FLAT, true)
FOORT_DEFINE_MIXED_METRIC(kRasheedLarsen, FOORT_MIXED_BODY_RASHEEDLARSEN, false)

// ---- Manko-Novikov, by forward-mode differentiation ---------------------------------
// Its metric functions are exponentials of sums of Legendre terms over powers of
// R = sqrt(x^2 + y^2 - 1) (Metric.cpp:511-566); sympy's expanded derivatives of them
// would be enormous. Instead the metric is evaluated once on dual numbers carrying the
// value and its derivatives in r and theta, which gives d_r g and d_theta g exactly up to
// rounding. Restated for the same values with these cancellation-free forms (x - 1 =
// (r - r_+)/k, so near the horizon nothing is formed as a difference of near-equal
// numbers):
//   x^2 - 1 = dp (x + 1) / k,  1 - y^2 = sin^2,  R^2 = (x^2 - 1) + y^2,
//   x^2 - y^2 = (x^2 - 1) + sin^2,  Delta = dp dm,  rho^2 = Delta + k^2 sin^2,
// and the inverse of the (t, phi) block from its determinant, exactly -Delta sin^2:
//   g^tt = -g_phiphi / (Delta sin^2), g^tphi = g_tphi / (Delta sin^2),
//   g^phiphi = -g_tt / (Delta sin^2).
template <typename T>
struct D2 {
    T v, r, h;  // value, d/dr, d/dtheta
};
template <typename T>
FOORT_HD D2<T> operator+(D2<T> a, D2<T> b) { return {a.v + b.v, a.r + b.r, a.h + b.h}; }
template <typename T>
FOORT_HD D2<T> operator-(D2<T> a, D2<T> b) { return {a.v - b.v, a.r - b.r, a.h - b.h}; }
template <typename T>
FOORT_HD D2<T> operator-(D2<T> a) { return {-a.v, -a.r, -a.h}; }
template <typename T>
FOORT_HD D2<T> operator*(D2<T> a, D2<T> b) { return {a.v * b.v, a.r * b.v + a.v * b.r, a.h * b.v + a.v * b.h}; }
template <typename T>
FOORT_HD D2<T> operator*(T c, D2<T> a) { return {c * a.v, c * a.r, c * a.h}; }
template <typename T>
FOORT_HD D2<T> operator+(T c, D2<T> a) { return {c + a.v, a.r, a.h}; }
template <typename T>
FOORT_HD D2<T> inv(D2<T> a) {  // 1 / a
    const T i = rcp(a.v), i2 = -i * i;
    return {i, i2 * a.r, i2 * a.h};
}
template <typename T>
FOORT_HD D2<T> d_sqrt(D2<T> a) {
    const T s = ::sqrt(a.v), d = T(0.5) * rcp(s);
    return {s, d * a.r, d * a.h};
}
template <typename T>
FOORT_HD D2<T> d_exp(D2<T> a) {
    const T e = ::exp(a.v);
    return {e, e * a.r, e * a.h};
}

template <typename T>
FOORT_HD D2<T> d_cast(D2<double> a) {
    return {T(a.v), T(a.r), T(a.h)};
}

// q: a, alpha3, alpha, k (make_metric_const). rd, dpd = r - r_+ (r_+ = 1 + k), sd, cd:
// the position in FP64; dp, dm, s, c: the same in T.
// The exponents' arguments are computed in FP64 from the FP64 position, whatever T is:
// - 1 - (x - y) S1 and -1 + (x + y) S2 are sums of O(1) terms whose leading orders cancel
//   through 1/x^2, so in FP32 arithmetic their absolute error stays ~6e-8 while the
//   values fall off like 1/x^3; an exponent's absolute error becomes the metric's
//   relative error (2e-6 at alpha3 = 13, the reference's Test.cfg value);
// - the exponents are sensitive to the position (factors of 2 alpha3): r and theta
//   rounded to FP32 put p99 7e-6 on the FP32 acceleration at alpha3 = 13, FP64 inputs
//   with only the exponentials rounded to FP32 2e-7 (measured on the CPU).
// ~250 FP64 operations per evaluation. The rest is in T.
template <typename T>
FOORT_HD void mn_eval(const T* q, double rd, double dpd, double sd, double cd, T dp, T dm, T s, T c, G5T<T>& dr,
                      G5T<T>& dh, G5T<T>& gu, T& grr) {
    // -- the exponents' arguments (FP64)
    const double a3d = q[1], kd = q[3], ikd = 1.0 / kd;
    const D2<double> X = {(rd - 1.0) * ikd, ikd, 0.0};
    const D2<double> Y = {cd, 0.0, -sd};
    const D2<double> XM1 = ikd * D2<double>{dpd, 1.0, 0.0};  // x - 1
    const D2<double> X2M1 = XM1 * (2.0 + XM1);                // x^2 - 1
    const D2<double> iR = inv(d_sqrt(X2M1 + Y * Y));
    const D2<double> t = X * Y * iR;  // the Legendre argument xy / R
    const D2<double> t2 = t * t;
    const D2<double> P1 = t;
    const D2<double> P2 = 0.5 * (3.0 * t2 + D2<double>{-1.0, 0.0, 0.0});
    const D2<double> P3 = 0.5 * t * (5.0 * t2 + D2<double>{-3.0, 0.0, 0.0});
    const D2<double> P4 = 0.125 * (35.0 * t2 * t2 - 30.0 * t2 + D2<double>{3.0, 0.0, 0.0});
    const D2<double> S1 = iR * (1.0 + iR * (P1 + iR * (P2 + iR * P3)));   // 1/R + P1/R^2 + P2/R^3 + P3/R^4
    const D2<double> S2 = iR * (1.0 + iR * (-P1 + iR * (P2 - iR * P3)));  // 1/R - P1/R^2 + P2/R^3 - P3/R^4
    const D2<double> iR4 = (iR * iR) * (iR * iR);
    const D2<double> Ea = (2.0 * a3d) * (1.0 + -((X - Y) * S1));
    const D2<double> Eb = (2.0 * a3d) * (-1.0 + (X + Y) * S2);
    const D2<double> psi2 = (2.0 * a3d) * (P3 * iR4);  // 2 psi
    const D2<double> gp2 = (4.0 * a3d * a3d) * ((P4 * P4 - P3 * P3) * (iR4 * iR4)) +
                           (4.0 * a3d) * ((-Y + iR * (X * P1 + iR * (-(Y * P2) + iR * (X * P3)))) * iR);  // 2 gamma'
    // -- the metric (T), without the reference's 1/AA: AA vanishes where g_tt does, and
    // omega and g_phiphi divide by it with terms that cancel there. With E = e^(2 psi),
    // G = e^(2 gamma'), c0 = 4 k alpha / (1 - alpha^2) and the identity
    //   4 CC^2 - (x^2 - 1)(1 - y^2) BB^2 = AA Q,
    //   Q = -s^2 (x-1)^4 a^2 b^2 + (x^2-1)(1+y)^4 a^2 - 2 s^2 (x^2-1)(x^2-y^2) a b
    //       + (x^2-1)(1-y)^4 b^2 - s^2 (x+1)^4     (a = aa, b = bb, s^2 = 1 - y^2),
    // the components are g_tt = -E AA/BB, g_tphi = (2k CC - c0 E AA)/BB,
    // g_phiphi = (-k^2 Q/E + 4k c0 CC - c0^2 E AA)/BB, g_thth = G rho^2 BB / (E (x^2 - y^2)
    // (1 - alpha^2)^2), g_rr = g_thth / Delta: the reference's expressions rearranged.
    const T al = q[2], k = q[3];
    const D2<T> y = d_cast<T>(Y);
    const D2<T> xm1 = d_cast<T>(XM1);
    const D2<T> xp1 = T(2) + xm1, x = T(1) + xm1;
    const D2<T> x2m1 = d_cast<T>(X2M1);
    const D2<T> s2 = {s * s, T(0), T(2) * s * c};
    const D2<T> aa = (-al) * d_exp(d_cast<T>(Ea));
    const D2<T> bb = al * d_exp(d_cast<T>(Eb));
    const D2<T> ab = aa * bb;
    const D2<T> ab1 = T(1) + ab;
    const D2<T> bma = bb - aa;
    const D2<T> AA = x2m1 * ab1 * ab1 - s2 * bma * bma;
    const D2<T> b1 = xp1 + xm1 * ab;
    const D2<T> yp1 = T(1) + y, ym1 = T(1) + -y;  // 1 + y, 1 - y
    const D2<T> b2 = yp1 * aa + ym1 * bb;
    const D2<T> BB = b1 * b1 + b2 * b2;
    const D2<T> CC = x2m1 * ab1 * (bma - y * (aa + bb)) + s2 * bma * (ab1 + x * (T(1) + -ab));
    const D2<T> xm1_2 = xm1 * xm1, xp1_2 = xp1 * xp1, yp1_2 = yp1 * yp1, ym1_2 = ym1 * ym1;
    const D2<T> x2my2 = x2m1 + s2;  // x^2 - y^2
    const D2<T> Q = -(s2 * (xm1_2 * xm1_2) * ab * ab) + x2m1 * (yp1_2 * yp1_2) * aa * aa -
                    T(2) * (s2 * x2m1 * x2my2 * ab) + x2m1 * (ym1_2 * ym1_2) * bb * bb - s2 * (xp1_2 * xp1_2);
    const T om2 = T(1) - al * al, c0 = T(4) * k * al * rcp(om2);
    const D2<T> E = d_exp(d_cast<T>(psi2)), Ei = d_exp(d_cast<T>(-psi2));
    const D2<T> iBB = inv(BB);
    const D2<T> EAA = E * AA;
    const D2<T> del = {dp * dm, dp + dm, T(0)};
    const D2<T> rho2 = del + (k * k) * s2;
    const D2<T> g_tt = -(EAA * iBB);
    const D2<T> g_tp = ((T(2) * k) * CC - c0 * EAA) * iBB;
    const D2<T> g_pp = ((-(k * k)) * (Q * Ei) + (T(4) * k * c0) * CC - (c0 * c0) * EAA) * iBB;
    const D2<T> g_hh = d_exp(d_cast<T>(gp2)) * rho2 * BB * Ei * inv((om2 * om2) * x2my2);
    const D2<T> g_rr = g_hh * inv(del);
    dr = {g_tt.r, g_tp.r, g_rr.r, g_hh.r, g_pp.r};
    dh = {g_tt.h, g_tp.h, g_rr.h, g_hh.h, g_pp.h};
    const T idet = rcp(del.v * s2.v);  // the (t, phi) block's determinant is -Delta sin^2
    gu = {-g_pp.v * idet, g_tp.v * idet, rcp(g_rr.v), rcp(g_hh.v), -g_tt.v * idet};
    grr = g_rr.v;
}

// The largest of |2 alpha3 (1 - (x - y) S1)|, |2 alpha3 (-1 + (x + y) S2)|, |2 psi| and
// |2 gamma'| (the arguments of Manko-Novikov's exponentials, mn_eval) over theta at
// radius r (n_theta - 1 interior angles, evenly spaced), in FP64 (host). FP32 carries an
// exponent with absolute error ~6e-8 times its size, which becomes the relative error of
// the metric; near the horizon the exponents grow without bound and the metric leaves
// FP32's range.
inline double mn_max_exponent(const MetricConst& M, double r, int n_theta = 180) {
    const double a3 = M.q[1], k = M.q[3];
    double worst = 0.0;
    for (int i = 1; i < n_theta; ++i) {
        const double th = 3.14159265358979323846 * i / n_theta, y = std::cos(th), s = std::sin(th);
        const double x = (r - 1.0) / k, x2m1 = (x - 1.0) * (x + 1.0);
        const double R = std::sqrt(x2m1 + y * y), iR = 1.0 / R, t = x * y * iR, t2 = t * t;
        const double P1 = t, P2 = 0.5 * (3 * t2 - 1), P3 = 0.5 * t * (5 * t2 - 3), P4 = 0.125 * (35 * t2 * t2 - 30 * t2 + 3);
        const double S1 = iR * (1 + iR * (P1 + iR * (P2 + iR * P3))), S2 = iR * (1 + iR * (-P1 + iR * (P2 - iR * P3)));
        const double iR4 = iR * iR * iR * iR;
        const double ea = 2 * a3 * (1 - (x - y) * S1), eb = 2 * a3 * (-1 + (x + y) * S2);
        const double psi = a3 * P3 * iR4;
        const double gp = 2 * a3 * a3 * (P4 * P4 - P3 * P3) * iR4 * iR4 +
                          2 * a3 * (-y + iR * (x * P1 + iR * (-y * P2 + iR * x * P3))) * iR;
        (void)s;
        const double m = std::fmax(std::fmax(std::fabs(ea), std::fabs(eb)), std::fmax(std::fabs(2 * psi), std::fabs(2 * gp)));
        if (!(m <= worst)) worst = m;  // a NaN counts as unbounded
    }
    return worst;
}

// The radius inside which Manko-Novikov's mixed-precision right-hand side is taken in
// FP64: scanning inward from r = 10^4 (r - r_+ shrinking by 0.8 per step), the first
// radius at which an exponent exceeds max_exponent, refined by bisection on r - r_+ to
// 0.1 %, then r - r_+ times 1.1 (everything inside it uses FP64). ~0.5 ms on the host.
constexpr double kMnMaxFp32Exponent = 8.0;
inline double mn_fp64_radius(const MetricConst& M, double max_exponent) {
    const double rp = 1.0 + M.q[3];
    double out = 1e4 - rp;  // r - r_+ known to be within bounds
    double in = out;
    while (in > 1e-9 && mn_max_exponent(M, rp + in) <= max_exponent) {
        out = in;
        in *= 0.8;
    }
    if (!(in > 1e-9)) return rp;
    while (out - in > 1e-3 * out) {  // exceeds at rp + in, within bounds at rp + out
        const double mid = 0.5 * (in + out);
        if (mn_max_exponent(M, rp + mid) <= max_exponent) out = mid; else in = mid;
    }
    return rp + out * 1.1;
}

template <>
struct MixedMetric<kMankoNovikov> {
    static constexpr bool kAvailable = true;
    static constexpr bool kInline = false;
    // from the position in T only (FP64 callers)
    template <typename T>
    static FOORT_HD void eval(const T* q, T r, T dp, T dm, T s, T c, G5T<T>& dr, G5T<T>& dh, G5T<T>& gu, T& grr) {
        (void)r;
        mn_eval<T>(q, double(r), double(dp), double(s), double(c), dp, dm, s, c, dr, dh, gu, grr);
    }
    // with the position also in FP64 (the mixed kernel has it in float-float)
    template <typename T>
    static FOORT_HD void eval_hi(const T* q, double rd, double dpd, double sd, double cd, T dp, T dm, T s, T c,
                                 G5T<T>& dr, G5T<T>& dh, G5T<T>& gu, T& grr) {
        (void)rd;
        mn_eval<T>(q, rd, dpd, sd, cd, dp, dm, s, c, dr, dh, gu, grr);
    }
};

// The plugins' constants q[]: the metric constants of make_metric_const for Kerr,
// Johannsen and flat space; for Rasheed-Larsen the slots of its rewritten form
// (gen_christoffel.py), from its rescaled m, a, p, q.
inline void mixed_metric_constants(int id, const MetricConst& M, double out[kMixedQ]) {
    for (int i = 0; i < kMixedQ; ++i) out[i] = 0.0;
    if (id == kRasheedLarsen) {
        const double a = M.q[0], m = M.q[1], p = M.q[2], qq = M.q[3];
        FOORT_MIXED_CONSTANTS_RASHEEDLARSEN
        return;
    }
    for (int i = 0; i < 6; ++i) out[i] = M.q[i];
}

// r_+ and r_- of the plugin's Delta = (r - r_+)(r - r_-) = r^2 - 2 m r + a^2: m = 1 for
// Kerr and Johannsen, Rasheed-Larsen's rescaled m; 1 -+ k for Manko-Novikov; none for
// flat space.
inline void mixed_horizons(int id, const MetricConst& M, double& rp, double& rm) {
    rp = rm = 0.0;
    if (id == kKerr || id == kJohannsen) {
        const double a = M.q[0];
        rp = 1.0 + std::sqrt(1.0 - a * a);
        rm = 1.0 - std::sqrt(1.0 - a * a);
    } else if (id == kRasheedLarsen) {
        const double a = M.q[0], m = M.q[1];
        rp = m + std::sqrt(m * m - a * a);
        rm = m - std::sqrt(m * m - a * a);
    } else if (id == kMankoNovikov) {  // Delta = (r - 1)^2 - k^2
        rp = 1.0 + M.q[3];
        rm = 1.0 - M.q[3];
    }
}

// d_x1 g and g^11 in log-r mode (x1 = ln r): d_x1 = r d_r, g_11 = r^2 g_rr,
// g^11 = g^rr / r^2.
template <typename T>
FOORT_HD void to_log_r(T r, T grr, G5T<T>& dr, G5T<T>& dh, G5T<T>& gu) {
    const T r2 = r * r;
    dr.tt *= r;
    dr.tp *= r;
    dr.hh *= r;
    dr.pp *= r;
    dr.rr = r * (T(2) * r * grr + r2 * dr.rr);
    dh.rr *= r2;
    gu.rr /= r2;
}

// a^mu = -1/2 g^{mu s} (2 u^n d_n g_{s p} u^p - d_s g_{n p} u^n u^p), with d_1 g, d_2 g
// the derivatives in the integration coordinates x1, x2.
template <typename T>
FOORT_HD void accel_lagrange(const G5T<T>& d1, const G5T<T>& d2, const G5T<T>& gu, const T u[4], T a[4]) {
    const T w1t = d1.tt * u[0] + d1.tp * u[3], w1r = d1.rr * u[1], w1h = d1.hh * u[2], w1p = d1.tp * u[0] + d1.pp * u[3];
    const T w2t = d2.tt * u[0] + d2.tp * u[3], w2r = d2.rr * u[1], w2h = d2.hh * u[2], w2p = d2.tp * u[0] + d2.pp * u[3];
    const T q1 = u[0] * w1t + u[1] * w1r + u[2] * w1h + u[3] * w1p;
    const T q2 = u[0] * w2t + u[1] * w2r + u[2] * w2h + u[3] * w2p;
    const T Ft = T(2) * (u[1] * w1t + u[2] * w2t);
    const T Fp = T(2) * (u[1] * w1p + u[2] * w2p);
    const T Fr = T(2) * (u[1] * w1r + u[2] * w2r) - q1;
    const T Fh = T(2) * (u[1] * w1h + u[2] * w2h) - q2;
    a[0] = T(-0.5) * (gu.tt * Ft + gu.tp * Fp);
    a[3] = T(-0.5) * (gu.tp * Ft + gu.pp * Fp);
    a[1] = T(-0.5) * gu.rr * Fr;
    a[2] = T(-0.5) * gu.hh * Fh;
}

// The acceleration in log-r mode (x1 = ln r). There d_x1 g_11 = 2 r^2 g_rr + r^3 d_r g_rr,
// and its first part contributes -1/2 g^11 (2 r^2 g_rr) (u^1)^2 = -(u^1)^2 to a^1 exactly:
// a pure coordinate term, at r = 1000 a thousand times the physical rest of a^1. It is
// added as -(u^1)^2 rather than through g^rr g_rr, which in FP32 differs from 1 by a
// few 1e-7: that would put a few 1e-7 of relative error on the dominant term of every
// step's radial acceleration.
template <typename T>
FOORT_HD void scale_log_r(T r, G5T<T>& dr, G5T<T>& dh, G5T<T>& gu) {
    const T r2 = r * r;
    dr.tt *= r;
    dr.tp *= r;
    dr.hh *= r;
    dr.pp *= r;
    dr.rr *= r2 * r;  // r^3 d_r g_rr: the physical part of d_x1 g_11
    dh.rr *= r2;
    gu.rr /= r2;
}
template <typename T>
FOORT_HD void accel_log_r(T r, G5T<T>& dr, G5T<T>& dh, G5T<T>& gu, const T u[4], T a[4]) {
    scale_log_r(r, dr, dh, gu);
    accel_lagrange(dr, dh, gu, u, a);
    a[1] -= u[1] * u[1];
}

}  // namespace foort
