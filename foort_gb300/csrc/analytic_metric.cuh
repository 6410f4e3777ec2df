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
// reciprocal (which sit on the critical path of every right-hand side). Infinite r0
// (x = 0) is passed through, where the refinement would give NaN.
FOORT_HD float rcp(float x) {
#ifdef __CUDA_ARCH__
    float r0;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r0) : "f"(x));
    const float r1 = __fmaf_rn(r0, __fmaf_rn(-x, r0, 1.0f), r0);
    return isinf(r0) ? r0 : r1;
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
// cache, and C2's five rounds take 695 ms inlined against 786 ms called on GB300.
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
// Kerr and Johannsen, Rasheed-Larsen's rescaled m; none for flat space.
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
