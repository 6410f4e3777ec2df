// Mixed-precision integration kernel: FP32 bulk, compensated state.
//
// Per lane the state (t, r, theta, phi), the 4-velocity and the affine parameter are
// float-float pairs (hi + lo, ~48 significant bits), updated each step with error-free
// transformations (Knuth's TwoSum, FMA-based TwoProd), so that rounding does not
// accumulate over the 10^4-10^5 steps of a geodesic. The right-hand side runs in FP32:
// analytic metric derivatives (gen_christoffel.inc) combined in Lagrangian form,
//     a^mu = -1/2 g^{mu s} (2 u^n d_n g_{s p} u^p - d_s g_{n p} u^n u^p),
// which needs only d_r g_ij and d_theta g_ij of the five non-zero components. The
// near-horizon factor Delta = (r - r_+)(r - r_-) is formed from the compensated radius.
//
// Decisions (terminations, equator crossings, closest radius) are taken on the
// compensated state; with DECIDE64 they are taken in FP64 on its exact double value,
// as the reference takes them, otherwise by float-float comparisons that agree with
// the FP64 ones except within 2^-48 (relative) of a threshold. Optionally, lanes inside
// the strong-field radius I.r_fp64 take their whole step in FP64 (step_fp64): there the
// ray bends most, and bending amplifies every error a step makes.
#pragma once

#include "analytic_metric.cuh"
#include "kernel_common.cuh"

namespace foort {

// ---- float-float arithmetic --------------------------------------------------------
struct ff {
    float hi, lo;
};

__device__ __forceinline__ ff two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}
__device__ __forceinline__ ff fast_two_sum(float a, float b) {  // |a| >= |b|
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ ff ff_add_f(ff a, float b) {
    ff s = two_sum(a.hi, b);
    s.lo = __fadd_rn(s.lo, a.lo);
    return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ ff ff_add(ff a, ff b) {
    ff s = two_sum(a.hi, b.hi);
    ff t = two_sum(a.lo, b.lo);
    s.lo = __fadd_rn(s.lo, t.hi);
    s = fast_two_sum(s.hi, s.lo);
    s.lo = __fadd_rn(s.lo, t.lo);
    return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ ff ff_neg(ff a) { return {-a.hi, -a.lo}; }
// exact product of two floats as a float-float (FMA-based TwoProd)
__device__ __forceinline__ ff two_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    return {p, __fmaf_rn(a, b, -p)};
}
__device__ __forceinline__ bool ff_lt(ff a, ff b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ bool ff_neg_sign(ff a) { return a.hi < 0.f || (a.hi == 0.f && a.lo < 0.f); }
__device__ __forceinline__ ff ff_abs(ff a) { return ff_neg_sign(a) ? ff_neg(a) : a; }
__device__ __forceinline__ double ff_d(ff a) { return static_cast<double>(a.hi) + static_cast<double>(a.lo); }
__device__ __forceinline__ float ff_f(ff a) { return a.hi + a.lo; }
__host__ __device__ inline void ff_split(double d, float& hi, float& lo) {
    hi = static_cast<float>(d);
    lo = static_cast<float>(d - static_cast<double>(hi));
}
__device__ __forceinline__ ff ff_of(const float* p) { return {p[0], p[1]}; }
__device__ __forceinline__ ff ff_from_d(double d) {
    const float hi = __double2float_rn(d);
    return {hi, __double2float_rn(d - static_cast<double>(hi))};
}
// a + (bh + bl) for a small second term bl (|bl| well below |bh|, or bh = 0): bh joins
// a's high part exactly (TwoSum), bl its low part.
__device__ __forceinline__ ff ff_add_f2(ff a, float bh, float bl) {
    ff s = two_sum(a.hi, bh);
    s.lo = __fadd_rn(s.lo, __fadd_rn(a.lo, bl));
    return fast_two_sum(s.hi, s.lo);
}

// The right-hand side in two parts: the metric part depends on the position only (the
// expensive part: angle, metric derivatives, inverse metric), the contraction with the
// velocity is cheap. Splitting them lets RK4 evaluate the metric at the next stage's
// position while the current stage's contraction waits for its velocity.
template <typename T>
struct MetricAt {
    G5T<T> d1, d2, gu;  // d_x1 g, d_theta g (scaled to x1 = ln r in log-r mode), g^uu
};

// Metric part at (x1, theta). `x1` and `th` are the compensated coordinates (x1 = r, or
// ln r in log-r mode); r_+ / r_- (and their logarithms) come from the image constants so
// that dp = r - r_+ and dm = r - r_- are accurate near the horizon.
template <int MID, typename T>
__device__ __forceinline__ MetricAt<T> metric_part(const T* q, const MixedConst& mc, bool rlog, ff x1, ff th) {
    T r, dp, dm;
    if (!rlog) {
        r = T(x1.hi) + T(x1.lo);
        dp = T(__fsub_rn(x1.hi, mc.rp[0])) + (T(x1.lo) - T(mc.rp[1]));
        dm = T(__fsub_rn(x1.hi, mc.rm[0])) + (T(x1.lo) - T(mc.rm[1]));
    } else {
        // exp(hi + lo) = exp(hi) (1 + lo): rounding ln r (up to 7 at r = 1000) to one
        // float first would cost 2.4e-7 of relative accuracy in r
        const T yp = (T(x1.hi) - T(mc.lrp[0])) + (T(x1.lo) - T(mc.lrp[1]));  // ln(r / r_+)
        if constexpr (sizeof(T) == sizeof(float)) {
            const float e = expf(x1.hi);
            r = fmaf(e, x1.lo, e);
            // r - r_+ from expm1 only where it cancels (r < e r_+): beyond, the float
            // argument's rounding (2.4e-7 at ln(r / r_+) = 6) would enter Delta and g_rr
            // as a relative error of that size. r - r_- never cancels (r >= r_+ > r_-).
            dp = (yp > 1.f) ? r - mc.rp[0] : mc.rp[0] * expm1f(yp);
            dm = r - mc.rm[0];
        } else {
            r = exp(T(x1.hi) + T(x1.lo));
            dp = T(mc.rpv) * expm1(yp);
            dm = (mc.rmv > 0.0) ? T(mc.rmv) * expm1((T(x1.hi) - T(mc.lrm[0])) + (T(x1.lo) - T(mc.lrm[1]))) : r;
        }
    }
    T s, c;
    if constexpr (sizeof(T) == sizeof(float)) {
        ff_sincos(th.hi, th.lo, s, c);
    } else {
        sincos(T(th.hi) + T(th.lo), &s, &c);
    }
    MetricAt<T> m;
    T grr;
    if constexpr (MID == kMankoNovikov && sizeof(T) == sizeof(float)) {
        // the plugin's FP64 block (its exponents) takes the position in FP64
        const double x1d = double(x1.hi) + double(x1.lo);
        const double rd = rlog ? exp(x1d) : x1d;
        double sd, cd;
        sincos(double(th.hi) + double(th.lo), &sd, &cd);
        MixedMetric<MID>::template eval_hi<T>(q, rd, rd - mc.rpv, sd, cd, dp, dm, s, c, m.d1, m.d2, m.gu, grr);
    } else {
        MixedMetric<MID>::template eval<T>(q, r, dp, dm, s, c, m.d1, m.d2, m.gu, grr);
    }
    if (rlog) scale_log_r(r, m.d1, m.d2, m.gu);
    return m;
}

// Metric part in FP64 at a double position (the strong-field steps). r - r_+ and r - r_-
// are formed in FP64 (in log-r mode through expm1 of ln(r / r_+)), so Delta keeps its
// relative accuracy down to the horizon.
template <int MID>
__device__ __forceinline__ MetricAt<double> metric_part_d(const double* q, const MixedConst& mc, bool rlog, double x1,
                                                          double th) {
    double r, dp, dm;
    if (!rlog) {
        r = x1;
        dp = x1 - mc.rpv;
        dm = x1 - mc.rmv;
    } else {
        r = exp(x1);
        const double lrp = double(mc.lrp[0]) + double(mc.lrp[1]);
        dp = (mc.rpv > 0.0) ? mc.rpv * expm1(x1 - lrp) : r;
        dm = (mc.rmv > 0.0) ? mc.rmv * expm1(x1 - (double(mc.lrm[0]) + double(mc.lrm[1]))) : r;
    }
    double s, c;
    sincos(th, &s, &c);
    MetricAt<double> m;
    double grr;
    MixedMetric<MID>::template eval<double>(q, r, dp, dm, s, c, m.d1, m.d2, m.gu, grr);
    if (rlog) scale_log_r(r, m.d1, m.d2, m.gu);
    return m;
}

// Contraction with the velocity (accel_lagrange; in log-r mode plus the exact coordinate
// term -(u^1)^2 of accel_log_r).
template <typename T>
__device__ __forceinline__ void accel_part(const MetricAt<T>& m, bool rlog, const T u[4], T a[4]) {
    accel_lagrange(m.d1, m.d2, m.gu, u, a);
    if (rlog) a[1] -= u[1] * u[1];
}

// Right-hand side at (x1, theta) with velocity u.
template <int MID, typename T>
__device__ __forceinline__ void rhs_analytic(const T* q, const MixedConst& mc, bool rlog, ff x1, ff th, const T u[4],
                                             T a[4]) {
    accel_part(metric_part<MID, T>(q, mc, rlog, x1, th), rlog, u, a);
}

// The called form of the FP32 right-hand side. Velocity and acceleration travel by value
// so that the call passes them in registers (arrays would go through the stack: a local
// store and load on the critical path of every evaluation; 7 % of a launch of the Kerr
// a = 0.99 adaptive run on its 509² grid).
struct F4 {
    float x, y, z, w;
};
template <int MID>
__device__ __noinline__ F4 rhs_f32_called(const float* q, const MixedConst& mc, bool rlog, ff x1, ff th, F4 uv) {
    const float u[4] = {uv.x, uv.y, uv.z, uv.w};
    float a[4];
    rhs_analytic<MID, float>(q, mc, rlog, x1, th, u, a);
    return F4{a[0], a[1], a[2], a[3]};
}

// The called form of the FP32 metric part (Verlet keeps it from step to step).
template <int MID>
__device__ __noinline__ MetricAt<float> metric_part_called(const float* q, const MixedConst& mc, bool rlog, ff x1,
                                                           ff th) {
    return metric_part<MID, float>(q, mc, rlog, x1, th);
}

// The increments of one step taken wholly in FP64, with its counts.
struct StepD {
    double dx[4], dv[4];
    double h;
    uint32_t rhs, err;
};

// One step in FP64 (the strong-field region): the reference's RK4 (Integrators.cpp:51-94)
// or velocity Verlet (Integrators.cpp:99-152) and its step rule (Integrators.cpp:34-46),
// with the analytic right-hand side, from the position (x1, theta) and the velocity u
// as doubles. Everything a step carries -- stage positions and velocities, the
// accelerations, the increments -- stays in FP64: an FP64 right-hand side fed with
// velocities rounded to FP32 would keep their 6e-8 relative error, which strongly bent
// rays amplify as much as the FP32 right-hand side's own.
template <int MID, int INTEG>
__device__ __noinline__ StepD step_fp64(const ImageConst& I, const RunConst& R, double x1, double th, double u0,
                                        double u1, double u2, double u3) {
    const bool rlog = R.rlog != 0;
    const double* q = I.qa;
    const double u[4] = {u0, u1, u2, u3};
    const double xs[4] = {0.0, x1, th, 0.0};
    StepD d;
    d.err = 0;
    const double h = adaptive_step_fp64(R, xs, u);
    d.h = h;
    if (INTEG == FOORT_INTEGRATOR_RK4) {
        double k1[4], k2[4], k3[4], k4[4], us[4];
        const double hh = 0.5 * h;
        accel_part(metric_part_d<MID>(q, I.mx, rlog, x1, th), rlog, u, k1);
#pragma unroll
        for (int i = 0; i < 4; ++i) us[i] = u[i] + hh * k1[i];
        accel_part(metric_part_d<MID>(q, I.mx, rlog, x1 + hh * u[1], th + hh * u[2]), rlog, us, k2);
#pragma unroll
        for (int i = 0; i < 4; ++i) us[i] = u[i] + hh * k2[i];
        accel_part(metric_part_d<MID>(q, I.mx, rlog, x1 + hh * (u[1] + hh * k1[1]), th + hh * (u[2] + hh * k1[2])),
                   rlog, us, k3);
#pragma unroll
        for (int i = 0; i < 4; ++i) us[i] = u[i] + h * k3[i];
        accel_part(metric_part_d<MID>(q, I.mx, rlog, x1 + h * (u[1] + hh * k2[1]), th + h * (u[2] + hh * k2[2])),
                   rlog, us, k4);
        const double h6 = h / 6.0;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            d.dv[i] = (((k1[i] + k2[i] * 2) + k3[i] * 2) + k4[i]) * h6;
            d.dx[i] = u[i] * h + ((k1[i] + k2[i]) + k3[i]) * (h * h6);
        }
        d.rhs = 4;
        return d;
    }
    double a0[4], a1[4], vi[4];
    accel_part(metric_part_d<MID>(q, I.mx, rlog, x1, th), rlog, u, a0);
    const double hh2 = h * h / 2.0;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        d.dx[i] = u[i] * h + a0[i] * hh2;
        vi[i] = u[i] + a0[i] * h;
    }
    const MetricAt<double> mn = metric_part_d<MID>(q, I.mx, rlog, x1 + d.dx[1], th + d.dx[2]);
    accel_part(mn, rlog, vi, a1);
    const double h2 = h / 2.0;
#pragma unroll
    for (int i = 0; i < 4; ++i) d.dv[i] = (a0[i] + a1[i]) * h2;
    d.rhs = 2;
    if (R.vtol > 0.0) {
        const double tol2 = R.vtol * R.vtol;
        for (int it = 0;; ++it) {
            double num = 0.0, den = 0.0;
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const double nv = u[i] + d.dv[i];
                const double e = nv - vi[i];
                num += e * e;
                den += nv * nv;
            }
            if (!(num / den > tol2)) break;
            if (it >= R.verlet_cap) {
                d.err |= FOORT_ERR_VERLET_ITER;
                break;
            }
#pragma unroll
            for (int i = 0; i < 4; ++i) vi[i] = u[i] + d.dv[i];
            accel_part(mn, rlog, vi, a1);
#pragma unroll
            for (int i = 0; i < 4; ++i) d.dv[i] = (a0[i] + a1[i]) * h2;
            d.rhs += 1;
        }
    }
    return d;
}

// Integrators::GetAdaptiveStep (Integrators.cpp:34-46) in FP32. Written as
//     h = eps / ((|u1| + d) + (|u2| + d) / m + |u3 + d|),  m = min(theta, pi - theta),
// which is the reference's expression with eps factored out, with eps carried as a
// float-float pair: the step size then has no systematic bias against the FP64 kernel's
// (a bias would shift every ray's affine parameter, and strongly bent rays turn a shift
// into an error of their end points). h = eps / s is formed as eps m / d with
// d = m (s1 + s3) + s2 (s = s1 + s2 / m + s3, m = min(theta, pi - theta)), so that one
// reciprocal sits on the step's chain, and from that reciprocal with its residual:
// q0 = eps_hi m (1/d), then q = q0 + (eps_hi m - q0 d + eps_lo m) / d. Taking eps_hi
// times the rounded 1/s instead is biased: far from the hole s = |u^1| + ... lies just
// below 1, where floats are twice as dense as just above 1, so every other 1/s falls just
// past a rounding midpoint and rounds up, making h about 3e-8 too large on average; over
// 10^5 steps that moved the end points of a Kerr a = 0.99, 60° view by 1e-6 on a tenth
// of its rays. pi - theta is
// formed from theta's float-float parts: near the pole both round to the same float, and a
// zero m would collapse the step to the smallest step size.
__device__ __forceinline__ float adaptive_step_f32(const RunConst& R, const MixedConst& mc, ff th, const float v[4]) {
    // pi - theta to float accuracy: near theta = pi the high parts' difference is exact
    // (Sterbenz) and the low parts carry the rest
    const float t = ff_f(th), pt = __fadd_rn(__fsub_rn(mc.pi[0], th.hi), __fsub_rn(mc.pi[1], th.lo));
    const float m = fabsf((pt < t) ? pt : t);
    const float s1 = __fadd_rn(fabsf(v[1]), 1e-20f);
    const float s2 = __fadd_rn(fabsf(v[2]), 1e-20f);
    const float s3 = fabsf(__fadd_rn(v[3], 1e-20f));
    // eps / (s1 + s2 / m + s3) = eps m / (m (s1 + s3) + s2): one reciprocal on the chain
    // instead of two (1 / m, then 1 / s)
    const float den = __fmaf_rn(m, __fadd_rn(s1, s3), s2);
    const float inv = rcp(den);
    const float num = __fmul_rn(mc.eps[0], m);
    const float q0 = __fmul_rn(num, inv);
    const float res = __fmaf_rn(-q0, den, num);  // num - q0 den, exact
    const float h = __fmaf_rn(__fmaf_rn(mc.eps[1], m, res), inv, q0);
    const float hmin = mc.hmin;
    return (h < hmin) ? hmin : h;
}

// DecideUpdate with a step counter, without branches: every == 0, or the counter
// reaching every (and restarting).
template <typename C>
__device__ __forceinline__ bool decide_nb(uint64_t every, C& cnt) {
    const C next = cnt + 1;
    const bool hit = (every == 0) | (static_cast<uint64_t>(next) >= every);
    cnt = (every == 0) ? cnt : (hit ? C(0) : next);
    return hit;
}

// FOORT_MIXED_FP64_TURNING_POINTS: FP64 steps where the radial or the polar speed is
// below this fraction of the ray's angular motion.
constexpr float kTurningFraction = 0.05f;

template <int MID, int INTEG, bool DECIDE64>
struct MixedEngine {
    // step_pair exists for RK4 with an inlined plugin, without the strong-field FP64 steps
    // (kept out of it, their call raised the two-lane kernel from 111 to 158 registers)
    static constexpr bool kPairCapable = INTEG == FOORT_INTEGRATOR_RK4 && MixedMetric<MID>::kInline;

    struct Lane {
        ff x[4], v[4];
        ff lam;
        uint64_t steps;
        TermState T;
        // diagnostics on the compensated state
        int32_t quad, passes;
        StepCount cE, cC;
        ff prev;      // previous theta sample (hi = -1: none yet)
        ff rmin;      // closest radius so far; ln r in log-r mode
        bool has_rmin;
        uint32_t err = 0;
        uint32_t img = 0;
        uint32_t rhs = 0;
        uint32_t fp64 = 0;
        int32_t term = 0;
        GeoposRec gp;  // set by the loop before init (dst null: not recording)
        MetricAt<float> mc;  // Verlet: the metric part at the current (x1, theta)
    };

    // Verlet keeps the metric part from step to step unless lanes may switch to FP64 steps
    // (the strong-field radius, turning points).
    static __device__ __forceinline__ bool verlet_cached(const ImageConst& I, const RunConst& R) {
        return INTEG == FOORT_INTEGRATOR_VERLET && !(I.mx.r_fp64 > 0.f) &&
               !(R.mixed_options & FOORT_MIXED_FP64_TURNING_POINTS);
    }

    // The FP32 metric part at (x1, theta): inlined for the inlined plugins, called otherwise.
    static __device__ __forceinline__ MetricAt<float> metric(const ImageConst& I, bool rlog, ff x1, ff th) {
        if constexpr (MixedMetric<MID>::kInline) {
            return metric_part<MID, float>(I.mx.q, I.mx, rlog, x1, th);
        } else {
            return metric_part_called<MID>(I.mx.q, I.mx, rlog, x1, th);
        }
    }

    // GeodesicPosition sample of the compensated position (second pass only)
    static __device__ __forceinline__ void geopos(Lane& L, const RunConst& R, double lam) {
        double x[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) x[i] = ff_d(L.x[i]);
        geopos_sample(L.gp, R, x, lam, L.term);
    }

    static __device__ __forceinline__ void load_double(const Lane& L, double x[4], double v[4]) {
        for (int i = 0; i < 4; ++i) {
            x[i] = ff_d(L.x[i]);
            v[i] = ff_d(L.v[i]);
        }
    }

    static __device__ __forceinline__ void init(Lane& L, const ImageConst& I, const RunConst& R, const foort_pixel& p) {
        double x[4], v[4];
        initial_conditions(I, p, x, v);
        for (int i = 0; i < 4; ++i) {
            ff_split(x[i], L.x[i].hi, L.x[i].lo);
            ff_split(v[i], L.v[i].hi, L.v[i].lo);
        }
        L.lam = {0.f, 0.f};
        L.steps = 0;
        L.err = 0;
        L.term = FOORT_TERMCODE_CONTINUE;
        L.img = p.image;
        L.quad = 0;
        L.passes = 0;
        L.cE = 0;
        L.cC = 0;
        L.prev = {-1.f, 0.f};
        L.rmin = {-1.f, 0.f};
        L.has_rmin = false;
        L.T.cH = L.T.cB = L.T.cT = L.T.cTh = 0;
        L.T.tcur = 0;
        if (verlet_cached(I, R)) L.mc = metric(I, R.rlog != 0, L.x[1], L.x[2]);
        diags(L, I, R, true);  // Geodesic::Reset's start sample at lambda = 0
        if (L.gp.dst) geopos(L, R, 0.0);
    }

    // EquatorialPasses and ClosestRadius updates (Diagnostics.cpp:351-380, :427-446) on
    // the compensated state; FourColorScreen at termination (Diagnostics.cpp:159-200).
    static __device__ __forceinline__ void diags(Lane& L, const ImageConst& I, const RunConst& R, bool at_start) {
        const double lamd = at_start ? 0.0 : 1.0;  // only compared with 0 by DecideUpdate
        // FourColorScreen's quadrant and EquatorialPasses' sign at the Horizon are taken at
        // termination from the final state, which no later step changes (write()).
        if (R.diag_flags & FOORT_DIAG_EQUATORIAL_PASSES) {
            if (DECIDE64) {
                if (diag_decide(R.eq_every, R.eq_start, R.eq_finish, L.cE, lamd, L.term)) {
                    const double th = ff_d(L.x[2]);
                    if (fabs(th - kRefPi / 2.0) > kRefPi / 2.0 * R.eq_thr) {
                        const double pv = ff_d(L.prev);
                        if (pv > 0 && ((pv - kRefPi / 2.0) * (th - kRefPi / 2.0)) < 0.0) ++L.passes;
                        L.prev = L.x[2];
                    }
                }
            } else {
                // without branches: a crossing counts where the sample is taken, theta is
                // away from the equator and on the other side of it than the last sample
                const bool d = (R.eq_every > 0) ? decide_nb(R.eq_every, L.cE)
                                                 : diag_decide(R.eq_every, R.eq_start, R.eq_finish, L.cE, lamd, L.term);
                const ff dt = ff_add(L.x[2], ff_of(I.mx.mpio2));
                const bool upd = d & ff_lt(ff_of(I.mx.eqthr), ff_abs(dt));
                const ff dprev = ff_add(L.prev, ff_of(I.mx.mpio2));
                const bool cross = upd & (L.prev.hi > 0.f) & (ff_neg_sign(dprev) != ff_neg_sign(dt));
                L.passes += cross ? 1 : 0;
                L.prev.hi = upd ? L.x[2].hi : L.prev.hi;
                L.prev.lo = upd ? L.x[2].lo : L.prev.lo;
            }
        }
        if (R.diag_flags & FOORT_DIAG_CLOSEST_RADIUS) {
            const bool d = (R.cr_every > 0) ? decide_nb(R.cr_every, L.cC)
                                             : diag_decide(R.cr_every, R.cr_start, R.cr_finish, L.cC, lamd, L.term);
            // in log-r mode ln r is tracked (exp is monotonic) and exponentiated once
            const bool upd = d & (!L.has_rmin | ff_lt(L.x[1], L.rmin));
            L.rmin.hi = upd ? L.x[1].hi : L.rmin.hi;
            L.rmin.lo = upd ? L.x[1].lo : L.rmin.lo;
            L.has_rmin = L.has_rmin | upd;
        }
    }

    static __device__ __forceinline__ int terms(Lane& L, const ImageConst& I, const RunConst& R) {
        if (DECIDE64) {
            const double x1 = ff_d(L.x[1]);
            const double r = R.rlog ? exp(x1) : x1;
            return check_terms(R, I.m.rh, I.h_eps, r, ff_d(L.x[2]), L.T);
        }
        // Same order and cadence as check_terms; thresholds precomputed as float-float
        // (in ln r in log-r mode). Without branches: every termination's counter advances,
        // and the checks run in reverse order so that the first in the reference's order
        // wins (the reference stops at it, and a finished geodesic's counters are unused).
        int code = FOORT_TERMCODE_CONTINUE;
        if (R.term_flags & FOORT_TERM_THETA_SINGULARITY) {
            const bool d = decide_nb(R.th_every, L.T.cTh);
            const ff e = ff_of(I.mx.theps);
            const bool hit = ff_lt(ff_abs(L.x[2]), e) | ff_lt(ff_abs(ff_add(ff_of(I.mx.pi), ff_neg(L.x[2]))), e);
            code = (d & hit) ? FOORT_TERMCODE_THETA_SINGULARITY : code;
        }
        if (R.term_flags & FOORT_TERM_TIMEOUT) {
            const bool d = decide_nb(R.t_every, L.T.cT);
            const bool hit = L.T.tcur >= R.t_max;
            code = (d & hit) ? FOORT_TERMCODE_TIMEOUT : code;
            L.T.tcur += (d & !hit) ? 1u : 0u;
        }
        if (R.term_flags & FOORT_TERM_BOUNDARY_SPHERE) {
            const bool d = decide_nb(R.b_every, L.T.cB);
            code = (d & ff_lt(ff_of(I.mx.bthr), L.x[1])) ? FOORT_TERMCODE_BOUNDARY_SPHERE : code;
        }
        if (R.term_flags & FOORT_TERM_HORIZON) {
            const bool d = decide_nb(R.h_every, L.T.cH);
            const bool hit = ff_lt(L.x[1], ff_of(I.mx.hthr)) | ((I.m.rh == 0.0) & ff_lt(L.x[1], ff_of(I.mx.hthr0)));
            code = (d & hit) ? FOORT_TERMCODE_HORIZON : code;
        }
        return code;
    }

    // A right-hand side through the plugin's FP32 form (inlined or called).
    static __device__ __forceinline__ void rhs(const ImageConst& I, const RunConst& R, ff x1, ff th, const float u[4],
                                               float a[4]) {
        const bool rlog = R.rlog != 0;
        if (MixedMetric<MID>::kInline) {
            rhs_analytic<MID, float>(I.mx.q, I.mx, rlog, x1, th, u, a);
        } else {
            const F4 r = rhs_f32_called<MID>(I.mx.q, I.mx, rlog, x1, th, F4{u[0], u[1], u[2], u[3]});
            a[0] = r.x;
            a[1] = r.y;
            a[2] = r.z;
            a[3] = r.w;
        }
    }

    // Whether this step is taken in FP64: lanes inside the strong-field radius r_fp64
    // (ln r in log-r mode; 0 = never), decided on the step's starting state.
    // With FOORT_MIXED_FP64_TURNING_POINTS, also near a turning point of r or of theta,
    // measured against the ray's own angular motion w = (u^theta, sin(theta) u^phi): a
    // radial turning point where |dr/dlambda| < kTurningFraction r |w|, a polar one where
    // |u^theta| < kTurningFraction |sin(theta) u^phi|.
    static __device__ __forceinline__ bool in_fp64_region(const ImageConst& I, const RunConst& R, const Lane& L) {
        if (I.mx.r_fp64 > 0.f && L.x[1].hi < I.mx.r_fp64) return true;
        if (R.mixed_options & FOORT_MIXED_FP64_TURNING_POINTS) {
            const float r = R.rlog ? __expf(L.x[1].hi) : L.x[1].hi;
            const float vr = R.rlog ? fabsf(L.v[1].hi) * r : fabsf(L.v[1].hi);
            const float vth = fabsf(L.v[2].hi), vph = fabsf(__sinf(L.x[2].hi) * L.v[3].hi);
            return vr < kTurningFraction * r * (vth + vph) || vth < kTurningFraction * vph;
        }
        return false;
    }

    // A step in FP64 (step_fp64) applied to the compensated state. `count`: this lane
    // counts the step's right-hand sides (both lanes of a pair take the same step).
    static __device__ __forceinline__ bool step_d(Lane& L, const ImageConst& I, const RunConst& R, bool count) {
        const StepD d = step_fp64<MID, INTEG>(I, R, ff_d(L.x[1]), ff_d(L.x[2]), ff_d(L.v[0]), ff_d(L.v[1]),
                                              ff_d(L.v[2]), ff_d(L.v[3]));
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            L.x[i] = ff_from_d(ff_d(L.x[i]) + d.dx[i]);
            L.v[i] = ff_from_d(ff_d(L.v[i]) + d.dv[i]);
        }
        if (count) {
            L.rhs += d.rhs;
            ++L.fp64;
        }
        L.err |= d.err;
        return after_step(L, I, R, ff_add(L.lam, ff_from_d(d.h)));
    }

    // One Geodesic::Update (Geodesic.cpp:61-88) through the integrator's step. Inside the
    // strong-field radius the whole step runs in FP64 (step_d). Otherwise the common cases
    // run inline: RK4 with an inlined plugin (stages reordered) and Verlet with its kept
    // metric part. Everything that evaluates right-hand sides through rhs() -- RK4 with a
    // called plugin, Verlet where the strong-field radius is set -- runs in step_general,
    // out of line: kept in the kernel, its calls' register needs made the Johannsen Verlet
    // kernel 22 % slower on GB300 although it never ran them.
    static __device__ __forceinline__ bool step(Lane& L, const ImageConst& I, const RunConst& R) {
        if (in_fp64_region(I, R, L)) return step_d(L, I, R, true);
        float uf[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) uf[i] = ff_f(L.v[i]);
        const float h = adaptive_step_f32(R, I.mx, L.x[2], uf);
        if (INTEG == FOORT_INTEGRATOR_VERLET && verlet_cached(I, R)) return step_verlet_cached(L, I, R, h, uf);
        if (INTEG == FOORT_INTEGRATOR_RK4 && MixedMetric<MID>::kInline) return step_rk4_inline(L, I, R, h, uf);
        const Incr d = step_general(I, R, L.x[1], L.x[2], L.v[1], L.v[2], F4{uf[0], uf[1], uf[2], uf[3]}, h);
        L.rhs += d.rhs;
        L.err |= d.err;
        return advance(L, I, R, h, d.du, d.dxc);
    }

    // RK4 with the inlined plugin. The stage positions need only the velocities of earlier
    // stages: x + h/2 u (stage 2) none, x + h/2 (u + h/2 k1) (stage 3) k1, x + h (u + h/2 k2)
    // (stage 4) k2. So the metric part of stage 2 runs beside stage 1's, and those of stages
    // 3 and 4 beside the contractions of stages 2 and 3: the dependent chain of a step is
    // two metric evaluations and three contractions instead of four of each. Same
    // operations, same results.
    static __device__ __forceinline__ bool step_rk4_inline(Lane& L, const ImageConst& I, const RunConst& R, float h,
                                                           const float uf[4]) {
        float k1[4], k2[4], k3[4], k4[4], us[4], du[4], dxc[4];
        const float hh = 0.5f * h;
        const bool rlog = R.rlog != 0;
        const MetricAt<float> m1 = metric_part<MID, float>(I.mx.q, I.mx, rlog, L.x[1], L.x[2]);
        const MetricAt<float> m2 = metric_part<MID, float>(I.mx.q, I.mx, rlog, ff_add_f(L.x[1], hh * uf[1]),
                                                           ff_add_f(L.x[2], hh * uf[2]));
        accel_part(m1, rlog, uf, k1);
#pragma unroll
        for (int i = 0; i < 4; ++i) us[i] = uf[i] + hh * k1[i];
        const MetricAt<float> m3 = metric_part<MID, float>(I.mx.q, I.mx, rlog, ff_add_f(L.x[1], hh * (uf[1] + hh * k1[1])),
                                                           ff_add_f(L.x[2], hh * (uf[2] + hh * k1[2])));
        accel_part(m2, rlog, us, k2);
#pragma unroll
        for (int i = 0; i < 4; ++i) us[i] = uf[i] + hh * k2[i];
        const MetricAt<float> m4 = metric_part<MID, float>(I.mx.q, I.mx, rlog, ff_add_f(L.x[1], h * (uf[1] + hh * k2[1])),
                                                           ff_add_f(L.x[2], h * (uf[2] + hh * k2[2])));
        accel_part(m3, rlog, us, k3);
#pragma unroll
        for (int i = 0; i < 4; ++i) us[i] = uf[i] + h * k3[i];
        accel_part(m4, rlog, us, k4);
        rk4_combine(h, k1, k2, k3, k4, du, dxc);
        L.rhs += 4;
        return advance(L, I, R, h, du, dxc);
    }

    // The increments of one step taken by step_general, with its counts.
    struct Incr {
        float du[4], dxc[4];
        uint32_t rhs, err;
    };

    // RK4 (Integrators.cpp:51-94) and velocity Verlet (Integrators.cpp:99-152) through
    // rhs(), from the coordinates x1, theta and the velocity; in Verlet the velocity change
    // of each iteration is formed as h/2 (a1_new - a1_old), free of cancellation.
    static __device__ __noinline__ Incr step_general(const ImageConst& I, const RunConst& R, ff x1, ff th, ff v1, ff v2,
                                                     F4 u4, float h) {
        Incr d;
        d.err = 0;
        const float uf[4] = {u4.x, u4.y, u4.z, u4.w};
        if (INTEG == FOORT_INTEGRATOR_RK4) {
            float k1[4], k2[4], k3[4], k4[4], us[4];
            const float hh = 0.5f * h;
            rhs(I, R, x1, th, uf, k1);
#pragma unroll
            for (int i = 0; i < 4; ++i) us[i] = uf[i] + hh * k1[i];
            rhs(I, R, ff_add_f(x1, hh * uf[1]), ff_add_f(th, hh * uf[2]), us, k2);
#pragma unroll
            for (int i = 0; i < 4; ++i) us[i] = uf[i] + hh * k2[i];
            rhs(I, R, ff_add_f(x1, hh * (uf[1] + hh * k1[1])), ff_add_f(th, hh * (uf[2] + hh * k1[2])), us, k3);
#pragma unroll
            for (int i = 0; i < 4; ++i) us[i] = uf[i] + h * k3[i];
            rhs(I, R, ff_add_f(x1, h * (uf[1] + hh * k2[1])), ff_add_f(th, h * (uf[2] + hh * k2[2])), us, k4);
            rk4_combine(h, k1, k2, k3, k4, d.du, d.dxc);
            d.rhs = 4;
            return d;
        }
        float a0[4], a1[4], vi[4];
        rhs(I, R, x1, th, uf, a0);
        const float hh2 = 0.5f * h * h;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            d.dxc[i] = hh2 * a0[i];
            vi[i] = uf[i] + h * a0[i];
        }
        const ff x1n = ff_add_f(ff_add(x1, two_prod(h, v1.hi)), __fmaf_rn(h, v1.lo, d.dxc[1]));
        const ff thn = ff_add_f(ff_add(th, two_prod(h, v2.hi)), __fmaf_rn(h, v2.lo, d.dxc[2]));
        rhs(I, R, x1n, thn, vi, a1);
        d.rhs = 2;
        const float h2 = 0.5f * h;
#pragma unroll
        for (int i = 0; i < 4; ++i) d.du[i] = h2 * (a0[i] + a1[i]);
        if (I.mx.vtol2 > 0.f) {
            const float tol2 = I.mx.vtol2;
            float dv[4];  // first correction: nv - vi = h/2 (a1 - a0)
#pragma unroll
            for (int i = 0; i < 4; ++i) dv[i] = h2 * (a1[i] - a0[i]);
            for (int it = 0;; ++it) {
                float num = 0.f, den = 0.f;
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const float nvi = uf[i] + d.du[i];
                    num += dv[i] * dv[i];
                    den += nvi * nvi;
                }
                if (!(num > tol2 * den)) break;  // num / den > tol2 with den = |v|^2 > 0
                if (it >= R.verlet_cap) {
                    d.err |= FOORT_ERR_VERLET_ITER;
                    break;
                }
                float a1n[4];
#pragma unroll
                for (int i = 0; i < 4; ++i) vi[i] = uf[i] + d.du[i];
                rhs(I, R, x1n, thn, vi, a1n);
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    dv[i] = h2 * (a1n[i] - a1[i]);
                    a1[i] = a1n[i];
                    d.du[i] = h2 * (a0[i] + a1[i]);
                }
                d.rhs += 1;
            }
        }
        return d;
    }

    // Velocity Verlet (Integrators.cpp:99-152) with one metric part per step. Every
    // right-hand side after the first is evaluated at the new position (x1n, thn), which
    // is where the next step's first one is evaluated: its metric part is computed once,
    // used for the new acceleration and every velocity iteration, and kept for the next
    // step. The new position's x1 and theta are stored as the metric saw them.
    static __device__ __forceinline__ bool step_verlet_cached(Lane& L, const ImageConst& I, const RunConst& R, float h,
                                                              const float uf[4]) {
        const bool rlog = R.rlog != 0;
        float a0[4], a1[4], vi[4], du[4], dxc[4];
        accel_part(L.mc, rlog, uf, a0);
        const float hh2 = 0.5f * h * h;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            dxc[i] = hh2 * a0[i];
            vi[i] = uf[i] + h * a0[i];
        }
        const ff x1n = ff_add_f(ff_add(L.x[1], two_prod(h, L.v[1].hi)), __fmaf_rn(h, L.v[1].lo, dxc[1]));
        const ff thn = ff_add_f(ff_add(L.x[2], two_prod(h, L.v[2].hi)), __fmaf_rn(h, L.v[2].lo, dxc[2]));
        // inlined for every plugin: this is the step's only metric part
        const MetricAt<float> mn = metric_part<MID, float>(I.mx.q, I.mx, rlog, x1n, thn);
        accel_part(mn, rlog, vi, a1);
        L.rhs += 2;
        const float h2 = 0.5f * h;
#pragma unroll
        for (int i = 0; i < 4; ++i) du[i] = h2 * (a0[i] + a1[i]);
        if (I.mx.vtol2 > 0.f) {
            const float tol2 = I.mx.vtol2;
            float dv[4];  // first correction: nv - vi = h/2 (a1 - a0)
#pragma unroll
            for (int i = 0; i < 4; ++i) dv[i] = h2 * (a1[i] - a0[i]);
            for (int it = 0;; ++it) {
                float num = 0.f, den = 0.f;
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const float nvi = uf[i] + du[i];
                    num += dv[i] * dv[i];
                    den += nvi * nvi;
                }
                if (!(num > tol2 * den)) break;
                if (it >= R.verlet_cap) {
                    L.err |= FOORT_ERR_VERLET_ITER;
                    break;
                }
                float a1n[4];
#pragma unroll
                for (int i = 0; i < 4; ++i) vi[i] = uf[i] + du[i];
                accel_part(mn, rlog, vi, a1n);
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    dv[i] = h2 * (a1n[i] - a1[i]);
                    a1[i] = a1n[i];
                    du[i] = h2 * (a0[i] + a1[i]);
                }
                L.rhs += 1;
            }
        }
        L.mc = mn;
        return advance(L, I, R, h, du, dxc, &x1n, &thn);
    }

    // RK4's velocity increment du = h/6 (k1 + 2 k2 + 2 k3 + k4) and the O(h^2) part of the
    // position increment dxc = h^2/6 (k1 + k2 + k3) (Integrators.cpp:91-92 rearranged).
    static __device__ __forceinline__ void rk4_combine(float h, const float k1[4], const float k2[4],
                                                       const float k3[4], const float k4[4], float du[4],
                                                       float dxc[4]) {
        // h / 6 is a quotient, not a product with a rounded 1/6: that constant is 3e-8
        // too large, which would scale every velocity increment by the same factor
        // and, amplified by strongly bent orbits, bias the escape direction by ~1e-7.
        // One Newton-Raphson correction of h * (1/6) gives the quotient to within an
        // ulp without that bias: q1 = q0 + (h - 6 q0) / 6.
        const float q0 = __fmul_rn(h, 0.166666672f);
        const float h6 = __fmaf_rn(__fmaf_rn(-6.f, q0, h), 0.166666672f, q0), hh6 = __fmul_rn(h, h6);
        // Each rounding is written out, so that the compiler cannot fuse the products that
        // produced k4 (one-lane kernel) into these sums: the two-lane kernel, whose k
        // arrive by shuffle, computes the same roundings.
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            du[i] = __fmul_rn(h6, __fadd_rn(__fmaf_rn(2.f, k3[i], __fmaf_rn(2.f, k2[i], k1[i])), k4[i]));
            dxc[i] = __fmul_rn(hh6, __fadd_rn(__fadd_rn(k1[i], k2[i]), k3[i]));
        }
    }

    // One RK4 step of one geodesic on two lanes (Kerr and flat space, the inlined
    // plugins). Both lanes hold the same state; in each of two rounds the even lane
    // evaluates the metric part at stage 1 (then 3) and the odd lane at stage 2 (then 4),
    // the positions that the reordered step of step() evaluates side by side. The four
    // contractions run on both lanes, each kept by the lane whose metric it used, and
    // each acceleration is sent to the partner with one shuffle. Both lanes then do the
    // same arithmetic on the same values as step(), so they stay in lockstep and their
    // results are step()'s. A lane does half the metric work of a step: where a launch
    // has fewer geodesics than the GPU has lanes, a step's latency is what sets the pace.
    static __device__ __forceinline__ bool step_pair(Lane& L, const ImageConst& I, const RunConst& R, bool odd,
                                                     unsigned pmask) {
        float uf[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) uf[i] = ff_f(L.v[i]);
        const float h = adaptive_step_f32(R, I.mx, L.x[2], uf);
        const float hh = 0.5f * h;
        const bool rlog = R.rlog != 0;
        float k1[4], k2[4], k3[4], k4[4], us[4], ka[4], du[4], dxc[4];
        // stages 1 (even lane) and 2 (odd lane)
        const ff p2r = ff_add_f(L.x[1], hh * uf[1]), p2t = ff_add_f(L.x[2], hh * uf[2]);
        MetricAt<float> m = metric_part<MID, float>(I.mx.q, I.mx, rlog, odd ? p2r : L.x[1], odd ? p2t : L.x[2]);
        accel_part(m, rlog, uf, ka);
#pragma unroll
        for (int i = 0; i < 4; ++i) k1[i] = __shfl_sync(pmask, ka[i], 0, 2);
#pragma unroll
        for (int i = 0; i < 4; ++i) us[i] = uf[i] + hh * k1[i];
        accel_part(m, rlog, us, ka);
#pragma unroll
        for (int i = 0; i < 4; ++i) k2[i] = __shfl_sync(pmask, ka[i], 1, 2);
        // stages 3 (even lane) and 4 (odd lane): each lane forms only its own position
        const float dr = odd ? h * (uf[1] + hh * k2[1]) : hh * (uf[1] + hh * k1[1]);
        const float dt = odd ? h * (uf[2] + hh * k2[2]) : hh * (uf[2] + hh * k1[2]);
        m = metric_part<MID, float>(I.mx.q, I.mx, rlog, ff_add_f(L.x[1], dr), ff_add_f(L.x[2], dt));
#pragma unroll
        for (int i = 0; i < 4; ++i) us[i] = uf[i] + hh * k2[i];
        accel_part(m, rlog, us, ka);
#pragma unroll
        for (int i = 0; i < 4; ++i) k3[i] = __shfl_sync(pmask, ka[i], 0, 2);
#pragma unroll
        for (int i = 0; i < 4; ++i) us[i] = uf[i] + h * k3[i];
        accel_part(m, rlog, us, ka);
#pragma unroll
        for (int i = 0; i < 4; ++i) k4[i] = __shfl_sync(pmask, ka[i], 1, 2);
        rk4_combine(h, k1, k2, k3, k4, du, dxc);
        L.rhs += 2;  // the pair evaluates four
        return advance(L, I, R, h, du, dxc);
    }

    // The end of a step: x += h u + dxc; u += du; lambda += h; terminations; diagnostics.
    static __device__ __forceinline__ bool advance(Lane& L, const ImageConst& I, const RunConst& R, float h,
                                                   const float du[4], const float dxc[4], const ff* x1n = nullptr,
                                                   const ff* thn = nullptr) {
        // h u is formed from the whole float-float velocity: its high part h u.hi exactly
        // (TwoProd) and joined to the position exactly (TwoSum); h u.lo, the product's
        // rounding error and the O(h^2) part dxc go to the low part. Rounding h u to one
        // float instead, or dropping u.lo, would put 6e-8 of relative error on every
        // position increment, which strongly bent rays amplify. du and dxc themselves
        // carry the FP32 right-hand side's error. x1n / thn: the new x1 and theta where
        // the caller already formed them.
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const ff t = two_prod(h, L.v[i].hi);
            L.x[i] = ff_add_f2(L.x[i], t.hi, __fadd_rn(t.lo, __fmaf_rn(h, L.v[i].lo, dxc[i])));
            L.v[i] = ff_add_f(L.v[i], du[i]);
        }
        if (x1n) {
            L.x[1] = *x1n;
            L.x[2] = *thn;
        }
        return after_step(L, I, R, ff_add_f(L.lam, h));
    }

    // Geodesic::Update after the integrator (Geodesic.cpp:66-87): the new affine
    // parameter, the step count, terminations, diagnostics.
    static __device__ __forceinline__ bool after_step(Lane& L, const ImageConst& I, const RunConst& R, ff lam) {
        L.lam = lam;
        ++L.steps;
        L.term = terms(L, I, R);
        diags(L, I, R, false);
        if (L.gp.dst) geopos(L, R, 1.0);  // lambda > 0 after a step; only compared with 0
        // A NaN or Inf anywhere in the state reaches r or u^r within one step through the
        // right-hand side, so those two words stand for the whole state here; the full
        // state is checked again when the geodesic's record is written.
        const bool bad = !(isfinite(L.x[1].hi) & isfinite(L.v[1].hi));
        L.err |= bad ? FOORT_ERR_NONFINITE : 0u;
        return (L.term == FOORT_TERMCODE_CONTINUE) & !(bad & !(R.term_flags & FOORT_TERM_TIMEOUT));
    }

    static __device__ __forceinline__ void write(const Lane& L, const RunConst& R, foort_result* o, int term,
                                                 uint32_t err) {
        double x[4], v[4];
        load_double(L, x, v);
        if (!(finite4(x) && finite4(v))) err |= FOORT_ERR_NONFINITE;
        DiagState D;
        D.quad = L.quad;
        if ((R.diag_flags & FOORT_DIAG_FOUR_COLOR_SCREEN) && term == FOORT_TERMCODE_BOUNDARY_SPHERE)
            D.quad = four_color_quadrant(x[2], x[3]);
        D.passes = ((R.diag_flags & FOORT_DIAG_EQUATORIAL_PASSES) && term == FOORT_TERMCODE_HORIZON) ? -L.passes : L.passes;
        double rm = -1.0;
        if (L.has_rmin) rm = R.rlog ? exp(ff_d(L.rmin)) : ff_d(L.rmin);
        if ((R.diag_flags & FOORT_DIAG_CLOSEST_RADIUS) && term == FOORT_TERMCODE_HORIZON) rm = 0.0;
        D.rmin = rm;
        write_result(o, term, err, L.steps, ff_d(L.lam), x, v, D);
    }

    static __device__ __forceinline__ void finish(const Lane& L, const RunConst& R, foort_result* o) {
        write(L, R, o, L.term, L.err);
    }
    static __device__ __forceinline__ void stop(const Lane& L, const RunConst& R, foort_result* o, uint32_t err) {
        write(L, R, o, FOORT_TERMCODE_CONTINUE, L.err | err);
    }
};

}  // namespace foort
