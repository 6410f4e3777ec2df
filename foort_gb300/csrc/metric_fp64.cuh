// FP64 metric plugins (host + device).
//
// Each metric returns the five independent components of a stationary, axisymmetric
// metric (g_tt, g_tphi, g_rr, g_thth, g_phiphi) with indices down (dd) or up (uu).
// The arguments are the radius r (already exponentiated in log-r mode), sin(theta) and
// cos(theta), so that a caller evaluating several points that share theta or r computes
// each transcendental once. The formulas keep the reference's association order
// (Metric.cpp:131-191 Kerr, :218-229 flat, :273-361 Rasheed-Larsen, :409-473 Johannsen,
// :511-626 Manko-Novikov) so that a strict build gives the reference's values.
#pragma once

#include <math.h>

#ifdef __CUDACC__
#define FOORT_HD __host__ __device__ __forceinline__
#else
#define FOORT_HD inline
#endif

namespace foort {

struct G5 {
    double tt, tp, rr, hh, pp;  // t-t, t-phi, r-r, theta-theta, phi-phi
};

// Derived metric constants, filled on the host from the user parameters.
struct MetricConst {
    double q[6];  // per-metric constants (see make_metric_const)
    double rh;    // horizon radius (0 for flat space)
};

// Number of constant slots of the analytic metric plugins (analytic_metric.cuh).
constexpr int kMixedQ = 20;

// Metric ids (include/foort_gpu.h FOORT_METRIC_*).
enum MetricId { kKerr = 0, kFlat = 1, kRasheedLarsen = 2, kJohannsen = 3, kMankoNovikov = 4 };

inline MetricConst make_metric_const(int id, const double* p) {
    MetricConst m{};
    switch (id) {
    case kKerr:  // Metric.cpp:111-128
        m.q[0] = p[0];
        m.rh = 1 + sqrt(1 - p[0] * p[0]);
        break;
    case kFlat:
        m.rh = 0.0;
        break;
    case kRasheedLarsen: {  // Metric.cpp:244-271: rescaled so that M = 1
        double mm = p[0], aa = p[1], pp = p[2], qq = p[3];
        m.q[0] = aa / ((pp + qq) / 4.0);
        m.q[1] = mm / ((pp + qq) / 4.0);
        m.q[2] = pp / ((pp + qq) / 4.0);
        m.q[3] = qq / ((pp + qq) / 4.0);
        m.rh = (mm + sqrt(mm * mm - aa * aa)) / ((pp + qq) / 4.0);
        break;
    }
    case kJohannsen:  // Metric.cpp:378-407 (Kerr horizon radius)
        for (int i = 0; i < 5; ++i) m.q[i] = p[i];
        m.rh = 1 + sqrt(1 - p[0] * p[0]);
        break;
    case kMankoNovikov:  // Metric.cpp:490-509
        m.q[0] = p[0];
        m.q[1] = p[1];
        m.q[2] = (p[0] == 0.0) ? 0.0 : (-1. + sqrt(1. - p[0] * p[0])) / p[0];
        m.q[3] = sqrt(1. - p[0] * p[0]);
        m.rh = 1 + sqrt(1. - p[0] * p[0]);
        break;
    default:
        break;
    }
    return m;
}

// ---- Kerr ---------------------------------------------------------------------------
FOORT_HD G5 kerr_dd(const MetricConst& M, double r, double s, double c, bool rlog) {
    const double a = M.q[0];
    double sig = r * r + a * a * c * c;
    double del = r * r + a * a - 2. * r;
    double A = (r * r + a * a) * (r * r + a * a) - del * a * a * s * s;
    G5 g;
    g.tt = -(1. - 2. * r / sig);
    g.rr = sig / del;
    g.hh = sig;
    g.pp = A / sig * s * s;
    g.tp = -2. * a * r * s * s / sig;
    if (rlog) g.rr *= (r * r);
    return g;
}
FOORT_HD G5 kerr_uu(const MetricConst& M, double r, double s, double c, bool rlog) {
    const double a = M.q[0];
    double sig = r * r + a * a * c * c;
    double del = r * r + a * a - 2. * r;
    double A = (r * r + a * a) * (r * r + a * a) - del * a * a * s * s;
    G5 g;
    g.tt = -A / (sig * del);
    g.rr = del / sig;
    g.hh = 1. / sig;
    g.pp = (del - a * a * s * s) / (sig * del * s * s);
    g.tp = -2. * a * r / (sig * del);
    if (rlog) g.rr *= 1.0 / (r * r);
    return g;
}

// ---- flat space (normal r; the reference has no log-r variant) -----------------------
FOORT_HD G5 flat_dd(const MetricConst&, double r, double s, double, bool) {
    G5 g;
    g.tt = -1; g.tp = 0; g.rr = 1; g.hh = r * r; g.pp = r * r * s * s;
    return g;
}
FOORT_HD G5 flat_uu(const MetricConst&, double r, double s, double, bool) {
    G5 g;
    g.tt = -1; g.tp = 0; g.rr = 1; g.hh = 1 / (r * r); g.pp = 1 / (r * r * s * s);
    return g;
}

// ---- Rasheed-Larsen -------------------------------------------------------------------
struct RLParts { double del, H3, Bp, H1, H2, sq, s2; };
FOORT_HD RLParts rl_parts(const MetricConst& M, double r, double s, double c) {
    const double a = M.q[0], mm = M.q[1], p = M.q[2], q = M.q[3];
    RLParts t;
    double r2 = r * r;
    t.s2 = s * s;
    double c2 = c * c;
    t.del = r2 + a * a - 2. * r * mm;
    t.H3 = r2 - 2. * r * mm + a * a * c2;
    t.Bp = sqrt(p * q) * a * t.s2 * (((p * q + 4. * mm * mm) * r
        - mm * (p - 2. * mm) * (q - 2. * mm)) / (2. * mm * (p + q) * t.H3));
    t.H1 = r2 + a * a * c2 + r * (p - 2. * mm)
        + (p / (p + q)) * ((p - 2. * mm) * (q - 2. * mm) / 2.)
        - (p / (2. * mm * (p + q))) * sqrt((p * p - 4. * mm * mm) * (q * q - 4. * mm * mm)) * a * c;
    t.H2 = r2 + a * a * c2 + r * (q - 2. * mm)
        + (q / (p + q)) * ((p - 2. * mm) * (q - 2. * mm) / 2.)
        + (q / (2. * mm * (p + q))) * sqrt((p * p - 4. * mm * mm) * (q * q - 4. * mm * mm)) * a * c;
    t.sq = sqrt(t.H1 * t.H2);
    return t;
}
FOORT_HD G5 rl_dd(const MetricConst& M, double r, double s, double c, bool rlog) {
    RLParts t = rl_parts(M, r, s, c);
    G5 g;
    g.tt = -t.H3 / t.sq;
    g.rr = t.sq / t.del;
    g.hh = t.sq;
    g.pp = -(t.H3 * t.Bp * t.Bp) / t.sq + (t.sq * t.del * t.s2) / t.H3;
    g.tp = -(t.H3 * t.Bp) / t.sq;
    if (rlog) g.rr *= (r * r);
    return g;
}
FOORT_HD G5 rl_uu(const MetricConst& M, double r, double s, double c, bool rlog) {
    RLParts t = rl_parts(M, r, s, c);
    G5 g;
    g.tt = ((t.H3 * t.H3 * t.Bp * t.Bp) / t.s2 - t.H1 * t.H2 * t.del) / (t.sq * t.H3 * t.del);
    g.rr = t.del / t.sq;
    g.hh = 1. / t.sq;
    g.pp = t.H3 / (t.sq * t.del * t.s2);
    g.tp = -(t.H3 * t.Bp) / (t.sq * t.del * t.s2);
    if (rlog) g.rr *= 1.0 / (r * r);
    return g;
}

// ---- Johannsen ------------------------------------------------------------------------
// pow(x, 2.) of the reference is written x * x: both are the correctly rounded square.
FOORT_HD G5 joh_dd(const MetricConst& M, double r, double s, double c, bool rlog) {
    const double a = M.q[0], a13 = M.q[1], a22 = M.q[2], a52 = M.q[3], e3 = M.q[4];
    double A1 = 1. + a13 / (r * r * r);
    double A2 = 1. + a22 / (r * r);
    double A5 = 1. + a52 / (r * r);
    double ef = e3 / r;
    double rho2 = r * r + a * a * c * c + ef;
    double del = r * r + a * a - 2. * r;
    double den = (r * r + a * a) * A1 - a * a * A2 * s * s;
    double den2 = den * den;
    double ra = (r * r + a * a) * A1;
    G5 g;
    g.tt = -rho2 * (del - a * a * A2 * A2 * s * s) / den2;
    g.rr = rho2 / (del * A5);
    g.hh = rho2;
    g.pp = rho2 * s * s * (ra * ra - a * a * del * s * s) / den2;
    g.tp = -a * ((r * r + a * a) * A1 * A2 - del) * rho2 * s * s / den2;
    if (rlog) g.rr *= (r * r);
    return g;
}
FOORT_HD G5 joh_uu(const MetricConst& M, double r, double s, double c, bool rlog) {
    const double a = M.q[0], a13 = M.q[1], a22 = M.q[2], a52 = M.q[3], e3 = M.q[4];
    double A1 = 1. + a13 / (r * r * r);
    double A2 = 1. + a22 / (r * r);
    double A5 = 1. + a52 / (r * r);
    double ef = e3 / r;
    double rho2 = r * r + a * a * c * c + ef;
    double del = r * r + a * a - 2. * r;
    double ra = (r * r + a * a) * A1;
    G5 g;
    g.tt = (-1. * (ra * ra) + a * a * del * s * s) / (del * rho2);
    g.rr = del * A5 / rho2;
    g.hh = 1. / rho2;
    g.pp = (-a * a * A2 * A2 * s * s + del) / (del * rho2 * s * s);
    g.tp = -a * (A2 * A1 * (r * r + a * a) - del) / (del * rho2);
    if (rlog) g.rr *= 1.0 / (r * r);
    return g;
}

// ---- Manko-Novikov --------------------------------------------------------------------
struct MNParts { double f, e2g, om, rho2, del; };
FOORT_HD MNParts mn_parts(const MetricConst& M, double r, double s, double c) {
    const double a3 = M.q[1], al = M.q[2], k = M.q[3];
    (void)s;
    MNParts t;
    double xx = (r - 1.) / k;
    double yy = c;
    double R = sqrt(xx * xx + yy * yy - 1.);
    double P1 = xx * yy / R;
    double P2 = 0.5 * (3. * xx * xx * yy * yy / (R * R) - 1.);
    double P3 = 0.5 * (5. * pow(xx * yy / R, 3.) - 3. * xx * yy / R);
    double P4 = 0.125 * (35. * pow(xx * yy / R, 4.) - 30. * xx * xx * yy * yy / (R * R) + 3.);
    double aa = -al * exp(2. * a3 * (1. - (xx - yy) * (1. / R + P1 / (R * R) + P2 / (R * R * R) + P3 / (R * R * R * R))));
    double bb = al * exp(2. * a3 * (-1. + (xx + yy) * (1. / R - P1 / (R * R) + P2 / (R * R * R) - P3 / (R * R * R * R))));
    double AA = (xx * xx - 1.) * (1. + aa * bb) * (1. + aa * bb) - (1. - yy * yy) * (bb - aa) * (bb - aa);
    double b1 = (xx + 1. + (xx - 1.) * aa * bb), b2 = ((1. + yy) * aa + (1. - yy) * bb);
    double BB = b1 * b1 + b2 * b2;
    double CC = (xx * xx - 1.) * (1. + aa * bb) * (bb - aa - yy * (aa + bb)) + (1. - yy * yy) * (bb - aa) * (1. + aa * bb + xx * (1. - aa * bb));
    double psi = a3 * P3 / (R * R * R * R);
    double gp = 2. * a3 * a3 * (P4 * P4 - P3 * P3) / (pow(R, 8.)) + 2. * a3 * (-yy + xx * P1 / R - yy * P2 / (R * R) + xx * P3 / (R * R * R)) / R;
    t.f = exp(2. * psi) * AA / BB;
    t.e2g = exp(2. * gp) * AA / ((xx * xx - yy * yy) * (1. - al * al) * (1. - al * al));
    t.om = 2. * k * exp(-2. * psi) * CC / AA - 4. * k * al / (1. - al * al);
    t.rho2 = (r - 1.) * (r - 1.) - k * k * c * c;
    t.del = (r - 1.) * (r - 1.) - k * k;
    return t;
}
FOORT_HD G5 mn_dd(const MetricConst& M, double r, double s, double c, bool rlog) {
    MNParts t = mn_parts(M, r, s, c);
    G5 g;
    g.tt = -t.f;
    g.hh = t.e2g * t.rho2 / t.f;
    g.rr = g.hh / t.del;
    g.pp = -t.f * t.om * t.om + t.del * s * s / t.f;
    g.tp = t.om * t.f;
    if (rlog) g.rr *= (r * r);
    return g;
}
FOORT_HD G5 mn_uu(const MetricConst& M, double r, double s, double c, bool rlog) {
    MNParts t = mn_parts(M, r, s, c);
    double bd = t.om * t.f;
    double gd = -t.f * t.om * t.om + t.del * s * s / t.f;
    double bu = bd / gd;
    double al2 = bu * bd + t.f;
    G5 g;
    g.tt = -1. / al2;
    g.hh = t.f / (t.e2g * t.rho2);
    g.rr = t.del * g.hh;
    g.pp = 1. / gd - bu * bu / al2;
    g.tp = bu / al2;
    if (rlog) g.rr *= 1.0 / (r * r);
    return g;
}

// Compile-time plugin wrappers used by the kernels.
template <int ID> struct MetricFP64;
template <> struct MetricFP64<kKerr> {
    static FOORT_HD G5 dd(const MetricConst& M, double r, double s, double c, bool l) { return kerr_dd(M, r, s, c, l); }
    static FOORT_HD G5 uu(const MetricConst& M, double r, double s, double c, bool l) { return kerr_uu(M, r, s, c, l); }
};
template <> struct MetricFP64<kFlat> {
    static FOORT_HD G5 dd(const MetricConst& M, double r, double s, double c, bool l) { return flat_dd(M, r, s, c, l); }
    static FOORT_HD G5 uu(const MetricConst& M, double r, double s, double c, bool l) { return flat_uu(M, r, s, c, l); }
};
template <> struct MetricFP64<kRasheedLarsen> {
    static FOORT_HD G5 dd(const MetricConst& M, double r, double s, double c, bool l) { return rl_dd(M, r, s, c, l); }
    static FOORT_HD G5 uu(const MetricConst& M, double r, double s, double c, bool l) { return rl_uu(M, r, s, c, l); }
};
template <> struct MetricFP64<kJohannsen> {
    static FOORT_HD G5 dd(const MetricConst& M, double r, double s, double c, bool l) { return joh_dd(M, r, s, c, l); }
    static FOORT_HD G5 uu(const MetricConst& M, double r, double s, double c, bool l) { return joh_uu(M, r, s, c, l); }
};
template <> struct MetricFP64<kMankoNovikov> {
    static FOORT_HD G5 dd(const MetricConst& M, double r, double s, double c, bool l) { return mn_dd(M, r, s, c, l); }
    static FOORT_HD G5 uu(const MetricConst& M, double r, double s, double c, bool l) { return mn_uu(M, r, s, c, l); }
};

// Run-time dispatch for host-side use (camera frame).
inline G5 metric_dd_host(int id, const MetricConst& M, double r, double s, double c, bool rlog) {
    switch (id) {
    case kKerr: return kerr_dd(M, r, s, c, rlog);
    case kFlat: return flat_dd(M, r, s, c, rlog);
    case kRasheedLarsen: return rl_dd(M, r, s, c, rlog);
    case kJohannsen: return joh_dd(M, r, s, c, rlog);
    default: return mn_dd(M, r, s, c, rlog);
    }
}
inline G5 metric_uu_host(int id, const MetricConst& M, double r, double s, double c, bool rlog) {
    switch (id) {
    case kKerr: return kerr_uu(M, r, s, c, rlog);
    case kFlat: return flat_uu(M, r, s, c, rlog);
    case kRasheedLarsen: return rl_uu(M, r, s, c, rlog);
    case kJohannsen: return joh_uu(M, r, s, c, rlog);
    default: return mn_uu(M, r, s, c, rlog);
    }
}

}  // namespace foort
