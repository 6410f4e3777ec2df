// ORACLE -- TEST INFRASTRUCTURE ONLY.
//
// CPU restatement of FOORT's integration stage (the pixel loop FOORT/Main.cpp:327-402
// and everything it calls), used by tests/, __graft_entry__.smoke() and the CPU
// baseline leg of bench.py as the CHECKER. The engine never links, loads or calls
// anything in this directory.
//
// Every function follows the reference file:line it cites, keeping the reference's
// order of floating-point operations (left-to-right association, the dense loops and
// their zero terms, operator/ as multiplication by the reciprocal, Geometry.h:181-184)
// so that a strict-IEEE build of this file (-O2 -ffp-contract=off) reproduces a
// strict-IEEE build of the reference bit for bit. The oracle is pinned in tests/ against
// (a) the golden .dat files shipped with the reference and (b) fixtures generated by the
// reference itself, compiled from its own sources (oracle/ref_driver.cpp).
//
// Build: oracle/Makefile (liboracle.so strict, liboracle_fast.so with the reference's
// -Ofast flags for the CPU-baseline timing).

#include "../include/foort_gpu.h"

#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

using real = double;
using V4 = std::array<real, 4>;
using M4 = std::array<V4, 4>;
using T4 = std::array<M4, 4>;

// Geometry.h:44 -- the reference's (truncated) pi, used in every angular test.
constexpr real kPi = 3.1415926535;
// Integrators.h:31 -- guard against division by zero in the step rule.
constexpr real kNoDiv0 = 1e-20;

// ---- tensor arithmetic, Geometry.h:141-184 ------------------------------------------
// a + b and a - b act elementwise; s * a and a * s multiply each element by s;
// a / s multiplies each element by (1 / s).
inline V4 vadd(const V4& a, const V4& b) { V4 t; for (int i = 0; i < 4; ++i) t[i] = a[i] + b[i]; return t; }
inline V4 vsub(const V4& a, const V4& b) { V4 t; for (int i = 0; i < 4; ++i) t[i] = a[i] - b[i]; return t; }
inline V4 vmul(const V4& a, real s) { V4 t; for (int i = 0; i < 4; ++i) t[i] = a[i] * s; return t; }
inline V4 vdiv(const V4& a, real s) { return vmul(a, 1 / s); }
inline M4 msub(const M4& a, const M4& b) { M4 t; for (int i = 0; i < 4; ++i) t[i] = vsub(a[i], b[i]); return t; }
inline M4 mmul(const M4& a, real s) { M4 t; for (int i = 0; i < 4; ++i) t[i] = vmul(a[i], s); return t; }
inline M4 mdiv(const M4& a, real s) { return mmul(a, 1 / s); }

inline real smin(real a, real b) { return (b < a) ? b : a; }  // std::min
inline real smax(real a, real b) { return (a < b) ? b : a; }  // std::max

inline M4 pack(real g00, real g03, real g11, real g22, real g33) {
    M4 g{};
    g[0][0] = g00; g[0][3] = g03; g[3][0] = g03;
    g[1][1] = g11; g[2][2] = g22; g[3][3] = g33;
    return g;
}

// ---- metrics, Metric.cpp ------------------------------------------------------------
struct MetricDef {
    int id;
    bool rlog;
    real p[6];   // raw parameters as given in foort_image_desc
    real q[6];   // derived parameters (rescaled / auxiliary), set by make_metric
    real rh;     // horizon radius (0 for flat space)
};

MetricDef make_metric(int id, const real* params, bool rlog) {
    MetricDef m{};
    m.id = id;
    m.rlog = rlog;
    for (int i = 0; i < 6; ++i) m.p[i] = params ? params[i] : 0.0;
    switch (id) {
    case FOORT_METRIC_KERR:  // Metric.cpp:111-128
        m.q[0] = m.p[0];
        m.rh = 1 + std::sqrt(1 - m.p[0] * m.p[0]);
        break;
    case FOORT_METRIC_FLAT:  // Metric.cpp:205-215
        m.rh = 0.0;
        break;
    case FOORT_METRIC_RASHEED_LARSEN: {  // Metric.cpp:244-271; params (m, a, p, q)
        real mm = m.p[0], aa = m.p[1], pp = m.p[2], qq = m.p[3];
        m.q[0] = aa / ((pp + qq) / 4.0);  // a
        m.q[1] = mm / ((pp + qq) / 4.0);  // m
        m.q[2] = pp / ((pp + qq) / 4.0);  // p
        m.q[3] = qq / ((pp + qq) / 4.0);  // q
        m.rh = (mm + std::sqrt(mm * mm - aa * aa)) / ((pp + qq) / 4.0);
        break;
    }
    case FOORT_METRIC_JOHANNSEN:  // Metric.cpp:378-407; params (a, a13, a22, a52, eps3)
        for (int i = 0; i < 5; ++i) m.q[i] = m.p[i];
        m.rh = 1 + std::sqrt(1 - m.p[0] * m.p[0]);
        break;
    case FOORT_METRIC_MANKO_NOVIKOV:  // Metric.cpp:490-509; params (a, alpha3)
        m.q[0] = m.p[0];
        m.q[1] = m.p[1];
        m.q[2] = (m.p[0] == 0.0) ? 0.0 : (-1. + std::sqrt(1. - m.p[0] * m.p[0])) / m.p[0];  // alpha
        m.q[3] = std::sqrt(1. - m.p[0] * m.p[0]);                                            // k
        m.rh = 1 + std::sqrt(1. - m.p[0] * m.p[0]);
        break;
    default:
        break;
    }
    return m;
}

// Kerr, Metric.cpp:131-159
M4 kerr_dd(const MetricDef& m, const V4& x) {
    const real a = m.q[0];
    real r = m.rlog ? std::exp(x[1]) : x[1];
    real th = x[2];
    real s = std::sin(th), c = std::cos(th);
    real sig = r * r + a * a * c * c;
    real del = r * r + a * a - 2. * r;
    real A = (r * r + a * a) * (r * r + a * a) - del * a * a * s * s;
    real g00 = -(1. - 2. * r / sig);
    real g11 = sig / del;
    real g22 = sig;
    real g33 = A / sig * s * s;
    real g03 = -2. * a * r * s * s / sig;
    if (m.rlog) g11 *= (r * r);
    return pack(g00, g03, g11, g22, g33);
}

// Kerr, Metric.cpp:162-191
M4 kerr_uu(const MetricDef& m, const V4& x) {
    const real a = m.q[0];
    real r = m.rlog ? std::exp(x[1]) : x[1];
    real th = x[2];
    real s = std::sin(th), c = std::cos(th);
    real sig = r * r + a * a * c * c;
    real del = r * r + a * a - 2. * r;
    real A = (r * r + a * a) * (r * r + a * a) - del * a * a * s * s;
    real g00 = -A / (sig * del);
    real g11 = del / sig;
    real g22 = 1. / sig;
    real g33 = (del - a * a * s * s) / (sig * del * s * s);
    real g03 = -2. * a * r / (sig * del);
    if (m.rlog) g11 *= 1.0 / (r * r);
    return pack(g00, g03, g11, g22, g33);
}

// FlatSpace, Metric.cpp:218-229 (normal r only; the reference ignores RLogScale here)
M4 flat_dd(const V4& x) {
    return pack(-1, 0, 1, x[1] * x[1], x[1] * x[1] * std::sin(x[2]) * std::sin(x[2]));
}
M4 flat_uu(const V4& x) {
    return pack(-1, 0, 1, 1 / (x[1] * x[1]), 1 / (x[1] * x[1] * std::sin(x[2]) * std::sin(x[2])));
}

// Rasheed-Larsen, Metric.cpp:273-361 (shared shorthands)
struct RLAux { real r, r2, s, c, s2, c2, del, H3, Bp, H1, H2, sq; };
RLAux rl_aux(const MetricDef& m, const V4& x) {
    const real a = m.q[0], mm = m.q[1], p = m.q[2], q = m.q[3];
    RLAux t;
    t.r = m.rlog ? std::exp(x[1]) : x[1];
    t.r2 = t.r * t.r;
    real th = x[2];
    t.s = std::sin(th);
    t.c = std::cos(th);
    t.s2 = t.s * t.s;
    t.c2 = t.c * t.c;
    const real r = t.r, r2 = t.r2;
    t.del = r2 + a * a - 2. * r * mm;
    t.H3 = r2 - 2. * r * mm + a * a * t.c2;
    t.Bp = std::sqrt(p * q) * a * t.s2 * (((p * q + 4. * mm * mm) * r
        - mm * (p - 2. * mm) * (q - 2. * mm)) / (2. * mm * (p + q) * t.H3));
    t.H1 = r2 + a * a * t.c2 + r * (p - 2. * mm)
        + (p / (p + q)) * ((p - 2. * mm) * (q - 2. * mm) / 2.)
        - (p / (2. * mm * (p + q))) * std::sqrt((p * p - 4. * mm * mm) * (q * q - 4. * mm * mm)) * a * t.c;
    t.H2 = r2 + a * a * t.c2 + r * (q - 2. * mm)
        + (q / (p + q)) * ((p - 2. * mm) * (q - 2. * mm) / 2.)
        + (q / (2. * mm * (p + q))) * std::sqrt((p * p - 4. * mm * mm) * (q * q - 4. * mm * mm)) * a * t.c;
    t.sq = std::sqrt(t.H1 * t.H2);
    return t;
}
M4 rl_dd(const MetricDef& m, const V4& x) {
    RLAux t = rl_aux(m, x);
    real g00 = -t.H3 / t.sq;
    real g11 = t.sq / t.del;
    real g22 = t.sq;
    real g33 = -(t.H3 * t.Bp * t.Bp) / t.sq + (t.sq * t.del * t.s2) / t.H3;
    real g03 = -(t.H3 * t.Bp) / t.sq;
    if (m.rlog) g11 *= (t.r * t.r);
    return pack(g00, g03, g11, g22, g33);
}
M4 rl_uu(const MetricDef& m, const V4& x) {
    RLAux t = rl_aux(m, x);
    real g00 = ((t.H3 * t.H3 * t.Bp * t.Bp) / t.s2 - t.H1 * t.H2 * t.del) / (t.sq * t.H3 * t.del);
    real g11 = t.del / t.sq;
    real g22 = 1. / t.sq;
    real g33 = t.H3 / (t.sq * t.del * t.s2);
    real g03 = -(t.H3 * t.Bp) / (t.sq * t.del * t.s2);
    if (m.rlog) g11 *= 1.0 / (t.r * t.r);
    return pack(g00, g03, g11, g22, g33);
}

// Johannsen, Metric.cpp:409-440
M4 joh_dd(const MetricDef& m, const V4& x) {
    const real a = m.q[0], a13 = m.q[1], a22 = m.q[2], a52 = m.q[3], e3 = m.q[4];
    real r = m.rlog ? std::exp(x[1]) : x[1];
    real th = x[2];
    real s = std::sin(th), c = std::cos(th);
    real A1 = 1. + a13 / (r * r * r);
    real A2 = 1. + a22 / (r * r);
    real A5 = 1. + a52 / (r * r);
    real ef = e3 / r;
    real rho2 = r * r + a * a * c * c + ef;
    real del = r * r + a * a - 2. * r;
    real g00 = -rho2 * (del - a * a * A2 * A2 * s * s) / std::pow((r * r + a * a) * A1 - a * a * A2 * s * s, 2.);
    real g11 = rho2 / (del * A5);
    real g22 = rho2;
    real g33 = rho2 * s * s * (std::pow((r * r + a * a) * A1, 2.) - a * a * del * s * s) / std::pow((r * r + a * a) * A1 - a * a * A2 * s * s, 2.);
    real g03 = -a * ((r * r + a * a) * A1 * A2 - del) * rho2 * s * s / std::pow((r * r + a * a) * A1 - a * a * A2 * s * s, 2.);
    if (m.rlog) g11 *= (r * r);
    return pack(g00, g03, g11, g22, g33);
}

// Johannsen, Metric.cpp:442-473
M4 joh_uu(const MetricDef& m, const V4& x) {
    const real a = m.q[0], a13 = m.q[1], a22 = m.q[2], a52 = m.q[3], e3 = m.q[4];
    real r = m.rlog ? std::exp(x[1]) : x[1];
    real th = x[2];
    real s = std::sin(th), c = std::cos(th);
    real A1 = 1. + a13 / (r * r * r);
    real A2 = 1. + a22 / (r * r);
    real A5 = 1. + a52 / (r * r);
    real ef = e3 / r;
    real rho2 = r * r + a * a * c * c + ef;
    real del = r * r + a * a - 2. * r;
    real g00 = (-1. * std::pow((r * r + a * a) * A1, 2.) + a * a * del * s * s) / (del * rho2);
    real g11 = del * A5 / rho2;
    real g22 = 1. / rho2;
    real g33 = (-a * a * A2 * A2 * s * s + del) / (del * rho2 * s * s);
    real g03 = -a * (A2 * A1 * (r * r + a * a) - del) / (del * rho2);
    if (m.rlog) g11 *= 1.0 / (r * r);
    return pack(g00, g03, g11, g22, g33);
}

// Manko-Novikov shared part, Metric.cpp:511-555 / 568-611
struct MNAux { real r, s, c, f, e2g, om, rho2, del; };
MNAux mn_aux(const MetricDef& m, const V4& x) {
    const real a3 = m.q[1], al = m.q[2], k = m.q[3];
    MNAux t;
    t.r = m.rlog ? std::exp(x[1]) : x[1];
    const real r = t.r;
    real th = x[2];
    t.s = std::sin(th);
    t.c = std::cos(th);
    real xx = (r - 1.) / k;
    real yy = t.c;
    real R = std::sqrt(xx * xx + yy * yy - 1.);
    real P1 = xx * yy / R;
    real P2 = 0.5 * (3. * xx * xx * yy * yy / (R * R) - 1.);
    real P3 = 0.5 * (5. * std::pow(xx * yy / R, 3.) - 3. * xx * yy / R);
    real P4 = 0.125 * (35. * std::pow(xx * yy / R, 4.) - 30. * xx * xx * yy * yy / (R * R) + 3.);
    real aa = -al * std::exp(2. * a3 * (1. - (xx - yy) * (1. / R + P1 / (R * R) + P2 / (R * R * R) + P3 / (R * R * R * R))));
    real bb = al * std::exp(2. * a3 * (-1. + (xx + yy) * (1. / R - P1 / (R * R) + P2 / (R * R * R) - P3 / (R * R * R * R))));
    real AA = (xx * xx - 1.) * (1. + aa * bb) * (1. + aa * bb) - (1. - yy * yy) * (bb - aa) * (bb - aa);
    real BB = std::pow((xx + 1. + (xx - 1.) * aa * bb), 2.) + std::pow(((1. + yy) * aa + (1. - yy) * bb), 2.);
    real CC = (xx * xx - 1.) * (1. + aa * bb) * (bb - aa - yy * (aa + bb)) + (1. - yy * yy) * (bb - aa) * (1. + aa * bb + xx * (1. - aa * bb));
    real psi = a3 * P3 / (R * R * R * R);
    real gp = 2. * a3 * a3 * (P4 * P4 - P3 * P3) / (std::pow(R, 8.)) + 2. * a3 * (-yy + xx * P1 / R - yy * P2 / (R * R) + xx * P3 / (R * R * R)) / R;
    t.f = std::exp(2. * psi) * AA / BB;
    t.e2g = std::exp(2. * gp) * AA / ((xx * xx - yy * yy) * (1. - al * al) * (1. - al * al));
    t.om = 2. * k * std::exp(-2. * psi) * CC / AA - 4. * k * al / (1. - al * al);
    t.rho2 = (r - 1.) * (r - 1.) - k * k * t.c * t.c;
    t.del = (r - 1.) * (r - 1.) - k * k;
    return t;
}
M4 mn_dd(const MetricDef& m, const V4& x) {
    MNAux t = mn_aux(m, x);
    real g00 = -t.f;
    real g22 = t.e2g * t.rho2 / t.f;
    real g11 = g22 / t.del;
    real g33 = -t.f * t.om * t.om + t.del * t.s * t.s / t.f;
    real g03 = t.om * t.f;
    if (m.rlog) g11 *= (t.r * t.r);
    return pack(g00, g03, g11, g22, g33);
}
M4 mn_uu(const MetricDef& m, const V4& x) {
    MNAux t = mn_aux(m, x);
    real bd = t.om * t.f;
    real gdd = -t.f * t.om * t.om + t.del * t.s * t.s / t.f;
    real bu = bd / gdd;
    real al2 = bu * bd + t.f;
    real g00 = -1. / al2;
    real g22 = t.f / (t.e2g * t.rho2);
    real g11 = t.del * g22;
    real g33 = 1. / gdd - bu * bu / al2;
    real g03 = bu / al2;
    if (m.rlog) g11 *= 1.0 / (t.r * t.r);
    return pack(g00, g03, g11, g22, g33);
}

M4 metric_dd(const MetricDef& m, const V4& x) {
    switch (m.id) {
    case FOORT_METRIC_KERR: return kerr_dd(m, x);
    case FOORT_METRIC_FLAT: return flat_dd(x);
    case FOORT_METRIC_RASHEED_LARSEN: return rl_dd(m, x);
    case FOORT_METRIC_JOHANNSEN: return joh_dd(m, x);
    default: return mn_dd(m, x);
    }
}
M4 metric_uu(const MetricDef& m, const V4& x) {
    switch (m.id) {
    case FOORT_METRIC_KERR: return kerr_uu(m, x);
    case FOORT_METRIC_FLAT: return flat_uu(x);
    case FOORT_METRIC_RASHEED_LARSEN: return rl_uu(m, x);
    case FOORT_METRIC_JOHANNSEN: return joh_uu(m, x);
    default: return mn_uu(m, x);
    }
}

// Metric::getChristoffel_udd, Metric.cpp:14-55. Every shipped metric declares the
// symmetries {0, 3} (t and phi), so only r and theta derivatives are taken.
T4 christoffel(const MetricDef& m, const V4& x, real h) {
    T4 dg{};  // dg[c][i][j] = d_c g_ij
    for (int c = 0; c < 4; ++c) {
        if (c == 0 || c == 3) continue;
        V4 sh{};
        sh[c] = h;
        dg[c] = mdiv(msub(metric_dd(m, vadd(x, sh)), metric_dd(m, vsub(x, sh))), 2 * h);
    }
    M4 gu = metric_uu(m, x);
    T4 G{};
    for (int mu = 0; mu < 4; ++mu)
        for (int nu = 0; nu < 4; ++nu)
            for (int rho = 0; rho < 4; ++rho)
                for (int sg = 0; sg < 4; ++sg)
                    G[mu][nu][rho] += 1.0 / 2 * gu[mu][sg] * (dg[nu][rho][sg] + dg[rho][nu][sg] - dg[sg][nu][rho]);
    return G;
}

// geoRHS lambda, Integrators.cpp:60-68 (NoSource: Geodesic.cpp:15-19 returns zero)
V4 geo_rhs(const MetricDef& m, const V4& x, const V4& v, real h) {
    T4 G = christoffel(m, x, h);
    V4 ret{0, 0, 0, 0};
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
            for (int k = 0; k < 4; ++k)
                ret[i] -= G[i][j][k] * v[j] * v[k];
    return ret;
}

struct Integ {
    int id;
    real eps, hfd, hmin, vtol;
};

// Integrators::GetAdaptiveStep, Integrators.cpp:34-46 (note fabs(u3 + delta) on :40)
real adaptive_step(const Integ& I, const V4& x, const V4& v) {
    real d1 = I.eps / (std::fabs(v[1]) + kNoDiv0);
    real d2 = I.eps * smin(x[2], kPi - x[2]) / (std::fabs(v[2]) + kNoDiv0);
    real d3 = I.eps / (std::fabs(v[3] + kNoDiv0));
    real h = 1 / (1 / std::fabs(d1) + 1 / std::fabs(d2) + 1 / std::fabs(d3));
    h = smax(h, I.hmin);
    return h;
}

// IntegrateGeodesicStep_RK4, Integrators.cpp:51-94
void step_rk4(const MetricDef& m, const Integ& I, const V4& x, const V4& v, V4& nx, V4& nv, real& hs, uint64_t& nrhs) {
    real h = adaptive_step(I, x, v);
    V4 k1 = geo_rhs(m, x, v, I.hfd);
    V4 l1 = v;
    V4 k2 = geo_rhs(m, vadd(x, vmul(l1, 0.5 * h)), vadd(v, vmul(k1, 0.5 * h)), I.hfd);
    V4 l2 = vadd(v, vmul(k1, 0.5 * h));
    V4 k3 = geo_rhs(m, vadd(x, vmul(l2, 0.5 * h)), vadd(v, vmul(k2, 0.5 * h)), I.hfd);
    V4 l3 = vadd(v, vmul(k2, 0.5 * h));
    V4 k4 = geo_rhs(m, vadd(x, vmul(l3, h)), vadd(v, vmul(k3, h)), I.hfd);
    V4 l4 = vadd(v, vmul(k3, h));
    nv = vadd(v, vmul(vadd(vadd(vadd(k1, vmul(k2, 2)), vmul(k3, 2)), k4), h / 6.0));
    nx = vadd(x, vmul(vadd(vadd(vadd(l1, vmul(l2, 2)), vmul(l3, 2)), l4), h / 6.0));
    hs = h;
    nrhs += 4;
}

inline real cartsq(const V4& a) { real r = 0; for (int i = 0; i < 4; ++i) r += a[i] * a[i]; return r; }

// IntegrateGeodesicStep_Verlet, Integrators.cpp:99-152. The reference iterates the
// velocity correction without bound; the oracle caps it at `iter_cap` to stay finite
// and reports the cap through `capped`.
void step_verlet(const MetricDef& m, const Integ& I, const V4& x, const V4& v, V4& nx, V4& nv, real& hs,
                 uint64_t& nrhs, bool& capped, int iter_cap) {
    real h = adaptive_step(I, x, v);
    V4 a0 = geo_rhs(m, x, v, I.hfd);
    nx = vadd(vadd(x, vmul(v, h)), vmul(a0, h * h / 2.0));
    V4 vi = vadd(v, vmul(a0, h));
    V4 a1 = geo_rhs(m, nx, vi, I.hfd);
    nv = vadd(v, vmul(vadd(a0, a1), h / 2.0));
    nrhs += 2;
    int it = 0;
    while (I.vtol > 0.0 && cartsq(vsub(nv, vi)) / cartsq(nv) > I.vtol * I.vtol) {
        if (it >= iter_cap) { capped = true; break; }
        vi = nv;
        a1 = geo_rhs(m, nx, vi, I.hfd);
        nv = vadd(v, vmul(vadd(a0, a1), h / 2.0));
        ++nrhs;
        ++it;
    }
    hs = h;
}

// ---- camera, ViewScreen.cpp ---------------------------------------------------------
struct Camera {
    M4 e;       // vielbein rows, m_Vielbein
    M4 gdd;     // m_Metric_dd at the camera
    V4 pos;     // m_Pos
    real size[2], center[2];
};

// ViewScreen::ConstructVielbein, ViewScreen.cpp:10-73 (including the theta-leg quirk at
// :56-58, which subtracts a multiple of the still-zero m_Vielbein[2])
Camera make_camera(const MetricDef& m, const foort_image_desc& im) {
    Camera C{};
    for (int i = 0; i < 4; ++i) C.pos[i] = im.cam_pos[i];
    C.size[0] = im.screen_size[0]; C.size[1] = im.screen_size[1];
    C.center[0] = im.screen_center[0]; C.center[1] = im.screen_center[1];
    V4 p = C.pos;
    p[1] = m.rlog ? std::log(p[1]) : p[1];
    M4 gdd = metric_dd(m, p);
    M4 guu = metric_uu(m, p);
    C.gdd = gdd;
    V4 sg{};
    auto ip = [&gdd](const V4& a, const V4& b) {
        real r = 0;
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j) r += a[i] * gdd[i][j] * b[j];
        return r;
    };
    M4 e{};
    e[0] = guu[0];
    real n = ip(e[0], e[0]);
    sg[0] = (n < 0) ? -1 : 1;
    e[0] = vdiv(vmul(e[0], sg[0]), std::sqrt(sg[0] * n));

    e[3] = vsub(guu[3], vmul(e[0], sg[0] * ip(guu[3], e[0])));
    n = ip(e[3], e[3]);
    sg[3] = (n < 0) ? -1 : 1;
    e[3] = vdiv(vmul(e[3], sg[3] * C.pos[1] * std::sin(C.pos[2])), std::sqrt(sg[3] * n));

    e[1] = vsub(vsub(guu[1], vmul(e[0], sg[0] * ip(guu[1], e[0]))), vmul(e[3], sg[3] * ip(guu[1], e[3])));
    n = ip(e[1], e[1]);
    sg[1] = (n < 0) ? -1 : 1;
    e[1] = vdiv(vmul(e[1], sg[1]), std::sqrt(sg[1] * n));

    e[2] = vsub(vsub(guu[2], vmul(e[0], sg[0] * ip(guu[2], e[0]))), vmul(e[2], sg[3] * ip(guu[2], e[3])));
    n = ip(e[2], e[2]);
    sg[2] = (n < 0) ? -1 : 1;
    e[2] = vdiv(vmul(e[2], sg[2] * C.pos[1]), std::sqrt(sg[2] * n));
    C.e = e;
    return C;
}

// ViewScreen::SetNewInitialConditions, ViewScreen.cpp:75-119, with the unit screen point
// of Mesh.cpp:49 / :671-672 (plus an optional offset used by the sensitivity tests).
void init_conditions(const MetricDef& m, const Camera& C, const foort_pixel& px, real du0, real du1, V4& pos, V4& vel) {
    pos = C.pos;
    pos[1] = m.rlog ? std::log(pos[1]) : pos[1];
    real u0 = px.row * 1.0 / static_cast<real>(px.grid - 1) + du0;
    real u1 = px.col * 1.0 / static_cast<real>(px.grid - 1) + du1;
    real alpha = C.center[0] + C.size[0] * (u0 - 0.5);
    real beta = C.center[1] + C.size[1] * (u1 - 0.5);
    real st0 = std::sin(pos[2]);
    const real R0 = C.pos[1];
    real den = std::sqrt(R0 * R0 + alpha * alpha + beta * beta);
    V4 pf{-1.0, -R0 / den, -beta / R0 / den, alpha / R0 / st0 / den};
    vel = V4{};
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) vel[i] += C.e[j][i] * pf[j];
    real energy = 1.0;
    real cur = 0;
    for (int i = 0; i < 4; ++i) cur += C.gdd[0][i] * vel[i];
    vel = vdiv(vmul(vel, energy), cur);
}

// ---- one geodesic: Geodesic::Reset/Update + Terminations + Diagnostics --------------
struct Opts {
    uint32_t term_flags, diag_flags;
    real h_eps, rh; uint64_t h_every;
    real b_rad; uint64_t b_every;
    uint64_t t_max, t_every;
    real th_eps; uint64_t th_every;
    foort_update_freq eq_f; real eq_thr;
    foort_update_freq cr_f;
    bool rlog;
};

struct Lane {
    V4 x, v;
    real lam;
    int term;
    uint64_t steps;
    // terminations (m_StepsSinceUpdated per class; TimeOut m_CurNrSteps)
    uint64_t cH, cB, cT, cTh, tcur;
    // diagnostics
    int quad;
    uint64_t cE; int passes; real prev;
    uint64_t cC; real rmin;
};

// Termination::DecideUpdate, Terminations.cpp:71-90
inline bool term_decide(uint64_t every, uint64_t& cnt) {
    if (every == 0) return true;
    ++cnt;
    if (cnt >= every) { cnt = 0; return true; }
    return false;
}

// Diagnostic::DecideUpdate, Diagnostics.cpp:113-140
inline bool diag_decide(const foort_update_freq& f, uint64_t& cnt, real lam, int term) {
    if (f.every_n > 0) {
        ++cnt;
        if (cnt >= f.every_n) { cnt = 0; return true; }
        return false;
    }
    if (f.at_start && lam == 0.0) return true;
    if (f.at_finish && term != FOORT_TERMCODE_CONTINUE) return true;
    return false;
}

// All Diagnostic::UpdateData of the value-first vector (Geodesic.cpp:82-85). The
// diagnostics are independent, so their order does not change any value.
void update_diags(const Opts& o, Lane& L) {
    if (o.diag_flags & FOORT_DIAG_FOUR_COLOR_SCREEN) {  // Diagnostics.cpp:159-200
        if (L.term == FOORT_TERMCODE_BOUNDARY_SPHERE) {
            V4 p = L.x;
            if (std::fabs(p[3]) < 2 * kPi * 1e5) {
                while (p[3] > 2 * kPi) p[3] -= 2 * kPi;
                while (p[3] < 0) p[3] += 2 * kPi;
            }
            int q = 0;
            if (p[2] < kPi / 2) q = (p[3] < kPi) ? 1 : 2;
            else q = (p[3] < kPi) ? 3 : 4;
            L.quad = q;
        }
    }
    if (o.diag_flags & FOORT_DIAG_EQUATORIAL_PASSES) {  // Diagnostics.cpp:351-380
        if (diag_decide(o.eq_f, L.cE, L.lam, L.term)) {
            real th = L.x[2];
            if (std::fabs(th - kPi / 2.0) > kPi / 2.0 * o.eq_thr) {
                if (L.prev > 0 && ((L.prev - kPi / 2.0) * (th - kPi / 2.0)) < 0.0) ++L.passes;
                L.prev = th;
            }
        }
        if (L.term == FOORT_TERMCODE_HORIZON) L.passes = -L.passes;
    }
    if (o.diag_flags & FOORT_DIAG_CLOSEST_RADIUS) {  // Diagnostics.cpp:427-446
        if (diag_decide(o.cr_f, L.cC, L.lam, L.term)) {
            real r = o.rlog ? std::exp(L.x[1]) : L.x[1];
            if (L.rmin < 0 || r < L.rmin) L.rmin = r;
        }
        if (L.term == FOORT_TERMCODE_HORIZON) L.rmin = 0.0;
    }
}

// Terminations in CreateTerminationVector order (Terminations.cpp:22-40); the first
// non-Continue result wins (Geodesic.cpp:74-79).
int check_terms(const Opts& o, Lane& L) {
    if (o.term_flags & FOORT_TERM_HORIZON) {  // Terminations.cpp:96-117
        if (term_decide(o.h_every, L.cH)) {
            real r = o.rlog ? std::exp(L.x[1]) : L.x[1];
            if ((r < o.rh * (1 + o.h_eps)) || (o.rh == 0.0 && r < o.h_eps)) return FOORT_TERMCODE_HORIZON;
        }
    }
    if (o.term_flags & FOORT_TERM_BOUNDARY_SPHERE) {  // Terminations.cpp:130-146
        if (term_decide(o.b_every, L.cB)) {
            real r = o.rlog ? std::exp(L.x[1]) : L.x[1];
            if (r > o.b_rad) return FOORT_TERMCODE_BOUNDARY_SPHERE;
        }
    }
    if (o.term_flags & FOORT_TERM_TIMEOUT) {  // Terminations.cpp:168-186
        if (term_decide(o.t_every, L.cT)) {
            if (L.tcur >= o.t_max) return FOORT_TERMCODE_TIMEOUT;
            ++L.tcur;
        }
    }
    if (o.term_flags & FOORT_TERM_THETA_SINGULARITY) {  // Terminations.cpp:200-214
        if (term_decide(o.th_every, L.cTh)) {
            real th = L.x[2];
            if (std::fabs(th) < o.th_eps || std::fabs(kPi - th) < o.th_eps) return FOORT_TERMCODE_THETA_SINGULARITY;
        }
    }
    return FOORT_TERMCODE_CONTINUE;
}

Opts make_opts(const foort_run_desc& d, const MetricDef& m, const foort_image_desc& im) {
    Opts o{};
    o.term_flags = d.term_flags;
    // Config.cpp:644-683: Horizon only exists for metrics with a horizon.
    if (d.metric_id == FOORT_METRIC_FLAT) o.term_flags &= ~FOORT_TERM_HORIZON;
    o.diag_flags = d.diag_flags;
    o.h_eps = im.horizon_eps > 0.0 ? im.horizon_eps : d.horizon_eps;
    o.rh = m.rh;
    o.h_every = d.horizon_every;
    o.b_rad = d.boundary_radius; o.b_every = d.boundary_every;
    o.t_max = d.timeout_max_steps; o.t_every = d.timeout_every;
    o.th_eps = d.theta_eps; o.th_every = d.theta_every;
    o.eq_f = d.equat_freq; o.eq_thr = d.equat_threshold;
    o.cr_f = d.closest_freq;
    o.rlog = d.rlog != 0 && d.metric_id != FOORT_METRIC_FLAT;
    return o;
}

// Geodesic::Reset (Geodesic.cpp:33-58) then the Update loop of Main.cpp:387-390.
void integrate_one(const MetricDef& m, const Integ& I, const Opts& o, const Camera& C, const foort_pixel& px,
                   real du0, real du1, uint64_t max_steps_guard, foort_result& out) {
    Lane L{};
    init_conditions(m, C, px, du0, du1, L.x, L.v);
    L.lam = 0.0;
    L.term = FOORT_TERMCODE_CONTINUE;
    L.quad = 0; L.cE = 0; L.passes = 0; L.prev = -1; L.cC = 0; L.rmin = -1;
    update_diags(o, L);
    L.cH = L.cB = L.cT = L.cTh = 0; L.tcur = 0;
    uint32_t err = 0;
    uint64_t nrhs = 0;
    while (L.term == FOORT_TERMCODE_CONTINUE) {
        if (max_steps_guard && L.steps >= max_steps_guard) { err |= FOORT_ERR_BUDGET; break; }
        V4 nx, nv;
        real h = 0;
        bool capped = false;
        if (I.id == FOORT_INTEGRATOR_RK4) step_rk4(m, I, L.x, L.v, nx, nv, h, nrhs);
        else step_verlet(m, I, L.x, L.v, nx, nv, h, nrhs, capped, 1 << 20);
        if (capped) err |= FOORT_ERR_VERLET_ITER;
        L.lam += h;
        L.x = nx;
        L.v = nv;
        ++L.steps;
        L.term = check_terms(o, L);
        update_diags(o, L);
        // A non-finite state is flagged; like the reference, integration then runs on
        // until a termination fires (TimeOut). Without TimeOut the reference would loop
        // forever, so the geodesic is stopped there instead.
        bool finite = true;
        for (int i = 0; i < 4; ++i) finite = finite && std::isfinite(L.x[i]) && std::isfinite(L.v[i]);
        if (!finite) {
            err |= FOORT_ERR_NONFINITE;
            if (L.term == FOORT_TERMCODE_CONTINUE && !(o.term_flags & FOORT_TERM_TIMEOUT)) break;
        }
    }
    out.term = L.term;
    out.err = err;
    out.steps = L.steps;
    out.lambda = L.lam;
    for (int i = 0; i < 4; ++i) { out.pos[i] = L.x[i]; out.vel[i] = L.v[i]; }
    out.quadrant = L.quad;
    out.equat_passes = L.passes;
    out.closest_r = L.rmin;
}

int validate(const foort_run_desc* d) {
    if (!d || d->n_images == 0 || !d->images) return FOORT_E_BADARG;
    if (d->metric_id < 0 || d->metric_id > 4) return FOORT_E_BADARG;
    if (d->integrator_id != FOORT_INTEGRATOR_RK4 && d->integrator_id != FOORT_INTEGRATOR_VERLET) return FOORT_E_BADARG;
    return FOORT_OK;
}

int run(const foort_run_desc* d, const foort_pixel* px, uint64_t n, real du0, real du1, foort_result* out,
        int nthreads, uint64_t max_steps_guard) {
    int rc = validate(d);
    if (rc) return rc;
    if (n && (!px || !out)) return FOORT_E_BADARG;
    std::vector<MetricDef> ms(d->n_images);
    std::vector<Camera> cs(d->n_images);
    std::vector<Opts> os(d->n_images);
    for (uint32_t i = 0; i < d->n_images; ++i) {
        ms[i] = make_metric(d->metric_id, d->images[i].metric_params, d->rlog != 0);
        if (d->metric_id == FOORT_METRIC_FLAT) ms[i].rlog = false;
        cs[i] = make_camera(ms[i], d->images[i]);
        os[i] = make_opts(*d, ms[i], d->images[i]);
    }
    for (uint64_t i = 0; i < n; ++i)
        if (px[i].image >= d->n_images) return FOORT_E_BADARG;
    Integ I{d->integrator_id, d->epsilon, d->derivative_h, d->smallest_step, d->verlet_tol};
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads)
#endif
    for (long long i = 0; i < static_cast<long long>(n); ++i) {
        const foort_pixel& p = px[i];
        integrate_one(ms[p.image], I, os[p.image], cs[p.image], p, du0, du1, max_steps_guard, out[i]);
    }
    (void)nthreads;
    return FOORT_OK;
}

}  // namespace

extern "C" {

// Integrate n pixels exactly as Main.cpp:348-402 does (nthreads <= 0: all threads).
int oracle_integrate(const foort_run_desc* d, const foort_pixel* px, uint64_t n, foort_result* out, int nthreads) {
    return run(d, px, n, 0.0, 0.0, out, nthreads, 0);
}

// Same with the unit screen point shifted by (du0, du1) and an optional per-geodesic
// step guard (0 = none); used to show that a mismatching pixel sits on a decision
// boundary (its outcome flips under a tiny shift of the initial condition).
int oracle_integrate_offset(const foort_run_desc* d, const foort_pixel* px, uint64_t n, double du0, double du1,
                            foort_result* out, int nthreads, uint64_t max_steps_guard) {
    return run(d, px, n, du0, du1, out, nthreads, max_steps_guard);
}

// Metric::getMetric_dd / getMetric_uu at one point, row-major 4x4.
int oracle_metric(int32_t metric_id, const double* params, int32_t rlog, const double* x, double* gdd, double* guu) {
    MetricDef m = make_metric(metric_id, params, rlog != 0);
    V4 p{x[0], x[1], x[2], x[3]};
    M4 a = metric_dd(m, p), b = metric_uu(m, p);
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) { gdd[4 * i + j] = a[i][j]; guu[4 * i + j] = b[i][j]; }
    return FOORT_OK;
}

// Metric::getChristoffel_udd at one point, gamma[16*mu + 4*nu + rho].
int oracle_christoffel(int32_t metric_id, const double* params, int32_t rlog, double h, const double* x, double* gamma) {
    MetricDef m = make_metric(metric_id, params, rlog != 0);
    V4 p{x[0], x[1], x[2], x[3]};
    T4 G = christoffel(m, p, h);
    for (int a = 0; a < 4; ++a)
        for (int b = 0; b < 4; ++b)
            for (int c = 0; c < 4; ++c) gamma[16 * a + 4 * b + c] = G[a][b][c];
    return FOORT_OK;
}

// Camera frame of image `image` (vielbein rows e[4*j + i] = e_j^i) and metric at the camera.
int oracle_camera(const foort_run_desc* d, uint32_t image, double* vielbein, double* gdd) {
    if (validate(d) || image >= d->n_images) return FOORT_E_BADARG;
    MetricDef m = make_metric(d->metric_id, d->images[image].metric_params, d->rlog != 0);
    Camera C = make_camera(m, d->images[image]);
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) { vielbein[4 * i + j] = C.e[i][j]; gdd[4 * i + j] = C.gdd[i][j]; }
    return FOORT_OK;
}

// Initial position and velocity of one pixel (ViewScreen::SetNewInitialConditions).
int oracle_initial_conditions(const foort_run_desc* d, const foort_pixel* px, double* pos, double* vel) {
    if (validate(d) || !px || px->image >= d->n_images) return FOORT_E_BADARG;
    MetricDef m = make_metric(d->metric_id, d->images[px->image].metric_params, d->rlog != 0);
    Camera C = make_camera(m, d->images[px->image]);
    V4 x, v;
    init_conditions(m, C, *px, 0.0, 0.0, x, v);
    for (int i = 0; i < 4; ++i) { pos[i] = x[i]; vel[i] = v[i]; }
    return FOORT_OK;
}

double oracle_horizon_radius(int32_t metric_id, const double* params) {
    return make_metric(metric_id, params, false).rh;
}

}  // extern "C"
