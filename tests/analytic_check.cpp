// FP32 accuracy of the analytic metric plugins (built and run by
// tests/test_analytic_metrics.py).
//
// For each metric, random points r in [r_+ + 0.01, 1000] (log-uniform) and theta, and
// random null velocities, the geodesic acceleration is evaluated with the plugin in
// double and in float (the float inputs prepared as the mixed kernel prepares them:
// r - r_+ and r - r_- from the exact radius, then rounded). Output, one line per case:
//   name p50 p90 p99 max
// of |a_float - a_double| / |a_double|_inf.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

#include "../foort_gb300/csrc/analytic_metric.cuh"

using namespace foort;

template <int MID>
void run(const char* name, const double* params, bool rlog, double r_from = 0.0) {
    MetricConst M = make_metric_const(MID, params);
    double qd[kMixedQ], rp, rm;
    mixed_metric_constants(MID, M, qd);
    mixed_horizons(MID, M, rp, rm);
    float qf[kMixedQ];
    for (int i = 0; i < kMixedQ; ++i) qf[i] = static_cast<float>(qd[i]);
    std::mt19937_64 rng(7);
    std::uniform_real_distribution<double> U(0.0, 1.0);
    std::vector<double> errs;
    const double rlo = r_from > 0.0 ? r_from : (rp > 0 ? rp : 1.0) + 0.01;
    for (int k = 0; k < 20000; ++k) {
        const double r = rlo * std::pow(1000.0 / rlo, U(rng));
        const double th = 0.05 + (M_PI - 0.1) * U(rng);
        const double s = std::sin(th), c = std::cos(th);
        G5T<double> dr, dh, gu;
        double grr;
        MixedMetric<MID>::template eval<double>(qd, r, r - rp, r - rm, s, c, dr, dh, gu, grr);
        G5 g = metric_dd_host(MID, M, r, s, c, false);
        // random spatial direction, u^t from the null condition with E = -u_t ~ 1
        double ur = 2 * U(rng) - 1, uh = (2 * U(rng) - 1) / r, up = (2 * U(rng) - 1) / (r * (s + 1e-3));
        double A = g.tt, B = 2 * g.tp * up, Cc = g.rr * ur * ur + g.hh * uh * uh + g.pp * up * up;
        double disc = B * B - 4 * A * Cc;
        if (disc < 0) continue;
        double ut = (-B - std::sqrt(disc)) / (2 * A);
        double u[4] = {ut, ur, uh, up};
        if (rlog) {
            to_log_r(r, grr, dr, dh, gu);
            u[1] = ur / r;  // d ln r / d lambda
        }
        double ad[4];
        accel_lagrange(dr, dh, gu, u, ad);
        // float path
        float rf = static_cast<float>(r), dpf = static_cast<float>(r - rp), dmf = static_cast<float>(r - rm);
        float sf, cf;  // as the kernel forms them, from the float-float angle
        const float th_hi = static_cast<float>(th);
        ff_sincos(th_hi, static_cast<float>(th - th_hi), sf, cf);
        G5T<float> fr, fh, fu;
        float frr;
        if constexpr (MID == kMankoNovikov) {  // as the kernel calls it: the position also in FP64
            MixedMetric<MID>::template eval_hi<float>(qf, r, r - rp, s, c, dpf, dmf, sf, cf, fr, fh, fu, frr);
        } else {
            MixedMetric<MID>::template eval<float>(qf, rf, dpf, dmf, sf, cf, fr, fh, fu, frr);
        }
        float uf[4] = {static_cast<float>(u[0]), static_cast<float>(u[1]), static_cast<float>(u[2]), static_cast<float>(u[3])};
        float af[4];
        if (rlog) {
            accel_log_r(rf, fr, fh, fu, uf, af);  // the kernel's log-r form
        } else {
            accel_lagrange(fr, fh, fu, uf, af);
        }
        double scale = 0, diff = 0;
        for (int i = 0; i < 4; ++i) {
            scale = std::max(scale, std::fabs(ad[i]));
            diff = std::max(diff, std::fabs(static_cast<double>(af[i]) - ad[i]));
        }
        if (!(scale > 0)) continue;
        errs.push_back(std::isfinite(diff) ? diff / scale : 1e30);
    }
    std::sort(errs.begin(), errs.end());
    auto q = [&](double f) { return errs[static_cast<size_t>(f * (errs.size() - 1))]; };
    std::printf("%s %.3e %.3e %.3e %.3e\n", name, q(0.5), q(0.9), q(0.99), errs.back());
}

// ff_sincos against long-double sin and cos of the exact float-float angle: relative
// error max(|ds| / |s|, |dc| / |c|), on angles across (-0.5, pi + 0.5) and within 1e-12 to
// 1e-3 of 0, pi/2 and pi, where the small one of sin and cos must stay accurate.
void sincos_check() {
    std::mt19937_64 rng(3);
    std::uniform_real_distribution<double> U(0.0, 1.0);
    const long double kPi = 3.141592653589793238462643383279503L;
    std::vector<double> errs;
    for (int k = 0; k < 200000; ++k) {
        long double th;
        const int kind = k % 4;
        if (kind == 0) {
            th = -0.5L + (kPi + 1.0L) * U(rng);
        } else {
            const long double off = std::pow(10.0L, -12.0L + 9.0L * U(rng)) * (U(rng) < 0.5 ? -1 : 1);
            th = (kind == 1 ? 0.0L : kind == 2 ? kPi / 2 : kPi) + off;
        }
        const float hi = static_cast<float>(th);
        const float lo = static_cast<float>(th - hi);
        const long double te = static_cast<long double>(hi) + lo;
        float s, c;
        ff_sincos(hi, lo, s, c);
        const long double se = std::sin(te), ce = std::cos(te);
        const double e = std::max(std::fabs((s - se) / se), std::fabs((c - ce) / ce));
        errs.push_back(std::isfinite(e) ? e : 1e30);
    }
    std::sort(errs.begin(), errs.end());
    auto q = [&](double f) { return errs[static_cast<size_t>(f * (errs.size() - 1))]; };
    std::printf("ff_sincos %.3e %.3e %.3e %.3e\n", q(0.5), q(0.9), q(0.99), errs.back());
}

int main() {
    sincos_check();
    const double kerr99[6] = {0.99}, kerr5[6] = {0.5}, kerr998[6] = {0.998};
    const double joh_c4[6] = {0.9, -0.5, 0, 0, 0}, joh_test[6] = {0.7, 2.0, 0, 0, 0}, joh_all[6] = {0.8, 1.0, 0.5, 0.2, 0.1};
    const double none[6] = {0};
    run<kKerr>("kerr_a0.99", kerr99, false);
    run<kKerr>("kerr_a0.5", kerr5, false);
    run<kKerr>("kerr_a0.998", kerr998, false);
    run<kKerr>("kerr_a0.5_logr", kerr5, true);
    run<kJohannsen>("johannsen_c4", joh_c4, false);
    run<kJohannsen>("johannsen_test_logr", joh_test, true);
    run<kJohannsen>("johannsen_all_params", joh_all, false);
    run<kFlat>("flat", none, false);
    // Rasheed-Larsen: the "Lorenzo" and "M1" parameter sets of the reference's Test.cfg
    // (M1 is extremal, m = a), and the reference's defaults (p = 2m: no dyonic terms)
    const double rl_lorenzo[6] = {0.3556562853309941, 0.2969060968239216, 3.057664971085168, 0.942335028914832};
    const double rl_m1[6] = {0.0000292676523070559347272298622578, 0.0000292676523070559347272298622578,
                             3.15470053516341633378322799917, 0.84529946483658456162619604143};
    const double rl_default[6] = {1.0, 0.5, 2.0, 2.0};
    run<kRasheedLarsen>("rasheed_larsen_lorenzo", rl_lorenzo, false);
    run<kRasheedLarsen>("rasheed_larsen_lorenzo_logr", rl_lorenzo, true);
    run<kRasheedLarsen>("rasheed_larsen_m1", rl_m1, false);
    run<kRasheedLarsen>("rasheed_larsen_default", rl_default, false);
    // Manko-Novikov (a, alpha3): the reference's Test.cfg value alpha3 = 13, its default 5,
    // and a mild 1; outside the radius inside which the kernel takes FP64
    const double mn_sets[3][6] = {{0.94, 13.0}, {0.9, 5.0}, {0.7, 1.0}};
    const char* mn_names[3] = {"manko_novikov_a0.94_alpha3_13", "manko_novikov_a0.9_alpha3_5",
                               "manko_novikov_a0.7_alpha3_1"};
    for (int i = 0; i < 3; ++i) {
        const MetricConst M = make_metric_const(kMankoNovikov, mn_sets[i]);
        run<kMankoNovikov>(mn_names[i], mn_sets[i], false, mn_fp64_radius(M, kMnMaxFp32Exponent));
    }
    return 0;
}
