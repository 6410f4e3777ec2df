// Host-side evaluation of the analytic metric plugins: the engine's counterpart of
// Metric::getChristoffel_udd (Metric.cpp:14-55), exact instead of finite differences.
#include <cmath>

#include "../../include/foort_gpu.h"
#include "analytic_metric.cuh"

using namespace foort;

namespace {

template <int MID>
int christoffel_host(const double* params, bool rlog, const double* x, double* gamma) {
    MetricConst M = make_metric_const(MID, params);
    double q[kMixedQ], rp, rm;
    mixed_metric_constants(MID, M, q);
    mixed_horizons(MID, M, rp, rm);
    const double r = rlog ? std::exp(x[1]) : x[1];
    const double s = std::sin(x[2]), c = std::cos(x[2]);
    G5T<double> dr, dh, gu;
    double grr;
    MixedMetric<MID>::template eval<double>(q, r, r - rp, r - rm, s, c, dr, dh, gu, grr);
    if (rlog) to_log_r(r, grr, dr, dh, gu);
    double d[4][4][4] = {}, g[4][4] = {};
    auto put = [](double m[4][4], const G5T<double>& v) {
        m[0][0] = v.tt; m[0][3] = m[3][0] = v.tp; m[1][1] = v.rr; m[2][2] = v.hh; m[3][3] = v.pp;
    };
    put(d[1], dr);
    put(d[2], dh);
    put(g, gu);
    for (int mu = 0; mu < 4; ++mu)
        for (int nu = 0; nu < 4; ++nu)
            for (int rho = 0; rho < 4; ++rho) {
                double acc = 0.0;
                for (int sg = 0; sg < 4; ++sg)
                    acc += 0.5 * g[mu][sg] * (d[nu][rho][sg] + d[rho][nu][sg] - d[sg][nu][rho]);
                gamma[16 * mu + 4 * nu + rho] = acc;
            }
    return FOORT_OK;
}

}  // namespace

extern "C" int foort_metric_christoffel(int32_t metric_id, const double* params, int32_t rlog, const double* x,
                                        double* gamma) {
    if (!params || !x || !gamma) return FOORT_E_BADARG;
    switch (metric_id) {
    case FOORT_METRIC_KERR: return christoffel_host<kKerr>(params, rlog != 0, x, gamma);
    case FOORT_METRIC_JOHANNSEN: return christoffel_host<kJohannsen>(params, rlog != 0, x, gamma);
    case FOORT_METRIC_FLAT: return christoffel_host<kFlat>(params, false, x, gamma);
    case FOORT_METRIC_RASHEED_LARSEN: return christoffel_host<kRasheedLarsen>(params, rlog != 0, x, gamma);
    case FOORT_METRIC_MANKO_NOVIKOV: return christoffel_host<kMankoNovikov>(params, rlog != 0, x, gamma);
    default: return FOORT_E_UNSUPPORTED;
    }
}
