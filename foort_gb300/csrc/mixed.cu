// Host side of the mixed-precision kernels: kernel registry and per-image constants.
#include <algorithm>
#include <cfloat>
#include <cmath>

#include "kernel_mixed.cuh"
#include "kernels.h"

namespace foort {

const void* mixed_kernel_kerr(int integrator, bool decide64);
const void* mixed_kernel_joh(int integrator, bool decide64);
const void* mixed_kernel_flat(int integrator, bool decide64);
const void* mixed_kernel_rl(int integrator, bool decide64);
const void* mixed_kernel_mn(int integrator, bool decide64);

// Mixed kernels for every metric: analytic derivatives generated by gen_christoffel.py,
// and for Manko-Novikov by forward-mode differentiation (analytic_metric.cuh).
const void* mixed_kernel_variant(int metric_id, int integ, bool decide64) {
    switch (metric_id) {
    case kKerr: return mixed_kernel_kerr(integ, decide64);
    case kJohannsen: return mixed_kernel_joh(integ, decide64);
    case kFlat: return mixed_kernel_flat(integ, decide64);
    case kRasheedLarsen: return mixed_kernel_rl(integ, decide64);
    case kMankoNovikov: return mixed_kernel_mn(integ, decide64);
    default: return nullptr;
    }
}

const void* mixed_kernel(int metric_id, int integ) { return mixed_kernel_variant(metric_id, integ, true); }

const void* mixed_pair_kernel_kerr(bool decide64);
const void* mixed_pair_kernel_flat(bool decide64);

// Two-lane kernels: RK4 with the inlined plugins (Kerr, flat space).
const void* mixed_pair_kernel_variant(int metric_id, int integ, bool decide64) {
    if (integ != FOORT_INTEGRATOR_RK4) return nullptr;
    switch (metric_id) {
    case kKerr: return mixed_pair_kernel_kerr(decide64);
    case kFlat: return mixed_pair_kernel_flat(decide64);
    default: return nullptr;
    }
}

void fill_mixed_constants(int metric_id, ImageConst& ic, const RunConst& rc) {
    MixedConst& mx = ic.mx;
    mixed_metric_constants(metric_id, ic.m, ic.qa);
    for (int i = 0; i < kMixedQ; ++i) mx.q[i] = static_cast<float>(ic.qa[i]);
    double rp, rm;
    mixed_horizons(metric_id, ic.m, rp, rm);
    mx.rpv = rp;
    mx.rmv = rm;
    ff_split(rp, mx.rp[0], mx.rp[1]);
    ff_split(rm, mx.rm[0], mx.rm[1]);
    ff_split(rp > 0 ? std::log(rp) : 0.0, mx.lrp[0], mx.lrp[1]);
    ff_split(rm > 0 ? std::log(rm) : 0.0, mx.lrm[0], mx.lrm[1]);
    const bool rlog = rc.rlog != 0;
    auto coord = [rlog](double r) { return rlog ? std::log(r) : r; };
    double r_fp64 = (rc.mixed_fp64_margin > 0.0 && rp > 0.0) ? rp + rc.mixed_fp64_margin : 0.0;
    // Manko-Novikov's exponents grow without bound toward the horizon and its metric
    // leaves FP32's range there: inside the radius where one exceeds 8 (e^8 ~ 3e3), the
    // right-hand side is always taken in FP64
    if (metric_id == kMankoNovikov) r_fp64 = std::max(r_fp64, mn_fp64_radius(ic.m, kMnMaxFp32Exponent));
    mx.r_fp64 = r_fp64 > 0.0 ? static_cast<float>(coord(r_fp64)) : 0.f;
    // FP64-analytic: every step in FP64 (x1 < +inf holds for every finite position)
    if (rc.precision == FOORT_PREC_FP64_ANALYTIC) mx.r_fp64 = HUGE_VALF;
    const double rh = ic.m.rh;
    ff_split(coord(rh * (1 + ic.h_eps)), mx.hthr[0], mx.hthr[1]);
    ff_split(ic.h_eps > 0 ? coord(ic.h_eps) : (rlog ? -HUGE_VAL : 0.0), mx.hthr0[0], mx.hthr0[1]);
    ff_split(coord(rc.b_rad), mx.bthr[0], mx.bthr[1]);
    ff_split(rc.th_eps, mx.theps[0], mx.theps[1]);
    ff_split(kRefPi, mx.pi[0], mx.pi[1]);
    ff_split(-(kRefPi / 2.0), mx.mpio2[0], mx.mpio2[1]);
    ff_split(kRefPi / 2.0 * rc.eq_thr, mx.eqthr[0], mx.eqthr[1]);
    ff_split(rc.eps, mx.eps[0], mx.eps[1]);
    mx.hmin = static_cast<float>(rc.hmin);
    // a positive tolerance whose square is below FP32's range still iterates (as with 0)
    mx.vtol2 = rc.vtol > 0.0 ? std::max(static_cast<float>(rc.vtol * rc.vtol), FLT_MIN) : 0.f;
}

}  // namespace foort
