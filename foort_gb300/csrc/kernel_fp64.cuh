// Plain FP64 integration kernel: the reference's algorithm on the GPU.
//
// One thread integrates one geodesic with its whole state in registers. The right-hand
// side is the reference's: finite-difference metric derivatives in r and theta
// (Metric.cpp:14-32) with h = Derivative_hval, the analytic inverse metric, the
// Christoffel symbols and the contraction with the velocity (Metric.cpp:39-53,
// Integrators.cpp:60-68), all in FP64. sin/cos/exp are evaluated once per distinct
// argument: the two radial shifts share theta, the two angular shifts share r.
#pragma once

#include "kernel_common.cuh"

namespace foort {

// The position-dependent part of the right-hand side: central differences of g_dd in x1
// and x2 and the inverse metric at x (Metric.cpp:14-38).
struct FdParts {
    G5 dr, dh, gu;
};

template <int MID>
__device__ __forceinline__ FdParts fd_parts_fp64(const MetricConst& M, bool rlog, double hfd, const double x[4]) {
    using Mt = MetricFP64<MID>;
    double r0, rp, rm;
    if (rlog) {
        r0 = exp(x[1]);
        rp = exp(x[1] + hfd);
        rm = exp(x[1] - hfd);
    } else {
        r0 = x[1];
        rp = x[1] + hfd;
        rm = x[1] - hfd;
    }
    double s0, c0, sp, cp, sm, cm;
    sincos(x[2], &s0, &c0);
    sincos(x[2] + hfd, &sp, &cp);
    sincos(x[2] - hfd, &sm, &cm);
    const G5 a = Mt::dd(M, rp, s0, c0, rlog);
    const G5 b = Mt::dd(M, rm, s0, c0, rlog);
    const G5 c = Mt::dd(M, r0, sp, cp, rlog);
    const G5 d = Mt::dd(M, r0, sm, cm, rlog);
    const G5 gu = Mt::uu(M, r0, s0, c0, rlog);
    const double inv = 1 / (2 * hfd);
    FdParts P;
    G5& dr = P.dr;
    G5& dh = P.dh;
    dr.tt = (a.tt - b.tt) * inv; dr.tp = (a.tp - b.tp) * inv; dr.rr = (a.rr - b.rr) * inv;
    dr.hh = (a.hh - b.hh) * inv; dr.pp = (a.pp - b.pp) * inv;
    dh.tt = (c.tt - d.tt) * inv; dh.tp = (c.tp - d.tp) * inv; dh.rr = (c.rr - d.rr) * inv;
    dh.hh = (c.hh - d.hh) * inv; dh.pp = (c.pp - d.pp) * inv;
    P.gu = gu;
    return P;
}

// The Christoffel symbols from the parts and their contraction with v (Metric.cpp:39-53,
// Integrators.cpp:60-68).
__device__ __forceinline__ void contract_fp64(const FdParts& P, const double v[4], double acc[4]) {
    const G5& dr = P.dr;
    const G5& dh = P.dh;
    const G5& gu = P.gu;
#include "gen_fd_christoffel.inc"
}

template <int MID>
__device__ __forceinline__ void rhs_fd_fp64(const MetricConst& M, bool rlog, double hfd, const double x[4],
                                            const double v[4], double acc[4]) {
    contract_fp64(fd_parts_fp64<MID>(M, rlog, hfd, x), v, acc);
}

template <int MID, int INTEG>
struct Fp64Engine {
    struct Lane {
        double x[4], v[4];
        double lam;
        uint64_t steps;
        TermState T;
        DiagState D;
        uint32_t err = 0;
        uint32_t img = 0;
        uint32_t rhs = 0;
        uint32_t fp64 = 0;
        int32_t term = 0;
        GeoposRec gp;  // set by the loop before init (dst null: not recording)
        FdParts P;     // Verlet: the parts at x (computed at the previous step's new position)
    };

    static __device__ __forceinline__ void init(Lane& L, const ImageConst& I, const RunConst& R, const foort_pixel& p) {
        initial_conditions(I, p, L.x, L.v);
        if (INTEG == FOORT_INTEGRATOR_VERLET) L.P = fd_parts_fp64<MID>(I.m, R.rlog != 0, R.hfd, L.x);
        L.lam = 0.0;
        L.steps = 0;
        L.err = 0;
        L.term = FOORT_TERMCODE_CONTINUE;
        L.img = p.image;
        reset_lane_state(R, L.x, L.D, L.T);
        if (L.gp.dst) geopos_sample(L.gp, R, L.x, 0.0, FOORT_TERMCODE_CONTINUE);  // Geodesic::Reset's sample
    }

    // One Geodesic::Update (Geodesic.cpp:61-88). Returns false once the geodesic ends.
    static __device__ __forceinline__ bool step(Lane& L, const ImageConst& I, const RunConst& R) {
        const MetricConst& M = I.m;
        const bool rlog = R.rlog != 0;
        double h = adaptive_step_fp64(R, L.x, L.v);
        double nx[4], nv[4];
        if (INTEG == FOORT_INTEGRATOR_RK4) {  // Integrators.cpp:51-94
            double k1[4], k2[4], k3[4], k4[4], l2[4], l3[4], l4[4], t[4];
            rhs_fd_fp64<MID>(M, rlog, R.hfd, L.x, L.v, k1);
            const double hh = 0.5 * h;
#pragma unroll
            for (int i = 0; i < 4; ++i) { t[i] = L.x[i] + L.v[i] * hh; l2[i] = L.v[i] + k1[i] * hh; }
            rhs_fd_fp64<MID>(M, rlog, R.hfd, t, l2, k2);
#pragma unroll
            for (int i = 0; i < 4; ++i) { t[i] = L.x[i] + l2[i] * hh; l3[i] = L.v[i] + k2[i] * hh; }
            rhs_fd_fp64<MID>(M, rlog, R.hfd, t, l3, k3);
#pragma unroll
            for (int i = 0; i < 4; ++i) { t[i] = L.x[i] + l3[i] * h; l4[i] = L.v[i] + k3[i] * h; }
            rhs_fd_fp64<MID>(M, rlog, R.hfd, t, l4, k4);
            const double h6 = h / 6.0;
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                nv[i] = L.v[i] + (((k1[i] + k2[i] * 2) + k3[i] * 2) + k4[i]) * h6;
                nx[i] = L.x[i] + (((L.v[i] + l2[i] * 2) + l3[i] * 2) + l4[i]) * h6;
            }
            L.rhs += 4;
        } else {  // Integrators.cpp:99-152
            // Every right-hand side after the first is evaluated at the new position nx,
            // which is where the next step's first one is evaluated: the metric parts
            // there are computed once and kept for the next step. The reference computes
            // them again from the same nx, so the values are the same.
            double a0[4], a1[4], vi[4];
            contract_fp64(L.P, L.v, a0);
            const double hh2 = h * h / 2.0;
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                nx[i] = (L.x[i] + L.v[i] * h) + a0[i] * hh2;
                vi[i] = L.v[i] + a0[i] * h;
            }
            const FdParts Pn = fd_parts_fp64<MID>(M, rlog, R.hfd, nx);
            contract_fp64(Pn, vi, a1);
            const double h2 = h / 2.0;
#pragma unroll
            for (int i = 0; i < 4; ++i) nv[i] = L.v[i] + (a0[i] + a1[i]) * h2;
            L.rhs += 2;
            if (R.vtol > 0.0) {
                const double tol2 = R.vtol * R.vtol;
                for (int it = 0;; ++it) {
                    double num = 0.0, den = 0.0;
#pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        const double d = nv[i] - vi[i];
                        num += d * d;
                        den += nv[i] * nv[i];
                    }
                    if (!(num / den > tol2)) break;
                    if (it >= R.verlet_cap) {
                        L.err |= FOORT_ERR_VERLET_ITER;
                        break;
                    }
#pragma unroll
                    for (int i = 0; i < 4; ++i) vi[i] = nv[i];
                    contract_fp64(Pn, vi, a1);
#pragma unroll
                    for (int i = 0; i < 4; ++i) nv[i] = L.v[i] + (a0[i] + a1[i]) * h2;
                    L.rhs += 1;
                }
            }
            L.P = Pn;
        }
        L.lam += h;
#pragma unroll
        for (int i = 0; i < 4; ++i) { L.x[i] = nx[i]; L.v[i] = nv[i]; }
        ++L.steps;
        const double r = radius_of(R, L.x[1]);
        L.term = check_terms(R, M.rh, I.h_eps, r, L.x[2], L.T);
        update_diags(R, r, L.x[2], L.x[3], L.lam, L.term, L.D);
        if (L.gp.dst) geopos_sample(L.gp, R, L.x, L.lam, L.term);
        if (!(finite4(L.x) && finite4(L.v))) {
            // The reference keeps integrating a non-finite state until TimeOut fires;
            // without TimeOut it would never stop, so the lane stops here.
            L.err |= FOORT_ERR_NONFINITE;
            if (L.term == FOORT_TERMCODE_CONTINUE && !(R.term_flags & FOORT_TERM_TIMEOUT)) return false;
        }
        return L.term == FOORT_TERMCODE_CONTINUE;
    }

    static __device__ __forceinline__ void finish(const Lane& L, const RunConst&, foort_result* o) {
        write_result(o, L.term, L.err, L.steps, L.lam, L.x, L.v, L.D);
    }
    static __device__ __forceinline__ void stop(const Lane& L, const RunConst&, foort_result* o, uint32_t err) {
        write_result(o, FOORT_TERMCODE_CONTINUE, L.err | err, L.steps, L.lam, L.x, L.v, L.D);
    }
};

template <int MID, int INTEG>
__global__ void __launch_bounds__(128) integrate_fp64_kernel(const __grid_constant__ LaunchArgs A,
                                                             const __grid_constant__ RunConst R) {
    persistent_loop<Fp64Engine<MID, INTEG>>(A, R);
}

}  // namespace foort
