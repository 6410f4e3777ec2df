// Device code shared by the FP64 and the mixed-precision integration kernels:
// initial conditions, terminations, diagnostics, result records and the persistent
// work-queue loop. All decisions (terminations, equator crossings, quadrants) are taken
// in FP64 on the FP64 view of the state, as the reference takes them.
#pragma once

#include <cuda_runtime.h>

#include "engine.h"

namespace foort {

constexpr unsigned kFullMask = 0xffffffffu;

// ---- terminations (Terminations.cpp) -------------------------------------------------
// Step counters of the terminations and diagnostics. The reference's are 64-bit. A kernel
// may keep them in 32 bits (StepCount), which saves registers and instructions on every
// step: they count at most a geodesic's steps, so they differ from the reference's only
// for an update frequency or TimeOut limit of 2^32 steps or more on a geodesic that runs
// that long (where a 32-bit counter wraps to 0 and restarts).
using StepCount = uint32_t;

template <typename C>
struct TermStateT {
    C cH, cB, cT, cTh;  // m_StepsSinceUpdated of each termination
    C tcur;             // TimeOutTermination::m_CurNrSteps
};
using TermState = TermStateT<StepCount>;

// Termination::DecideUpdate, Terminations.cpp:71-90
template <typename C>
__device__ __forceinline__ bool term_decide(uint64_t every, C& cnt) {
    if (every == 0) return true;
    ++cnt;
    if (cnt >= every) {
        cnt = 0;
        return true;
    }
    return false;
}

// Radius of the current position (exp(u) in log-r mode), as every termination and
// diagnostic computes it (Terminations.cpp:106-107, :139-140; Diagnostics.cpp:433).
__device__ __forceinline__ double radius_of(const RunConst& R, double x1) { return R.rlog ? exp(x1) : x1; }

// Terminations in CreateTerminationVector order (Terminations.cpp:22-40): Horizon,
// BoundarySphere, TimeOut, ThetaSingularity; the first non-Continue wins
// (Geodesic.cpp:74-79) and the later ones are not consulted.
template <typename C>
__device__ __forceinline__ int check_terms(const RunConst& R, double rh, double heps, double r, double th,
                                           TermStateT<C>& T) {
    if (R.term_flags & FOORT_TERM_HORIZON) {  // Terminations.cpp:96-117
        if (term_decide(R.h_every, T.cH)) {
            if ((r < rh * (1 + heps)) || (rh == 0.0 && r < heps)) return FOORT_TERMCODE_HORIZON;
        }
    }
    if (R.term_flags & FOORT_TERM_BOUNDARY_SPHERE) {  // Terminations.cpp:130-146
        if (term_decide(R.b_every, T.cB)) {
            if (r > R.b_rad) return FOORT_TERMCODE_BOUNDARY_SPHERE;
        }
    }
    if (R.term_flags & FOORT_TERM_TIMEOUT) {  // Terminations.cpp:159-186
        if (term_decide(R.t_every, T.cT)) {
            if (T.tcur >= R.t_max) return FOORT_TERMCODE_TIMEOUT;
            ++T.tcur;
        }
    }
    if (R.term_flags & FOORT_TERM_THETA_SINGULARITY) {  // Terminations.cpp:200-214
        if (term_decide(R.th_every, T.cTh)) {
            if (fabs(th) < R.th_eps || fabs(kRefPi - th) < R.th_eps) return FOORT_TERMCODE_THETA_SINGULARITY;
        }
    }
    return FOORT_TERMCODE_CONTINUE;
}

// ---- diagnostics (Diagnostics.cpp) ---------------------------------------------------
struct DiagState {
    int32_t quad;     // FourColorScreenDiagnostic::m_quadrant
    int32_t passes;   // EquatorialPassesDiagnostic::m_EquatPasses
    StepCount cE, cC;  // m_StepsSinceUpdated of EquatorialPasses / ClosestRadius
    double prev;       // m_PrevTheta
    double rmin;      // ClosestRadiusDiagnostic::m_ClosestRadius
};

// Diagnostic::DecideUpdate, Diagnostics.cpp:113-140
template <typename C>
__device__ __forceinline__ bool diag_decide(uint64_t every, int32_t at_start, int32_t at_finish, C& cnt, double lam,
                                            int term) {
    if (every > 0) {
        ++cnt;
        if (cnt >= every) {
            cnt = 0;
            return true;
        }
        return false;
    }
    if (at_start && lam == 0.0) return true;
    if (at_finish && term != FOORT_TERMCODE_CONTINUE) return true;
    return false;
}

// GeodesicPosition (Diagnostics.cpp:246-284), recorded on a second, identical pass.
// The reference saves every sampled position and at the end keeps the samples i with
// i % j == 0, j = M / OutputSteps (M samples in all), the last kept one replaced by the
// final sample. The first pass gives M (from the step count), so this pass writes each
// kept sample straight to its slot: sample i goes to slot i / j, sample M - 1 to slot
// (M - 1) / j. Samples beyond the M the plan allows are not written.
__device__ __forceinline__ void geopos_sample(GeoposRec& g, const RunConst& R, const double x[4], double lam,
                                              int term) {
    if (!diag_decide(R.gp_every, R.gp_start, R.gp_finish, g.cnt, lam, term)) return;
    const uint64_t i = g.i++;
    if (i >= g.M) return;
    uint64_t slot;
    if (i % g.j == 0) {
        slot = i / g.j;
    } else if (i == g.M - 1) {
        slot = (g.M - 1) / g.j;
    } else {
        return;
    }
    double* d = g.dst + 4 * slot;
    d[0] = x[0];
    d[1] = x[1];
    d[2] = x[2];
    d[3] = x[3];
}

// FourColorScreenDiagnostic::UpdateData, Diagnostics.cpp:159-200 (only on BoundarySphere)
static __device__ __noinline__ int32_t four_color_quadrant(double th, double ph) {
    if (fabs(ph) < 2 * kRefPi * 1e5) {
        while (ph > 2 * kRefPi) ph -= 2 * kRefPi;
        while (ph < 0) ph += 2 * kRefPi;
    }
    if (th < kRefPi / 2) return (ph < kRefPi) ? 1 : 2;
    return (ph < kRefPi) ? 3 : 4;
}

// Every Diagnostic::UpdateData of one Geodesic::Update (Geodesic.cpp:82-85). The
// diagnostics are independent, so their order does not change any value.
__device__ __forceinline__ void update_diags(const RunConst& R, double r, double th, double ph, double lam, int term,
                                             DiagState& D) {
    if (R.diag_flags & FOORT_DIAG_FOUR_COLOR_SCREEN) {
        if (term == FOORT_TERMCODE_BOUNDARY_SPHERE) D.quad = four_color_quadrant(th, ph);
    }
    if (R.diag_flags & FOORT_DIAG_EQUATORIAL_PASSES) {  // Diagnostics.cpp:351-380
        if (diag_decide(R.eq_every, R.eq_start, R.eq_finish, D.cE, lam, term)) {
            if (fabs(th - kRefPi / 2.0) > kRefPi / 2.0 * R.eq_thr) {
                if (D.prev > 0 && ((D.prev - kRefPi / 2.0) * (th - kRefPi / 2.0)) < 0.0) ++D.passes;
                D.prev = th;
            }
        }
        if (term == FOORT_TERMCODE_HORIZON) D.passes = -D.passes;
    }
    if (R.diag_flags & FOORT_DIAG_CLOSEST_RADIUS) {  // Diagnostics.cpp:427-446
        if (diag_decide(R.cr_every, R.cr_start, R.cr_finish, D.cC, lam, term)) {
            if (D.rmin < 0 || r < D.rmin) D.rmin = r;
        }
        if (term == FOORT_TERMCODE_HORIZON) D.rmin = 0.0;
    }
}

// Diagnostic and Termination Reset (Geodesic.cpp:47-57) and the start sample taken by
// Geodesic::Reset at lambda = 0.
__device__ __forceinline__ void reset_lane_state(const RunConst& R, const double x[4], DiagState& D, TermState& T) {
    D.quad = 0;
    D.passes = 0;
    D.cE = 0;
    D.cC = 0;
    D.prev = -1;
    D.rmin = -1;
    update_diags(R, radius_of(R, x[1]), x[2], x[3], 0.0, FOORT_TERMCODE_CONTINUE, D);
    T.cH = T.cB = T.cT = T.cTh = 0;
    T.tcur = 0;
}

// ---- step size ------------------------------------------------------------------------
// Integrators::GetAdaptiveStep, Integrators.cpp:34-46
__device__ __forceinline__ double adaptive_step_fp64(const RunConst& R, const double x[4], const double v[4]) {
    double d1 = R.eps / (fabs(v[1]) + 1e-20);
    double m = (kRefPi - x[2] < x[2]) ? kRefPi - x[2] : x[2];
    double d2 = R.eps * m / (fabs(v[2]) + 1e-20);
    double d3 = R.eps / fabs(v[3] + 1e-20);
    double h = 1 / (1 / fabs(d1) + 1 / fabs(d2) + 1 / fabs(d3));
    return (h < R.hmin) ? R.hmin : h;
}

// ---- initial conditions (ViewScreen.cpp:75-119) ----------------------------------------
__device__ __forceinline__ void initial_conditions(const ImageConst& I, const foort_pixel& p, double x[4], double v[4]) {
    for (int i = 0; i < 4; ++i) x[i] = I.pos0[i];
    // unit screen point, Mesh.cpp:49 and :671-672
    double u0 = p.row * 1.0 / static_cast<double>(p.grid - 1);
    double u1 = p.col * 1.0 / static_cast<double>(p.grid - 1);
    double alpha = I.center[0] + I.size[0] * (u0 - 0.5);
    double beta = I.center[1] + I.size[1] * (u1 - 0.5);
    const double R0 = I.R0;
    double den = sqrt(R0 * R0 + alpha * alpha + beta * beta);
    double pf[4] = {-1.0, -R0 / den, -beta / R0 / den, alpha / R0 / I.sin_th0 / den};
    for (int i = 0; i < 4; ++i) {
        double acc = 0.0;
        for (int j = 0; j < 4; ++j) acc += I.e[j][i] * pf[j];
        v[i] = acc;
    }
    double cur = 0.0;
    for (int i = 0; i < 4; ++i) cur += I.gdd0[i] * v[i];
    const double inv = 1 / cur;
    for (int i = 0; i < 4; ++i) v[i] = (v[i] * 1.0) * inv;
}

// ---- results ----------------------------------------------------------------------------
__device__ __forceinline__ void write_result(foort_result* o, int term, uint32_t err, uint64_t steps, double lam,
                                             const double x[4], const double v[4], const DiagState& D) {
    o->term = term;
    o->err = err;
    o->steps = steps;
    o->lambda = lam;
    for (int i = 0; i < 4; ++i) {
        o->pos[i] = x[i];
        o->vel[i] = v[i];
    }
    o->quadrant = D.quad;
    o->equat_passes = D.passes;
    o->closest_r = D.rmin;
}

__device__ __forceinline__ void write_unstarted(foort_result* o, uint32_t err) {
    o->term = FOORT_TERMCODE_CONTINUE;
    o->err = err | FOORT_ERR_UNFINISHED;
    o->steps = 0;
    o->lambda = 0.0;
    for (int i = 0; i < 4; ++i) {
        o->pos[i] = 0.0;
        o->vel[i] = 0.0;
    }
    o->quadrant = 0;
    o->equat_passes = 0;
    o->closest_r = -1.0;
}

__device__ __forceinline__ bool finite4(const double a[4]) {
    return isfinite(a[0]) && isfinite(a[1]) && isfinite(a[2]) && isfinite(a[3]);
}

// ---- persistent work-queue loop -------------------------------------------------------
// Engine interface (per lane):
//   struct Lane;                       lane state
//   init(L, I, R, px)                  Geodesic::Reset with the pixel's initial conditions
//   step(L, I, R) -> bool              one Geodesic::Update; true while the lane runs
//   finish(L, R, out)                  write the lane's record
//   stop(L, R, out, err)               write a partial record (budget / cancel)
//   counters: L.rhs, L.fp64            accumulated per lane, flushed at each poll
//
// Every warp takes pixels from one global counter (one atomic per warp, shared by the
// lanes that need work) and keeps integrating until the queue is empty. Lanes whose
// geodesics terminated take the next pixels at the warp's next refill, at most
// R.refill_steps steps later (the regrouping cadence; 1 = at once), so lanes of a warp
// stay busy while geodesics of very different lengths run side by side; a longer cadence
// refills several lanes with one atomic and one pass of the initial conditions. Every
// R.poll_steps iterations a
// warp publishes its step count, checks the step budget and the host cancel flag, and
// learns whether another warp has asked every lane to stop. No loop waits on another
// thread or on the host.
//
// PAIR: lanes 2k and 2k+1 integrate one geodesic together (E::step_pair). Both take the
// same pixel, hold the same state and so leave the loop together; the even lane writes
// the record and counts the step.
template <class E, bool PAIR = false>
__device__ __forceinline__ void persistent_loop(const LaunchArgs& A, const RunConst& R) {
    const unsigned lane = threadIdx.x & 31u;
    const bool odd = PAIR && (lane & 1u);
    const unsigned slot_lane = PAIR ? (lane & ~1u) : lane;  // the lane that numbers the slot
    const unsigned lt_mask = (1u << slot_lane) - 1u;
    const unsigned slots = PAIR ? 0x55555555u : kFullMask;  // one bit per geodesic slot
    const unsigned pmask = 3u << (lane & ~1u);
    typename E::Lane L;
    ImageConst Ic;  // PAIR: the lane's image constants in registers, copied at each refill
    bool active = false;
    bool drained = false;
    bool stopping = false;
    uint32_t stop_err = 0;
    uint64_t idx = 0;
    unsigned long long lane_steps = 0, lane_done = 0;
    int since_poll = 0, since_refill = 0;

    for (;;) {
        // Refill idle lanes from the queue.
        since_refill = 0;
        if (!drained) {
            const unsigned need = __ballot_sync(kFullMask, !active) & slots;
            if (need) {
                const int leader = __ffs(need) - 1;
                const unsigned cnt = __popc(need);
                unsigned long long base = 0;
                if (lane == static_cast<unsigned>(leader)) base = atomicAdd(&A.ctr[kCtrHead], (unsigned long long)cnt);
                base = __shfl_sync(kFullMask, base, leader);
                if (base + cnt >= A.n) drained = true;
                if (!active) {
                    const uint64_t my = base + __popc(need & lt_mask);
                    if (my < A.n) {
                        const foort_pixel p = A.px[my];
                        if (stopping) {
                            if (!odd) write_unstarted(&A.out[my], stop_err);
                        } else if (p.image >= A.n_images || p.grid < 2) {
                            if (!odd) write_unstarted(&A.out[my], FOORT_ERR_BADPIXEL);
                        } else {
                            idx = my;
                            // i and cnt start at 0 as literals: copying them from the record
                            // made the Johannsen Verlet kernel 3 % slower on GB300
                            L.gp = (A.gp_plan && !odd && A.gp_plan[my].M > 0 && A.gp_plan[my].j > 0)
                                       ? GeoposRec{A.gp_plan[my].dst, A.gp_plan[my].j, A.gp_plan[my].M, 0, 0}
                                       : GeoposRec{nullptr, 1, 0, 0, 0};
                            E::init(L, A.images[p.image], R, p);
                            if constexpr (PAIR) Ic = A.images[p.image];
                            active = true;
                        }
                    }
                }
            }
        }
        if (!__any_sync(kFullMask, active)) {
            if (drained) break;
            continue;
        }
        // Integrate until a lane needs new work (while work remains) or a poll is due.
        for (;;) {
            if (active) {
                bool more;
                if constexpr (PAIR) {
                    more = E::step_pair(L, Ic, R, odd, pmask);
                } else {
                    more = E::step(L, A.images[L.img], R);
                }
                lane_steps += odd ? 0u : 1u;
                if (!more) {
                    if (!odd) {
                        E::finish(L, R, &A.out[idx]);
                        ++lane_done;
                    }
                    active = false;
                }
            }
            ++since_poll;
            ++since_refill;
            if (since_poll >= R.poll_steps) break;
            const unsigned idle = __ballot_sync(kFullMask, !active);
            if (idle == kFullMask) break;
            if (idle && !drained && since_refill >= R.refill_steps) break;
        }
        if (since_poll >= R.poll_steps || drained) {
            since_poll = 0;
            // Publish progress; read the global stop request.
            unsigned long long ws = __reduce_add_sync(kFullMask, static_cast<unsigned>(lane_steps));
            unsigned long long wr = __reduce_add_sync(kFullMask, static_cast<unsigned>(L.rhs));
            unsigned long long wf = __reduce_add_sync(kFullMask, static_cast<unsigned>(L.fp64));
            unsigned long long wd = __reduce_add_sync(kFullMask, static_cast<unsigned>(lane_done));
            lane_steps = 0;
            lane_done = 0;
            L.rhs = 0;
            L.fp64 = 0;
            unsigned long long st = 0;
            if (lane == 0) {
                unsigned long long before = atomicAdd(&A.ctr[kCtrSteps], ws);
                if (wr) atomicAdd(&A.ctr[kCtrRhs], wr);
                if (wf) atomicAdd(&A.ctr[kCtrFp64Steps], wf);
                if (wd) atomicAdd(&A.ctr[kCtrDone], wd);
                if (A.budget && before + ws > A.budget) atomicOr(&A.ctr[kCtrStatus], kStatusBudget);
                if (A.cancel && *A.cancel) atomicOr(&A.ctr[kCtrStatus], kStatusCancelled);
                st = *reinterpret_cast<volatile unsigned long long*>(&A.ctr[kCtrStatus]);
            }
            st = __shfl_sync(kFullMask, st, 0);
            if (!stopping && (st & (kStatusBudget | kStatusCancelled))) {
                stopping = true;
                stop_err = (st & kStatusCancelled) ? FOORT_ERR_CANCELLED : FOORT_ERR_BUDGET;
                if (active) {
                    if (!odd) E::stop(L, R, &A.out[idx], stop_err);
                    active = false;
                }
            }
        }
    }
    // Flush what is left.
    unsigned long long ws = __reduce_add_sync(kFullMask, static_cast<unsigned>(lane_steps));
    unsigned long long wr = __reduce_add_sync(kFullMask, static_cast<unsigned>(L.rhs));
    unsigned long long wf = __reduce_add_sync(kFullMask, static_cast<unsigned>(L.fp64));
    unsigned long long wd = __reduce_add_sync(kFullMask, static_cast<unsigned>(lane_done));
    if (lane == 0) {
        if (ws) atomicAdd(&A.ctr[kCtrSteps], ws);
        if (wr) atomicAdd(&A.ctr[kCtrRhs], wr);
        if (wf) atomicAdd(&A.ctr[kCtrFp64Steps], wf);
        if (wd) atomicAdd(&A.ctr[kCtrDone], wd);
    }
}

}  // namespace foort
