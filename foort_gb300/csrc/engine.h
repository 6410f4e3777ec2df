// Internal structures shared by the host library and the kernels.
#pragma once

#include <stdint.h>

#include "../../include/foort_gpu.h"
#include "metric_fp64.cuh"

namespace foort {

// Truncated pi of the reference (Geometry.h:44); every angular test uses it.
constexpr double kRefPi = 3.1415926535;

// Constants of the mixed-precision kernel (per image). Pairs [2] are float-float
// (hi, lo) splits of a double; thresholds are in ln r in log-r mode.
struct MixedConst {
    float q[kMixedQ];  // analytic plugin constants in FP32 (ImageConst::qa)
    float rp[2];       // r_+ (Delta = (r - r_+)(r - r_-))
    float rm[2];       // r_-
    float lrp[2];      // ln r_+
    float lrm[2];      // ln r_- (unused when r_- = 0)
    double rpv, rmv;   // r_+, r_- as doubles
    float r_fp64;      // lanes with x1 below this use the FP64 right-hand side (0: never)
    float hthr[2];     // Horizon: r_h (1 + eps)
    float hthr0[2];    // Horizon with r_h = 0: eps
    float bthr[2];     // BoundarySphere radius
    float theps[2];    // ThetaSingularity epsilon
    float pi[2];       // the reference's pi
    float mpio2[2];    // -pi / 2
    float eqthr[2];    // EquatorialPasses threshold: pi / 2 * Threshold
    float eps[2];      // Integrators::epsilon
    float hmin;        // Integrators::SmallestPossibleStepsize
    float vtol2;       // VerletVelocityTolerance squared (0: no velocity iterations)
};

// Per-image constants, computed once on the host (ViewScreen.cpp:10-73).
struct ImageConst {
    MetricConst m;
    double e[4][4];     // vielbein rows: e[j][i] = e_j^i
    double gdd0[4];     // g_dd[0][*] at the camera, for the E = 1 rescaling
    double pos0[4];     // initial position (r replaced by ln r in log-r mode)
    double R0;          // camera radius (ordinary r)
    double sin_th0;     // sin(theta) at the camera
    double size[2];     // screen size
    double center[2];   // screen center
    double h_eps;       // Epsilon_Horizon of this image (relative)
    double qa[kMixedQ]; // analytic plugin constants (mixed_metric_constants)
    MixedConst mx;
};

// Run options (process globals in the reference, Config.cpp:11-28 and
// Integrators.h:31-57), passed by value to every launch.
struct RunConst {
    int32_t metric_id;
    int32_t rlog;
    int32_t integrator;
    int32_t precision;
    double eps, hfd, hmin, vtol;
    uint32_t term_flags, diag_flags;
    double h_eps;
    uint64_t h_every;
    double b_rad;
    uint64_t b_every;
    uint64_t t_max, t_every;
    double th_eps;
    uint64_t th_every;
    uint64_t eq_every;
    int32_t eq_start, eq_finish;
    double eq_thr;
    uint64_t cr_every;
    int32_t cr_start, cr_finish;
    int32_t verlet_cap;   // cap on Verlet velocity iterations (the reference has none)
    int32_t poll_steps;   // steps between budget / cancel polls
    uint32_t mixed_options;
    int32_t refill_steps;  // steps a warp runs between refills of its idle lanes (>= 1)
    double mixed_fp64_margin;
    uint64_t gp_every;  // GeodesicPosition update frequency (recorded on a second pass)
    int32_t gp_start, gp_finish;
};

// Scratch counters of one launch (device memory, zeroed before each launch).
enum Ctr {
    kCtrHead = 0,      // next pixel index to hand out (work queue)
    kCtrSteps = 1,     // integration steps, all geodesics
    kCtrRhs = 2,       // right-hand-side evaluations
    kCtrFp64Steps = 3, // mixed kernel: steps evaluated on the FP64 path
    kCtrDone = 4,      // geodesics finished
    kCtrStatus = 5,    // FOORT_STATUS_* bits
    kNumCtr = 8
};

// Steps between budget / cancel polls unless a launch shape says otherwise.
constexpr uint32_t kDefaultPollSteps = 512;

// Status bits written by the kernel.
constexpr unsigned long long kStatusBudget = 1ull;
constexpr unsigned long long kStatusCancelled = 2ull;
constexpr unsigned long long kStatusNonfinite = 4ull;

// GeodesicPosition recording of one geodesic (the second pass of foort_gpu_positions):
// one record per pixel in device memory, prepared by the host; a lane copies dst, j and
// M into its state and counts i and cnt there. (Keeping only a pointer to the record in
// the lane made the Kerr a = 0.99 adaptive run (509² grid, 26,547 geodesics) 1.7 % slower on GB300.)
struct GeoposRec {
    double* dst;    // the geodesic's first slot (4 doubles per kept position)
    uint64_t j, M;  // keep sample i where i % j == 0, and the last of M samples
    uint64_t i;     // samples taken so far
    uint64_t cnt;   // steps since the last sample (DecideUpdate)
};

struct LaunchArgs {
    const foort_pixel* px;
    foort_result* out;
    uint64_t n;
    const ImageConst* images;
    uint32_t n_images;
    uint32_t pad;
    unsigned long long* ctr;          // kNumCtr counters
    const volatile int32_t* cancel;   // host flag in mapped pinned memory (may be null)
    unsigned long long budget;        // 0 = unlimited
    GeoposRec* gp_plan;               // GeodesicPosition second pass: a record per pixel (else null)
};

}  // namespace foort
