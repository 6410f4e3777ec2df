// Host library of the geodesic engine: the C ABI of include/foort_gpu.h.
//
// Per context: the run options (RunConst), the per-image constants (ImageConst, with
// the camera frame of ViewScreen::ConstructVielbein), a stream, a small block of
// device counters (work-queue head, step/RHS counters, status) and a cancel flag in
// mapped pinned host memory. A launch is one persistent kernel over all pixels.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "engine.h"
#include "kernels.h"

using namespace foort;

struct foort_ctx {
    foort_run_desc desc{};
    std::vector<foort_image_desc> images;
    RunConst rc{};
    std::vector<ImageConst> hic;
    ImageConst* d_images = nullptr;
    unsigned long long* d_ctr = nullptr;
    // Pinned, so that the copy of the counters after a launch does not hold the host until
    // the kernel ends (a copy into pageable memory returns only once it is done).
    unsigned long long* h_ctr = nullptr;
    // pinned pixels and results of foort_gpu_run's launches (foort_ctx_stage)
    foort_pixel* h_stage_px = nullptr;
    foort_result* h_stage = nullptr;
    uint64_t stage_cap = 0;
    int32_t* h_cancel = nullptr;
    int32_t* d_cancel = nullptr;
    cudaStream_t stream = nullptr;
    cudaStream_t last_stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    foort_pixel* d_px = nullptr;
    foort_result* d_out = nullptr;
    uint64_t cap = 0;
    uint64_t budget = 0;
    uint64_t last_n = 0;
    uint32_t block_size = 0, blocks_per_sm = 0;
    uint32_t lanes = 0;  // lanes per geodesic: 0 chosen per launch, 1, 2
    int device = 0, num_sms = 0;
    bool pending = false;
    bool autotune = false;  // search shapes for launches without a cache entry
    uint32_t schedule = FOORT_SCHEDULE_WAVES;  // foort_gpu_run
    uint64_t lookahead = FOORT_LOOKAHEAD_AUTO;
    uint32_t run_launches = 0, run_schedule = 0;
    bool record = false;  // keep the last run's launch pixel lists
    std::vector<std::vector<foort_pixel>> launch_px;
    foort_stats stats{};
    std::string err;
};

namespace {

std::mutex g_err_mu;
std::string g_create_err = "no error";

int fail(foort_ctx* c, int code, const std::string& msg) {
    if (c) {
        c->err = msg;
    } else {
        std::lock_guard<std::mutex> lk(g_err_mu);
        g_create_err = msg;
    }
    return code;
}

int cuda_fail(foort_ctx* c, cudaError_t e, const char* what) {
    return fail(c, FOORT_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(call)                                                   \
    do {                                                           \
        cudaError_t e_ = (call);                                   \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call);   \
    } while (0)

// ViewScreen::ConstructVielbein (ViewScreen.cpp:10-73), in FP64 on the host, with the
// reference's dense loops so that the frame is the reference's to the last bit.
void camera_frame(int metric_id, bool rlog, const foort_image_desc& im, ImageConst& ic) {
    double p[4] = {im.cam_pos[0], im.cam_pos[1], im.cam_pos[2], im.cam_pos[3]};
    p[1] = rlog ? std::log(p[1]) : p[1];
    const double r = rlog ? std::exp(p[1]) : p[1];
    const double s = std::sin(p[2]), c = std::cos(p[2]);
    G5 a = metric_dd_host(metric_id, ic.m, r, s, c, rlog);
    G5 b = metric_uu_host(metric_id, ic.m, r, s, c, rlog);
    double gdd[4][4] = {}, guu[4][4] = {};
    gdd[0][0] = a.tt; gdd[0][3] = gdd[3][0] = a.tp; gdd[1][1] = a.rr; gdd[2][2] = a.hh; gdd[3][3] = a.pp;
    guu[0][0] = b.tt; guu[0][3] = guu[3][0] = b.tp; guu[1][1] = b.rr; guu[2][2] = b.hh; guu[3][3] = b.pp;
    auto ip = [&gdd](const double* u, const double* w) {
        double acc = 0;
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j) acc += u[i] * gdd[i][j] * w[j];
        return acc;
    };
    double e[4][4] = {};
    double sg[4] = {};
    auto scale = [](double* v, double f) { for (int i = 0; i < 4; ++i) v[i] = v[i] * f; };
    // t leg
    for (int i = 0; i < 4; ++i) e[0][i] = guu[0][i];
    double n = ip(e[0], e[0]);
    sg[0] = (n < 0) ? -1 : 1;
    scale(e[0], sg[0]);
    scale(e[0], 1 / std::sqrt(sg[0] * n));
    // phi leg
    double f0 = sg[0] * ip(guu[3], e[0]);
    for (int i = 0; i < 4; ++i) e[3][i] = guu[3][i] - e[0][i] * f0;
    n = ip(e[3], e[3]);
    sg[3] = (n < 0) ? -1 : 1;
    scale(e[3], sg[3] * im.cam_pos[1] * std::sin(im.cam_pos[2]));
    scale(e[3], 1 / std::sqrt(sg[3] * n));
    // r leg
    f0 = sg[0] * ip(guu[1], e[0]);
    double f3 = sg[3] * ip(guu[1], e[3]);
    for (int i = 0; i < 4; ++i) e[1][i] = (guu[1][i] - e[0][i] * f0) - e[3][i] * f3;
    n = ip(e[1], e[1]);
    sg[1] = (n < 0) ? -1 : 1;
    scale(e[1], sg[1]);
    scale(e[1], 1 / std::sqrt(sg[1] * n));
    // theta leg: the reference subtracts a multiple of the (still zero) theta leg itself
    // instead of the phi leg (ViewScreen.cpp:56-58); kept as written.
    f0 = sg[0] * ip(guu[2], e[0]);
    f3 = sg[3] * ip(guu[2], e[3]);
    double prev2[4] = {e[2][0], e[2][1], e[2][2], e[2][3]};
    for (int i = 0; i < 4; ++i) e[2][i] = (guu[2][i] - e[0][i] * f0) - prev2[i] * f3;
    n = ip(e[2], e[2]);
    sg[2] = (n < 0) ? -1 : 1;
    scale(e[2], sg[2] * im.cam_pos[1]);
    scale(e[2], 1 / std::sqrt(sg[2] * n));
    for (int j = 0; j < 4; ++j)
        for (int i = 0; i < 4; ++i) ic.e[j][i] = e[j][i];
    for (int i = 0; i < 4; ++i) ic.gdd0[i] = gdd[0][i];
    for (int i = 0; i < 4; ++i) ic.pos0[i] = im.cam_pos[i];
    ic.pos0[1] = p[1];
    ic.R0 = im.cam_pos[1];
    ic.sin_th0 = std::sin(p[2]);
    ic.size[0] = im.screen_size[0];
    ic.size[1] = im.screen_size[1];
    ic.center[0] = im.screen_center[0];
    ic.center[1] = im.screen_center[1];
}

int validate(const foort_run_desc* d, std::string& why) {
    if (!d) { why = "descriptor is NULL"; return FOORT_E_BADARG; }
    if (d->metric_id < 0 || d->metric_id > 4) { why = "unknown metric_id"; return FOORT_E_BADARG; }
    if (d->integrator_id != FOORT_INTEGRATOR_RK4 && d->integrator_id != FOORT_INTEGRATOR_VERLET) {
        why = "unknown integrator_id";
        return FOORT_E_BADARG;
    }
    if (d->precision != FOORT_PREC_FP64 && d->precision != FOORT_PREC_MIXED && d->precision != FOORT_PREC_FP64_ANALYTIC) {
        why = "unknown precision";
        return FOORT_E_BADARG;
    }
    if (d->n_images == 0 || !d->images) { why = "no images"; return FOORT_E_BADARG; }
    if (d->term_flags == 0) { why = "no terminations turned on"; return FOORT_E_BADARG; }
    if (d->term_flags & ~0xFu) { why = "unknown termination flag"; return FOORT_E_BADARG; }
    if (d->diag_flags & ~0xFu) { why = "unknown diagnostic flag"; return FOORT_E_BADARG; }
    if (!(d->epsilon > 0.0) || !(d->derivative_h > 0.0)) { why = "epsilon and derivative_h must be > 0"; return FOORT_E_BADARG; }
    for (uint32_t i = 0; i < d->n_images; ++i) {
        const foort_image_desc& im = d->images[i];
        if (!(im.cam_pos[1] > 0.0)) { why = "camera radius must be > 0"; return FOORT_E_BADARG; }
    }
    return FOORT_OK;
}

RunConst make_run_const(const foort_run_desc& d) {
    RunConst R{};
    R.metric_id = d.metric_id;
    // Flat space is not a SphericalHorizonMetric: no log-r scale (ViewScreen.h:49-50)
    // and no Horizon termination (Config.cpp:649-657).
    R.rlog = (d.rlog && d.metric_id != kFlat) ? 1 : 0;
    R.integrator = d.integrator_id;
    R.precision = d.precision;
    R.eps = d.epsilon;
    R.hfd = d.derivative_h;
    R.hmin = d.smallest_step;
    R.vtol = d.verlet_tol;
    R.term_flags = d.term_flags;
    if (d.metric_id == kFlat) R.term_flags &= ~FOORT_TERM_HORIZON;
    R.diag_flags = d.diag_flags;
    R.h_eps = d.horizon_eps;
    R.h_every = d.horizon_every;
    R.b_rad = d.boundary_radius;
    R.b_every = d.boundary_every;
    R.t_max = d.timeout_max_steps;
    R.t_every = d.timeout_every;
    R.th_eps = d.theta_eps;
    R.th_every = d.theta_every;
    R.eq_every = d.equat_freq.every_n;
    R.eq_start = d.equat_freq.at_start;
    R.eq_finish = d.equat_freq.at_finish;
    R.eq_thr = d.equat_threshold;
    R.cr_every = d.closest_freq.every_n;
    R.cr_start = d.closest_freq.at_start;
    R.cr_finish = d.closest_freq.at_finish;
    R.verlet_cap = 1000;
    R.poll_steps = kDefaultPollSteps;
    R.refill_steps = 1;
    R.mixed_options = d.mixed_options;
    R.mixed_fp64_margin = (d.mixed_options & FOORT_MIXED_FP64_NEAR_HORIZON) ? d.mixed_fp64_margin : 0.0;
    R.gp_every = d.geopos_freq.every_n;
    R.gp_start = d.geopos_freq.at_start;
    R.gp_finish = d.geopos_freq.at_finish;
    return R;
}

// The analytic-derivative kernels serve FOORT_PREC_MIXED and FOORT_PREC_FP64_ANALYTIC
// (the latter takes every step in FP64).
bool analytic_family(int precision) { return precision == FOORT_PREC_MIXED || precision == FOORT_PREC_FP64_ANALYTIC; }

const void* select_kernel(const RunConst& R) {
    if (analytic_family(R.precision))
        return mixed_kernel_variant(R.metric_id, R.integrator, (R.mixed_options & FOORT_MIXED_FP64_DECISIONS) != 0);
    return fp64_kernel(R.metric_id, R.integrator);
}

// The two-lanes-per-geodesic kernel for these options, or nullptr (FP64, FP64-analytic,
// Verlet, the called plugins, the strong-field FP64 steps).
const void* select_pair_kernel(const RunConst& R) {
    if (R.precision != FOORT_PREC_MIXED || R.mixed_fp64_margin > 0.0 ||
        (R.mixed_options & FOORT_MIXED_FP64_TURNING_POINTS))
        return nullptr;
    return mixed_pair_kernel_variant(R.metric_id, R.integrator, (R.mixed_options & FOORT_MIXED_FP64_DECISIONS) != 0);
}

struct LaunchShape {
    const void* fn = nullptr;
    uint32_t grid = 0, block = 0, lanes = 1, refill = 1, poll = kDefaultPollSteps;
};

// Kernel and grid of a launch of n geodesics in the requested shape (zero fields: the
// built-in rule): a persistent grid of at most the resident CTAs. The rule takes 128
// threads, as many CTAs per SM as fit, and two lanes per geodesic where that kernel exists
// and all n geodesics fit on the GPU's resident lanes that way (then a step's latency,
// not the GPU's throughput, sets the pace, and two lanes halve the metric work on it).
int choose_launch(foort_ctx* ctx, const RunConst& R, uint64_t n, int num_sms, const foort_launch_shape& want,
                  LaunchShape& out) {
    const uint32_t bs = want.block_size ? want.block_size : 128;
    auto resident = [&](const void* fn, int& per_sm) -> int {
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, static_cast<int>(bs), 0));
        if (want.blocks_per_sm) per_sm = std::min<int>(per_sm, static_cast<int>(want.blocks_per_sm));
        return FOORT_OK;
    };
    const void* fn = select_kernel(R);
    if (!fn) return fail(ctx, FOORT_E_UNSUPPORTED, "no kernel for this metric / integrator / precision");
    int per_sm = 0, rc = 0;
    uint32_t lanes = 1;
    const void* fn2 = (want.lanes != 1) ? select_pair_kernel(R) : nullptr;
    if (fn2) {
        int per_sm2 = 0;
        if ((rc = resident(fn2, per_sm2))) return rc;
        const uint64_t cap2 = static_cast<uint64_t>(per_sm2) * static_cast<uint64_t>(num_sms) * bs;
        if (per_sm2 > 0 && (want.lanes == 2 || 2 * n <= cap2)) {
            fn = fn2;
            per_sm = per_sm2;
            lanes = 2;
        }
    }
    if (lanes == 1 && (rc = resident(fn, per_sm))) return rc;
    if (per_sm <= 0) return fail(ctx, FOORT_E_CUDA, "kernel does not fit on an SM with this block size");
    const uint64_t full = static_cast<uint64_t>(per_sm) * static_cast<uint64_t>(num_sms);
    const uint64_t need = (lanes * n + bs - 1) / bs;
    out.fn = fn;
    out.grid = static_cast<uint32_t>(std::max<uint64_t>(1, std::min(full, need)));
    out.block = bs;
    out.lanes = lanes;
    out.refill = want.refill_steps ? want.refill_steps : 1;
    out.poll = want.poll_steps ? want.poll_steps : kDefaultPollSteps;
    return FOORT_OK;
}

// The shape a launch of n geodesics asks for: the cached tuned shape for the context's
// key, with the context's forced settings (foort_gpu_set_launch / _set_lanes) over it.
foort_launch_shape requested_shape(const foort_ctx* ctx, uint64_t n, bool* cached = nullptr) {
    foort_launch_shape s{};
    char key[160];
    const bool hit = foort_tune_key(&ctx->desc, ctx->num_sms, n, key, sizeof(key)) == FOORT_OK &&
                     foort_tune_get(key, &s) == FOORT_OK;
    if (!hit) s = foort_launch_shape{};
    if (cached) *cached = hit;
    if (ctx->block_size) s.block_size = ctx->block_size;
    if (ctx->blocks_per_sm) s.blocks_per_sm = ctx->blocks_per_sm;
    if (ctx->lanes) s.lanes = ctx->lanes;
    return s;
}

int ensure_capacity(foort_ctx* ctx, uint64_t n) {
    if (n <= ctx->cap) return FOORT_OK;
    if (ctx->d_px) cudaFree(ctx->d_px);
    if (ctx->d_out) cudaFree(ctx->d_out);
    ctx->d_px = nullptr;
    ctx->d_out = nullptr;
    ctx->cap = 0;
    CK(cudaMalloc(&ctx->d_px, n * sizeof(foort_pixel)));
    CK(cudaMalloc(&ctx->d_out, n * sizeof(foort_result)));
    ctx->cap = n;
    return FOORT_OK;
}

int autotune_launch(foort_ctx* ctx, const foort_pixel* d_px, uint64_t n, foort_result* d_out, cudaStream_t st,
                    foort_launch_shape* best);

// One launch over n pixels: the explicit shape if given, else the requested one (with
// the search first where autotuning is on and the cache has no entry).
int launch(foort_ctx* ctx, const foort_pixel* d_px, uint64_t n, foort_result* d_out, cudaStream_t st,
           GeoposRec* gp_plan = nullptr, const foort_launch_shape* shape = nullptr) {
    bool cached = false;
    const foort_launch_shape want = shape ? *shape : requested_shape(ctx, n, &cached);
    if (!shape && !cached && ctx->autotune && !gp_plan && n > 0) return autotune_launch(ctx, d_px, n, d_out, st, nullptr);
    LaunchShape ls;
    int rc = choose_launch(ctx, ctx->rc, n, ctx->num_sms, want, ls);
    if (rc) return rc;
    const void* fn = ls.fn;
    const uint32_t bs = ls.block, grid = ls.grid;
    *ctx->h_cancel = 0;
    CK(cudaMemsetAsync(ctx->d_ctr, 0, kNumCtr * sizeof(unsigned long long), st));
    LaunchArgs A{};
    A.px = d_px;
    A.out = d_out;
    A.n = n;
    A.images = ctx->d_images;
    A.n_images = static_cast<uint32_t>(ctx->hic.size());
    A.ctr = ctx->d_ctr;
    A.cancel = ctx->d_cancel;
    A.budget = ctx->budget;
    A.gp_plan = gp_plan;
    if (!A.budget && !(ctx->rc.term_flags & FOORT_TERM_TIMEOUT)) {
        // Without TimeOut a geodesic may never terminate (the reference would loop
        // forever); a finite default budget keeps every launch finite.
        A.budget = std::max<unsigned long long>(100000000ull, 1000000ull * n);
    }
    RunConst R = ctx->rc;
    R.refill_steps = static_cast<int32_t>(ls.refill);
    R.poll_steps = static_cast<int32_t>(ls.poll);
    void* args[2] = {&A, &R};
    CK(cudaEventRecord(ctx->ev0, st));
    if (n > 0) CK(cudaLaunchKernel(fn, dim3(grid), dim3(bs), args, 0, st));
    CK(cudaEventRecord(ctx->ev1, st));
    CK(cudaMemcpyAsync(ctx->h_ctr, ctx->d_ctr, kNumCtr * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    ctx->stats.n_blocks = grid;
    ctx->stats.block_size = bs;
    ctx->stats.lanes_per_geodesic = ls.lanes;
    ctx->stats.refill_steps = ls.refill;
    ctx->stats.poll_steps = ls.poll;
    ctx->last_n = n;
    ctx->last_stream = st;
    ctx->pending = true;
    return FOORT_OK;
}

// GeodesicPosition samples of one geodesic (M) and the stride j of the kept ones, from its
// step count. DecideUpdate (Diagnostics.cpp:113-140) runs at Geodesic::Reset and after
// every step, so with UpdateFrequency N > 0 a geodesic of S steps has floor((S + 1) / N)
// samples, with N = 0 one at the start and / or one at the finish. Geodesics that did not
// terminate (stopped by the budget or a cancel, or skipped) have none. The end of
// GeodesicPositionDiagnostic::UpdateData (:255-283) keeps every j-th sample, j =
// M / OutputSteps, when OutputSteps is below M: (M - 1) / j + 1 of them.
void geopos_plan(const foort_run_desc& d, uint64_t steps, int32_t term, uint64_t& M, uint64_t& j, uint64_t& kept) {
    M = 0;
    if (term != FOORT_TERMCODE_CONTINUE) {
        const uint64_t every = d.geopos_freq.every_n;
        if (every > 0)
            M = (steps + 1) / every;
        else
            M = (d.geopos_freq.at_start ? 1u : 0u) + (d.geopos_freq.at_finish ? 1u : 0u);
    }
    const uint64_t K = d.geopos_output_steps;
    j = (K > 0 && K < M) ? M / K : 1;
    kept = M ? (M - 1) / j + 1 : 0;
}

int finish(foort_ctx* ctx) {
    if (!ctx->pending) return FOORT_OK;
    ctx->pending = false;
    CK(cudaStreamSynchronize(ctx->last_stream));
    CK(cudaGetLastError());
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    ctx->stats.kernel_ms = ms;
    ctx->stats.steps = ctx->h_ctr[kCtrSteps];
    ctx->stats.rhs_evals = ctx->h_ctr[kCtrRhs];
    ctx->stats.fp64_steps = ctx->h_ctr[kCtrFp64Steps];
    ctx->stats.geodesics = ctx->h_ctr[kCtrDone];
    const unsigned long long st = ctx->h_ctr[kCtrStatus];
    int rc = FOORT_OK;
    if (st & kStatusCancelled) rc = fail(ctx, FOORT_E_CANCELLED, "launch cancelled by foort_gpu_cancel");
    else if (st & kStatusBudget) rc = fail(ctx, FOORT_E_BUDGET, "global step budget exhausted; unfinished geodesics are marked");
    ctx->stats.status = static_cast<uint32_t>(rc);
    return rc;
}

// The search (foort_gpu_autotune). Candidates: lanes per geodesic (1, and 2 where the
// two-lane kernel exists) times CTA sizes 32, 64, 128, at refill cadence 1 and the default
// poll interval; then, around the fastest, refill cadences 4 and 16 and poll intervals
// 128 and 2048; the two fastest are timed once more and the smaller time counts. Each
// candidate is one launch over the pixels (or a prefix, for launches much larger than the
// GPU's resident lanes), timed with CUDA events. The last launch integrates all n pixels
// in the winning shape.
int autotune_launch(foort_ctx* ctx, const foort_pixel* d_px, uint64_t n, foort_result* d_out, cudaStream_t st,
                    foort_launch_shape* best_out) {
    LaunchShape probe;
    int rc = choose_launch(ctx, ctx->rc, 1, ctx->num_sms, foort_launch_shape{128, 0, 1, 1, kDefaultPollSteps, 0, 0.0},
                           probe);
    if (rc) return rc;
    int per_sm = 0;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, probe.fn, 128, 0));
    const uint64_t resident = static_cast<uint64_t>(std::max(per_sm, 1)) * ctx->num_sms * 128;
    const uint64_t m = std::min<uint64_t>(n, FOORT_TUNE_SAMPLE_LANES_X * resident);
    const bool has_pair = select_pair_kernel(ctx->rc) != nullptr;
    std::vector<foort_launch_shape> tried;
    auto time_shape = [&](foort_launch_shape s, double& ms) -> int {
        int r = launch(ctx, d_px, m, d_out, st, nullptr, &s);
        if (r) return r;
        r = finish(ctx);
        if (r != FOORT_OK) return r;
        ms = ctx->stats.kernel_ms;
        return FOORT_OK;
    };
    auto consider = [&](foort_launch_shape s) -> int {
        for (const auto& t : tried)
            if (t.block_size == s.block_size && t.lanes == s.lanes && t.refill_steps == s.refill_steps &&
                t.poll_steps == s.poll_steps && t.blocks_per_sm == s.blocks_per_sm)
                return FOORT_OK;
        double ms = 0.0;
        int r = time_shape(s, ms);
        if (r) return r;
        s.ms = ms;
        tried.push_back(s);
        return FOORT_OK;
    };
    auto fastest = [&]() {
        size_t b = 0;
        for (size_t i = 1; i < tried.size(); ++i)
            if (tried[i].ms < tried[b].ms) b = i;
        return tried[b];
    };
    // one untimed launch: module load and first-touch costs stay out of the comparison
    double warm = 0.0;
    if ((rc = time_shape(foort_launch_shape{128, 0, 1, 1, kDefaultPollSteps, 0, 0.0}, warm))) return rc;
    for (uint32_t lanes = 1; lanes <= (has_pair ? 2u : 1u); ++lanes)
        for (uint32_t bs : {32u, 64u, 128u})
            if ((rc = consider(foort_launch_shape{bs, 0, lanes, 1, kDefaultPollSteps, 0, 0.0}))) return rc;
    foort_launch_shape b = fastest();
    for (uint32_t refill : {4u, 16u}) {
        foort_launch_shape c = b;
        c.refill_steps = refill;
        if ((rc = consider(c))) return rc;
    }
    b = fastest();
    for (uint32_t poll : {128u, 2048u}) {
        foort_launch_shape c = b;
        c.poll_steps = poll;
        if ((rc = consider(c))) return rc;
    }
    // the two fastest once more
    std::sort(tried.begin(), tried.end(),
              [](const foort_launch_shape& x, const foort_launch_shape& y) { return x.ms < y.ms; });
    for (size_t i = 0; i < std::min<size_t>(2, tried.size()); ++i) {
        double ms = 0.0;
        if ((rc = time_shape(tried[i], ms))) return rc;
        tried[i].ms = std::min(tried[i].ms, ms);
    }
    b = fastest();
    char key[160];
    if (foort_tune_key(&ctx->desc, ctx->num_sms, n, key, sizeof(key)) == FOORT_OK) foort_tune_put(key, &b);
    if (best_out) *best_out = b;
    // the real launch: every pixel, the winning shape
    return launch(ctx, d_px, n, d_out, st, nullptr, &b);
}

}  // namespace

extern "C" {

void foort_gpu_default_desc(foort_run_desc* d) {
    if (!d) return;
    std::memset(d, 0, sizeof(*d));
    d->metric_id = FOORT_METRIC_KERR;
    d->integrator_id = FOORT_INTEGRATOR_RK4;
    d->precision = FOORT_PREC_FP64;
    d->epsilon = 0.03;
    d->derivative_h = 1e-7;
    d->smallest_step = 1e-12;
    d->verlet_tol = 0.001;
    d->term_flags = FOORT_TERM_BOUNDARY_SPHERE | FOORT_TERM_TIMEOUT;
    d->diag_flags = FOORT_DIAG_FOUR_COLOR_SCREEN;
    d->value_diag = FOORT_DIAG_FOUR_COLOR_SCREEN;
    d->horizon_eps = 0.01;
    d->horizon_every = 1;
    d->boundary_radius = 1000.0;
    d->boundary_every = 1;
    d->timeout_max_steps = 10000;
    d->timeout_every = 1;
    d->theta_eps = 1e-5;
    d->theta_every = 1;
    d->equat_freq = foort_update_freq{1, 1, 1};
    d->equat_threshold = 0.01;
    d->closest_freq = foort_update_freq{1, 1, 1};
    d->geopos_freq = foort_update_freq{1, 0, 1};
}

int foort_gpu_create(const foort_run_desc* desc, foort_ctx** out_ctx) {
    if (!out_ctx) return fail(nullptr, FOORT_E_BADARG, "out_ctx is NULL");
    *out_ctx = nullptr;
    std::string why;
    int v = validate(desc, why);
    if (v) return fail(nullptr, v, why);
    foort_ctx* ctx = new foort_ctx();
    ctx->desc = *desc;
    ctx->images.assign(desc->images, desc->images + desc->n_images);
    ctx->desc.images = ctx->images.data();
    ctx->rc = make_run_const(*desc);
    ctx->hic.resize(desc->n_images);
    for (uint32_t i = 0; i < desc->n_images; ++i) {
        ImageConst& ic = ctx->hic[i];
        std::memset(&ic, 0, sizeof(ic));
        ic.m = make_metric_const(desc->metric_id, desc->images[i].metric_params);
        camera_frame(desc->metric_id, ctx->rc.rlog != 0, desc->images[i], ic);
        ic.h_eps = desc->images[i].horizon_eps > 0.0 ? desc->images[i].horizon_eps : desc->horizon_eps;
        if (analytic_family(ctx->rc.precision)) fill_mixed_constants(desc->metric_id, ic, ctx->rc);
    }
    auto bail = [&](int rc) {
        std::string m = ctx->err;
        foort_gpu_destroy(ctx);
        return fail(nullptr, rc, m);
    };
    cudaError_t e = cudaGetDevice(&ctx->device);
    if (e != cudaSuccess) return bail(cuda_fail(ctx, e, "cudaGetDevice"));
    e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, ctx->device);
    if (e != cudaSuccess) return bail(cuda_fail(ctx, e, "cudaDeviceGetAttribute"));
    if (!select_kernel(ctx->rc)) return bail(fail(ctx, FOORT_E_UNSUPPORTED, "no kernel for this metric / integrator / precision"));
    e = cudaMalloc(&ctx->d_images, ctx->hic.size() * sizeof(ImageConst));
    if (e != cudaSuccess) return bail(cuda_fail(ctx, e, "cudaMalloc(images)"));
    e = cudaMemcpy(ctx->d_images, ctx->hic.data(), ctx->hic.size() * sizeof(ImageConst), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return bail(cuda_fail(ctx, e, "cudaMemcpy(images)"));
    e = cudaMalloc(&ctx->d_ctr, kNumCtr * sizeof(unsigned long long));
    if (e != cudaSuccess) return bail(cuda_fail(ctx, e, "cudaMalloc(counters)"));
    e = cudaHostAlloc(reinterpret_cast<void**>(&ctx->h_ctr), kNumCtr * sizeof(unsigned long long), cudaHostAllocDefault);
    if (e != cudaSuccess) return bail(cuda_fail(ctx, e, "cudaHostAlloc(counters)"));
    std::memset(ctx->h_ctr, 0, kNumCtr * sizeof(unsigned long long));
    e = cudaHostAlloc(reinterpret_cast<void**>(&ctx->h_cancel), sizeof(int32_t), cudaHostAllocMapped);
    if (e != cudaSuccess) return bail(cuda_fail(ctx, e, "cudaHostAlloc(cancel)"));
    *ctx->h_cancel = 0;
    e = cudaHostGetDevicePointer(reinterpret_cast<void**>(&ctx->d_cancel), ctx->h_cancel, 0);
    if (e != cudaSuccess) return bail(cuda_fail(ctx, e, "cudaHostGetDevicePointer(cancel)"));
    e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return bail(cuda_fail(ctx, e, "cudaStreamCreate"));
    if ((e = cudaEventCreate(&ctx->ev0)) != cudaSuccess || (e = cudaEventCreate(&ctx->ev1)) != cudaSuccess)
        return bail(cuda_fail(ctx, e, "cudaEventCreate"));
    *out_ctx = ctx;
    return FOORT_OK;
}

int foort_gpu_integrate(foort_ctx* ctx, const foort_pixel* px, uint64_t n, foort_result* out) {
    if (!ctx) return fail(nullptr, FOORT_E_BADARG, "ctx is NULL");
    if (n && (!px || !out)) return fail(ctx, FOORT_E_BADARG, "NULL pixel or result buffer");
    for (uint64_t i = 0; i < n; ++i)
        if (px[i].image >= ctx->hic.size() || px[i].grid < 2)
            return fail(ctx, FOORT_E_BADARG, "pixel " + std::to_string(i) + " has an invalid image index or grid < 2");
    int rc = finish(ctx);
    if (rc != FOORT_OK && rc != FOORT_E_BUDGET && rc != FOORT_E_CANCELLED) return rc;
    if ((rc = ensure_capacity(ctx, n))) return rc;
    cudaStream_t st = ctx->stream;
    if (n) CK(cudaMemcpyAsync(ctx->d_px, px, n * sizeof(foort_pixel), cudaMemcpyHostToDevice, st));
    if ((rc = launch(ctx, ctx->d_px, n, ctx->d_out, st))) return rc;
    if (n) CK(cudaMemcpyAsync(out, ctx->d_out, n * sizeof(foort_result), cudaMemcpyDeviceToHost, st));
    return finish(ctx);
}

int foort_gpu_integrate_async(foort_ctx* ctx, const foort_pixel* d_px, uint64_t n, foort_result* d_out,
                              void* cuda_stream) {
    if (!ctx) return fail(nullptr, FOORT_E_BADARG, "ctx is NULL");
    if (n && (!d_px || !d_out)) return fail(ctx, FOORT_E_BADARG, "NULL pixel or result buffer");
    int rc = finish(ctx);
    if (rc != FOORT_OK && rc != FOORT_E_BUDGET && rc != FOORT_E_CANCELLED) return rc;
    return launch(ctx, d_px, n, d_out, static_cast<cudaStream_t>(cuda_stream));
}

int foort_gpu_positions(foort_ctx* ctx, const foort_pixel* px, uint64_t n, const foort_result* first, uint64_t* counts,
                        double* points, uint64_t cap_points, uint64_t* total_points) {
    if (!ctx) return fail(nullptr, FOORT_E_BADARG, "ctx is NULL");
    if (n && (!px || !first || !counts)) return fail(ctx, FOORT_E_BADARG, "NULL pixel, result or count buffer");
    if (!(ctx->desc.diag_flags & FOORT_DIAG_GEODESIC_POSITION))
        return fail(ctx, FOORT_E_BADARG, "the GeodesicPosition diagnostic is not turned on");
    std::vector<GeoposRec> plan(n);
    std::vector<uint64_t> first_slot(n);
    uint64_t total = 0;
    for (uint64_t i = 0; i < n; ++i) {
        uint64_t M, j, kept;
        geopos_plan(ctx->desc, first[i].steps, first[i].term, M, j, kept);
        first_slot[i] = total;
        plan[i] = GeoposRec{nullptr, j, M, 0, 0};
        counts[i] = kept;
        total += kept;
    }
    if (total_points) *total_points = total;
    if (!points || n == 0) return FOORT_OK;
    if (cap_points < total)
        return fail(ctx, FOORT_E_BADARG, "the points buffer holds " + std::to_string(cap_points) + " of the " +
                                             std::to_string(total) + " positions");
    int rc = finish(ctx);
    if (rc != FOORT_OK && rc != FOORT_E_BUDGET && rc != FOORT_E_CANCELLED) return rc;
    if ((rc = ensure_capacity(ctx, n))) return rc;
    GeoposRec* d_plan = nullptr;
    double* d_pts = nullptr;
    std::vector<foort_result> again(n);
    auto body = [&]() -> int {
        cudaStream_t st = ctx->stream;
        CK(cudaMalloc(&d_plan, plan.size() * sizeof(GeoposRec)));
        CK(cudaMalloc(&d_pts, std::max<uint64_t>(1, total) * 4 * sizeof(double)));
        CK(cudaMemsetAsync(d_pts, 0xFF, std::max<uint64_t>(1, total) * 4 * sizeof(double), st));  // NaN
        for (uint64_t i = 0; i < n; ++i) plan[i].dst = d_pts + 4 * first_slot[i];  // device addresses
        CK(cudaMemcpyAsync(ctx->d_px, px, n * sizeof(foort_pixel), cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(d_plan, plan.data(), plan.size() * sizeof(GeoposRec), cudaMemcpyHostToDevice, st));
        int r = launch(ctx, ctx->d_px, n, ctx->d_out, st, d_plan);
        if (r) return r;
        CK(cudaMemcpyAsync(points, d_pts, total * 4 * sizeof(double), cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(again.data(), ctx->d_out, n * sizeof(foort_result), cudaMemcpyDeviceToHost, st));
        return finish(ctx);
    };
    rc = body();
    if (d_plan) cudaFree(d_plan);
    if (d_pts) cudaFree(d_pts);
    if (rc != FOORT_OK) return rc;
    // the second pass must retrace the first: same steps for every recorded geodesic
    for (uint64_t i = 0; i < n; ++i)
        if (plan[i].M && again[i].steps != first[i].steps)
            return fail(ctx, FOORT_E_NUMERIC, "geodesic " + std::to_string(i) + " took " +
                                                  std::to_string(again[i].steps) + " steps on the second pass, " +
                                                  std::to_string(first[i].steps) + " on the first");
    return FOORT_OK;
}

int foort_geopos_count(const foort_run_desc* desc, uint64_t steps, int32_t term, uint64_t* samples, uint64_t* kept) {
    if (!desc) return FOORT_E_BADARG;
    uint64_t M, j, k;
    geopos_plan(*desc, steps, term, M, j, k);
    if (samples) *samples = M;
    if (kept) *kept = k;
    return FOORT_OK;
}

int foort_gpu_sync(foort_ctx* ctx) {
    if (!ctx) return fail(nullptr, FOORT_E_BADARG, "ctx is NULL");
    return finish(ctx);
}

int foort_gpu_set_budget(foort_ctx* ctx, uint64_t max_total_steps) {
    if (!ctx) return fail(nullptr, FOORT_E_BADARG, "ctx is NULL");
    ctx->budget = max_total_steps;
    return FOORT_OK;
}

int foort_gpu_cancel(foort_ctx* ctx) {
    if (!ctx) return fail(nullptr, FOORT_E_BADARG, "ctx is NULL");
    *reinterpret_cast<volatile int32_t*>(ctx->h_cancel) = 1;
    return FOORT_OK;
}

int foort_gpu_set_launch(foort_ctx* ctx, uint32_t block_size, uint32_t blocks_per_sm) {
    if (!ctx) return fail(nullptr, FOORT_E_BADARG, "ctx is NULL");
    if (block_size && (block_size % 32 || block_size > 128))
        return fail(ctx, FOORT_E_BADARG, "block_size must be a multiple of 32 and at most 128");
    ctx->block_size = block_size;
    ctx->blocks_per_sm = blocks_per_sm;
    return FOORT_OK;
}

int foort_gpu_set_lanes(foort_ctx* ctx, uint32_t lanes_per_geodesic) {
    if (!ctx) return fail(nullptr, FOORT_E_BADARG, "ctx is NULL");
    if (lanes_per_geodesic > 2) return fail(ctx, FOORT_E_BADARG, "lanes_per_geodesic must be 0 (automatic), 1 or 2");
    ctx->lanes = lanes_per_geodesic;
    return FOORT_OK;
}

int foort_gpu_autotune(foort_ctx* ctx, const foort_pixel* d_px, uint64_t n, foort_result* d_out, void* cuda_stream,
                       foort_launch_shape* best) {
    if (!ctx) return fail(nullptr, FOORT_E_BADARG, "ctx is NULL");
    if (n == 0 || !d_px || !d_out) return fail(ctx, FOORT_E_BADARG, "autotuning needs pixels and a result buffer");
    int rc = finish(ctx);
    if (rc != FOORT_OK && rc != FOORT_E_BUDGET && rc != FOORT_E_CANCELLED) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
    if ((rc = autotune_launch(ctx, d_px, n, d_out, st, best))) return rc;
    return finish(ctx);
}

int foort_gpu_set_autotune(foort_ctx* ctx, int32_t on) {
    if (!ctx) return fail(nullptr, FOORT_E_BADARG, "ctx is NULL");
    ctx->autotune = on != 0;
    return FOORT_OK;
}

int foort_gpu_launch_shape(foort_ctx* ctx, uint64_t n, foort_launch_shape* shape) {
    if (!ctx || !shape) return fail(ctx, FOORT_E_BADARG, "NULL argument");
    const foort_launch_shape want = requested_shape(ctx, n);
    LaunchShape ls;
    const int rc = choose_launch(ctx, ctx->rc, n, ctx->num_sms, want, ls);
    if (rc) return rc;
    *shape = foort_launch_shape{ls.block, want.blocks_per_sm, ls.lanes, ls.refill, ls.poll, 0, want.ms};
    return FOORT_OK;
}

int foort_gpu_set_schedule(foort_ctx* ctx, uint32_t schedule) {
    if (!ctx) return fail(nullptr, FOORT_E_BADARG, "ctx is NULL");
    if (schedule > FOORT_SCHEDULE_ROUNDS) return fail(ctx, FOORT_E_BADARG, "unknown schedule");
    ctx->schedule = schedule;
    return FOORT_OK;
}

int foort_gpu_run_info(const foort_ctx* ctx, uint32_t* launches, uint32_t* schedule) {
    if (!ctx) return FOORT_E_BADARG;
    if (launches) *launches = ctx->run_launches;
    if (schedule) *schedule = ctx->run_schedule;
    return FOORT_OK;
}

int foort_gpu_set_lookahead(foort_ctx* ctx, uint64_t max_geodesics) {
    if (!ctx) return fail(nullptr, FOORT_E_BADARG, "ctx is NULL");
    ctx->lookahead = max_geodesics;
    return FOORT_OK;
}

int foort_gpu_set_record_launches(foort_ctx* ctx, int32_t on) {
    if (!ctx) return fail(nullptr, FOORT_E_BADARG, "ctx is NULL");
    ctx->record = on != 0;
    if (!ctx->record) ctx->launch_px.clear();
    return FOORT_OK;
}

int foort_gpu_run_launch(const foort_ctx* ctx, uint32_t k, foort_pixel* out, uint64_t cap, uint64_t* n) {
    if (!ctx || !n || k >= ctx->launch_px.size()) return FOORT_E_BADARG;
    const auto& v = ctx->launch_px[k];
    *n = v.size();
    if (!out) return FOORT_OK;
    if (cap < v.size()) return FOORT_E_BADARG;
    std::copy(v.begin(), v.end(), out);
    return FOORT_OK;
}

uint32_t foort_ctx_schedule(const foort_ctx* ctx) { return ctx->schedule; }
uint64_t foort_ctx_lookahead(const foort_ctx* ctx) {
    return ctx->lookahead == FOORT_LOOKAHEAD_AUTO ? 128ull * static_cast<uint64_t>(ctx->num_sms) : ctx->lookahead;
}
void foort_ctx_launched(foort_ctx* ctx, const foort_pixel* px, uint64_t n, bool first) {
    if (first) ctx->launch_px.clear();
    if (ctx->record) ctx->launch_px.emplace_back(px, px + n);
}
uint64_t foort_ctx_budget(const foort_ctx* ctx) { return ctx->budget; }
void foort_ctx_set_run_info(foort_ctx* ctx, uint32_t launches, uint32_t schedule) {
    ctx->run_launches = launches;
    ctx->run_schedule = schedule;
}
// Pinned room for n pixels and n results, kept by the context from run to run.
int foort_ctx_stage(foort_ctx* ctx, uint64_t n, foort_pixel** px, foort_result** res) {
    if (n > ctx->stage_cap) {
        if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
        if (ctx->h_stage_px) cudaFreeHost(ctx->h_stage_px);
        ctx->h_stage = nullptr;
        ctx->h_stage_px = nullptr;
        ctx->stage_cap = 0;
        CK(cudaHostAlloc(reinterpret_cast<void**>(&ctx->h_stage), n * sizeof(foort_result), cudaHostAllocDefault));
        CK(cudaHostAlloc(reinterpret_cast<void**>(&ctx->h_stage_px), n * sizeof(foort_pixel), cudaHostAllocDefault));
        ctx->stage_cap = n;
    }
    if (px) *px = ctx->h_stage_px;
    if (res) *res = ctx->h_stage;
    return FOORT_OK;
}
// foort_gpu_integrate in two halves, for foort_gpu_run to work on the host while a launch
// runs: begin enqueues the copy of n pixels from host memory, the launch and the copy of
// the results into the pinned staging, and returns; end waits for them and copies the
// results out (out == NULL: they stay in the staging, foort_ctx_stage). px may be the
// staging's own pixels. Nothing else may launch on the context in between.
int foort_ctx_integrate_begin(foort_ctx* ctx, const foort_pixel* px, uint64_t n) {
    if (!ctx) return fail(nullptr, FOORT_E_BADARG, "ctx is NULL");
    if (n && !px) return fail(ctx, FOORT_E_BADARG, "NULL pixel buffer");
    for (uint64_t i = 0; i < n; ++i)
        if (px[i].image >= ctx->hic.size() || px[i].grid < 2)
            return fail(ctx, FOORT_E_BADARG, "pixel " + std::to_string(i) + " has an invalid image index or grid < 2");
    int rc = finish(ctx);
    if (rc != FOORT_OK && rc != FOORT_E_BUDGET && rc != FOORT_E_CANCELLED) return rc;
    if ((rc = ensure_capacity(ctx, n))) return rc;
    if (n > ctx->stage_cap) {
        if (px == ctx->h_stage_px) return fail(ctx, FOORT_E_BADARG, "staged pixels beyond the staging");
        if ((rc = foort_ctx_stage(ctx, n, nullptr, nullptr))) return rc;
    }
    cudaStream_t st = ctx->stream;
    if (n) CK(cudaMemcpyAsync(ctx->d_px, px, n * sizeof(foort_pixel), cudaMemcpyHostToDevice, st));
    if ((rc = launch(ctx, ctx->d_px, n, ctx->d_out, st))) return rc;
    if (n) CK(cudaMemcpyAsync(ctx->h_stage, ctx->d_out, n * sizeof(foort_result), cudaMemcpyDeviceToHost, st));
    return FOORT_OK;
}
int foort_ctx_integrate_end(foort_ctx* ctx, foort_result* out, uint64_t n) {
    const int rc = finish(ctx);
    if (out && n && (rc == FOORT_OK || rc == FOORT_E_BUDGET || rc == FOORT_E_CANCELLED))
        std::memcpy(out, ctx->h_stage, n * sizeof(foort_result));
    return rc;
}

int foort_gpu_get_desc(const foort_ctx* ctx, foort_run_desc* desc) {
    if (!ctx || !desc) return FOORT_E_BADARG;
    *desc = ctx->desc;  // images: the context's own copy
    return FOORT_OK;
}

int foort_gpu_get_stats(const foort_ctx* ctx, foort_stats* stats) {
    if (!ctx || !stats) return FOORT_E_BADARG;
    *stats = ctx->stats;
    return FOORT_OK;
}

void foort_gpu_destroy(foort_ctx* ctx) {
    if (!ctx) return;
    if (ctx->pending && ctx->last_stream) cudaStreamSynchronize(ctx->last_stream);
    if (ctx->d_px) cudaFree(ctx->d_px);
    if (ctx->d_out) cudaFree(ctx->d_out);
    if (ctx->d_images) cudaFree(ctx->d_images);
    if (ctx->d_ctr) cudaFree(ctx->d_ctr);
    if (ctx->h_cancel) cudaFreeHost(ctx->h_cancel);
    if (ctx->h_ctr) cudaFreeHost(ctx->h_ctr);
    if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
    if (ctx->h_stage_px) cudaFreeHost(ctx->h_stage_px);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

const char* foort_gpu_last_error(const foort_ctx* ctx) {
    if (ctx) return ctx->err.c_str();
    std::lock_guard<std::mutex> lk(g_err_mu);
    return g_create_err.c_str();
}

double foort_horizon_radius(int32_t metric_id, const double* metric_params) {
    if (!metric_params || metric_id < 0 || metric_id > 4) return 0.0;
    return make_metric_const(metric_id, metric_params).rh;
}

int foort_gpu_has_kernel(int32_t metric_id, int32_t integrator_id, int32_t precision) {
    if (metric_id < 0 || metric_id > 4) return 0;
    if (integrator_id != FOORT_INTEGRATOR_RK4 && integrator_id != FOORT_INTEGRATOR_VERLET) return 0;
    if (precision == FOORT_PREC_FP64) return fp64_kernel(metric_id, integrator_id) != nullptr;
    if (analytic_family(precision)) return mixed_kernel(metric_id, integrator_id) != nullptr;
    return 0;
}

// Sizes of the ABI structs, for binding checks (0 pixel, 1 result, 2 run_desc,
// 3 image_desc, 4 stats, 5 output_desc, 6 config).
uint64_t foort_abi_size(int32_t which) {
    switch (which) {
    case 0: return sizeof(foort_pixel);
    case 1: return sizeof(foort_result);
    case 2: return sizeof(foort_run_desc);
    case 3: return sizeof(foort_image_desc);
    case 4: return sizeof(foort_stats);
    case 5: return sizeof(foort_output_desc);
    case 6: return sizeof(foort_config);
    default: return 0;
    }
}

}  // extern "C"

namespace foort {

const void* fp64_kernel_kerr(int);
const void* fp64_kernel_flat(int);
const void* fp64_kernel_rl(int);
const void* fp64_kernel_joh(int);
const void* fp64_kernel_mn(int);

const void* fp64_kernel(int metric_id, int integ) {
    switch (metric_id) {
    case kKerr: return fp64_kernel_kerr(integ);
    case kFlat: return fp64_kernel_flat(integ);
    case kRasheedLarsen: return fp64_kernel_rl(integ);
    case kJohannsen: return fp64_kernel_joh(integ);
    case kMankoNovikov: return fp64_kernel_mn(integ);
    default: return nullptr;
    }
}

}  // namespace foort

// ---------------------------------------------------------------------------------------
// Allocation-free entry point (foort_gpu_integrate_noalloc).
//
// The launch counters and the per-image constants that foort_gpu_create() puts in
// cudaMalloc'd memory live here in one statically declared device array instead. On the
// host, foort_noalloc_scratch names that array only as a symbol: its device address on
// the current device comes from cudaGetSymbolAddress, looked up on every call.

static_assert(sizeof(ImageConst) == 672, "FOORT_NOALLOC_SCRATCH_BYTES assumes 672-byte image constants");
static_assert(kNumCtr * sizeof(unsigned long long) <= 256, "the counters take the first 256 bytes");

static __device__ __align__(256) unsigned char foort_noalloc_scratch[FOORT_NOALLOC_SCRATCH_BYTES];

namespace {

constexpr int kNoAllocMaxDevices = 64;

struct NoAllocDevice {
    unsigned char* scratch = nullptr;  // device address of foort_noalloc_scratch
    int num_sms = 0;
};

std::mutex g_noalloc_mu;
NoAllocDevice g_noalloc_dev[kNoAllocMaxDevices];

// The current device's array address and SM count. The address is looked up on every
// call (cheap once the module is loaded): a context made anew after cudaDeviceReset loads
// the module again, possibly elsewhere. The SM count is the device's and is kept. Takes
// no stream operation.
int noalloc_device(int dev, NoAllocDevice& out) {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    NoAllocDevice& d = g_noalloc_dev[dev];
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, foort_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaGetSymbolAddress(foort_noalloc_scratch)");
    d.scratch = static_cast<unsigned char*>(p);
    if (!d.num_sms) {
        int sms = 0;
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaDeviceGetAttribute");
        d.num_sms = sms;
    }
    out = d;
    return FOORT_OK;
}

}  // namespace

extern "C" int foort_gpu_integrate_noalloc(const foort_run_desc* desc, const foort_pixel* d_px, uint64_t n,
                                           foort_result* d_out, void* cuda_stream, foort_stats* stats) {
    foort_ctx* ctx = nullptr;  // errors go to foort_gpu_last_error(NULL)
    std::string why;
    int v = validate(desc, why);
    if (v) return fail(nullptr, v, why);
    if (desc->n_images > FOORT_NOALLOC_MAX_IMAGES)
        return fail(nullptr, FOORT_E_BADARG,
                    "n_images = " + std::to_string(desc->n_images) + " exceeds the " +
                        std::to_string(FOORT_NOALLOC_MAX_IMAGES) +
                        " images that the allocation-free entry point has room for");
    if (n && (!d_px || !d_out)) return fail(nullptr, FOORT_E_BADARG, "NULL pixel or result buffer");
    const RunConst R0 = make_run_const(*desc);
    const void* fn = select_kernel(R0);
    if (!fn) return fail(nullptr, FOORT_E_UNSUPPORTED, "no kernel for this metric / integrator / precision");

    int dev = 0;
    CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNoAllocMaxDevices)
        return fail(nullptr, FOORT_E_BADARG, "device index beyond the " + std::to_string(kNoAllocMaxDevices) +
                                                 " devices the allocation-free entry point tracks");
    NoAllocDevice nd;
    int rc = noalloc_device(dev, nd);
    if (rc) return rc;
    unsigned long long* d_ctr = reinterpret_cast<unsigned long long*>(nd.scratch);
    ImageConst* d_images = reinterpret_cast<ImageConst*>(nd.scratch + 256);
    cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);

    // Image constants, one at a time from the stack: a copy from pageable memory returns
    // once the source has been staged, so the next image may reuse the buffer.
    for (uint32_t i = 0; i < desc->n_images; ++i) {
        ImageConst ic;
        std::memset(&ic, 0, sizeof(ic));
        ic.m = make_metric_const(desc->metric_id, desc->images[i].metric_params);
        camera_frame(desc->metric_id, R0.rlog != 0, desc->images[i], ic);
        ic.h_eps = desc->images[i].horizon_eps > 0.0 ? desc->images[i].horizon_eps : desc->horizon_eps;
        if (analytic_family(R0.precision)) fill_mixed_constants(desc->metric_id, ic, R0);
        CK(cudaMemcpyAsync(d_images + i, &ic, sizeof(ic), cudaMemcpyHostToDevice, st));
    }
    CK(cudaMemsetAsync(d_ctr, 0, kNumCtr * sizeof(unsigned long long), st));

    LaunchShape ls;
    if ((rc = choose_launch(nullptr, R0, n, nd.num_sms, foort_launch_shape{}, ls))) return rc;
    const uint32_t bs = ls.block, grid = ls.grid;
    fn = ls.fn;
    LaunchArgs A{};
    A.px = d_px;
    A.out = d_out;
    A.n = n;
    A.images = d_images;
    A.n_images = desc->n_images;
    A.ctr = d_ctr;
    A.cancel = nullptr;
    A.budget = 0;
    if (!(R0.term_flags & FOORT_TERM_TIMEOUT)) A.budget = std::max<unsigned long long>(100000000ull, 1000000ull * n);
    RunConst R = R0;
    R.refill_steps = static_cast<int32_t>(ls.refill);
    R.poll_steps = static_cast<int32_t>(ls.poll);
    void* args[2] = {&A, &R};
    if (n > 0) CK(cudaLaunchKernel(fn, dim3(grid), dim3(bs), args, 0, st));
    if (!stats) return FOORT_OK;

    unsigned long long h_ctr[kNumCtr] = {};
    CK(cudaMemcpyAsync(h_ctr, d_ctr, sizeof(h_ctr), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    std::memset(stats, 0, sizeof(*stats));
    stats->geodesics = h_ctr[kCtrDone];
    stats->steps = h_ctr[kCtrSteps];
    stats->rhs_evals = h_ctr[kCtrRhs];
    stats->fp64_steps = h_ctr[kCtrFp64Steps];
    stats->n_blocks = grid;
    stats->block_size = bs;
    stats->lanes_per_geodesic = ls.lanes;
    stats->refill_steps = ls.refill;
    stats->poll_steps = ls.poll;
    rc = FOORT_OK;
    if (h_ctr[kCtrStatus] & kStatusBudget)
        rc = fail(nullptr, FOORT_E_BUDGET, "global step budget exhausted; unfinished geodesics are marked");
    stats->status = static_cast<uint32_t>(rc);
    return rc;
}
