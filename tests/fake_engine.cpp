// Test infrastructure: the engine entry points that foort_gpu_run (csrc/run.cpp) calls,
// without a GPU. Linked with run.cpp, mesh.cpp and output.cpp into a library of its own,
// it lets CPU tests run whole foort_gpu_run calls under every schedule. A pixel's result
// is a pure function of its grid cell (like an integration, whose result does not depend
// on the launch it runs in), and every launch is recorded.
#include <cstdint>
#include <cstring>
#include <vector>

#include "foort_gpu.h"

struct foort_ctx {
    foort_run_desc desc{};
    uint32_t schedule = FOORT_SCHEDULE_WAVES;
    uint64_t lookahead = 0;
    uint64_t budget = 0;
    uint32_t run_launches = 0, run_schedule = 0;
    std::vector<uint64_t> launch_sizes;
    std::vector<foort_pixel> stage_px;
    std::vector<foort_result> stage_res;
    bool pending = false;
    uint64_t pending_n = 0;
    int64_t fail_at = -1;  // the launch (0-based) that reports fail_code instead of running
    int fail_code = 0;
    uint64_t calls = 0;
};

namespace {

// Quadrants in bands that cross the grid at angles, a shadow disc in the middle, and
// pass counts and closest radii that vary from cell to cell.
foort_result result_of(const foort_pixel& p) {
    foort_result r;
    std::memset(&r, 0, sizeof r);
    const int64_t R = static_cast<int64_t>(p.grid), row = static_cast<int64_t>(p.row), col = static_cast<int64_t>(p.col);
    const int64_t dr = 2 * row - R, dc = 2 * col - R;
    int32_t quad = 1 + ((row * 3 + col * 5) / (R / 6 + 1)) % 4;
    if (dr * dr + 2 * dc * dc < (R * R) / 9) quad = 0;
    r.term = quad == 0 ? FOORT_TERMCODE_HORIZON : FOORT_TERMCODE_BOUNDARY_SPHERE;
    r.steps = static_cast<uint64_t>(100 + (row * 31 + col * 17) % 997);
    r.lambda = 0.5 * static_cast<double>(r.steps);
    r.pos[1] = quad == 0 ? 1.9 : 1000.5;
    r.pos[2] = 0.001 * static_cast<double>(row % 1000);
    r.pos[3] = 0.002 * static_cast<double>(col % 1000);
    r.vel[0] = 1.0;
    r.quadrant = quad;
    r.equat_passes = quad == 0 ? -static_cast<int32_t>((row + col) % 3) : static_cast<int32_t>((row * col) % 4);
    r.closest_r = quad == 0 ? 0.0 : 2.0 + static_cast<double>((row * 7 + col * 13) % 50) / 8.0;
    return r;
}

void compute(const foort_pixel* px, uint64_t n, foort_result* out) {
    for (uint64_t i = 0; i < n; ++i) out[i] = result_of(px[i]);
}

}  // namespace

extern "C" {

// ---- the test's handle on the fake context
foort_ctx* fake_ctx_create(uint32_t diag_flags, uint32_t value_diag, uint32_t schedule, uint64_t lookahead) {
    auto* c = new foort_ctx();
    c->desc.diag_flags = diag_flags;
    c->desc.value_diag = value_diag;
    c->schedule = schedule;
    c->lookahead = lookahead;
    return c;
}
void fake_ctx_destroy(foort_ctx* c) { delete c; }
uint64_t fake_ctx_launches(const foort_ctx* c) { return c->launch_sizes.size(); }
uint64_t fake_ctx_launch_size(const foort_ctx* c, uint64_t k) { return c->launch_sizes[k]; }
uint32_t fake_ctx_run_schedule(const foort_ctx* c) { return c->run_schedule; }
uint32_t fake_ctx_run_launches(const foort_ctx* c) { return c->run_launches; }
void fake_ctx_fail_at(foort_ctx* c, int64_t launch, int code) {
    c->fail_at = launch;
    c->fail_code = code;
}

// ---- what run.cpp calls
uint32_t foort_ctx_schedule(const foort_ctx* c) { return c->schedule; }
uint64_t foort_ctx_budget(const foort_ctx* c) { return c->budget; }
uint64_t foort_ctx_lookahead(const foort_ctx* c) { return c->lookahead; }
void foort_ctx_set_run_info(foort_ctx* c, uint32_t launches, uint32_t schedule) {
    c->run_launches = launches;
    c->run_schedule = schedule;
}
void foort_ctx_launched(foort_ctx* c, const foort_pixel*, uint64_t n, bool first) {
    if (first) c->launch_sizes.clear();
    c->launch_sizes.push_back(n);
}
int foort_ctx_stage(foort_ctx* c, uint64_t n, foort_pixel** px, foort_result** res) {
    if (c->pending) return FOORT_E_BADARG;  // the staging is not reallocated under a launch
    if (n > c->stage_px.size()) {
        c->stage_px.resize(n);
        c->stage_res.resize(n);
    }
    if (px) *px = c->stage_px.data();
    if (res) *res = c->stage_res.data();
    return FOORT_OK;
}
int foort_ctx_integrate_begin(foort_ctx* c, const foort_pixel* px, uint64_t n) {
    if (c->pending) return FOORT_E_BADARG;  // one launch in flight at a time
    if (static_cast<int64_t>(c->calls++) == c->fail_at) return c->fail_code;
    if (n > c->stage_res.size()) {
        if (px == c->stage_px.data()) return FOORT_E_BADARG;
        c->stage_px.resize(n);
        c->stage_res.resize(n);
    }
    compute(px, n, c->stage_res.data());
    c->pending = true;
    c->pending_n = n;
    return FOORT_OK;
}
int foort_ctx_integrate_end(foort_ctx* c, foort_result* out, uint64_t n) {
    if (!c->pending || n != c->pending_n) return FOORT_E_BADARG;
    c->pending = false;
    if (out && n) std::memcpy(out, c->stage_res.data(), n * sizeof(foort_result));
    return FOORT_OK;
}
int foort_gpu_get_desc(const foort_ctx* c, foort_run_desc* d) {
    *d = c->desc;
    return FOORT_OK;
}
int foort_gpu_integrate(foort_ctx* c, const foort_pixel* px, uint64_t n, foort_result* out) {
    if (c->pending) return FOORT_E_BADARG;
    if (static_cast<int64_t>(c->calls++) == c->fail_at) return c->fail_code;
    compute(px, n, out);
    return FOORT_OK;
}
int foort_gpu_positions(foort_ctx*, const foort_pixel*, uint64_t, const foort_result*, uint64_t*, double*, uint64_t,
                        uint64_t*) {
    return FOORT_E_UNSUPPORTED;
}

}  // extern "C"
