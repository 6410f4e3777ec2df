// ORACLE -- TEST INFRASTRUCTURE ONLY.
//
// Driver that runs the reference implementation itself. It is linked against the
// reference's own translation units (Diagnostics, Geodesic, InputOutput, Integrators,
// Mesh, Metric, Terminations, Utilities, ViewScreen), compiled unmodified from where
// they lie by oracle/Makefile. Config.cpp and Main.cpp are left out: Config.cpp needs
// libconfig, so this file defines the static option objects that Config.cpp:11-28
// would define, and the loops below restate Main.cpp:313-427.
//
// The library it produces (oracle/_ref/libfoort_ref*.so) exists only where the
// reference sources exist; it generates the golden fixtures under tests/golden/ and
// validates the restatement in oracle/foort_oracle.cpp.

#include "Diagnostics.h"
#include "Geodesic.h"
#include "InputOutput.h"
#include "Integrators.h"
#include "Mesh.h"
#include "Metric.h"
#include "Terminations.h"
#include "Utilities.h"
#include "ViewScreen.h"

#include "../include/foort_gpu.h"
#include "ref_driver.h"

#include <omp.h>

#include <chrono>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

// Static option objects (Config.cpp:11-28 defines these in the reference build).
std::unique_ptr<GeodesicPositionOptions> GeodesicPositionDiagnostic::DiagOptions;
std::unique_ptr<EquatorialPassesOptions> EquatorialPassesDiagnostic::DiagOptions;
std::unique_ptr<ClosestRadiusOptions> ClosestRadiusDiagnostic::DiagOptions;
std::unique_ptr<HorizonTermOptions> HorizonTermination::TermOptions;
std::unique_ptr<BoundarySphereTermOptions> BoundarySphereTermination::TermOptions;
std::unique_ptr<TimeOutTermOptions> TimeOutTermination::TermOptions;
std::unique_ptr<ThetaSingularityTermOptions> ThetaSingularityTermination::TermOptions;

namespace {

// A Mesh (the reference's plugin interface, Mesh.h:24-61) that hands out an explicit
// list of pixels with the unit-point convention of Mesh.cpp:49 / :671-672.
class ListMesh final : public Mesh {
public:
    ListMesh(std::vector<foort_pixel> px, DiagBitflag valdiag) : Mesh(valdiag), m_px(std::move(px)) {}
    largecounter getCurNrGeodesics() const final { return m_px.size(); }
    void getNewInitConds(largecounter index, ScreenPoint& p, ScreenIndex& s) const final {
        const foort_pixel& q = m_px[index];
        s = ScreenIndex{q.row, q.col};
        p = ScreenPoint{q.row * 1.0 / static_cast<real>(q.grid - 1), q.col * 1.0 / static_cast<real>(q.grid - 1)};
    }
    void GeodesicFinished(largecounter, std::vector<real>) final {}
    void EndCurrentLoop() final { m_done = true; }
    bool IsFinished() const final { return m_done; }

private:
    std::vector<foort_pixel> m_px;
    bool m_done{false};
};

std::unique_ptr<Metric> make_metric(const foort_run_desc* d, const double* p) {
    bool rl = d->rlog != 0;
    switch (d->metric_id) {
    case FOORT_METRIC_KERR: return std::unique_ptr<Metric>(new KerrMetric(p[0], rl));
    case FOORT_METRIC_FLAT: return std::unique_ptr<Metric>(new FlatSpaceMetric());
    case FOORT_METRIC_RASHEED_LARSEN: return std::unique_ptr<Metric>(new RasheedLarsenMetric(p[0], p[1], p[2], p[3], rl));
    case FOORT_METRIC_JOHANNSEN: return std::unique_ptr<Metric>(new JohannsenMetric(p[0], p[1], p[2], p[3], p[4], rl));
    default: return std::unique_ptr<Metric>(new MankoNovikovMetric(p[0], p[1], rl));
    }
}

// Set the process-global options the way Config.cpp:393-1071 would for these settings.
GeodesicIntegratorFunc set_globals(const foort_run_desc* d, const Metric* M, TermBitflag& terms, double heps) {
    SetOutputLevel(OutputLevel::Level_0_WARNING);
    const SphericalHorizonMetric* sm = dynamic_cast<const SphericalHorizonMetric*>(M);
    bool rl = sm && sm->getrLogScale();
    terms = static_cast<TermBitflag>(d->term_flags);
    if (terms & Term_Horizon) {
        if (!sm) terms &= static_cast<TermBitflag>(~Term_Horizon);
        else HorizonTermination::TermOptions.reset(new HorizonTermOptions{sm->getHorizonRadius(), rl, heps, d->horizon_every});
    }
    BoundarySphereTermination::TermOptions.reset(new BoundarySphereTermOptions{d->boundary_radius, rl, d->boundary_every});
    TimeOutTermination::TermOptions.reset(new TimeOutTermOptions{d->timeout_max_steps, d->timeout_every});
    ThetaSingularityTermination::TermOptions.reset(new ThetaSingularityTermOptions{d->theta_eps, d->theta_every});
    EquatorialPassesDiagnostic::DiagOptions.reset(new EquatorialPassesOptions(
        d->equat_threshold, UpdateFrequency{d->equat_freq.every_n, d->equat_freq.at_start != 0, d->equat_freq.at_finish != 0}));
    ClosestRadiusDiagnostic::DiagOptions.reset(new ClosestRadiusOptions(
        rl, UpdateFrequency{d->closest_freq.every_n, d->closest_freq.at_start != 0, d->closest_freq.at_finish != 0}));
    GeodesicPositionDiagnostic::DiagOptions.reset(new GeodesicPositionOptions(
        d->geopos_output_steps, UpdateFrequency{d->geopos_freq.every_n, d->geopos_freq.at_start != 0, d->geopos_freq.at_finish != 0}));
    Integrators::epsilon = d->epsilon;
    Integrators::Derivative_hval = d->derivative_h;
    Integrators::SmallestPossibleStepsize = d->smallest_step;
    Integrators::VerletVelocityTolerance = d->verlet_tol;
    if (d->integrator_id == FOORT_INTEGRATOR_VERLET) {
        Integrators::IntegratorDescription = "Verlet";
        return Integrators::IntegrateGeodesicStep_Verlet;
    }
    Integrators::IntegratorDescription = "RK4";
    return Integrators::IntegrateGeodesicStep_RK4;
}

void fill_result(const Geodesic& g, uint64_t steps, uint32_t diag_flags, uint32_t valdiag, foort_result& o) {
    o.term = static_cast<int32_t>(g.getTermCondition());
    o.err = 0;
    o.steps = steps;
    o.lambda = g.getCurrentLambda();
    Point p = g.getCurrentPos();
    OneIndex v = g.getCurrentVel();
    for (int i = 0; i < 4; ++i) { o.pos[i] = p[i]; o.vel[i] = v[i]; }
    // Output strings in CreateDiagnosticVector order (Diagnostics.cpp:14-99): appended in
    // the order FourColor, GeodesicPosition, EquatorialPasses, ClosestRadius; appending
    // the value diagnostic rotates the vector left by one (std::rotate(b, b + 1, e)).
    std::vector<std::string> s = g.getAllOutputStr();
    std::vector<uint32_t> order;
    const uint32_t all[4] = {FOORT_DIAG_FOUR_COLOR_SCREEN, FOORT_DIAG_GEODESIC_POSITION, FOORT_DIAG_EQUATORIAL_PASSES,
                             FOORT_DIAG_CLOSEST_RADIUS};
    for (uint32_t f : all) {
        if (!(diag_flags & f)) continue;
        order.push_back(f);
        if (valdiag & f) { order.push_back(order.front()); order.erase(order.begin()); }
    }
    o.quadrant = 0;
    o.equat_passes = 0;
    o.closest_r = -1;
    for (size_t k = 0; k < order.size() && k + 1 < s.size(); ++k) {
        const std::string& t = s[k + 1];
        if (order[k] == FOORT_DIAG_FOUR_COLOR_SCREEN) o.quadrant = std::stoi(t);
        if (order[k] == FOORT_DIAG_EQUATORIAL_PASSES) o.equat_passes = std::stoi(t);
        if (order[k] == FOORT_DIAG_CLOSEST_RADIUS) o.closest_r = std::stod(t);
    }
    // The first diagnostic's value is available at full precision.
    std::vector<real> val = g.getDiagnosticFinalValue();
    if (!order.empty() && order[0] == FOORT_DIAG_CLOSEST_RADIUS && !val.empty()) o.closest_r = val[0];
}

}  // namespace

extern "C" {

// Integrate an explicit pixel list with the reference's own objects (Main.cpp:327-402),
// one image after the other. `lines` (optional, n * line_stride bytes) receives each
// geodesic's output line as GeodesicOutputHandler would write it for diagnostic 0.
int ref_integrate(const foort_run_desc* d, const foort_pixel* px, uint64_t n, foort_result* out, int nthreads,
                  char* lines, uint64_t line_stride) {
    if (!d || !d->images || d->n_images == 0) return FOORT_E_BADARG;
    if (nthreads <= 0) nthreads = omp_get_max_threads();
    for (uint32_t im = 0; im < d->n_images; ++im) {
        std::vector<foort_pixel> sub;
        std::vector<uint64_t> where;
        for (uint64_t i = 0; i < n; ++i)
            if (px[i].image == im) { sub.push_back(px[i]); where.push_back(i); }
        if (sub.empty()) continue;
        const foort_image_desc& I = d->images[im];
        std::unique_ptr<Metric> M = make_metric(d, I.metric_params);
        std::unique_ptr<Source> S(new NoSource(M.get()));
        TermBitflag terms;
        GeodesicIntegratorFunc integ = set_globals(d, M.get(), terms, I.horizon_eps > 0.0 ? I.horizon_eps : d->horizon_eps);
        DiagBitflag diags = static_cast<DiagBitflag>(d->diag_flags), vd = static_cast<DiagBitflag>(d->value_diag);
        ViewScreen view(Point{I.cam_pos[0], I.cam_pos[1], I.cam_pos[2], I.cam_pos[3]},
                        OneIndex{I.cam_dir[0], I.cam_dir[1], I.cam_dir[2], I.cam_dir[3]},
                        ScreenPoint{I.screen_size[0], I.screen_size[1]}, ScreenPoint{I.screen_center[0], I.screen_center[1]},
                        std::unique_ptr<Mesh>(new ListMesh(sub, vd)), M.get());
        long long N = static_cast<long long>(sub.size());
#pragma omp parallel num_threads(nthreads)
        {
            Geodesic g(M.get(), S.get(), diags, vd, terms, integ);
#pragma omp for schedule(dynamic, 4)
            for (long long k = 0; k < N; ++k) {
                Point p;
                OneIndex v;
                ScreenIndex si;
                view.SetNewInitialConditions(static_cast<largecounter>(k), p, v, si);
                g.Reset(si, p, v);
                uint64_t steps = 0;
                while (g.getTermCondition() == Term::Continue) { g.Update(); ++steps; }
                fill_result(g, steps, d->diag_flags, d->value_diag, out[where[k]]);
                if (lines && line_stride) {
                    std::vector<std::string> s = g.getAllOutputStr();
                    std::string line = s[0] + " " + (s.size() > 1 ? s[1] : std::string());
                    char* dst = lines + where[k] * line_stride;
                    std::strncpy(dst, line.c_str(), line_stride - 1);
                    dst[line_stride - 1] = 0;
                }
            }
        }
    }
    return FOORT_OK;
}

static std::unique_ptr<Mesh> make_mesh(const ref_mesh_spec* ms, DiagBitflag vd) {
    if (ms->kind == 0) return std::unique_ptr<Mesh>(new SimpleSquareMesh(ms->total_pixels, vd));
    return std::unique_ptr<Mesh>(new SquareSubdivisionMeshV2(ms->max_pixels, ms->initial_pixels, ms->max_subdivide,
                                                             ms->iteration_pixels, ms->initial_sub_to_final != 0, vd));
}

}  // extern "C"

// A full run of image 0 as Main.cpp:313-427 does it, writing the reference's .dat files
// through GeodesicOutputHandler; each round's geodesics are integrated by `body`.
int ref_run_rounds(const foort_run_desc* d, const ref_mesh_spec* ms, const char* prefix, const char* timestamp,
                   const char* ext, uint64_t to_cache, uint64_t per_file, int32_t first_line, const RefRoundBody& body,
                   uint64_t* n_geod, uint32_t* n_rounds, double* seconds) {
    if (!d || !ms || !d->images) return FOORT_E_BADARG;
    const foort_image_desc& I = d->images[0];
    std::unique_ptr<Metric> M = make_metric(d, I.metric_params);
    std::unique_ptr<Source> S(new NoSource(M.get()));
    TermBitflag terms;
    GeodesicIntegratorFunc integ = set_globals(d, M.get(), terms, I.horizon_eps > 0.0 ? I.horizon_eps : d->horizon_eps);
    DiagBitflag diags = static_cast<DiagBitflag>(d->diag_flags), vd = static_cast<DiagBitflag>(d->value_diag);
    std::unique_ptr<ViewScreen> view(new ViewScreen(
        Point{I.cam_pos[0], I.cam_pos[1], I.cam_pos[2], I.cam_pos[3]}, OneIndex{I.cam_dir[0], I.cam_dir[1], I.cam_dir[2], I.cam_dir[3]},
        ScreenPoint{I.screen_size[0], I.screen_size[1]}, ScreenPoint{I.screen_center[0], I.screen_center[1]}, make_mesh(ms, vd),
        M.get()));
    std::string info = first_line ? Utilities::GetFirstLineInfoString(M.get(), S.get(), diags, vd, terms, view.get()) : "";
    GeodesicOutputHandler outh(prefix ? prefix : "", timestamp ? timestamp : "", ext ? ext : "",
                               Utilities::GetDiagNameStrings(diags, vd), to_cache, per_file, info);
    auto t0 = std::chrono::steady_clock::now();
    uint64_t total = 0;
    uint32_t rounds = 0;
    while (!view->IsFinished()) {
        total += static_cast<uint64_t>(view->getCurNrGeodesics());
        ++rounds;
        const int rc = body(view.get(), &outh, RefRunObjects{M.get(), S.get(), diags, vd, terms, integ});
        if (rc != FOORT_OK) return rc;
        view->EndCurrentLoop();
    }
    outh.OutputFinished();
    if (n_geod) *n_geod = total;
    if (n_rounds) *n_rounds = rounds;
    if (seconds) *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return FOORT_OK;
}

extern "C" {

// ref_run_rounds with the reference's own round body: the OpenMP loop of Main.cpp:327-402.
int ref_run(const foort_run_desc* d, const ref_mesh_spec* ms, const char* prefix, const char* timestamp,
            const char* ext, uint64_t to_cache, uint64_t per_file, int32_t first_line, int nthreads,
            uint64_t* n_geod, uint32_t* n_rounds, double* seconds) {
    if (nthreads <= 0) nthreads = omp_get_max_threads();
    auto body = [nthreads](ViewScreen* view, GeodesicOutputHandler* outh, const RefRunObjects& o) {
        long long N = static_cast<long long>(view->getCurNrGeodesics());
#pragma omp parallel num_threads(nthreads)
        {
#pragma omp single
            outh->PrepareForOutput(static_cast<largecounter>(N));
            Geodesic g(o.metric, o.source, o.diags, o.valdiag, o.terms, o.integrator);
#pragma omp for schedule(dynamic, 4)
            for (long long k = 0; k < N; ++k) {
                Point p;
                OneIndex v;
                ScreenIndex si;
                view->SetNewInitialConditions(static_cast<largecounter>(k), p, v, si);
                g.Reset(si, p, v);
                while (g.getTermCondition() == Term::Continue) g.Update();
                view->GeodesicFinished(static_cast<largecounter>(k), g.getDiagnosticFinalValue());
                outh->NewGeodesicOutput(static_cast<largecounter>(k), g.getAllOutputStr());
            }
        }
        return static_cast<int>(FOORT_OK);
    };
    return ref_run_rounds(d, ms, prefix, timestamp, ext, to_cache, per_file, first_line, body, n_geod, n_rounds,
                          seconds);
}

// The run-description line the reference writes first in every output file
// (Utilities.cpp:52-84), for image 0 of `d` and mesh `ms`.
int ref_first_line(const foort_run_desc* d, const ref_mesh_spec* ms, char* buf, uint64_t len) {
    if (!d || !ms || !buf || !len) return FOORT_E_BADARG;
    const foort_image_desc& I = d->images[0];
    std::unique_ptr<Metric> M = make_metric(d, I.metric_params);
    std::unique_ptr<Source> S(new NoSource(M.get()));
    TermBitflag terms;
    set_globals(d, M.get(), terms, I.horizon_eps > 0.0 ? I.horizon_eps : d->horizon_eps);
    DiagBitflag diags = static_cast<DiagBitflag>(d->diag_flags), vd = static_cast<DiagBitflag>(d->value_diag);
    ViewScreen view(Point{I.cam_pos[0], I.cam_pos[1], I.cam_pos[2], I.cam_pos[3]},
                    OneIndex{I.cam_dir[0], I.cam_dir[1], I.cam_dir[2], I.cam_dir[3]},
                    ScreenPoint{I.screen_size[0], I.screen_size[1]}, ScreenPoint{I.screen_center[0], I.screen_center[1]},
                    make_mesh(ms, vd), M.get());
    std::string s = Utilities::GetFirstLineInfoString(M.get(), S.get(), diags, vd, terms, &view);
    std::strncpy(buf, s.c_str(), len - 1);
    buf[len - 1] = 0;
    return FOORT_OK;
}

// Synthetic per-pixel values for mesh-only traces: a pure function of (row, col, grid)
// with the value ranges of the three scalar diagnostics. Restated identically by the
// tests that replay these traces.
static double synth_value(int kind, uint64_t row, uint64_t col, uint64_t grid) {
    long long R = static_cast<long long>(grid);
    long long dr = 2 * static_cast<long long>(row) - R, dc = 2 * static_cast<long long>(col) - R;
    if (kind == 0) {  // quadrant-like: 0 inside a disk, 1..4 by sector outside
        if (dr * dr + 3 * dc * dc < (R * R) / 3) return 0.0;
        return static_cast<double>(1 + (row < col ? 0 : 1) + (static_cast<long long>(row + col) < R ? 0 : 2));
    }
    if (kind == 1) {  // pass-count-like integers in [-2, 3]
        long long w = R / 8 + 1;
        return static_cast<double>(((static_cast<long long>(row) * 31 + static_cast<long long>(col) * 17) / w) % 6 - 2);
    }
    // radius-like continuous values; every operation is exact (a power-of-two scale),
    // so the value does not depend on floating-point flags
    long long h = (static_cast<long long>(row) * 7919 + static_cast<long long>(col) * 104729) % 1009;
    return 1.5 + static_cast<double>(h) * 0.0009765625 * static_cast<double>((row + col) % 3);
}

// Drive a reference Mesh with synthetic values and record every round's queue:
// rows/cols/round_of receive the pixels in the order getNewInitConds hands them out.
int ref_mesh_trace(const ref_mesh_spec* ms, uint32_t value_diag, int32_t value_kind, uint64_t* rows, uint64_t* cols,
                   uint32_t* round_of, uint64_t cap, uint64_t* n_out, uint32_t* n_rounds) {
    if (!ms) return FOORT_E_BADARG;
    SetOutputLevel(OutputLevel::Level_0_WARNING);
    std::unique_ptr<Mesh> mesh = make_mesh(ms, static_cast<DiagBitflag>(value_diag));
    uint64_t k = 0;
    uint32_t rnd = 0;
    while (!mesh->IsFinished()) {
        largecounter N = mesh->getCurNrGeodesics();
        for (largecounter i = 0; i < N; ++i) {
            ScreenPoint up;
            ScreenIndex si;
            mesh->getNewInitConds(i, up, si);
            // The grid size is recovered from the unit point: col = up * (R - 1).
            uint64_t grid = 0;
            if (ms->kind == 0) grid = static_cast<uint64_t>(std::sqrt(static_cast<double>(ms->total_pixels)));
            else {
                uint64_t s = static_cast<uint64_t>(std::sqrt(static_cast<double>(ms->initial_pixels)));
                grid = (s - 1) * (1ull << (ms->max_subdivide - 1)) + 1;
            }
            if (k < cap) { rows[k] = si[0]; cols[k] = si[1]; round_of[k] = rnd; }
            ++k;
            mesh->GeodesicFinished(i, std::vector<real>{synth_value(value_kind, si[0], si[1], grid)});
        }
        mesh->EndCurrentLoop();
        ++rnd;
    }
    if (n_out) *n_out = k;
    if (n_rounds) *n_rounds = rnd;
    return FOORT_OK;
}

}  // extern "C"
