// ORACLE -- TEST INFRASTRUCTURE ONLY.
//
// Runs the engine's FOORT-side binding (foort_gb300/shim/foort_round.cpp) inside the
// reference's own round loop: the reference's ViewScreen, Mesh and GeodesicOutputHandler
// (compiled from its sources by oracle/Makefile) with IntegrateRoundOnGPU as the body of
// each round. The engine call is the oracle restatement (oracle_integrate), standing in
// for the GPU on a machine without one; the library is linked with libfoort_gpu.so as a
// FOORT program would be, so the binding's default engine call resolves as it does there.
#include "ref_driver.h"

#include "../foort_gb300/shim/foort_round.h"

#include <cmath>

extern "C" int oracle_integrate(const foort_run_desc* d, const foort_pixel* px, uint64_t n, foort_result* out,
                                int nthreads);

namespace {

const foort_run_desc* g_desc = nullptr;
int g_threads = 0;

// foort_gpu_integrate's contract on the CPU: the oracle with the reference's flags.
int oracle_as_engine(foort_ctx*, const foort_pixel* px, uint64_t n, foort_result* out) {
    return oracle_integrate(g_desc, px, n, out, g_threads);
}

uint64_t mesh_grid(const ref_mesh_spec* ms) {
    if (ms->kind == 0) return static_cast<uint64_t>(std::llround(std::sqrt(static_cast<double>(ms->total_pixels))));
    const uint64_t s = static_cast<uint64_t>(std::llround(std::sqrt(static_cast<double>(ms->initial_pixels))));
    return (s - 1) * (1ull << (ms->max_subdivide - 1)) + 1;  // Mesh.h:306
}

}  // namespace

extern "C" int shim_run(const foort_run_desc* d, const ref_mesh_spec* ms, const char* prefix, const char* timestamp,
                        const char* ext, uint64_t to_cache, uint64_t per_file, int32_t first_line, int nthreads,
                        uint64_t* n_geod, uint32_t* n_rounds) {
    if (!d || !ms) return FOORT_E_BADARG;
    g_desc = d;
    g_threads = nthreads;
    const uint64_t grid = mesh_grid(ms);
    auto body = [grid](ViewScreen* view, GeodesicOutputHandler* outh, const RefRunObjects& o) {
        return IntegrateRoundOnGPU(view, outh, nullptr, grid, o.diags, o.valdiag, oracle_as_engine);
    };
    return ref_run_rounds(d, ms, prefix, timestamp, ext, to_cache, per_file, first_line, body, n_geod, n_rounds,
                          nullptr);
}
