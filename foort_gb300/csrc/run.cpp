// A whole run: the round loop of Main.cpp:313-419 over the engine, the meshes and the
// output files, all through the C ABI.
//
// Per round every unfinished image's mesh hands out its pixels (ViewScreen::
// getCurNrGeodesics / SetNewInitialConditions); the pixels of all images go to the GPU
// in one launch (foort_gpu_integrate); the results go back to each mesh
// (GeodesicFinished, Main.cpp:399) and to each image's output files
// (NewGeodesicOutput, Main.cpp:400); then each mesh ends its round (EndCurrentLoop,
// Main.cpp:410). Images advance in lockstep, so a round is one launch over all images.
#include <algorithm>
#include <cstring>
#include <vector>

#include "../../include/foort_gpu.h"
#include "diag_order.h"

extern "C" int foort_gpu_run(foort_ctx* ctx, foort_mesh* const* meshes, foort_output* const* outputs,
                             uint32_t n_images, uint64_t* geodesics, uint32_t* rounds) {
    if (!ctx || !meshes || n_images == 0) return FOORT_E_BADARG;
    for (uint32_t i = 0; i < n_images; ++i)
        if (!meshes[i]) return FOORT_E_BADARG;
    foort_run_desc desc;
    if (foort_gpu_get_desc(ctx, &desc)) return FOORT_E_BADARG;
    const bool geopos = (desc.diag_flags & FOORT_DIAG_GEODESIC_POSITION) != 0;
    const std::vector<uint32_t> order = foort::diagnostic_order(desc.diag_flags, desc.value_diag);
    const uint32_t value_first = order.empty() ? 0u : order[0];
    uint64_t total = 0;
    uint32_t n_rounds = 0;
    std::vector<foort_pixel> px;
    std::vector<foort_result> res;
    std::vector<uint64_t> count(n_images);
    int rc = FOORT_OK;
    for (;;) {
        uint64_t n = 0;
        for (uint32_t i = 0; i < n_images; ++i) {
            const int fin = foort_mesh_is_finished(meshes[i]);
            if (fin < 0) return fin;
            count[i] = fin ? 0 : foort_mesh_cur_nr_geodesics(meshes[i]);
            n += count[i];
        }
        bool any = false;
        for (uint32_t i = 0; i < n_images; ++i) any = any || foort_mesh_is_finished(meshes[i]) == 0;
        if (!any) break;
        px.resize(n);
        res.resize(n);
        uint64_t k = 0;
        for (uint32_t i = 0; i < n_images; ++i) {
            if (foort_mesh_is_finished(meshes[i])) continue;
            if ((rc = foort_mesh_get_pixels(meshes[i], i, px.data() + k))) return rc;
            k += count[i];
        }
        rc = foort_gpu_integrate(ctx, px.data(), n, res.data());
        if (rc != FOORT_OK) return rc;
        // GeodesicPosition: a second pass records the positions (foort_gpu_positions)
        std::vector<uint64_t> counts, first;
        std::vector<double> points;
        if (geopos) {
            counts.resize(n);
            first.resize(n);
            uint64_t total = 0;
            if ((rc = foort_gpu_positions(ctx, px.data(), n, res.data(), counts.data(), nullptr, 0, &total))) return rc;
            points.resize(4 * std::max<uint64_t>(total, 1));
            if ((rc = foort_gpu_positions(ctx, px.data(), n, res.data(), counts.data(), points.data(), total, &total)))
                return rc;
            uint64_t s = 0;
            for (uint64_t g = 0; g < n; ++g) {
                first[g] = s;
                s += counts[g];
            }
        }
        k = 0;
        for (uint32_t i = 0; i < n_images; ++i) {
            if (foort_mesh_is_finished(meshes[i])) continue;
            if (value_first == FOORT_DIAG_GEODESIC_POSITION) {
                // getFinalDataVal: (theta, phi) of the last kept position (Diagnostics.cpp:304-309)
                for (uint64_t g = 0; g < count[i]; ++g) {
                    const uint64_t q = k + g;
                    double v[2] = {res[q].pos[2], res[q].pos[3]};
                    if (counts[q]) {
                        v[0] = points[4 * (first[q] + counts[q] - 1) + 2];
                        v[1] = points[4 * (first[q] + counts[q] - 1) + 3];
                    }
                    if ((rc = foort_mesh_geodesic_finished(meshes[i], g, v, 2))) return rc;
                }
            } else if ((rc = foort_mesh_set_results(meshes[i], res.data() + k, count[i]))) {
                return rc;
            }
            if (outputs && outputs[i]) {
                rc = geopos ? foort_output_round_positions(outputs[i], px.data() + k, res.data() + k, count[i],
                                                           counts.data() + k, points.data() + 4 * (k < n ? first[k] : 0))
                            : foort_output_round(outputs[i], px.data() + k, res.data() + k, count[i]);
                if (rc) return rc;
            }
            if ((rc = foort_mesh_end_current_loop(meshes[i]))) return rc;
            k += count[i];
        }
        total += n;
        ++n_rounds;
    }
    if (outputs)
        for (uint32_t i = 0; i < n_images; ++i)
            if (outputs[i] && (rc = foort_output_finish(outputs[i]))) return rc;
    if (geodesics) *geodesics = total;
    if (rounds) *rounds = n_rounds;
    return FOORT_OK;
}
