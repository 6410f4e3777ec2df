// Output files of a run, byte for byte as FOORT writes them.
//
// The first line of every file (Utilities::GetFirstLineInfoString, Utilities.cpp:52-84)
// describes the metric, source, diagnostics, terminations, view screen, mesh and
// integrator with the reference's wording and number formats (std::to_string is "%f",
// the integrator's constants are std::scientific, i.e. "%e"). The data lines are
// "row col " + " " + the diagnostic's string (Geodesic.cpp:111-139,
// InputOutput.cpp:196-200), one file per diagnostic in the order of the diagnostic vector,
// named prefix_[timestamp_]Name[_n].ext (InputOutput.cpp:271-299). Outputs are cached and
// written when the cache would overflow and at the end, split over files of at most
// geodesics_per_file lines (GeodesicOutputHandler::WriteCachedOutputToFile,
// InputOutput.cpp:129-269), so that caching and splitting give the reference's files.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <string>
#include <thread>
#include <vector>

#include "../../include/foort_gpu.h"
#include "diag_order.h"

namespace {

std::string f6(double x) {  // std::to_string(double)
    char b[512];
    std::snprintf(b, sizeof(b), "%f", x);
    return b;
}

std::string e6(double x) {  // std::stringstream << std::scientific
    char b[64];
    std::snprintf(b, sizeof(b), "%e", x);
    return b;
}

const char* diag_name(uint32_t f) {  // Diagnostic::getNameStr
    switch (f) {
    case FOORT_DIAG_FOUR_COLOR_SCREEN: return "FourColorScreen";
    case FOORT_DIAG_GEODESIC_POSITION: return "GeodesicPosition";
    case FOORT_DIAG_EQUATORIAL_PASSES: return "EquatPasses";
    case FOORT_DIAG_CLOSEST_RADIUS: return "ClosestRadius";
    default: return "";
    }
}

// Metric::getFullDescriptionStr (Metric.cpp:194-196, 232-234, 364-368, 476-480, 629-632)
std::string metric_description(int32_t id, const double* p, bool rlog) {
    const std::string coord = rlog ? "using logarithmic r coord" : "using normal r coord";
    switch (id) {
    case FOORT_METRIC_KERR: return "Kerr (a = " + f6(p[0]) + ", " + coord + ")";
    case FOORT_METRIC_FLAT: return "Flat space";
    case FOORT_METRIC_RASHEED_LARSEN:
        return "Rasheed-Larsen (m = " + f6(p[0]) + ", a = " + f6(p[1]) + ", p = " + f6(p[2]) + ", q = " + f6(p[3]) +
               ", " + coord + ")";
    case FOORT_METRIC_JOHANNSEN:
        return "Johannsen (a = " + f6(p[0]) + ", alpha13 = " + f6(p[1]) + ", alpha22 = " + f6(p[2]) +
               ", alpha52 = " + f6(p[3]) + ", epsilon3 = " + f6(p[4]) + ", " + coord + ")";
    case FOORT_METRIC_MANKO_NOVIKOV: return "Manko-Novikov (a = " + f6(p[0]) + ", alpha3 = " + f6(p[1]) + ", " + coord + ")";
    default: return "";
    }
}

// Diagnostic::getFullDescriptionStr (Diagnostics.cpp:229-232, 330-334, 409-412, 472-475)
std::string diag_description(uint32_t f, const foort_run_desc& d) {
    switch (f) {
    case FOORT_DIAG_FOUR_COLOR_SCREEN: return "Four-color screen";
    case FOORT_DIAG_GEODESIC_POSITION:
        return "Geodesic position (output " + std::to_string(d.geopos_output_steps) + " steps, updates every " +
               std::to_string(d.geopos_freq.every_n) + " steps)";
    case FOORT_DIAG_EQUATORIAL_PASSES: return "Equatorial passes (threshold = " + f6(d.equat_threshold) + ")";
    case FOORT_DIAG_CLOSEST_RADIUS: return "Closest radius";
    default: return "";
    }
}

std::string first_line(const foort_run_desc& d, uint32_t image, const std::string& mesh_desc) {
    const foort_image_desc& im = d.images[image];
    const bool flat = d.metric_id == FOORT_METRIC_FLAT;
    std::string diags = "Diagnostics: ";
    for (uint32_t f : foort::diagnostic_order(d.diag_flags, d.value_diag)) diags += diag_description(f, d) + ", ";
    // CreateTerminationVector order (Terminations.cpp:22-40); flat space gets no Horizon
    // termination (Config.cpp:649-657). Terminations.cpp:119-219 for the wording.
    std::string terms = "Terminations: ";
    const double heps = im.horizon_eps > 0.0 ? im.horizon_eps : d.horizon_eps;
    if ((d.term_flags & FOORT_TERM_HORIZON) && !flat) terms += "Horizon (stop at " + f6(1 + heps) + "x(horizon radius)), ";
    if (d.term_flags & FOORT_TERM_BOUNDARY_SPHERE) terms += "Boundary sphere (R = " + f6(d.boundary_radius) + "), ";
    if (d.term_flags & FOORT_TERM_TIMEOUT)
        terms += "Time out (max integration steps: " + std::to_string(d.timeout_max_steps) + "), ";
    if (d.term_flags & FOORT_TERM_THETA_SINGULARITY) terms += "Theta singularity (epsilon: " + f6(d.theta_eps) + "), ";
    // ViewScreen::getFullDescriptionStr (ViewScreen.cpp:214-218) with toString of the
    // position and screen size (Geometry.h:100-115)
    const std::string view = "ViewScreen position: (" + f6(im.cam_pos[0]) + ", " + f6(im.cam_pos[1]) + ", " +
                             f6(im.cam_pos[2]) + ", " + f6(im.cam_pos[3]) + "), screen size: (" + f6(im.screen_size[0]) +
                             ", " + f6(im.screen_size[1]) + "), " + mesh_desc;
    // Integrators::GetFullIntegratorDescription (Integrators.cpp:11-31)
    std::string integ = "Integrator: ";
    if (d.integrator_id == FOORT_INTEGRATOR_VERLET)
        integ += "Verlet (velocity tolerance: " + e6(d.verlet_tol) + ")";
    else
        integ += "RK4";
    integ += ", basic step size: " + e6(d.epsilon) + ", min. step size: " + e6(d.smallest_step) +
             ", derivative h: " + e6(d.derivative_h);
    return "Metric: " + metric_description(d.metric_id, im.metric_params, d.rlog != 0 && !flat) + "; " +
           "Source: No source; " + diags + "; " + terms + "; " + view + "; " + integ;
}

}  // namespace

struct foort_output {
    std::string prefix, timestamp, extension, first;
    std::vector<uint32_t> diags;
    uint64_t cache_max = 0, per_file = 0;
    // cached outputs: per diagnostic one text block, and where each geodesic's line starts
    std::vector<std::string> text;
    std::vector<std::vector<uint64_t>> starts;
    uint64_t cached = 0;
    uint64_t full_files = 0, in_file = 0;  // m_CurrentFullFiles, m_CurrentGeodesicsInFile

    std::string file_name(size_t diag, uint64_t filenr) const {  // InputOutput.cpp:271-299
        std::string s = prefix + "_";
        if (!timestamp.empty()) s += timestamp + "_";
        s += diag_name(diags[diag]);
        if (filenr > 1) s += "_" + std::to_string(filenr);
        if (!extension.empty()) s += "." + extension;
        return s;
    }

    bool open_first(const std::string& name) const {  // InputOutput.cpp:301-330
        const auto pos = name.find_last_of('/');
        if (pos != std::string::npos) {
            std::error_code ec;
            std::filesystem::create_directories(name.substr(0, pos), ec);
        }
        std::ofstream f(name, std::ios::out | std::ios::trunc | std::ios::binary);
        if (!f) return false;
        if (!first.empty()) f << first << "\n";
        return static_cast<bool>(f);
    }

    // Lines [a, b) of the cache for diagnostic k, appended to file `name`.
    bool append(const std::string& name, size_t k, uint64_t a, uint64_t b) const {
        std::ofstream f(name, std::ios::out | std::ios::app | std::ios::binary);
        if (!f) return false;
        const uint64_t lo = starts[k][a], hi = (b < cached) ? starts[k][b] : text[k].size();
        f.write(text[k].data() + lo, static_cast<std::streamsize>(hi - lo));
        return static_cast<bool>(f);
    }

    // WriteCachedOutputToFile (InputOutput.cpp:129-269)
    int flush() {
        if (cached == 0) return FOORT_OK;
        uint64_t nrfiles = 1;
        while (in_file + cached > nrfiles * per_file) ++nrfiles;
        uint64_t curfile = 1, curgeod = 0, lastcount = 0;
        if (in_file == 0)
            for (size_t k = 0; k < diags.size(); ++k)
                if (!open_first(file_name(k, full_files + curfile))) return FOORT_E_IO;
        while (curfile <= nrfiles) {
            const uint64_t loopmax = (curfile == 1) ? std::min(cached, per_file - in_file)
                                                    : std::min(cached - curgeod, per_file);
            for (size_t k = 0; k < diags.size(); ++k)
                if (!append(file_name(k, full_files + curfile), k, curgeod, curgeod + loopmax)) return FOORT_E_IO;
            ++curfile;
            if (curfile <= nrfiles) {
                curgeod += loopmax;
                for (size_t k = 0; k < diags.size(); ++k)
                    if (!open_first(file_name(k, full_files + curfile))) return FOORT_E_IO;
            } else {
                lastcount = loopmax;
            }
        }
        full_files += nrfiles - 1;
        if (lastcount == per_file) {
            ++full_files;
            lastcount = 0;
        }
        in_file = (nrfiles == 1) ? in_file + lastcount : lastcount;
        for (size_t k = 0; k < diags.size(); ++k) {
            text[k].clear();
            starts[k].clear();
        }
        cached = 0;
        return FOORT_OK;
    }

    // The lines of geodesics [a, b) of a round for diagnostic k. GeodesicPosition's string
    // is the number of positions, " ;; ", then every coordinate with a space after it
    // (Diagnostics.cpp:286-302).
    static void format(uint32_t diag, const foort_pixel* px, const foort_result* res, const uint64_t* counts,
                       const uint64_t* first, const double* points, uint64_t a, uint64_t b, std::string& out,
                       std::vector<uint64_t>& st, uint64_t base) {
        char line[512];
        for (uint64_t i = a; i < b; ++i) {
            int n;
            const unsigned long long row = px[i].row, col = px[i].col;
            st.push_back(base + out.size());
            switch (diag) {
            case FOORT_DIAG_FOUR_COLOR_SCREEN: n = std::snprintf(line, sizeof(line), "%llu %llu  %d\n", row, col, res[i].quadrant); break;
            case FOORT_DIAG_EQUATORIAL_PASSES: n = std::snprintf(line, sizeof(line), "%llu %llu  %d\n", row, col, res[i].equat_passes); break;
            case FOORT_DIAG_GEODESIC_POSITION: {
                n = std::snprintf(line, sizeof(line), "%llu %llu  %llu ;; ", row, col,
                                  static_cast<unsigned long long>(counts[i]));
                out.append(line, static_cast<size_t>(n));
                const double* p = points + 4 * first[i];
                for (uint64_t k = 0; k < 4 * counts[i]; ++k) {
                    n = std::snprintf(line, sizeof(line), "%f ", p[k]);
                    out.append(line, static_cast<size_t>(n));
                }
                out += '\n';
                continue;
            }
            default: n = std::snprintf(line, sizeof(line), "%llu %llu  %f\n", row, col, res[i].closest_r); break;
            }
            out.append(line, static_cast<size_t>(n));
        }
    }

    // PrepareForOutput + NewGeodesicOutput for a whole round (InputOutput.cpp:95-121)
    int round(const foort_pixel* px, const foort_result* res, uint64_t n, const uint64_t* counts = nullptr,
              const double* points = nullptr) {
        const bool geopos = std::find(diags.begin(), diags.end(), FOORT_DIAG_GEODESIC_POSITION) != diags.end();
        if (geopos && n && (!counts || !points)) return FOORT_E_BADARG;
        std::vector<uint64_t> first;
        if (geopos) {
            first.resize(n);
            uint64_t s = 0;
            for (uint64_t i = 0; i < n; ++i) {
                first[i] = s;
                s += counts[i];
            }
        }
        if (cached + n > cache_max) {
            const int rc = flush();
            if (rc) return rc;
        }
        // large rounds are formatted in parallel chunks, joined in order
        const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
        const uint64_t chunk = 1 << 16;
        const uint64_t nchunks = (n + chunk - 1) / chunk;
        for (size_t k = 0; k < diags.size(); ++k) {
            if (nchunks <= 1 || hw == 1) {
                format(diags[k], px, res, counts, first.data(), points, 0, n, text[k], starts[k], 0);
                continue;
            }
            std::vector<std::string> parts(nchunks);
            std::vector<std::vector<uint64_t>> pst(nchunks);
            std::vector<std::thread> pool;
            const uint64_t nt = std::min<uint64_t>(hw, nchunks);
            for (uint64_t t = 0; t < nt; ++t)
                pool.emplace_back([&, t]() {
                    for (uint64_t c = t; c < nchunks; c += nt)
                        format(diags[k], px, res, counts, first.data(), points, c * chunk, std::min(n, (c + 1) * chunk), parts[c],
                               pst[c], 0);
                });
            for (auto& th : pool) th.join();
            for (uint64_t c = 0; c < nchunks; ++c) {
                const uint64_t base = text[k].size();
                for (uint64_t s : pst[c]) starts[k].push_back(base + s);
                text[k] += parts[c];
            }
        }
        cached += n;
        return FOORT_OK;
    }
};

extern "C" {

int foort_first_line_info(const foort_run_desc* desc, uint32_t image, const foort_mesh* mesh, char* buf, uint64_t cap) {
    if (!desc || !mesh || !buf || cap == 0 || image >= desc->n_images || !desc->images) return FOORT_E_BADARG;
    char mbuf[1024];
    if (foort_mesh_description(mesh, mbuf, sizeof(mbuf))) return FOORT_E_BADARG;
    const std::string s = first_line(*desc, image, mbuf);
    if (s.size() + 1 > cap) return FOORT_E_BADARG;
    std::memcpy(buf, s.c_str(), s.size() + 1);
    return FOORT_OK;
}

int foort_output_create(const foort_output_desc* od, foort_output** out) {
    if (!od || !out || !od->prefix) return FOORT_E_BADARG;
    *out = nullptr;
    // An empty prefix or zero geodesics per file means console output in the reference
    // (InputOutput.cpp:80-82); this writer only writes files.
    if (od->prefix[0] == '\0' || od->geodesics_per_file == 0) return FOORT_E_UNSUPPORTED;
    const std::vector<uint32_t> order = foort::diagnostic_order(od->diag_flags, od->value_diag);
    if (order.empty()) return FOORT_E_BADARG;
    auto* o = new foort_output();
    o->prefix = od->prefix;
    o->timestamp = od->timestamp ? od->timestamp : "";
    o->extension = od->extension ? od->extension : "";
    o->first = od->first_line ? od->first_line : "";
    o->diags = order;
    o->cache_max = od->outputs_to_cache;  // 0: every round is written before the next is cached
    o->per_file = od->geodesics_per_file;
    o->text.resize(order.size());
    o->starts.resize(order.size());
    *out = o;
    return FOORT_OK;
}

int foort_output_round(foort_output* o, const foort_pixel* px, const foort_result* res, uint64_t n) {
    if (!o || (n && (!px || !res))) return FOORT_E_BADARG;
    return o->round(px, res, n);
}

int foort_output_round_positions(foort_output* o, const foort_pixel* px, const foort_result* res, uint64_t n,
                                 const uint64_t* counts, const double* points) {
    if (!o || (n && (!px || !res))) return FOORT_E_BADARG;
    return o->round(px, res, n, counts, points);
}

int foort_output_finish(foort_output* o) {
    if (!o) return FOORT_E_BADARG;
    return o->flush();
}

void foort_output_destroy(foort_output* o) { delete o; }

}  // extern "C"
