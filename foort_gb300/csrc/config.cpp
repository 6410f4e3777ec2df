// FOORT configuration files (.cfg) into engine descriptors.
//
// The reference reads its settings with libconfig (Main.cpp:161-200, Config.cpp:94-1155).
// This file has its own reader for the libconfig syntax those files use and the
// reference's interpretation of the settings:
//
// * Syntax (libconfig's grammar): `name = value` or `name : value`, optional `;` / `,`
//   after a setting, groups `{ ... }`, lists `( ... )`, arrays `[ ... ]`, comments `#`,
//   `//`, `/* */`; values are booleans (true / false, any case), integers (decimal or
//   0x hex, `L` suffix or too large for 32 bits: 64-bit), floats (with a point or an
//   exponent) and strings ("..." with escapes; adjacent strings are joined).
//   `@include` is not supported.
// * Typed lookups as libconfig's Setting::lookupValue does them without automatic
//   conversion: a double setting must be written as a float (`a = 1;` is an integer and
//   is not found, so the default stays), a bool as a boolean, a string as a string; the
//   reference reads counts as a 64-bit integer, else as an unsigned int (negative values
//   become 0), Config.cpp:45-90.
// * The reference's defaults, fallbacks and choices per section: metric names matched in
//   lower case (Config.cpp:137-330), diagnostics with their UseForMesh choice of the
//   value diagnostic and FourColorScreen fallback (:405-620), terminations with Horizon
//   only for metrics with a horizon and BoundarySphere + TimeOut as fallback (:628-800),
//   view screen (:800-870), meshes (:874-1000), integrator (:1002-1090) and output
//   (:1094-1155).
#include <algorithm>
#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <fstream>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/foort_gpu.h"

namespace {

// ---- a libconfig document ---------------------------------------------------------------
struct Node {
    enum Type { Group, List, Array, Int, Int64, Float, Bool, String } type = Group;
    std::string name;
    long long i = 0;
    double f = 0.0;
    bool b = false;
    std::string s;
    std::vector<std::unique_ptr<Node>> kids;

    const Node* get(const char* n) const {
        for (const auto& k : kids)
            if (k->name == n) return k.get();
        return nullptr;
    }
};

struct Parser {
    const std::string& t;
    size_t p = 0;
    int line = 1;
    std::string err;

    explicit Parser(const std::string& text) : t(text) {}

    bool fail(const std::string& m) {
        if (err.empty()) err = "line " + std::to_string(line) + ": " + m;
        return false;
    }

    void skip() {
        for (;;) {
            while (p < t.size() && std::isspace(static_cast<unsigned char>(t[p]))) {
                if (t[p] == '\n') ++line;
                ++p;
            }
            if (p < t.size() && t[p] == '#') {
                while (p < t.size() && t[p] != '\n') ++p;
            } else if (p + 1 < t.size() && t[p] == '/' && t[p + 1] == '/') {
                while (p < t.size() && t[p] != '\n') ++p;
            } else if (p + 1 < t.size() && t[p] == '/' && t[p + 1] == '*') {
                p += 2;
                while (p + 1 < t.size() && !(t[p] == '*' && t[p + 1] == '/')) {
                    if (t[p] == '\n') ++line;
                    ++p;
                }
                p = std::min(t.size(), p + 2);
            } else {
                return;
            }
        }
    }

    static bool name_start(char c) { return std::isalpha(static_cast<unsigned char>(c)) || c == '*'; }
    static bool name_char(char c) {
        return std::isalnum(static_cast<unsigned char>(c)) || c == '-' || c == '_' || c == '*';
    }

    // settings until `close` (0: end of text)
    bool settings(Node& g, char close) {
        for (;;) {
            skip();
            if (p >= t.size()) return close == 0 ? true : fail("unexpected end of file");
            if (t[p] == close) {
                ++p;
                return true;
            }
            if (t[p] == '@') return fail("@include is not supported");
            if (!name_start(t[p])) return fail(std::string("unexpected '") + t[p] + "'");
            const size_t a = p;
            while (p < t.size() && name_char(t[p])) ++p;
            auto n = std::make_unique<Node>();
            n->name = t.substr(a, p - a);
            if (g.get(n->name.c_str())) return fail("duplicate setting name " + n->name);
            skip();
            if (p >= t.size() || (t[p] != '=' && t[p] != ':')) return fail("expected '=' or ':' after " + n->name);
            ++p;
            if (!value(*n)) return false;
            skip();
            if (p < t.size() && (t[p] == ';' || t[p] == ',')) ++p;
            g.kids.push_back(std::move(n));
        }
    }

    bool value(Node& n) {
        skip();
        if (p >= t.size()) return fail("missing value");
        const char c = t[p];
        if (c == '{') {
            ++p;
            n.type = Node::Group;
            return settings(n, '}');
        }
        if (c == '(' || c == '[') {
            ++p;
            n.type = (c == '(') ? Node::List : Node::Array;
            const char close = (c == '(') ? ')' : ']';
            for (;;) {
                skip();
                if (p < t.size() && t[p] == close) {
                    ++p;
                    return true;
                }
                auto k = std::make_unique<Node>();
                if (!value(*k)) return false;
                n.kids.push_back(std::move(k));
                skip();
                if (p < t.size() && t[p] == ',') ++p;
            }
        }
        if (c == '"') {
            n.type = Node::String;
            while (p < t.size() && t[p] == '"') {
                ++p;
                while (p < t.size() && t[p] != '"') {
                    char ch = t[p++];
                    if (ch == '\\' && p < t.size()) {
                        const char e = t[p++];
                        switch (e) {
                        case 'n': ch = '\n'; break;
                        case 't': ch = '\t'; break;
                        case 'r': ch = '\r'; break;
                        case 'f': ch = '\f'; break;
                        case 'x': {
                            if (p + 2 > t.size()) return fail("bad \\x escape");
                            ch = static_cast<char>(std::strtol(t.substr(p, 2).c_str(), nullptr, 16));
                            p += 2;
                            break;
                        }
                        default: ch = e;
                        }
                    }
                    n.s += ch;
                }
                if (p >= t.size()) return fail("unterminated string");
                ++p;
                skip();
            }
            return true;
        }
        // a word: boolean or number
        const size_t a = p;
        while (p < t.size() && (std::isalnum(static_cast<unsigned char>(t[p])) || t[p] == '.' || t[p] == '-' ||
                                t[p] == '+'))
            ++p;
        std::string w = t.substr(a, p - a);
        std::string lw = w;
        for (char& ch : lw) ch = static_cast<char>(std::tolower(static_cast<unsigned char>(ch)));
        if (lw == "true" || lw == "false") {
            n.type = Node::Bool;
            n.b = lw == "true";
            return true;
        }
        if (w.empty()) return fail("missing value");
        const bool hex = lw.size() > 2 && (lw.rfind("0x", 0) == 0 || lw.rfind("-0x", 0) == 0 || lw.rfind("+0x", 0) == 0);
        bool is_float = !hex && (lw.find('.') != std::string::npos || lw.find('e') != std::string::npos);
        if (is_float) {
            char* end = nullptr;
            n.f = std::strtod(w.c_str(), &end);
            if (end == w.c_str() || *end) return fail("bad number " + w);
            n.type = Node::Float;
            return true;
        }
        bool longsuf = false;
        while (!lw.empty() && lw.back() == 'l') {
            lw.pop_back();
            longsuf = true;
        }
        char* end = nullptr;
        errno = 0;
        const long long v = std::strtoll(lw.c_str(), &end, hex ? 16 : 10);
        if (end == lw.c_str() || *end || errno) return fail("bad number " + w);
        n.i = v;
        n.type = (longsuf || v > 2147483647LL || v < -2147483648LL) ? Node::Int64 : Node::Int;
        return true;
    }
};

// Setting::lookupValue without automatic conversion
bool get_double(const Node* g, const char* n, double& v) {
    const Node* x = g ? g->get(n) : nullptr;
    if (!x || x->type != Node::Float) return false;
    v = x->f;
    return true;
}
bool get_bool(const Node* g, const char* n, bool& v) {
    const Node* x = g ? g->get(n) : nullptr;
    if (!x || x->type != Node::Bool) return false;
    v = x->b;
    return true;
}
bool get_string(const Node* g, const char* n, std::string& v) {
    const Node* x = g ? g->get(n) : nullptr;
    if (!x || x->type != Node::String) return false;
    v = x->s;
    return true;
}
bool get_int(const Node* g, const char* n, int& v) {
    const Node* x = g ? g->get(n) : nullptr;
    if (!x || x->type != Node::Int) return false;
    v = static_cast<int>(x->i);
    return true;
}
// Config::lookupValuelargecounter (Config.cpp:45-90): as a 64-bit integer, else as an
// unsigned int (libconfig clamps a negative int to 0).
bool get_count(const Node* g, const char* n, uint64_t& v) {
    const Node* x = g ? g->get(n) : nullptr;
    if (!x) return false;
    if (x->type == Node::Int64) {
        v = static_cast<uint64_t>(x->i);
        return true;
    }
    if (x->type == Node::Int) {
        v = x->i < 0 ? 0u : static_cast<uint64_t>(x->i);
        return true;
    }
    return false;
}

std::string lower(std::string s) {
    for (char& c : s) c = static_cast<char>(std::tolower(static_cast<unsigned char>(c)));
    return s;
}

constexpr double kRefPi = 3.1415926535;  // Geometry.h:44
constexpr uint64_t kCounterMax = ~0ull;   // LARGECOUNTER_MAX

struct Notes {
    std::string text;
    void add(const std::string& s) { text += s + "\n"; }
};

void set_update(foort_update_freq& u, const Node* g, bool start_default, bool finish_default) {
    uint64_t every = 1;
    bool start = start_default, finish = finish_default;
    get_count(g, "UpdateFrequency", every);
    if (every == 0) {
        get_bool(g, "UpdateStart", start);
        get_bool(g, "UpdateFinish", finish);
    }
    u.every_n = every;
    u.at_start = start ? 1 : 0;
    u.at_finish = finish ? 1 : 0;
}

void interpret(const Node& root, foort_config& c, Notes& notes) {
    foort_run_desc& d = c.run;
    foort_image_desc& im = c.image;
    // ---- Metric (Config.cpp:132-330)
    d.metric_id = FOORT_METRIC_KERR;
    im.metric_params[0] = 0.5;
    d.rlog = 0;
    {
        const Node* m = root.get("Metric");
        std::string name;
        if (!m || !get_string(m, "Name", name)) {
            notes.add("No metric settings found. Using default metric (Kerr with a = 0.5).");
        } else {
            name = lower(name);
            bool rlog = false;
            double* p = im.metric_params;
            auto param = [&](const char* key, double def, int i) {
                p[i] = def;
                if (!get_double(m, key, p[i])) notes.add(std::string("Metric: no value for ") + key + " given; default used.");
            };
            if (name == "kerr") {
                d.metric_id = FOORT_METRIC_KERR;
                param("a", 0.5, 0);
                get_bool(m, "RLogScale", rlog);
            } else if (name == "flatspace") {
                d.metric_id = FOORT_METRIC_FLAT;
                p[0] = 0.0;
            } else if (name == "rasheedlarsen" || name == "rasheed-larsen") {
                d.metric_id = FOORT_METRIC_RASHEED_LARSEN;
                param("m", 1.0, 0);
                param("a", 0.5, 1);
                param("p", 2.0, 2);
                param("q", 2.0, 3);
                get_bool(m, "RLogScale", rlog);
            } else if (name == "johannsen") {
                d.metric_id = FOORT_METRIC_JOHANNSEN;
                param("a", 0.7, 0);
                param("alpha13", 2.0, 1);
                param("alpha22", 0.0, 2);
                param("alpha52", 0.0, 3);
                param("epsilon3", 0.0, 4);
                get_bool(m, "RLogScale", rlog);
            } else if (name == "mankonovikov" || name == "manko-novikov") {
                d.metric_id = FOORT_METRIC_MANKO_NOVIKOV;
                param("a", 0.0, 0);
                param("alpha3", 5.0, 1);
                get_bool(m, "RLogScale", rlog);
            } else {
                notes.add("No metric settings found. Using default metric (Kerr with a = 0.5).");
            }
            d.rlog = rlog ? 1 : 0;
        }
    }
    const bool has_horizon = d.metric_id != FOORT_METRIC_FLAT;  // SphericalHorizonMetric
    // ---- Source (Config.cpp:333-400): only NoSource exists
    // ---- Diagnostics (Config.cpp:402-620)
    d.diag_flags = 0;
    d.value_diag = 0;
    d.equat_freq = foort_update_freq{1, 1, 1};
    d.equat_threshold = 0.01;
    d.closest_freq = foort_update_freq{1, 1, 1};
    d.geopos_freq = foort_update_freq{1, 0, 1};
    d.geopos_output_steps = 0;
    {
        const Node* ds = root.get("Diagnostics");
        bool ok = ds != nullptr;
        if (ok) {
            auto on = [&](const char* n) {
                const Node* g = ds->get(n);
                bool v = false;
                return g && get_bool(g, "On", v) && v;
            };
            auto use_for_mesh = [&](const char* n, uint32_t flag) {
                bool v = false;
                if (d.value_diag == 0 && get_bool(ds->get(n), "UseForMesh", v) && v) d.value_diag = flag;
            };
            if (on("FourColorScreen")) {
                d.diag_flags |= FOORT_DIAG_FOUR_COLOR_SCREEN;
                use_for_mesh("FourColorScreen", FOORT_DIAG_FOUR_COLOR_SCREEN);
            }
            if (on("GeodesicPosition")) {
                const Node* g = ds->get("GeodesicPosition");
                d.diag_flags |= FOORT_DIAG_GEODESIC_POSITION;
                set_update(d.geopos_freq, g, false, true);
                get_count(g, "OutputSteps", d.geopos_output_steps);
                use_for_mesh("GeodesicPosition", FOORT_DIAG_GEODESIC_POSITION);
            }
            if (on("EquatorialPasses")) {
                const Node* g = ds->get("EquatorialPasses");
                d.diag_flags |= FOORT_DIAG_EQUATORIAL_PASSES;
                set_update(d.equat_freq, g, true, true);
                get_double(g, "Threshold", d.equat_threshold);
                use_for_mesh("EquatorialPasses", FOORT_DIAG_EQUATORIAL_PASSES);
            }
            if (on("ClosestRadius")) {
                const Node* g = ds->get("ClosestRadius");
                d.diag_flags |= FOORT_DIAG_CLOSEST_RADIUS;
                set_update(d.closest_freq, g, true, true);
                use_for_mesh("ClosestRadius", FOORT_DIAG_CLOSEST_RADIUS);
            }
            if (d.diag_flags == 0) ok = false;
            if (ok && d.value_diag == 0) {
                if (d.diag_flags & FOORT_DIAG_FOUR_COLOR_SCREEN) {
                    notes.add("No mesh diagnostic set; using FourColorScreen.");
                    d.value_diag = FOORT_DIAG_FOUR_COLOR_SCREEN;
                } else {
                    ok = false;
                }
            }
        }
        if (!ok) {
            notes.add("Diagnostics not usable. Using default diagnostic(s) (FourColorScreen).");
            d.diag_flags = FOORT_DIAG_FOUR_COLOR_SCREEN;
            d.value_diag = FOORT_DIAG_FOUR_COLOR_SCREEN;
        }
    }
    // ---- Terminations (Config.cpp:623-800)
    d.term_flags = 0;
    d.horizon_eps = 0.01;
    d.horizon_every = 1;
    d.boundary_radius = 1000.0;
    d.boundary_every = 1;
    d.timeout_max_steps = 10000;
    d.timeout_every = 1;
    d.theta_eps = 1e-5;
    d.theta_every = 1;
    {
        const Node* ts = root.get("Terminations");
        auto on = [&](const char* n) {
            const Node* g = ts ? ts->get(n) : nullptr;
            bool v = false;
            return g && get_bool(g, "On", v) && v;
        };
        if (ts) {
            if (on("Horizon")) {
                if (!has_horizon) {
                    notes.add("Horizon Termination turned on but metric does not have horizon! Turning off Horizon Termination.");
                } else {
                    const Node* g = ts->get("Horizon");
                    d.term_flags |= FOORT_TERM_HORIZON;
                    get_double(g, "Epsilon_Horizon", d.horizon_eps);
                    get_count(g, "UpdateFrequency", d.horizon_every);
                }
            }
            if (on("BoundarySphere")) {
                const Node* g = ts->get("BoundarySphere");
                d.term_flags |= FOORT_TERM_BOUNDARY_SPHERE;
                get_double(g, "SphereRadius", d.boundary_radius);
                get_count(g, "UpdateFrequency", d.boundary_every);
            }
            if (on("TimeOut")) {
                const Node* g = ts->get("TimeOut");
                d.term_flags |= FOORT_TERM_TIMEOUT;
                get_count(g, "MaxSteps", d.timeout_max_steps);
                get_count(g, "UpdateFrequency", d.timeout_every);
            }
            if (on("ThetaSingularity")) {
                const Node* g = ts->get("ThetaSingularity");
                d.term_flags |= FOORT_TERM_THETA_SINGULARITY;
                get_double(g, "Epsilon", d.theta_eps);
                get_count(g, "UpdateFrequency", d.theta_every);
            }
        }
        if (d.term_flags == 0) {
            notes.add("No terminations turned on. Using default termination(s) (BoundarySphere and TimeOut).");
            d.term_flags = FOORT_TERM_BOUNDARY_SPHERE | FOORT_TERM_TIMEOUT;
            d.boundary_radius = 1000.0;
            d.boundary_every = 1;
            d.timeout_max_steps = 10000;
            d.timeout_every = 1;
        }
    }
    // ---- ViewScreen (Config.cpp:800-870)
    const double pos0[4] = {0.0, 1000.0, kRefPi / 2.0, 0.0};
    const double dir0[4] = {0.0, -1.0, 0.0, 0.0};
    for (int i = 0; i < 4; ++i) {
        im.cam_pos[i] = pos0[i];
        im.cam_dir[i] = dir0[i];
    }
    im.screen_size[0] = im.screen_size[1] = 10.0;
    im.screen_center[0] = im.screen_center[1] = 0.0;
    im.horizon_eps = 0.0;
    const Node* vs = root.get("ViewScreen");
    if (!vs) {
        notes.add("No view screen settings found. Using default ViewScreen Settings.");
    } else {
        const char* coords[4] = {"t", "r", "theta", "phi"};
        if (const Node* g = vs->get("Position"))
            for (int i = 0; i < 4; ++i) get_double(g, coords[i], im.cam_pos[i]);
        if (const Node* g = vs->get("Direction"))
            for (int i = 0; i < 4; ++i) get_double(g, coords[i], im.cam_dir[i]);
        if (const Node* g = vs->get("ScreenSize")) {
            get_double(g, "x", im.screen_size[0]);
            get_double(g, "y", im.screen_size[1]);
        }
        if (const Node* g = vs->get("ScreenCenter")) {
            get_double(g, "x", im.screen_center[0]);
            get_double(g, "y", im.screen_center[1]);
        }
    }
    // ---- Mesh (Config.cpp:874-1000)
    c.mesh_kind = FOORT_CONFIG_MESH_SIMPLE;
    c.total_pixels = 100 * 100;
    {
        const Node* ms = vs ? vs->get("Mesh") : nullptr;
        std::string type;
        if (!ms || !get_string(ms, "Type", type)) {
            notes.add("No Mesh settings found. Using default (SimpleSquareMesh with 100x100 pixels).");
        } else if (type == "SimpleSquareMesh" || type == "InputCertainPixelsMesh") {
            c.mesh_kind = type == "SimpleSquareMesh" ? FOORT_CONFIG_MESH_SIMPLE : FOORT_CONFIG_MESH_INPUT_PIXELS;
            get_count(ms, "TotalPixels", c.total_pixels);
        } else if (type == "SquareSubdivisionMesh" || type == "SquareSubdivisionMeshV2") {
            c.mesh_kind = type == "SquareSubdivisionMesh" ? FOORT_CONFIG_MESH_SUBDIVISION : FOORT_CONFIG_MESH_SUBDIVISION_V2;
            c.initial_pixels = 100;
            c.max_pixels = 100;
            c.iteration_pixels = 100;
            int maxsub = 1;
            bool to_final = false;
            get_count(ms, "InitialPixels", c.initial_pixels);
            get_count(ms, "MaxPixels", c.max_pixels);
            get_count(ms, "IterationPixels", c.iteration_pixels);
            get_int(ms, "MaxSubdivide", maxsub);
            if (c.max_pixels < c.initial_pixels) c.max_pixels = c.initial_pixels;
            if (maxsub < 1) {
                notes.add("Invalid MaxSubdivide level given. Using MaxSubdivide = 1.");
                maxsub = 1;
            }
            get_bool(ms, "InitialSubdivisionToFinal", to_final);
            c.max_subdivide = maxsub;
            c.initial_sub_to_final = to_final ? 1 : 0;
        } else {
            notes.add("Incorrect Mesh Type specified. Using default (SimpleSquareMesh with 100x100 pixels).");
        }
    }
    // ---- Integrator (Config.cpp:1002-1090); step sizes are read before the type
    d.integrator_id = FOORT_INTEGRATOR_RK4;
    d.epsilon = 0.03;
    d.derivative_h = 1e-7;
    d.smallest_step = 1e-12;
    d.verlet_tol = 0.001;
    {
        const Node* is = root.get("Integrator");
        std::string type;
        if (!is) {
            notes.add("No integrator settings found. Using default integrator (RK4 integrator).");
        } else {
            get_double(is, "StepSize", d.epsilon);
            get_double(is, "DerivativeH", d.derivative_h);
            get_double(is, "SmallestPossibleStepsize", d.smallest_step);
            if (!get_string(is, "Type", type)) {
                notes.add("No integrator settings found. Using default integrator (RK4 integrator).");
            } else if (lower(type) == "rk4") {
                d.integrator_id = FOORT_INTEGRATOR_RK4;
            } else if (lower(type) == "verlet") {
                d.integrator_id = FOORT_INTEGRATOR_VERLET;
                get_double(is, "VerletVelocityTolerance", d.verlet_tol);
            } else {
                notes.add("No integrator settings found. Using default integrator (RK4 integrator).");
            }
        }
    }
    // ---- Output (Config.cpp:94-116, :1094-1155)
    c.file_prefix[0] = c.file_extension[0] = '\0';
    c.timestamp = 1;
    c.outputs_to_cache = kCounterMax - 1;
    c.geodesics_per_file = kCounterMax;
    c.first_line_info = 1;
    c.screen_output_level = 4;
    c.loop_message_frequency = kCounterMax;
    const Node* os = root.get("Output");
    if (os) {
        int lvl = 4;
        get_int(os, "ScreenOutputLevel", lvl);
        c.screen_output_level = std::max(0, std::min(lvl, 4));
        get_count(os, "LoopMessageFrequency", c.loop_message_frequency);
    }
    std::string prefix;
    if (!os || !get_string(os, "FilePrefix", prefix)) {
        notes.add("No output file name prefix found. Will do all output to console.");
    } else {
        std::string ext;
        get_string(os, "FileExtension", ext);
        bool ts = true, first = true;
        get_bool(os, "TimeStamp", ts);
        get_count(os, "GeodesicsToCache", c.outputs_to_cache);
        get_count(os, "GeodesicsPerFile", c.geodesics_per_file);
        if (c.geodesics_per_file == 0) c.geodesics_per_file = kCounterMax;
        get_bool(os, "FirstLineInfo", first);
        std::snprintf(c.file_prefix, sizeof(c.file_prefix), "%s", prefix.c_str());
        std::snprintf(c.file_extension, sizeof(c.file_extension), "%s", ext.c_str());
        c.timestamp = ts ? 1 : 0;
        c.first_line_info = first ? 1 : 0;
    }
    d.n_images = 1;
    d.images = nullptr;  // the caller points it at c.image
}

int parse_into(const std::string& text, foort_config* out, char* notes, uint64_t cap) {
    if (!out) return FOORT_E_BADARG;
    Node root;
    Parser ps(text);
    if (!ps.settings(root, 0)) {
        if (notes && cap) std::snprintf(notes, cap, "parse error: %s", ps.err.c_str());
        return FOORT_E_BADARG;
    }
    std::memset(out, 0, sizeof(*out));
    foort_gpu_default_desc(&out->run);
    Notes n;
    interpret(root, *out, n);
    if (notes && cap) std::snprintf(notes, cap, "%s", n.text.c_str());
    return FOORT_OK;
}

}  // namespace

extern "C" {

int foort_config_parse(const char* text, foort_config* out, char* notes, uint64_t cap) {
    if (!text) return FOORT_E_BADARG;
    return parse_into(std::string(text), out, notes, cap);
}

int foort_config_load(const char* path, foort_config* out, char* notes, uint64_t cap) {
    if (!path) return FOORT_E_BADARG;
    std::ifstream f(path, std::ios::binary);
    if (!f) {
        if (notes && cap) std::snprintf(notes, cap, "cannot read %s", path);
        return FOORT_E_IO;
    }
    std::stringstream ss;
    ss << f.rdbuf();
    return parse_into(ss.str(), out, notes, cap);
}

int foort_config_create_mesh(const foort_config* c, foort_mesh** out) {
    if (!c || !out) return FOORT_E_BADARG;
    switch (c->mesh_kind) {
    case FOORT_CONFIG_MESH_SIMPLE:
        return foort_mesh_create_simple(c->total_pixels, c->run.diag_flags, c->run.value_diag, out);
    case FOORT_CONFIG_MESH_SUBDIVISION_V2:
        return foort_mesh_create_v2(c->max_pixels, c->initial_pixels, c->max_subdivide, c->iteration_pixels,
                                    c->initial_sub_to_final, c->run.diag_flags, c->run.value_diag, out);
    default:
        return FOORT_E_UNSUPPORTED;  // SquareSubdivisionMesh (V1), InputCertainPixelsMesh
    }
}

// Utilities::GetTimeStampString (Utilities.cpp:28-36): local time as %y%m%d-%H%M%S.
int foort_timestamp_string(char* buf, uint64_t cap) {
    if (!buf || cap < 14) return FOORT_E_BADARG;
    const std::time_t t = std::time(nullptr);
    std::tm tm{};
    localtime_r(&t, &tm);
    return std::strftime(buf, cap, "%y%m%d-%H%M%S", &tm) ? FOORT_OK : FOORT_E_BADARG;
}

}  // extern "C"
