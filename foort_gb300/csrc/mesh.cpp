// Host meshes: which pixels each integration round gets (Mesh.h:24-61).
//
// SimpleSquareMesh (Mesh.h:66-106, Mesh.cpp:25-73): one round over an n x n grid.
// SquareSubdivisionMeshV2 (Mesh.h:285-423, Mesh.cpp:660-1186): a seed grid, then rounds
// that subdivide the squares whose corner values differ most. The adaptive mesh is
// integer / index work and must hand out exactly the reference's pixels in the
// reference's order: the data flow below follows Mesh.cpp step for step (the order in
// which pixels enter the queue, the weight-update list and the active list, and the
// std::sort of the active list with the reference's comparator, whose tie order
// depends on that input order).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <deque>
#include <string>
#include <vector>

#include "../../include/foort_gpu.h"
#include "diag_order.h"

namespace {

// Value vector of one geodesic for the mesh: getFinalDataVal() of the FIRST diagnostic
// of the value-first diagnostic vector (Geodesic.cpp:141-149, Diagnostics.cpp:14-99).
// That vector is built in the order FourColor, GeodesicPosition, EquatorialPasses,
// ClosestRadius, and appending the value diagnostic rotates it left by one.
uint32_t first_diagnostic(uint32_t diag_flags, uint32_t value_diag) {
    const std::vector<uint32_t> order = foort::diagnostic_order(diag_flags, value_diag);
    return order.empty() ? 0u : order[0];
}

// A pixel's value vector as the distances read it: its length and its first two entries
// (no distance reads further).
struct Value {
    double v[2] = {0.0, 0.0};
    uint32_t n = 0;
    void set(const double* x, uint32_t len) {
        n = len;
        for (uint32_t i = 0; i < len && i < 2; ++i) v[i] = x[i];
    }
};

// FinalDataValDistance of the value diagnostic (Diagnostics.cpp:214-221, :311-322,
// :395-401, :460-464).
double distance(uint32_t value_diag, const Value& a, const Value& b) {
    if (a.n == 0 || b.n == 0) return 0.0;
    switch (value_diag) {
    case FOORT_DIAG_FOUR_COLOR_SCREEN: return std::fabs(a.v[0] - b.v[0]) < 1.0 ? 0.0 : 1.0;
    case FOORT_DIAG_GEODESIC_POSITION:
        if (a.n != 2 || b.n != 2) return 0.0;
        return std::acos(std::cos(a.v[0]) * std::cos(b.v[0]) +
                         std::sin(a.v[0]) * std::sin(b.v[0]) * std::cos(a.v[1] - b.v[1]));
    case FOORT_DIAG_EQUATORIAL_PASSES: return std::fabs(a.v[0] - b.v[0]);  // pass counts are integers
    default: return std::fabs(a.v[0] - b.v[0]);
    }
}

uint64_t pow2(int e) {
    uint64_t v = 1;
    while (e-- > 0) v *= 2;
    return v;
}

}  // namespace

struct foort_mesh {
    int kind = 0;  // 0 simple, 1 V2
    uint32_t value_diag = 0, diag_flags = 0;
    uint64_t grid = 0;  // m_RowColumnSize
    std::string err;
    virtual ~foort_mesh() = default;
    virtual uint64_t cur() const = 0;
    virtual void pixel(uint64_t i, uint64_t& row, uint64_t& col) const = 0;
    virtual void finished(uint64_t i, const double* v, uint32_t n) = 0;
    virtual void end_loop() = 0;
    virtual bool done() const = 0;
    virtual uint64_t rounds() const = 0;
    virtual std::string description() const = 0;  // Mesh::getFullDescriptionStr
    // The same mesh, unstarted, with every square of positive weight subdivided in each
    // round (foort_mesh_create_waves); null where that is not this mesh's pixel set.
    virtual foort_mesh* wave_clone() const = 0;
    // Every pixel the next round could hand out: the five candidates of each square that
    // awaits its weight (foort_mesh_lookahead); cells, each once.
    virtual void lookahead(std::vector<uint64_t>&) const {}
    // Most pixels the mesh hands out over a run (0: no limit).
    virtual uint64_t pixel_cap() const = 0;
};

namespace {

// SimpleSquareMesh, Mesh.cpp:25-73
struct SimpleMesh final : foort_mesh {
    uint64_t total = 0;
    bool fin = false;
    uint64_t cur() const override { return total; }
    void pixel(uint64_t i, uint64_t& row, uint64_t& col) const override {
        row = i / grid;  // the reference counts rows up one by one (Mesh.cpp:40-43)
        col = i - row * grid;
    }
    void finished(uint64_t, const double*, uint32_t) override {}
    void end_loop() override { fin = true; }
    bool done() const override { return fin; }
    uint64_t rounds() const override { return fin ? 1 : 0; }
    // Mesh.cpp:69-73
    std::string description() const override {
        return "Mesh: simple square grid (" + std::to_string(grid) + "^2 pixels)";
    }
    uint64_t pixel_cap() const override { return total; }
    foort_mesh* wave_clone() const override {
        if (fin) return nullptr;
        auto* m = new SimpleMesh(*this);
        m->err.clear();
        return m;
    }
};

// SquareSubdivisionMeshV2, Mesh.cpp:660-1186
struct V2Mesh final : foort_mesh {
    struct Px {
        uint64_t row, col;
        int level;
        double weight = -1;
        Value value;
        Px *left = nullptr, *right = nullptr, *up = nullptr, *down = nullptr, *se = nullptr;
        Px(uint64_t r, uint64_t c, int l) : row(r), col(c), level(l) {}
    };
    uint64_t initial = 0, iteration = 0, max_pixels = 0, left_px = 0, integrated = 0;
    int max_sub = 1;
    bool infinite = true, sub_to_final = false;
    uint64_t n_rounds = 0;
    bool waves = false;                    // a copy of level waves (wave_clone)
    std::deque<Px> all;                    // owns every pixel (stable addresses, few allocations)
    std::vector<Px*> active, queue, updating;

    Px* make(uint64_t r, uint64_t c, int l) {
        all.emplace_back(r, c, l);
        return &all.back();
    }

    // InitializeFirstGrid, Mesh.cpp:741-802
    void init_grid() {
        const uint64_t n = static_cast<uint64_t>(std::sqrt(static_cast<double>(initial)));
        const uint64_t scale = pow2(max_sub - 1);
        std::vector<Px*> g(n * n);
        for (uint64_t r = 0; r < n; ++r)
            for (uint64_t c = 0; c < n; ++c) {
                int lvl = (r == n - 1 || c == n - 1) ? max_sub : 1;
                g[r * n + c] = make(static_cast<uint64_t>(static_cast<double>(r) * static_cast<double>(scale)),
                                    static_cast<uint64_t>(static_cast<double>(c) * static_cast<double>(scale)), lvl);
            }
        for (uint64_t r = 0; r + 1 < n; ++r)
            for (uint64_t c = 0; c + 1 < n; ++c) {
                Px* p = g[r * n + c];
                p->right = g[r * n + c + 1];
                g[r * n + c + 1]->left = p;
                p->down = g[(r + 1) * n + c];
                g[(r + 1) * n + c]->up = p;
                p->se = g[(r + 1) * n + c + 1];
            }
        for (uint64_t i = 0; i < n * n; ++i) {
            queue.push_back(g[i]);
            if (g[i]->level < max_sub) updating.push_back(g[i]);
        }
        if (!infinite) left_px -= queue.size();
    }

    // UpdateAllWeights, Mesh.cpp:809-841
    void update_weights() {
        for (Px* p : updating) {
            double d0 = distance(value_diag, p->value, p->right->value);
            double d1 = distance(value_diag, p->value, p->down->value);
            double d2 = distance(value_diag, p->value, p->se->value);
            p->weight = std::max(d0, std::max(d1, d2));
            if (p->weight > 0.0) active.push_back(p);
        }
        updating.clear();
    }

    // GetUp / GetDown / GetLeft / GetRight, Mesh.cpp:844-939
    Px* get_up(Px* p, int s) const {
        if (!p || !p->up || p->up->level < s) return nullptr;
        if (p->up->level == s) return p->up;
        return get_up(get_up(p, s + 1), s + 1);
    }
    Px* get_down(Px* p, int s) const {
        if (!p || !p->down || p->level < s) return nullptr;
        if (p->level == s) return p->down;
        return get_down(get_down(p, s + 1), s + 1);
    }
    Px* get_left(Px* p, int s) const {
        if (!p || !p->left || p->left->level < s) return nullptr;
        if (p->left->level == s) return p->left;
        return get_left(get_left(p, s + 1), s + 1);
    }
    Px* get_right(Px* p, int s) const {
        if (!p || !p->right || p->level < s) return nullptr;
        if (p->level == s) return p->right;
        return get_right(get_right(p, s + 1), s + 1);
    }

    // SubdivideAndQueue, Mesh.cpp:944-1086: square (1, 3, 7, 9) gets pixels 2, 4, 5, 6, 8.
    void subdivide(uint64_t ind) {
        Px* p1 = active[ind];
        Px* p3 = p1->right;
        Px* p7 = p1->down;
        Px* p9 = p1->se;
        const int ns = p1->level + 1;
        const uint64_t step = pow2(max_sub - ns);
        p1->level = ns;
        if (ns < max_sub) updating.push_back(p1);
        Px* p2 = get_down(get_right(get_up(p1, ns), ns), ns);
        if (!p2) {
            p2 = make(p1->row, p1->col + step, ns);
            queue.push_back(p2);
        } else {
            p2->level = ns;
        }
        if (ns < max_sub) updating.push_back(p2);
        Px* p4 = get_right(get_down(get_left(p1, ns), ns), ns);
        if (!p4) {
            p4 = make(p1->row + step, p1->col, ns);
            queue.push_back(p4);
        } else {
            p4->level = ns;
        }
        if (ns < max_sub) updating.push_back(p4);
        Px* p5 = make(p1->row + step, p1->col + step, ns);
        queue.push_back(p5);
        if (ns < max_sub) updating.push_back(p5);
        Px* p6 = get_down(p3, ns);
        if (!p6) {
            p6 = make(p1->row + step, p1->col + 2 * step, 0);
            queue.push_back(p6);
        }
        Px* p8 = get_right(p7, ns);
        if (!p8) {
            p8 = make(p1->row + 2 * step, p1->col + step, 0);
            queue.push_back(p8);
        }
        p1->right = p2; p2->left = p1; p1->down = p4; p4->up = p1; p1->se = p5;
        p2->right = p3; p3->left = p2; p2->down = p5; p5->up = p2; p2->se = p6;
        p4->right = p5; p5->left = p4; p4->down = p7; p7->up = p4; p4->se = p8;
        p5->right = p6; p6->left = p5; p5->down = p8; p8->up = p5; p5->se = p9;
    }

    uint64_t cur() const override { return queue.size(); }
    void pixel(uint64_t i, uint64_t& row, uint64_t& col) const override {
        row = queue[i]->row;
        col = queue[i]->col;
    }
    void finished(uint64_t i, const double* v, uint32_t n) override { queue[i]->value.set(v, n); }
    bool done() const override { return queue.empty(); }
    uint64_t rounds() const override { return n_rounds; }
    // Mesh.cpp:697-707
    std::string description() const override {
        const uint64_t n = static_cast<uint64_t>(std::sqrt(static_cast<double>(initial)));
        return "Mesh: square subdivision v2 (initial pixels: " + std::to_string(n) +
               "^2; max subdivision: " + std::to_string(max_sub) +
               "; pixels subdivided per iteration: " + std::to_string(iteration) +
               "; max total pixels: " + (infinite ? std::string("infinite") : std::to_string(max_pixels)) +
               "; if pixel is initially subdivided, will continue to max: " + std::to_string(sub_to_final ? 1 : 0) +
               "; row/column size: " + std::to_string(grid) + ")";
    }

    // With unlimited MaxPixels the reference's rounds continue until no square of
    // positive weight is left, so every such square is subdivided in some round: the
    // run's pixel set is fixed by the values alone, and IterationPixels only spreads it
    // over rounds. With IterationPixels unlimited, round k hands out the pixels of
    // subdivision level k. The copy is unlimited also where this mesh is not: its pixels
    // then hold this mesh's (at most MaxPixels of them, cut in the round order).
    foort_mesh* wave_clone() const override {
        if (n_rounds != 0) return nullptr;
        auto* m = new V2Mesh();
        m->kind = kind;
        m->grid = grid;
        m->diag_flags = diag_flags;
        m->value_diag = value_diag;
        m->initial = initial;
        m->max_sub = max_sub;
        m->iteration = UINT64_MAX;
        m->sub_to_final = sub_to_final;
        m->waves = true;
        m->init_grid();
        return m;
    }

    // The squares of the updating list get their weights at the end of this round; the
    // next round subdivides some of them (all that get a positive weight, in a wave mesh),
    // and each subdivision hands out at most its square's p2, p4, p5, p6 and p8.
    uint64_t pixel_cap() const override { return infinite ? 0 : max_pixels; }
    void lookahead(std::vector<uint64_t>& cells) const override {
        cells.clear();
        cells.reserve(5 * updating.size());
        for (const Px* p : updating) {
            const uint64_t h = pow2(max_sub - p->level - 1);  // half the square's side
            const uint64_t r = p->row, c = p->col;
            const uint64_t cand[5][2] = {{r, c + h}, {r + h, c}, {r + h, c + h}, {r + h, c + 2 * h}, {r + 2 * h, c + h}};
            for (const auto& q : cand) cells.push_back(q[0] * grid + q[1]);
        }
        // ascending and each once: a bitmap of the grid where it is not much larger than
        // the list (a seed round's 5 x 16,384 candidates: 0.2 ms instead of 4 ms of sort)
        const uint64_t words = (grid * grid + 63) / 64;
        if (words <= 4 * cells.size()) {
            std::vector<uint64_t> bits(words, 0);
            for (const uint64_t c : cells) bits[c >> 6] |= uint64_t{1} << (c & 63);
            cells.clear();
            for (uint64_t w = 0; w < words; ++w)
                for (uint64_t b = bits[w]; b; b &= b - 1)
                    cells.push_back(64 * w + static_cast<uint64_t>(__builtin_ctzll(b)));
            return;
        }
        std::sort(cells.begin(), cells.end());
        cells.erase(std::unique(cells.begin(), cells.end()), cells.end());
    }

    // The reference's std::sort of the active list (Mesh.cpp:1126-1130), on records that
    // carry each square's weight and level beside its pointer: std::sort's permutation
    // depends only on the element count and the comparisons' outcomes, which are the same
    // as on the pointers, so the order (ties included) is the reference's, without a
    // pointer dereference per comparison.
    struct SortKey {
        double weight;
        int level;
        Px* p;
    };
    std::vector<SortKey> keys;
    void sort_active() {
        keys.resize(active.size());
        for (size_t i = 0; i < active.size(); ++i) keys[i] = SortKey{active[i]->weight, active[i]->level, active[i]};
        std::sort(keys.begin(), keys.end(), [](const SortKey& a, const SortKey& b) {
            if (a.weight > b.weight) return true;
            if (a.weight == b.weight && a.level < b.level) return true;
            return false;
        });
        for (size_t i = 0; i < active.size(); ++i) active[i] = keys[i].p;
    }

    // EndCurrentLoop, Mesh.cpp:1092-1186
    void end_loop() override {
        ++n_rounds;
        integrated += queue.size();
        queue.clear();
        if (infinite || left_px > 0) {
            update_weights();
            // A wave copy subdivides every square of positive weight: the pixels it
            // creates, their levels and links do not depend on the order (a shared
            // pixel is made by one square and found by the other), only the order in
            // which they are handed out does, and no result depends on that.
            if (!waves) sort_active();
            const uint64_t lim = std::min<uint64_t>(active.size(), iteration);
            for (uint64_t i = 0; i < lim; ++i) subdivide(i);
            active.erase(active.begin(), active.begin() + static_cast<std::ptrdiff_t>(lim));
            if (!infinite && queue.size() > left_px) queue.erase(queue.begin() + static_cast<std::ptrdiff_t>(left_px), queue.end());
            if (!infinite) left_px -= queue.size();
        }
    }
};

thread_local std::string g_mesh_err;

}  // namespace

extern "C" {

int foort_mesh_create_simple(uint64_t total_pixels, uint32_t diag_flags, uint32_t value_diag, foort_mesh** out) {
    if (!out) return FOORT_E_BADARG;
    auto* m = new SimpleMesh();
    m->kind = 0;
    m->grid = static_cast<uint64_t>(std::sqrt(static_cast<double>(total_pixels)));
    m->total = m->grid * m->grid;
    m->diag_flags = diag_flags;
    m->value_diag = value_diag;
    *out = m;
    return FOORT_OK;
}

int foort_mesh_create_v2(uint64_t max_pixels, uint64_t initial_pixels, int32_t max_subdivide, uint64_t iteration_pixels,
                         int32_t initial_sub_to_final, uint32_t diag_flags, uint32_t value_diag, foort_mesh** out) {
    if (!out || max_subdivide < 1 || initial_pixels < 4) return FOORT_E_BADARG;
    // InitialSubdivisionToFinal is stored by the reference's V2 mesh but never read
    // (Mesh.h:344, Mesh.cpp:660-1186); it is accepted and has no effect here either.
    auto* m = new V2Mesh();
    m->kind = 1;
    const uint64_t n = static_cast<uint64_t>(std::sqrt(static_cast<double>(initial_pixels)));
    m->initial = n * n;
    m->max_sub = max_subdivide;
    m->grid = static_cast<uint64_t>((std::sqrt(static_cast<double>(initial_pixels)) - 1) *
                                    static_cast<double>(pow2(max_subdivide - 1)) + 1);
    m->max_pixels = max_pixels;
    m->left_px = max_pixels;
    m->infinite = max_pixels == 0;
    m->iteration = iteration_pixels;
    m->sub_to_final = initial_sub_to_final != 0;
    m->diag_flags = diag_flags;
    m->value_diag = value_diag;
    m->init_grid();
    *out = m;
    return FOORT_OK;
}

int foort_mesh_is_finished(const foort_mesh* m) { return m ? (m->done() ? 1 : 0) : FOORT_E_BADARG; }

uint64_t foort_mesh_cur_nr_geodesics(const foort_mesh* m) { return m ? m->cur() : 0; }

uint64_t foort_mesh_grid(const foort_mesh* m) { return m ? m->grid : 0; }

uint64_t foort_mesh_rounds(const foort_mesh* m) { return m ? m->rounds() : 0; }

int foort_mesh_get_pixels(const foort_mesh* m, uint32_t image, foort_pixel* out) {
    if (!m || (!out && m->cur())) return FOORT_E_BADARG;
    const uint64_t n = m->cur();
    for (uint64_t i = 0; i < n; ++i) {
        foort_pixel& p = out[i];
        p.image = image;
        p.reserved = 0;
        m->pixel(i, p.row, p.col);
        p.grid = m->grid;
    }
    return FOORT_OK;
}

int foort_mesh_geodesic_finished(foort_mesh* m, uint64_t index, const double* values, uint32_t n_values) {
    if (!m || index >= m->cur() || (n_values && !values)) return FOORT_E_BADARG;
    m->finished(index, values, n_values);
    return FOORT_OK;
}

int foort_mesh_set_results(foort_mesh* m, const foort_result* res, uint64_t n) {
    if (!m || n != m->cur() || (n && !res)) return FOORT_E_BADARG;
    const uint32_t first = first_diagnostic(m->diag_flags, m->value_diag);
    if (first == FOORT_DIAG_GEODESIC_POSITION) return FOORT_E_UNSUPPORTED;
    for (uint64_t i = 0; i < n; ++i) {
        double v = 0.0;
        if (first == FOORT_DIAG_FOUR_COLOR_SCREEN) v = res[i].quadrant;
        else if (first == FOORT_DIAG_EQUATORIAL_PASSES) v = res[i].equat_passes;
        else if (first == FOORT_DIAG_CLOSEST_RADIUS) v = res[i].closest_r;
        m->finished(i, &v, 1);
    }
    return FOORT_OK;
}

int foort_mesh_end_current_loop(foort_mesh* m) {
    if (!m) return FOORT_E_BADARG;
    m->end_loop();
    return FOORT_OK;
}

void foort_mesh_destroy(foort_mesh* m) { delete m; }

uint64_t foort_mesh_max_pixels(const foort_mesh* m) { return m ? m->pixel_cap() : 0; }
int foort_mesh_kind(const foort_mesh* m) { return m ? m->kind : FOORT_E_BADARG; }

int foort_mesh_lookahead(const foort_mesh* m, uint32_t image, foort_pixel* out, uint64_t cap, uint64_t* n) {
    if (!m || !n) return FOORT_E_BADARG;
    std::vector<uint64_t> cells;
    m->lookahead(cells);
    *n = cells.size();
    if (!out) return FOORT_OK;
    if (cap < cells.size()) return FOORT_E_BADARG;
    for (uint64_t i = 0; i < cells.size(); ++i)
        out[i] = foort_pixel{image, 0u, cells[i] / m->grid, cells[i] % m->grid, m->grid};
    return FOORT_OK;
}

int foort_mesh_create_waves(const foort_mesh* m, foort_mesh** out) {
    if (!m || !out) return FOORT_E_BADARG;
    *out = m->wave_clone();
    return *out ? FOORT_OK : FOORT_E_UNSUPPORTED;
}

int foort_mesh_description(const foort_mesh* m, char* buf, uint64_t cap) {
    if (!m || !buf || cap == 0) return FOORT_E_BADARG;
    const std::string s = m->description();
    if (s.size() + 1 > cap) return FOORT_E_BADARG;
    std::memcpy(buf, s.c_str(), s.size() + 1);
    return FOORT_OK;
}

}  // extern "C"
