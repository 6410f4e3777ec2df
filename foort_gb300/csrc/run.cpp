// A whole run: the round loop of Main.cpp:313-419 over the engine, the meshes and the
// output files, all through the C ABI.
//
// Per round every unfinished image's mesh hands out its pixels (ViewScreen::
// getCurNrGeodesics / SetNewInitialConditions); the pixels of all images go to the GPU
// in one launch (foort_gpu_integrate); the results go back to each mesh
// (GeodesicFinished, Main.cpp:399) and to each image's output files
// (NewGeodesicOutput, Main.cpp:400); then each mesh ends its round (EndCurrentLoop,
// Main.cpp:410). Images advance in lockstep, so a round is one launch over all images.
//
// Level waves (FOORT_SCHEDULE_WAVES). A launch lasts as long as its slowest geodesic, and
// on the adaptive mesh's rounds that is most of the launch: in the Kerr a = 0.99 run on a
// 509² grid the geodesics all take 66,000-71,000 steps, so a round of 1,079 geodesics
// takes as long as one of 16,384. With unlimited MaxPixels the mesh's pixel set is fixed
// by the values alone (foort_mesh_create_waves), and it splits into one wave per
// subdivision level, each depending only on the results of the waves before. The run
// integrates the waves first, a wave's launch also taking the next wave's candidates
// (foort_mesh_lookahead) while it stays within the context's lookahead cap (that run: two
// launches where the reference has five rounds), then replays the meshes' rounds from the
// stored results, so meshes and output files see the reference's rounds. With a finite MaxPixels an image's waves stop at that
// budget, and its rounds integrate what the waves did not. While a wave's launch runs, the
// host replays the rounds whose results are already stored.
#include <algorithm>
#include <cstring>
#include <vector>

#include "../../include/foort_gpu.h"
#include "diag_order.h"

// engine.cu (internal)
extern "C" {
uint32_t foort_ctx_schedule(const foort_ctx* ctx);
uint64_t foort_ctx_budget(const foort_ctx* ctx);
uint64_t foort_ctx_lookahead(const foort_ctx* ctx);
void foort_ctx_set_run_info(foort_ctx* ctx, uint32_t launches, uint32_t schedule);
void foort_ctx_launched(foort_ctx* ctx, const foort_pixel* px, uint64_t n, bool first);
int foort_ctx_stage(foort_ctx* ctx, uint64_t n, foort_pixel** px, foort_result** res);
int foort_ctx_integrate_begin(foort_ctx* ctx, const foort_pixel* px, uint64_t n);
int foort_ctx_integrate_end(foort_ctx* ctx, foort_result* out, uint64_t n);
}

namespace {

// How many pixels each unfinished mesh hands out this round: count[i] of image i (0 for a
// finished mesh), n in all. any: some mesh is unfinished.
int count_pixels(foort_mesh* const* meshes, uint32_t n_images, std::vector<uint64_t>& count, bool& any,
                 uint64_t& n) {
    n = 0;
    any = false;
    for (uint32_t i = 0; i < n_images; ++i) {
        const int fin = foort_mesh_is_finished(meshes[i]);
        if (fin < 0) return fin;
        count[i] = fin ? 0 : foort_mesh_cur_nr_geodesics(meshes[i]);
        any = any || !fin;
        n += count[i];
    }
    return FOORT_OK;
}

// Those pixels, image after image, into px.
int fill_pixels(foort_mesh* const* meshes, uint32_t n_images, const std::vector<uint64_t>& count, foort_pixel* px) {
    uint64_t k = 0;
    for (uint32_t i = 0; i < n_images; ++i) {
        if (foort_mesh_is_finished(meshes[i])) continue;
        const int rc = foort_mesh_get_pixels(meshes[i], i, px + k);
        if (rc) return rc;
        k += count[i];
    }
    return FOORT_OK;
}

// Map from a pixel (image, grid cell) to an index: open addressing with linear probing
// over a power-of-two table of (key, value) slots kept at most half full, sized ahead of
// each batch of inserts (reserve). For the 187k results of a Kerr a = 0.998 run on a
// 4097² grid, one insert and two lookups each take 10 ms on an x86-64 host core (20 ms
// with keys and values in separate arrays and growth by doubling, 42 ms with
// std::unordered_map).
class PixelMap {
  public:
    static uint64_t key(const foort_pixel& p) { return (static_cast<uint64_t>(p.image) << 42) | (p.row * p.grid + p.col); }
    bool get(uint64_t k, uint64_t& v) const {
        if (slots_.empty()) return false;
        for (uint64_t i = mix(k) & mask_;; i = (i + 1) & mask_) {
            const Slot& s = slots_[i];
            if (s.key == k) {
                v = s.val;
                return true;
            }
            if (s.key == kEmpty) return false;
        }
    }
    bool has(uint64_t k) const {
        uint64_t v;
        return get(k, v);
    }
    // Room for n entries in all without a rehash.
    void reserve(uint64_t n) {
        uint64_t cap = 64;
        while (cap < 2 * n) cap *= 2;
        if (cap > slots_.size()) rehash(cap);
    }
    void put(uint64_t k, uint64_t v) {
        if (2 * (size_ + 1) > slots_.size()) rehash(std::max<uint64_t>(64, 2 * slots_.size()));
        for (uint64_t i = mix(k) & mask_;; i = (i + 1) & mask_) {
            Slot& s = slots_[i];
            if (s.key == k) {
                s.val = v;
                return;
            }
            if (s.key == kEmpty) {
                s = Slot{k, v};
                ++size_;
                return;
            }
        }
    }

  private:
    struct Slot {
        uint64_t key, val;
    };
    static constexpr uint64_t kEmpty = ~0ull;  // no pixel has this key (image < 2^22)
    static uint64_t mix(uint64_t x) {  // the splitmix64 finaliser
        x ^= x >> 30;
        x *= 0xbf58476d1ce4e5b9ull;
        x ^= x >> 27;
        x *= 0x94d049bb133111ebull;
        return x ^ (x >> 31);
    }
    void rehash(uint64_t cap) {
        std::vector<Slot> old(cap, Slot{kEmpty, 0});
        std::swap(old, slots_);
        mask_ = cap - 1;
        size_ = 0;
        for (const Slot& s : old)
            if (s.key != kEmpty) put(s.key, s.val);
    }
    std::vector<Slot> slots_;
    uint64_t mask_ = 0, size_ = 0;
};

// Results of integrated pixels by image and grid cell.
struct ResultStore {
    PixelMap slot;  // pixel -> index in res
    std::vector<foort_result> res;
};

// One launch of the run (foort_gpu_integrate), counted and recorded.
int launch(foort_ctx* ctx, const std::vector<foort_pixel>& px, std::vector<foort_result>& res, uint32_t& launches) {
    res.resize(px.size());
    foort_ctx_launched(ctx, px.data(), px.size(), launches == 0);
    ++launches;
    return foort_gpu_integrate(ctx, px.data(), px.size(), res.data());
}

// The same launch in two halves: `during` runs on the host while it is in flight.
template <typename F>
int launch_overlapped(foort_ctx* ctx, const std::vector<foort_pixel>& px, std::vector<foort_result>& res,
                      uint32_t& launches, F&& during) {
    res.resize(px.size());
    foort_ctx_launched(ctx, px.data(), px.size(), launches == 0);
    ++launches;
    int rc = foort_ctx_integrate_begin(ctx, px.data(), px.size());
    if (rc) return rc;
    const int rc_host = during();
    rc = foort_ctx_integrate_end(ctx, res.data(), px.size());
    return rc ? rc : rc_host;
}

// The next wave's candidates (foort_mesh_lookahead) of the images marked in `use` that have
// no result yet and are not in `todo`, appended to `spec`. Stops, with `over` set, once
// there are more than `limit` of them: the launch then cannot take them.
int lookahead_candidates(foort_mesh* const* waves, uint32_t n_images, const std::vector<bool>& use,
                         const ResultStore& store, const std::vector<foort_pixel>& todo, uint64_t limit,
                         std::vector<foort_pixel>& spec, bool& over) {
    over = false;
    std::vector<uint64_t> raw(n_images, 0);
    uint64_t known = store.res.size() + todo.size();  // candidates that can drop out, at most
    uint64_t all = 0;
    for (uint32_t i = 0; i < n_images; ++i) {
        if (!use[i]) continue;
        const int rc = foort_mesh_lookahead(waves[i], i, nullptr, 0, &raw[i]);
        if (rc) return rc;
        all += raw[i];
    }
    if (all > limit + known) {  // more than `limit` remain whatever drops out
        over = true;
        return FOORT_OK;
    }
    PixelMap now;
    now.reserve(todo.size());
    for (const foort_pixel& p : todo) now.put(PixelMap::key(p), 0);
    std::vector<foort_pixel> cand;
    for (uint32_t i = 0; i < n_images; ++i) {
        if (!use[i] || raw[i] == 0) continue;
        uint64_t n = raw[i];
        cand.resize(n);
        const int rc = foort_mesh_lookahead(waves[i], i, cand.data(), n, &n);
        if (rc) return rc;
        for (const foort_pixel& p : cand) {
            const uint64_t k = PixelMap::key(p);
            if (!store.slot.has(k) && !now.has(k)) spec.push_back(p);
        }
        if (spec.size() > limit) {
            over = true;
            return FOORT_OK;
        }
    }
    return FOORT_OK;
}

// Integrate the meshes' level waves, one launch per wave over all images, and keep every
// result. An image's waves stop before the one that would take them past the mesh's
// foort_mesh_max_pixels (its rounds then find the rest missing and integrate it).
// FOORT_E_UNSUPPORTED (nothing integrated) where a mesh has no waves.
template <typename F>
int integrate_waves(foort_ctx* ctx, foort_mesh* const* meshes, uint32_t n_images, ResultStore& store,
                    uint32_t& launches, F&& during) {
    std::vector<foort_mesh*> waves(n_images, nullptr);
    auto release = [&]() {
        for (foort_mesh* w : waves) foort_mesh_destroy(w);
    };
    std::vector<uint64_t> budget(n_images), handed(n_images, 0), count(n_images);
    for (uint32_t i = 0; i < n_images; ++i) {
        if (foort_mesh_create_waves(meshes[i], &waves[i]) != FOORT_OK) {
            release();
            return FOORT_E_UNSUPPORTED;
        }
        budget[i] = foort_mesh_max_pixels(meshes[i]);
        if (budget[i] == 0) budget[i] = UINT64_MAX;
    }
    const uint64_t ahead = foort_ctx_lookahead(ctx);
    std::vector<bool> live(n_images, true), use(n_images, false);
    std::vector<foort_pixel> px, todo;
    std::vector<foort_result> res, got;
    int rc = FOORT_OK;
    for (;;) {
        // this wave's pixels, image after image
        px.clear();
        for (uint32_t i = 0; i < n_images; ++i) {
            count[i] = 0;
            if (live[i] && foort_mesh_is_finished(waves[i])) live[i] = false;
            if (!live[i]) continue;
            const uint64_t n = foort_mesh_cur_nr_geodesics(waves[i]);
            if (n > budget[i] - handed[i]) {
                live[i] = false;
                continue;
            }
            px.resize(px.size() + n);
            if ((rc = foort_mesh_get_pixels(waves[i], i, px.data() + px.size() - n))) break;
            count[i] = n;
            handed[i] += n;
        }
        if (rc || px.empty()) break;
        // the pixels without a result (none where the last launch looked ahead)
        todo.clear();
        for (const foort_pixel& p : px)
            if (!store.slot.has(PixelMap::key(p))) todo.push_back(p);
        if (!todo.empty()) {
            if (ahead > todo.size()) {
                std::vector<foort_pixel> spec;
                bool over = false;
                for (uint32_t i = 0; i < n_images; ++i) use[i] = count[i] > 0;
                if ((rc = lookahead_candidates(waves.data(), n_images, use, store, todo, ahead - todo.size(), spec,
                                               over)))
                    break;
                // candidates within each image's budget only
                std::vector<uint64_t> per(n_images, 0);
                for (const foort_pixel& p : spec) ++per[p.image];
                bool fits = !over && todo.size() + spec.size() <= ahead;
                for (uint32_t i = 0; i < n_images && fits; ++i) fits = per[i] <= budget[i] - handed[i];
                if (fits) todo.insert(todo.end(), spec.begin(), spec.end());
            }
            if ((rc = launch_overlapped(ctx, todo, got, launches, during))) break;
            store.slot.reserve(store.res.size() + todo.size());
            store.res.reserve(store.res.size() + todo.size());
            for (uint64_t g = 0; g < todo.size(); ++g) {
                store.slot.put(PixelMap::key(todo[g]), store.res.size());
                store.res.push_back(got[g]);
            }
        }
        res.resize(px.size());
        for (uint64_t g = 0; g < px.size(); ++g) {
            uint64_t at = 0;
            store.slot.get(PixelMap::key(px[g]), at);  // stored above, or by an earlier launch
            res[g] = store.res[at];
        }
        uint64_t k = 0;
        for (uint32_t i = 0; i < n_images && rc == FOORT_OK; ++i) {
            if (!count[i]) continue;
            rc = foort_mesh_set_results(waves[i], res.data() + k, count[i]);
            if (!rc) rc = foort_mesh_end_current_loop(waves[i]);
            k += count[i];
        }
        if (rc) break;
    }
    release();
    return rc;
}

// The round's results from the store; the pixels it lacks are integrated in one launch.
int results_from_store(foort_ctx* ctx, const ResultStore& store, const std::vector<foort_pixel>& px,
                       std::vector<foort_result>& res, uint32_t& launches) {
    std::vector<uint64_t> miss;
    for (uint64_t g = 0; g < px.size(); ++g) {
        uint64_t at = 0;
        if (store.slot.get(PixelMap::key(px[g]), at)) {
            res[g] = store.res[at];
        } else {
            miss.push_back(g);
        }
    }
    if (miss.empty()) return FOORT_OK;
    std::vector<foort_pixel> mp(miss.size());
    std::vector<foort_result> mr;
    for (uint64_t j = 0; j < miss.size(); ++j) mp[j] = px[miss[j]];
    const int rc = launch(ctx, mp, mr, launches);
    if (rc) return rc;
    for (uint64_t j = 0; j < miss.size(); ++j) res[miss[j]] = mr[j];
    return FOORT_OK;
}

// The reference's round loop (Main.cpp:313-419), one round per call of next().
struct Rounds {
    foort_ctx* ctx;
    foort_mesh* const* meshes;
    foort_output* const* outputs;
    uint32_t n_images;
    bool geopos;
    uint32_t value_first;
    uint64_t total = 0;
    uint32_t n_rounds = 0;
    bool done = false;
    std::vector<foort_pixel> px;
    std::vector<foort_result> res;
    std::vector<uint64_t> count;

    // One round over every unfinished mesh. Its results come from `store` where given
    // (with one launch for the pixels it lacks), else from a launch, whose pixels and
    // results stay in the context's pinned staging. stored_only: run the round only if the
    // store holds all of its results (ran tells), and never launch.
    int next(const ResultStore* store, uint32_t& launches, bool stored_only, bool& ran) {
        ran = false;
        if (done) return FOORT_OK;
        bool any = false;
        uint64_t n = 0;
        count.resize(n_images);
        int rc = count_pixels(meshes, n_images, count, any, n);
        if (rc) return rc;
        if (!any) {
            done = true;
            return FOORT_OK;
        }
        foort_pixel* P = nullptr;
        foort_result* Rs = nullptr;
        if (store) {
            px.resize(n);
            res.resize(n);
            P = px.data();
            Rs = res.data();
            if ((rc = fill_pixels(meshes, n_images, count, P))) return rc;
            if (stored_only) {
                if (geopos) return FOORT_OK;
                for (uint64_t g = 0; g < n; ++g) {
                    uint64_t at = 0;
                    if (!store->slot.get(PixelMap::key(P[g]), at)) return FOORT_OK;
                    Rs[g] = store->res[at];
                }
            } else if ((rc = results_from_store(ctx, *store, px, res, launches))) {
                return rc;
            }
        } else {
            if (stored_only) return FOORT_OK;
            if ((rc = foort_ctx_stage(ctx, n, &P, &Rs))) return rc;
            if ((rc = fill_pixels(meshes, n_images, count, P))) return rc;
            foort_ctx_launched(ctx, P, n, launches == 0);
            ++launches;
            if ((rc = foort_ctx_integrate_begin(ctx, P, n))) return rc;
            if ((rc = foort_ctx_integrate_end(ctx, nullptr, n))) return rc;
        }
        // GeodesicPosition: a second pass records the positions (foort_gpu_positions)
        std::vector<uint64_t> counts, first;
        std::vector<double> points;
        if (geopos) {
            counts.resize(n);
            first.resize(n);
            uint64_t total_pts = 0;
            if ((rc = foort_gpu_positions(ctx, P, n, Rs, counts.data(), nullptr, 0, &total_pts)))
                return rc;
            points.resize(4 * std::max<uint64_t>(total_pts, 1));
            if ((rc = foort_gpu_positions(ctx, P, n, Rs, counts.data(), points.data(), total_pts,
                                          &total_pts)))
                return rc;
            uint64_t s = 0;
            for (uint64_t g = 0; g < n; ++g) {
                first[g] = s;
                s += counts[g];
            }
        }
        uint64_t k = 0;
        for (uint32_t i = 0; i < n_images; ++i) {
            if (foort_mesh_is_finished(meshes[i])) continue;
            if (value_first == FOORT_DIAG_GEODESIC_POSITION) {
                // getFinalDataVal: (theta, phi) of the last kept position (Diagnostics.cpp:304-309)
                for (uint64_t g = 0; g < count[i]; ++g) {
                    const uint64_t q = k + g;
                    double v[2] = {Rs[q].pos[2], Rs[q].pos[3]};
                    if (counts[q]) {
                        v[0] = points[4 * (first[q] + counts[q] - 1) + 2];
                        v[1] = points[4 * (first[q] + counts[q] - 1) + 3];
                    }
                    if ((rc = foort_mesh_geodesic_finished(meshes[i], g, v, 2))) return rc;
                }
            } else if ((rc = foort_mesh_set_results(meshes[i], Rs + k, count[i]))) {
                return rc;
            }
            if (outputs && outputs[i]) {
                rc = geopos ? foort_output_round_positions(outputs[i], P + k, Rs + k, count[i],
                                                           counts.data() + k, points.data() + 4 * (k < n ? first[k] : 0))
                            : foort_output_round(outputs[i], P + k, Rs + k, count[i]);
                if (rc) return rc;
            }
            if ((rc = foort_mesh_end_current_loop(meshes[i]))) return rc;
            k += count[i];
        }
        total += n;
        ++n_rounds;
        ran = true;
        return FOORT_OK;
    }
};

int run(foort_ctx* ctx, foort_mesh* const* meshes, foort_output* const* outputs, uint32_t n_images,
        uint64_t* geodesics, uint32_t* rounds, uint32_t& launches, uint32_t& schedule) {
    foort_run_desc desc;
    if (foort_gpu_get_desc(ctx, &desc)) return FOORT_E_BADARG;
    const bool geopos = (desc.diag_flags & FOORT_DIAG_GEODESIC_POSITION) != 0;
    const std::vector<uint32_t> order = foort::diagnostic_order(desc.diag_flags, desc.value_diag);
    Rounds R{ctx, meshes, outputs, n_images, geopos, order.empty() ? 0u : order[0]};
    int rc = FOORT_OK;
    ResultStore store;
    schedule = FOORT_SCHEDULE_ROUNDS;
    // A SimpleSquareMesh is its own single wave: without an adaptive mesh the waves are
    // the rounds, and storing the results would only cost time.
    bool adaptive = false;
    for (uint32_t i = 0; i < n_images; ++i) adaptive = adaptive || foort_mesh_kind(meshes[i]) == FOORT_MESH_SUBDIVISION_V2;
    if (adaptive && foort_ctx_schedule(ctx) == FOORT_SCHEDULE_WAVES && !geopos && foort_ctx_budget(ctx) == 0) {
        // while a launch runs: the rounds whose results are all stored
        auto replay = [&]() -> int {
            bool ran = true;
            while (ran) {
                const int r = R.next(&store, launches, true, ran);
                if (r) return r;
            }
            return FOORT_OK;
        };
        rc = integrate_waves(ctx, meshes, n_images, store, launches, replay);
        if (rc == FOORT_OK) {
            schedule = FOORT_SCHEDULE_WAVES;
        } else if (rc != FOORT_E_UNSUPPORTED) {
            return rc;
        }
    }
    const ResultStore* from = schedule == FOORT_SCHEDULE_WAVES ? &store : nullptr;
    for (;;) {
        bool ran = false;
        if ((rc = R.next(from, launches, false, ran))) return rc;
        if (!ran) break;
    }
    if (outputs)
        for (uint32_t i = 0; i < n_images; ++i)
            if (outputs[i] && (rc = foort_output_finish(outputs[i]))) return rc;
    if (geodesics) *geodesics = R.total;
    if (rounds) *rounds = R.n_rounds;
    return FOORT_OK;
}

}  // namespace

extern "C" int foort_gpu_run(foort_ctx* ctx, foort_mesh* const* meshes, foort_output* const* outputs,
                             uint32_t n_images, uint64_t* geodesics, uint32_t* rounds) {
    if (!ctx || !meshes || n_images == 0) return FOORT_E_BADARG;
    for (uint32_t i = 0; i < n_images; ++i)
        if (!meshes[i]) return FOORT_E_BADARG;
    uint32_t launches = 0, schedule = FOORT_SCHEDULE_ROUNDS;
    const int rc = run(ctx, meshes, outputs, n_images, geodesics, rounds, launches, schedule);
    foort_ctx_set_run_info(ctx, launches, schedule);
    return rc;
}
