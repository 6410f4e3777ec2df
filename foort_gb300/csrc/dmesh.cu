// Device-resident SquareSubdivisionMeshV2 (Mesh.h:285-423, Mesh.cpp:660-1186): the
// adaptive mesh's grid, values and pixel lists in device memory, so that a round's
// pixels go from the mesh to the integration kernels and the results back to the mesh
// without leaving the GPU.
//
// State, for the R x R grid of the mesh (R = (sqrt(InitialPixels) - 1) 2^(MaxSubdivide-1)
// + 1, Mesh.cpp:671-672), one entry per grid cell:
//   level[cell]  -1: no pixel; 0: a pixel that is no square's top-left corner; s >= 1:
//                the top-left corner of a square of side 2^(MaxSubdivide - s)
//   value[cell]  the pixel's value (Geodesic::getDiagnosticFinalValue, Geodesic.cpp:141-149)
//   claim[cell]  scratch of the subdivision step (below)
// and the reference's lists: the round's queue (pixels to integrate), "updating" (pixels
// whose square needs a weight) and "active" (squares with a positive weight that are not
// yet subdivided).
//
// End of a round (EndCurrentLoop, Mesh.cpp:1092-1186):
//   1. each queued pixel's value goes to its cell;
//   2. each updating pixel's square gets its weight, the largest FinalDataValDistance
//      from the top-left corner's value to the other three corners' (UpdateAllWeights,
//      Mesh.cpp:809-841); the positive ones are appended to the active list in the
//      updating list's order (a stable compaction);
//   3. the active list is sorted by weight (descending), then level (ascending), with the
//      reference's comparator. std::sort is not stable, and the order it leaves equal keys
//      in -- the rule with FourColorScreen, whose weights are 0 or 1 -- decides which
//      squares the next step takes. FOORT_DMESH_ORDER_REFERENCE keeps a host copy of the
//      active list (24 bytes per square: weight, level, cell) and sorts it with
//      libstdc++'s std::sort, which, given the same sequence, leaves it in the
//      reference's order; only the new squares come from the device and only the squares
//      to subdivide go back. FOORT_DMESH_ORDER_DEVICE sorts on the device with the cell
//      as a last key: the same rounds wherever no tie straddles the cut.
//   4. the first IterationPixels squares are subdivided (SubdivideAndQueue,
//      Mesh.cpp:944-1086), all at once. Square i has five candidate pixels in slots
//      5i + (0..4): the top and left edge midpoints and the centre get the new level; the
//      right and bottom edge midpoints are created at level 0 where absent. Levels rise
//      by atomicMax, which gives every cell the level the reference's sequential pass
//      leaves. A cell absent at the start of the step is created by the first slot that
//      names it -- the lowest, found by atomicMin on claim[cell] -- as in the reference,
//      which creates a pixel the first time its neighbour links do not find one; the new
//      queue is the stable compaction of the creating slots, i.e. the reference's
//      creation order. The updating list is p1, p2, p4, p5 of each square whose new
//      level is below MaxSubdivide, in square order.
//   5. with a finite MaxPixels, the queue is cut to the pixels left, in that order.
// With FOORT_DMESH_ORDER_REFERENCE the rounds hand out the reference's pixels in the
// reference's order.
//
// A whole run (foort_gpu_run_dmesh) launches by level waves where the mesh's MaxPixels is
// unlimited: a device copy of the mesh with unlimited IterationPixels hands out one
// subdivision level per round, each launch also takes the next level's candidates (the
// five of every square awaiting its weight, deduplicated on the device) while it stays
// within the context's lookahead cap, and every result is kept in a pool indexed by
// slot[cell]. The mesh's own rounds then gather their results from the pool.
#include <cuda_runtime.h>

#include <cub/device/device_merge_sort.cuh>
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_select.cuh>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/foort_gpu.h"
#include "diag_order.h"

namespace {

struct ActiveSq {
    double weight;
    int32_t level;
    uint32_t pad;
    uint64_t cell;
};
static_assert(sizeof(ActiveSq) == 24, "ActiveSq layout");

// The reference's comparator (Mesh.cpp:1137-1148).
struct RefOrder {
    bool operator()(const ActiveSq& a, const ActiveSq& b) const {
        if (a.weight > b.weight) return true;
        if (a.weight == b.weight && a.level < b.level) return true;
        return false;
    }
};

// The same, then the cell: a strict total order for the device sort.
struct DeviceOrder {
    __host__ __device__ bool operator()(const ActiveSq& a, const ActiveSq& b) const {
        if (a.weight != b.weight) return a.weight > b.weight;
        if (a.level != b.level) return a.level < b.level;
        return a.cell < b.cell;
    }
};

struct PositiveWeight {
    __host__ __device__ bool operator()(const ActiveSq& a) const { return a.weight > 0.0; }
};

constexpr uint32_t kNoClaim = 0xFFFFFFFFu;

// FinalDataValDistance of the value diagnostic (Diagnostics.cpp:214-221, :395-401,
// :460-464).
__device__ __forceinline__ double value_distance(uint32_t value_diag, double a, double b) {
    if (value_diag == FOORT_DIAG_FOUR_COLOR_SCREEN) return fabs(a - b) < 1.0 ? 0.0 : 1.0;
    return fabs(a - b);
}

// std::max(a, b): b only where a < b, so a NaN in a is kept.
__device__ __forceinline__ double std_max(double a, double b) { return a < b ? b : a; }

__device__ __forceinline__ double result_value(uint32_t kind, const foort_result& r) {
    if (kind == FOORT_DIAG_FOUR_COLOR_SCREEN) return static_cast<double>(r.quadrant);
    if (kind == FOORT_DIAG_EQUATORIAL_PASSES) return static_cast<double>(r.equat_passes);
    if (kind == FOORT_DIAG_CLOSEST_RADIUS) return r.closest_r;
    return 0.0;
}

#define DM_FOR(i, n)                                                                  \
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; \
         i < (n); i += static_cast<uint64_t>(gridDim.x) * blockDim.x)

__global__ void k_scatter_results(const uint64_t* q, const foort_result* res, uint64_t n, uint32_t kind,
                                  double* value) {
    DM_FOR(i, n) value[q[i]] = result_value(kind, res[i]);
}

__global__ void k_scatter_values(const uint64_t* q, const double* v, uint64_t n, double* value) {
    DM_FOR(i, n) value[q[i]] = v[i];
}

// Step 2: the weight of each updating pixel's square (Mesh.cpp:809-841); its corners are
// `s` cells to the right, below and diagonally.
__global__ void k_weights(const uint64_t* upd, uint64_t nu, const int32_t* level, const double* value, uint64_t R,
                          int max_sub, uint32_t value_diag, ActiveSq* cand) {
    DM_FOR(i, nu) {
        const uint64_t c = upd[i];
        const int lvl = level[c];
        const uint64_t s = 1ull << (max_sub - lvl);
        const double v = value[c];
        const double d0 = value_distance(value_diag, v, value[c + s]);
        const double d1 = value_distance(value_diag, v, value[c + s * R]);
        const double d2 = value_distance(value_diag, v, value[c + s * R + s]);
        cand[i] = ActiveSq{std_max(d0, std_max(d1, d2)), lvl, 0u, c};
    }
}

struct Square {
    uint64_t c[5];  // p2, p4, p5, p6, p8
    uint64_t c1;
    int ns;
};

__device__ __forceinline__ Square square_of(const ActiveSq& a, uint64_t R, int max_sub) {
    Square q;
    q.c1 = a.cell;
    q.ns = a.level + 1;
    const uint64_t h = 1ull << (max_sub - q.ns);  // half the side
    q.c[0] = q.c1 + h;
    q.c[1] = q.c1 + h * R;
    q.c[2] = q.c[1] + h;
    q.c[3] = q.c[2] + h;
    q.c[4] = q.c[2] + h * R;
    return q;
}

// Step 4a: the lowest slot naming each absent cell.
__global__ void k_claim(const ActiveSq* sub, uint64_t k, const int32_t* level, uint64_t R, int max_sub,
                        uint32_t* claim) {
    DM_FOR(i, k) {
        const Square q = square_of(sub[i], R, max_sub);
#pragma unroll
        for (int j = 0; j < 5; ++j)
            if (level[q.c[j]] == -1) atomicMin(&claim[q.c[j]], static_cast<uint32_t>(5 * i + j));
    }
}

// Step 4b: new levels; the creating slots; the next updating list's slots.
__global__ void k_subdivide(const ActiveSq* sub, uint64_t k, int32_t* level, const uint32_t* claim, uint64_t R,
                            int max_sub, uint64_t* qslot, uint8_t* qflag, uint64_t* uslot, uint8_t* uflag) {
    DM_FOR(i, k) {
        const Square q = square_of(sub[i], R, max_sub);
        atomicMax(&level[q.c1], q.ns);
        atomicMax(&level[q.c[0]], q.ns);
        atomicMax(&level[q.c[1]], q.ns);
        atomicMax(&level[q.c[2]], q.ns);
        atomicMax(&level[q.c[3]], 0);
        atomicMax(&level[q.c[4]], 0);
#pragma unroll
        for (int j = 0; j < 5; ++j) {
            qslot[5 * i + j] = q.c[j];
            qflag[5 * i + j] = claim[q.c[j]] == static_cast<uint32_t>(5 * i + j) ? 1 : 0;
        }
        const uint8_t up = q.ns < max_sub ? 1 : 0;
        uslot[4 * i + 0] = q.c1;
        uslot[4 * i + 1] = q.c[0];
        uslot[4 * i + 2] = q.c[1];
        uslot[4 * i + 3] = q.c[2];
        uflag[4 * i + 0] = uflag[4 * i + 1] = uflag[4 * i + 2] = uflag[4 * i + 3] = up;
    }
}

// Step 4c: clear the claims of the created cells (the only cells that hold one).
__global__ void k_unclaim(const uint64_t* cells, const long long* n, uint32_t* claim) {
    const uint64_t cnt = static_cast<uint64_t>(*n);
    DM_FOR(i, cnt) claim[cells[i]] = kNoClaim;
}

__global__ void k_cells_to_pixels(const uint64_t* cells, uint64_t n, uint64_t R, uint32_t image, foort_pixel* px) {
    DM_FOR(i, n) {
        const uint64_t c = cells[i];
        px[i] = foort_pixel{image, 0u, c / R, c % R, R};
    }
}

// The seed grid (InitializeFirstGrid, Mesh.cpp:741-802): n x n pixels `scale` cells apart,
// level 1, or MaxSubdivide in the last row and column, queued row by row; the level-1
// ones are the updating list, in the same order.
__global__ void k_seed(uint64_t n, uint64_t scale, uint64_t R, int max_sub, int32_t* level, uint64_t* queue,
                       uint64_t* upd) {
    DM_FOR(i, n * n) {
        const uint64_t r = i / n, c = i % n;
        const uint64_t cell = r * scale * R + c * scale;
        const bool edge = r == n - 1 || c == n - 1;
        level[cell] = edge ? max_sub : 1;
        queue[i] = cell;
        if (!edge && max_sub > 1) upd[r * (n - 1) + c] = cell;
    }
}

// ---- level waves on the device (foort_gpu_run_dmesh with FOORT_SCHEDULE_WAVES)
constexpr uint32_t kNoSlot = 0xFFFFFFFFu;

// Cells of q without a stored result.
__global__ void k_flag_unstored(const uint64_t* q, uint64_t n, const uint32_t* slot, uint8_t* flag) {
    DM_FOR(i, n) flag[i] = slot[q[i]] == kNoSlot ? 1 : 0;
}

// The five candidates of each updating pixel's square (p2, p4, p5, p6, p8 of a square of
// half-side h = 2^(MaxSubdivide - level - 1)), flagged where no result is stored.
__global__ void k_candidates(const uint64_t* upd, uint64_t nu, const int32_t* level, const uint32_t* slot, uint64_t R,
                             int max_sub, uint64_t* out, uint8_t* flag) {
    DM_FOR(i, nu) {
        const uint64_t c = upd[i];
        const uint64_t h = 1ull << (max_sub - level[c] - 1);
        const uint64_t cand[5] = {c + h, c + h * R, c + h * R + h, c + h * R + 2 * h, c + 2 * h * R + h};
#pragma unroll
        for (int j = 0; j < 5; ++j) {
            out[5 * i + j] = cand[j];
            flag[5 * i + j] = slot[cand[j]] == kNoSlot ? 1 : 0;
        }
    }
}

// The launch's results are pool[base .. base + n): point the cells' slots at them.
__global__ void k_set_slots(const uint64_t* cells, uint64_t n, uint32_t base, uint32_t* slot) {
    DM_FOR(i, n) slot[cells[i]] = base + static_cast<uint32_t>(i);
}

// Values of the queued cells from their stored results.
__global__ void k_values_from_pool(const uint64_t* q, uint64_t n, const uint32_t* slot, const foort_result* pool,
                                   uint32_t kind, double* value) {
    DM_FOR(i, n) value[q[i]] = result_value(kind, pool[slot[q[i]]]);
}

// The round's results in the round's order.
__global__ void k_gather(const uint64_t* q, uint64_t n, const uint32_t* slot, const foort_result* pool,
                         foort_result* out) {
    DM_FOR(i, n) out[i] = pool[slot[q[i]]];
}

unsigned grid_for(uint64_t n) {
    return static_cast<unsigned>(std::max<uint64_t>(1, std::min<uint64_t>((n + 255) / 256, 152ull * 16)));
}

uint64_t pow2(int e) { return 1ull << e; }

}  // namespace

struct foort_dmesh {
    uint64_t R = 0, initial = 0, initial_arg = 0, iteration = 0, max_pixels = 0, left_px = 0;
    int max_sub = 1;
    bool infinite = true;
    uint32_t value_diag = 0, value_kind = 0, image = 0, order = 0;
    cudaStream_t st = nullptr;
    // grid
    int32_t* level = nullptr;
    double* value = nullptr;
    uint32_t* claim = nullptr;
    // lists, with their capacities in entries
    uint64_t* qcells = nullptr;
    foort_pixel* qpx = nullptr;
    uint64_t cap_q = 0;
    uint64_t* upd = nullptr;
    uint64_t cap_upd = 0;
    ActiveSq* cand = nullptr;
    ActiveSq* newact = nullptr;
    uint64_t cap_w = 0;
    ActiveSq* sub = nullptr;
    uint64_t cap_k = 0;
    uint64_t* qslot = nullptr;
    uint64_t* uslot = nullptr;
    uint64_t cap_slots = 0;
    uint8_t* qflag = nullptr;
    uint8_t* uflag = nullptr;
    uint64_t cap_flags = 0;
    ActiveSq* active = nullptr;  // FOORT_DMESH_ORDER_DEVICE
    ActiveSq* active_tmp = nullptr;
    uint64_t cap_a = 0;
    long long* num = nullptr;  // device counters: 0 new actives, 1 queue, 2 updating, 3 scratch
    void* tmp = nullptr;
    size_t tmp_bytes = 0;
    std::vector<ActiveSq> mirror;  // FOORT_DMESH_ORDER_REFERENCE: the active list
    bool unordered = false;        // wave copy: the queue's order does not matter
    uint64_t n_queue = 0, n_upd = 0, n_active = 0, rounds = 0, integrated = 0;
    bool values_set = false;
    std::string err;
};

namespace {

int fail(foort_dmesh* m, cudaError_t e, const char* what) {
    m->err = std::string(what) + ": " + cudaGetErrorString(e);
    return FOORT_E_CUDA;
}

#define DM_CK(call)                                       \
    do {                                                  \
        cudaError_t e_ = (call);                          \
        if (e_ != cudaSuccess) return fail(m, e_, #call); \
    } while (0)

// Device buffer of at least `need` entries; contents are not kept.
template <class T>
int grow(foort_dmesh* m, T*& p, uint64_t& cap, uint64_t need, const char* what) {
    if (p && need <= cap) return FOORT_OK;
    const uint64_t n = std::max<uint64_t>({need, cap + cap / 2, 1});
    if (p) DM_CK(cudaFreeAsync(p, m->st));
    p = nullptr;
    cap = 0;
    const cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&p), n * sizeof(T), m->st);
    if (e != cudaSuccess) return fail(m, e, what);
    cap = n;
    return FOORT_OK;
}

// Two buffers of one capacity.
template <class T, class U>
int grow2(foort_dmesh* m, T*& p, U*& q, uint64_t& cap, uint64_t need, const char* what) {
    if (p && q && need <= cap) return FOORT_OK;
    uint64_t c1 = p && q ? cap : 0, c2 = c1;
    int rc = grow(m, p, c1, need, what);
    if (!rc) rc = grow(m, q, c2, c1, what);
    cap = rc ? 0 : std::min(c1, c2);
    return rc;
}

int ensure_tmp(foort_dmesh* m, size_t bytes) {
    if (m->tmp && bytes <= m->tmp_bytes) return FOORT_OK;
    if (m->tmp) DM_CK(cudaFreeAsync(m->tmp, m->st));
    m->tmp = nullptr;
    m->tmp_bytes = 0;
    DM_CK(cudaMallocAsync(&m->tmp, std::max<size_t>(bytes, 16), m->st));
    m->tmp_bytes = std::max<size_t>(bytes, 16);
    return FOORT_OK;
}

int fetch(foort_dmesh* m, long long* h, int first, int count) {
    DM_CK(cudaMemcpyAsync(h + first, m->num + first, count * sizeof(long long), cudaMemcpyDeviceToHost, m->st));
    DM_CK(cudaStreamSynchronize(m->st));
    return FOORT_OK;
}

void free_all(foort_dmesh* m) {
    void* ptrs[] = {m->level, m->value, m->claim, m->qcells, m->qpx, m->upd, m->cand, m->newact, m->sub,
                    m->qslot, m->uslot, m->qflag, m->uflag, m->active, m->active_tmp, m->num, m->tmp};
    for (void* p : ptrs)
        if (p) cudaFreeAsync(p, m->st);
    cudaStreamSynchronize(m->st);
}

// Steps 2-3 with FOORT_DMESH_ORDER_REFERENCE: the new squares join the host copy of the
// active list, which std::sort orders; the first k go to the device.
int order_reference(foort_dmesh* m, uint64_t n_new, uint64_t& k) {
    const uint64_t old = m->mirror.size();
    m->mirror.resize(old + n_new);
    if (n_new) {
        DM_CK(cudaMemcpyAsync(m->mirror.data() + old, m->newact, n_new * sizeof(ActiveSq), cudaMemcpyDeviceToHost,
                              m->st));
        DM_CK(cudaStreamSynchronize(m->st));
    }
    std::sort(m->mirror.begin(), m->mirror.end(), RefOrder());
    k = std::min<uint64_t>(m->mirror.size(), m->iteration);
    int rc = grow(m, m->sub, m->cap_k, k, "cudaMallocAsync(sub)");
    if (rc) return rc;
    if (k) {
        DM_CK(cudaMemcpyAsync(m->sub, m->mirror.data(), k * sizeof(ActiveSq), cudaMemcpyHostToDevice, m->st));
        // the host copy's first k entries are erased next: the copy must have read them
        DM_CK(cudaStreamSynchronize(m->st));
    }
    m->mirror.erase(m->mirror.begin(), m->mirror.begin() + static_cast<std::ptrdiff_t>(k));
    m->n_active = m->mirror.size();
    return FOORT_OK;
}

// Steps 2-3 with FOORT_DMESH_ORDER_DEVICE: the active list stays on the device.
int order_device(foort_dmesh* m, uint64_t n_new, uint64_t& k) {
    const uint64_t n = m->n_active + n_new;
    if (!m->active || n > m->cap_a) {
        ActiveSq *a = nullptr, *b = nullptr;
        uint64_t cap = 0;
        int rc = grow2(m, a, b, cap, std::max<uint64_t>(n, m->cap_a + m->cap_a / 2), "cudaMallocAsync(active)");
        if (rc) return rc;
        if (m->n_active)
            DM_CK(cudaMemcpyAsync(a, m->active, m->n_active * sizeof(ActiveSq), cudaMemcpyDeviceToDevice, m->st));
        if (m->active) DM_CK(cudaFreeAsync(m->active, m->st));
        if (m->active_tmp) DM_CK(cudaFreeAsync(m->active_tmp, m->st));
        m->active = a;
        m->active_tmp = b;
        m->cap_a = cap;
    }
    if (n_new)
        DM_CK(cudaMemcpyAsync(m->active + m->n_active, m->newact, n_new * sizeof(ActiveSq), cudaMemcpyDeviceToDevice,
                              m->st));
    if (n > 1 && !(m->unordered && m->iteration >= n)) {
        size_t bytes = 0;
        DM_CK(cub::DeviceMergeSort::SortKeysCopy(nullptr, bytes, m->active, m->active_tmp, static_cast<int64_t>(n),
                                                 DeviceOrder(), m->st));
        int rc = ensure_tmp(m, bytes);
        if (rc) return rc;
        DM_CK(cub::DeviceMergeSort::SortKeysCopy(m->tmp, bytes, m->active, m->active_tmp, static_cast<int64_t>(n),
                                                 DeviceOrder(), m->st));
        std::swap(m->active, m->active_tmp);
    }
    k = std::min<uint64_t>(n, m->iteration);
    int rc = grow(m, m->sub, m->cap_k, k, "cudaMallocAsync(sub)");
    if (rc) return rc;
    if (k) DM_CK(cudaMemcpyAsync(m->sub, m->active, k * sizeof(ActiveSq), cudaMemcpyDeviceToDevice, m->st));
    if (k && n > k) {
        DM_CK(cudaMemcpyAsync(m->active_tmp, m->active + k, (n - k) * sizeof(ActiveSq), cudaMemcpyDeviceToDevice,
                              m->st));
        std::swap(m->active, m->active_tmp);
    }
    m->n_active = n - k;
    return FOORT_OK;
}

// Cells in ascending order (in and out distinct).
int sort_cells(foort_dmesh* m, const uint64_t* in, uint64_t* out, uint64_t n) {
    if (n == 0) return FOORT_OK;
    size_t bytes = 0;
    DM_CK(cub::DeviceRadixSort::SortKeys(nullptr, bytes, in, out, static_cast<int64_t>(n), 0, 64, m->st));
    const int rc = ensure_tmp(m, bytes);
    if (rc) return rc;
    DM_CK(cub::DeviceRadixSort::SortKeys(m->tmp, bytes, in, out, static_cast<int64_t>(n), 0, 64, m->st));
    return FOORT_OK;
}

template <class T>
int select_flagged(foort_dmesh* m, const T* in, const uint8_t* flags, T* out, long long* count, uint64_t n) {
    size_t bytes = 0;
    DM_CK(cub::DeviceSelect::Flagged(nullptr, bytes, in, flags, out, count, static_cast<int64_t>(n), m->st));
    int rc = ensure_tmp(m, bytes);
    if (rc) return rc;
    DM_CK(cub::DeviceSelect::Flagged(m->tmp, bytes, in, flags, out, count, static_cast<int64_t>(n), m->st));
    return FOORT_OK;
}

}  // namespace

extern "C" {

int foort_dmesh_create_v2(uint64_t max_pixels, uint64_t initial_pixels, int32_t max_subdivide,
                          uint64_t iteration_pixels, int32_t initial_sub_to_final, uint32_t diag_flags,
                          uint32_t value_diag, uint32_t image, uint32_t order, void* cuda_stream, foort_dmesh** out) {
    (void)initial_sub_to_final;  // stored by the reference's V2 mesh but never read
    if (!out) return FOORT_E_BADARG;
    *out = nullptr;
    if (max_subdivide < 1 || max_subdivide > 30 || initial_pixels < 4 || order > FOORT_DMESH_ORDER_DEVICE)
        return FOORT_E_BADARG;
    const std::vector<uint32_t> diag = foort::diagnostic_order(diag_flags, value_diag);
    if (diag.empty() || diag[0] == FOORT_DIAG_GEODESIC_POSITION || value_diag == FOORT_DIAG_GEODESIC_POSITION)
        return FOORT_E_UNSUPPORTED;
    const uint64_t n = static_cast<uint64_t>(std::sqrt(static_cast<double>(initial_pixels)));
    const uint64_t scale = pow2(max_subdivide - 1);
    const double Rd = (std::sqrt(static_cast<double>(initial_pixels)) - 1) * static_cast<double>(scale) + 1;
    if (!(Rd * Rd <= static_cast<double>(FOORT_DMESH_MAX_CELLS))) return FOORT_E_BADARG;
    foort_dmesh* m = new foort_dmesh();
    m->R = static_cast<uint64_t>(Rd);
    m->initial = n * n;
    m->initial_arg = initial_pixels;
    m->iteration = iteration_pixels;
    m->max_pixels = max_pixels;
    m->left_px = max_pixels;
    m->infinite = max_pixels == 0;
    m->max_sub = max_subdivide;
    m->value_diag = value_diag;
    m->value_kind = diag[0];
    m->image = image;
    m->order = order;
    m->st = static_cast<cudaStream_t>(cuda_stream);
    const uint64_t cells = m->R * m->R;
    auto init = [&]() -> int {
        uint64_t c0 = 0, c1 = 0, c2 = 0, c3 = 0;
        int rc = grow(m, m->level, c0, cells, "cudaMallocAsync(level)");
        if (!rc) rc = grow(m, m->value, c1, cells, "cudaMallocAsync(value)");
        if (!rc) rc = grow(m, m->claim, c2, cells, "cudaMallocAsync(claim)");
        if (!rc) rc = grow(m, m->num, c3, 4, "cudaMallocAsync(counters)");
        if (!rc) rc = grow2(m, m->qcells, m->qpx, m->cap_q, n * n, "cudaMallocAsync(queue)");
        if (!rc) rc = grow(m, m->upd, m->cap_upd, (n - 1) * (n - 1), "cudaMallocAsync(updating)");
        if (rc) return rc;
        DM_CK(cudaMemsetAsync(m->level, 0xFF, cells * sizeof(int32_t), m->st));
        DM_CK(cudaMemsetAsync(m->value, 0, cells * sizeof(double), m->st));
        DM_CK(cudaMemsetAsync(m->claim, 0xFF, cells * sizeof(uint32_t), m->st));
        k_seed<<<grid_for(n * n), 256, 0, m->st>>>(n, scale, m->R, max_subdivide, m->level, m->qcells, m->upd);
        DM_CK(cudaGetLastError());
        k_cells_to_pixels<<<grid_for(n * n), 256, 0, m->st>>>(m->qcells, n * n, m->R, m->image, m->qpx);
        DM_CK(cudaGetLastError());
        DM_CK(cudaStreamSynchronize(m->st));
        return FOORT_OK;
    };
    const int rc = init();
    if (rc) {
        free_all(m);
        delete m;
        return rc;
    }
    m->n_queue = n * n;
    m->n_upd = max_subdivide > 1 ? (n - 1) * (n - 1) : 0;
    if (!m->infinite) m->left_px -= m->n_queue;  // unsigned, as the reference's count
    *out = m;
    return FOORT_OK;
}

int foort_dmesh_is_finished(const foort_dmesh* m) { return m ? (m->n_queue == 0 ? 1 : 0) : FOORT_E_BADARG; }
uint64_t foort_dmesh_cur_nr_geodesics(const foort_dmesh* m) { return m ? m->n_queue : 0; }
uint64_t foort_dmesh_grid(const foort_dmesh* m) { return m ? m->R : 0; }
uint64_t foort_dmesh_rounds(const foort_dmesh* m) { return m ? m->rounds : 0; }
uint64_t foort_dmesh_active(const foort_dmesh* m) { return m ? m->n_active : 0; }
const foort_pixel* foort_dmesh_pixels(const foort_dmesh* m) { return m ? m->qpx : nullptr; }
const char* foort_dmesh_last_error(const foort_dmesh* m) { return m ? m->err.c_str() : "mesh is NULL"; }

int foort_dmesh_get_pixels(foort_dmesh* m, foort_pixel* out) {
    if (!m || (m->n_queue && !out)) return FOORT_E_BADARG;
    if (m->n_queue) {
        DM_CK(cudaMemcpyAsync(out, m->qpx, m->n_queue * sizeof(foort_pixel), cudaMemcpyDeviceToHost, m->st));
        DM_CK(cudaStreamSynchronize(m->st));
    }
    return FOORT_OK;
}

int foort_dmesh_set_results(foort_dmesh* m, const foort_result* d_res, uint64_t n) {
    if (!m || (n && !d_res) || n != m->n_queue) return FOORT_E_BADARG;
    if (n) {
        k_scatter_results<<<grid_for(n), 256, 0, m->st>>>(m->qcells, d_res, n, m->value_kind, m->value);
        DM_CK(cudaGetLastError());
    }
    m->values_set = true;
    return FOORT_OK;
}

int foort_dmesh_set_values(foort_dmesh* m, const double* d_values, uint64_t n) {
    if (!m || (n && !d_values) || n != m->n_queue) return FOORT_E_BADARG;
    if (n) {
        k_scatter_values<<<grid_for(n), 256, 0, m->st>>>(m->qcells, d_values, n, m->value);
        DM_CK(cudaGetLastError());
    }
    m->values_set = true;
    return FOORT_OK;
}

int foort_dmesh_end_current_loop(foort_dmesh* m) {
    if (!m) return FOORT_E_BADARG;
    if (m->n_queue == 0) return FOORT_OK;
    if (!m->values_set) {
        m->err = "the round's values were not set";
        return FOORT_E_BADARG;
    }
    m->values_set = false;
    ++m->rounds;
    m->integrated += m->n_queue;
    m->n_queue = 0;
    if (!m->infinite && m->left_px == 0) return FOORT_OK;
    long long h[3] = {0, 0, 0};
    int rc;
    // 2. weights, and the positive ones in order
    uint64_t n_new = 0;
    if (m->n_upd) {
        if ((rc = grow2(m, m->cand, m->newact, m->cap_w, m->n_upd, "cudaMallocAsync(weights)"))) return rc;
        k_weights<<<grid_for(m->n_upd), 256, 0, m->st>>>(m->upd, m->n_upd, m->level, m->value, m->R, m->max_sub,
                                                         m->value_diag, m->cand);
        DM_CK(cudaGetLastError());
        size_t bytes = 0;
        DM_CK(cub::DeviceSelect::If(nullptr, bytes, m->cand, m->newact, m->num, static_cast<int64_t>(m->n_upd),
                                    PositiveWeight(), m->st));
        if ((rc = ensure_tmp(m, bytes))) return rc;
        DM_CK(cub::DeviceSelect::If(m->tmp, bytes, m->cand, m->newact, m->num, static_cast<int64_t>(m->n_upd),
                                    PositiveWeight(), m->st));
        if ((rc = fetch(m, h, 0, 1))) return rc;
        n_new = static_cast<uint64_t>(h[0]);
    }
    m->n_upd = 0;
    // 3. order
    uint64_t k = 0;
    rc = m->order == FOORT_DMESH_ORDER_REFERENCE ? order_reference(m, n_new, k) : order_device(m, n_new, k);
    if (rc) return rc;
    if (k == 0) return FOORT_OK;
    // 4. subdivide
    if ((rc = grow2(m, m->qslot, m->uslot, m->cap_slots, 5 * k, "cudaMallocAsync(slots)"))) return rc;
    if ((rc = grow2(m, m->qflag, m->uflag, m->cap_flags, 5 * k, "cudaMallocAsync(flags)"))) return rc;
    if ((rc = grow2(m, m->qcells, m->qpx, m->cap_q, 5 * k, "cudaMallocAsync(queue)"))) return rc;
    if ((rc = grow(m, m->upd, m->cap_upd, 4 * k, "cudaMallocAsync(updating)"))) return rc;
    k_claim<<<grid_for(k), 256, 0, m->st>>>(m->sub, k, m->level, m->R, m->max_sub, m->claim);
    DM_CK(cudaGetLastError());
    k_subdivide<<<grid_for(k), 256, 0, m->st>>>(m->sub, k, m->level, m->claim, m->R, m->max_sub, m->qslot, m->qflag,
                                                m->uslot, m->uflag);
    DM_CK(cudaGetLastError());
    if ((rc = select_flagged(m, m->qslot, m->qflag, m->qcells, m->num + 1, 5 * k))) return rc;
    if ((rc = select_flagged(m, m->uslot, m->uflag, m->upd, m->num + 2, 4 * k))) return rc;
    k_unclaim<<<grid_for(5 * k), 256, 0, m->st>>>(m->qcells, m->num + 1, m->claim);
    DM_CK(cudaGetLastError());
    if ((rc = fetch(m, h, 1, 2))) return rc;
    m->n_queue = static_cast<uint64_t>(h[1]);
    m->n_upd = static_cast<uint64_t>(h[2]);
    // 5. a finite MaxPixels cuts the queue
    if (!m->infinite) {
        m->n_queue = std::min<uint64_t>(m->n_queue, m->left_px);
        m->left_px -= m->n_queue;
    }
    if (m->n_queue) {
        k_cells_to_pixels<<<grid_for(m->n_queue), 256, 0, m->st>>>(m->qcells, m->n_queue, m->R, m->image, m->qpx);
        DM_CK(cudaGetLastError());
    }
    return FOORT_OK;
}

void foort_dmesh_destroy(foort_dmesh* m) {
    if (!m) return;
    free_all(m);
    delete m;
}

}  // extern "C"

// engine.cu (internal)
extern "C" {
uint32_t foort_ctx_schedule(const foort_ctx* ctx);
uint64_t foort_ctx_budget(const foort_ctx* ctx);
uint64_t foort_ctx_lookahead(const foort_ctx* ctx);
void foort_ctx_set_run_info(foort_ctx* ctx, uint32_t launches, uint32_t schedule);
}

namespace {

// Results of a run's pixels on the device: slot[cell] indexes pool (kNoSlot: none yet).
struct DevStore {
    uint32_t* slot = nullptr;
    foort_result* pool = nullptr;
    uint64_t cap = 0, used = 0;
    uint64_t* list = nullptr;  // launch list (cells) and its scratch
    uint64_t* sorted = nullptr;
    uint8_t* flag = nullptr;
    foort_pixel* px = nullptr;
    uint64_t cap_list = 0;
};

void free_store(DevStore& S, cudaStream_t st) {
    void* ptrs[] = {S.slot, S.pool, S.list, S.sorted, S.flag, S.px};
    for (void* p : ptrs)
        if (p) cudaFreeAsync(p, st);
    cudaStreamSynchronize(st);
}

// Room for `need` more results in the pool, keeping those stored.
int grow_pool(foort_dmesh* m, DevStore& S, uint64_t need) {
    if (S.used + need <= S.cap && S.pool) return FOORT_OK;
    const uint64_t cap = std::max<uint64_t>(S.used + need, 2 * S.cap);
    if (cap >= kNoSlot) {
        m->err = "too many results for 32-bit slots";
        return FOORT_E_BADARG;
    }
    foort_result* p = nullptr;
    DM_CK(cudaMallocAsync(reinterpret_cast<void**>(&p), cap * sizeof(foort_result), m->st));
    if (S.used) DM_CK(cudaMemcpyAsync(p, S.pool, S.used * sizeof(foort_result), cudaMemcpyDeviceToDevice, m->st));
    if (S.pool) DM_CK(cudaFreeAsync(S.pool, m->st));
    S.pool = p;
    S.cap = cap;
    return FOORT_OK;
}

int grow_list(foort_dmesh* m, DevStore& S, uint64_t need) {
    if (S.list && need <= S.cap_list) return FOORT_OK;
    uint64_t c1 = S.list ? S.cap_list : 0, c2 = c1, c3 = c1, c4 = c1;
    int rc = grow(m, S.list, c1, need, "cudaMallocAsync(launch list)");
    if (!rc) rc = grow(m, S.sorted, c2, c1, "cudaMallocAsync(launch list)");
    if (!rc) rc = grow(m, S.flag, c3, c1, "cudaMallocAsync(launch list)");
    if (!rc) rc = grow(m, S.px, c4, c1, "cudaMallocAsync(launch list)");
    S.cap_list = rc ? 0 : c1;
    return rc;
}

// Integrate the cells of S.list[0, n) of image `image` (one launch) and store the results.
int launch_cells(foort_ctx* ctx, foort_dmesh* m, DevStore& S, uint64_t n, uint32_t& launches) {
    int rc = grow_pool(m, S, n);
    if (rc) return rc;
    k_cells_to_pixels<<<grid_for(n), 256, 0, m->st>>>(S.list, n, m->R, m->image, S.px);
    DM_CK(cudaGetLastError());
    if ((rc = foort_gpu_integrate_async(ctx, S.px, n, S.pool + S.used, m->st))) return rc;
    ++launches;
    if ((rc = foort_gpu_sync(ctx))) return rc;
    k_set_slots<<<grid_for(n), 256, 0, m->st>>>(S.list, n, static_cast<uint32_t>(S.used), S.slot);
    DM_CK(cudaGetLastError());
    S.used += n;
    return FOORT_OK;
}

// The queued cells of `q` without a result, compacted into S.list; returns the count.
int unstored(foort_dmesh* m, DevStore& S, const uint64_t* q, uint64_t nq, uint64_t& n) {
    n = 0;
    if (!nq) return FOORT_OK;
    int rc = grow_list(m, S, nq);
    if (rc) return rc;
    k_flag_unstored<<<grid_for(nq), 256, 0, m->st>>>(q, nq, S.slot, S.flag);
    DM_CK(cudaGetLastError());
    if ((rc = select_flagged(m, q, S.flag, S.list, m->num + 3, nq))) return rc;
    long long h[4];
    if ((rc = fetch(m, h, 3, 1))) return rc;
    n = static_cast<uint64_t>(h[3]);
    return FOORT_OK;
}

// The wave schedule: the level waves of a copy of `m` with unlimited IterationPixels, each
// launch also taking the next wave's candidates while it stays within the lookahead cap;
// then m's own rounds, each with its results gathered from the store.
int run_dmesh_waves(foort_ctx* ctx, foort_dmesh* m, foort_result* d_out, uint64_t cap_out,
                    foort_dmesh_round_fn on_round, void* user, uint64_t& total, uint32_t& nr, uint32_t& launches) {
    foort_dmesh* w = nullptr;
    int rc = foort_dmesh_create_v2(0, m->initial_arg, m->max_sub, UINT64_MAX, 0, FOORT_DIAG_FOUR_COLOR_SCREEN,
                                   FOORT_DIAG_FOUR_COLOR_SCREEN, m->image, FOORT_DMESH_ORDER_DEVICE, m->st, &w);
    if (rc) return rc;
    w->value_diag = m->value_diag;
    w->value_kind = m->value_kind;
    w->unordered = true;
    DevStore S;
    auto done = [&](int code) {
        free_store(S, m->st);
        foort_dmesh_destroy(w);
        return code;
    };
    const uint64_t cells = m->R * m->R, ahead = foort_ctx_lookahead(ctx);
    uint64_t c0 = 0;
    if ((rc = grow(m, S.slot, c0, cells, "cudaMallocAsync(slots)"))) return done(rc);
    DM_CK(cudaMemsetAsync(S.slot, 0xFF, cells * sizeof(uint32_t), m->st));
    while (w->n_queue) {
        // every list of this wave in one allocation round: the launch list holds the wave's
        // cells without a result and then at most nc candidates; the scratch list holds
        // the nc raw candidates and their compaction
        const uint64_t nc = ahead > 0 ? 5 * w->n_upd : 0;
        if ((rc = grow_list(m, S, std::max<uint64_t>(w->n_queue + nc, 2 * nc)))) return done(rc);
        uint64_t n = 0;
        if ((rc = unstored(m, S, w->qcells, w->n_queue, n))) return done(rc);
        if (n) {
            const uint64_t n_todo = n;
            if (ahead > n_todo && nc) {
                // candidates: 5 per updating pixel, those without a result, each once
                uint64_t* raw = S.sorted;       // nc raw candidates, later their sorted copy
                uint64_t* kept = S.sorted + nc;  // those without a result
                k_candidates<<<grid_for(w->n_upd), 256, 0, m->st>>>(w->upd, w->n_upd, w->level, S.slot, m->R,
                                                                    m->max_sub, raw, S.flag);
                DM_CK(cudaGetLastError());
                if ((rc = select_flagged(m, raw, S.flag, kept, m->num + 3, nc))) return done(rc);
                long long h[4];
                if ((rc = fetch(m, h, 3, 1))) return done(rc);
                const uint64_t nf = static_cast<uint64_t>(h[3]);
                if (nf) {  // neighbouring squares share edge midpoints: each cell once
                    if ((rc = sort_cells(m, kept, raw, nf))) return done(rc);
                    size_t bytes = 0;
                    DM_CK(cub::DeviceSelect::Unique(nullptr, bytes, raw, S.list + n_todo, m->num + 3,
                                                    static_cast<int64_t>(nf), m->st));
                    if ((rc = ensure_tmp(m, bytes))) return done(rc);
                    DM_CK(cub::DeviceSelect::Unique(m->tmp, bytes, raw, S.list + n_todo, m->num + 3,
                                                    static_cast<int64_t>(nf), m->st));
                    if ((rc = fetch(m, h, 3, 1))) return done(rc);
                    if (n_todo + static_cast<uint64_t>(h[3]) <= ahead) n = n_todo + static_cast<uint64_t>(h[3]);
                }
            }
            if ((rc = launch_cells(ctx, m, S, n, launches))) return done(rc);
        }
        k_values_from_pool<<<grid_for(w->n_queue), 256, 0, m->st>>>(w->qcells, w->n_queue, S.slot, S.pool,
                                                                     w->value_kind, w->value);
        DM_CK(cudaGetLastError());
        w->values_set = true;
        if ((rc = foort_dmesh_end_current_loop(w))) {
            m->err = w->err;
            return done(rc);
        }
    }
    // m's rounds from the store
    while (m->n_queue) {
        const uint64_t n = m->n_queue;
        if (n > cap_out) {
            m->err = "the result buffer holds " + std::to_string(cap_out) + " results, the round has " +
                     std::to_string(n);
            return done(FOORT_E_BADARG);
        }
        uint64_t miss = 0;
        if ((rc = unstored(m, S, m->qcells, n, miss))) return done(rc);
        if (miss && (rc = launch_cells(ctx, m, S, miss, launches))) return done(rc);
        k_gather<<<grid_for(n), 256, 0, m->st>>>(m->qcells, n, S.slot, S.pool, d_out);
        DM_CK(cudaGetLastError());
        DM_CK(cudaStreamSynchronize(m->st));
        if (on_round && (rc = on_round(user, m->qpx, d_out, n, nr))) return done(rc);
        if ((rc = foort_dmesh_set_results(m, d_out, n))) return done(rc);
        if ((rc = foort_dmesh_end_current_loop(m))) return done(rc);
        total += n;
        ++nr;
    }
    return done(FOORT_OK);
}

}  // namespace

extern "C" {

int foort_gpu_run_dmesh(foort_ctx* ctx, foort_dmesh* m, foort_result* d_out, uint64_t cap_out,
                        foort_dmesh_round_fn on_round, void* user, uint64_t* geodesics, uint32_t* rounds) {
    if (!ctx || !m || !d_out) return FOORT_E_BADARG;
    uint64_t total = 0;
    uint32_t nr = 0, launches = 0;
    if (foort_ctx_schedule(ctx) == FOORT_SCHEDULE_WAVES && m->infinite && m->rounds == 0 && foort_ctx_budget(ctx) == 0) {
        const int rc = run_dmesh_waves(ctx, m, d_out, cap_out, on_round, user, total, nr, launches);
        foort_ctx_set_run_info(ctx, launches, FOORT_SCHEDULE_WAVES);
        if (rc) return rc;
        if (geodesics) *geodesics = total;
        if (rounds) *rounds = nr;
        return FOORT_OK;
    }
    while (m->n_queue) {
        const uint64_t n = m->n_queue;
        if (n > cap_out) {
            m->err = "the result buffer holds " + std::to_string(cap_out) + " results, the round has " +
                     std::to_string(n);
            return FOORT_E_BADARG;
        }
        int rc = foort_gpu_integrate_async(ctx, m->qpx, n, d_out, m->st);
        if (rc) return rc;
        ++launches;
        foort_ctx_set_run_info(ctx, launches, FOORT_SCHEDULE_ROUNDS);
        if ((rc = foort_gpu_sync(ctx))) return rc;
        if (on_round && (rc = on_round(user, m->qpx, d_out, n, nr))) return rc;
        if ((rc = foort_dmesh_set_results(m, d_out, n))) return rc;
        if ((rc = foort_dmesh_end_current_loop(m))) return rc;
        total += n;
        ++nr;
    }
    foort_ctx_set_run_info(ctx, launches, FOORT_SCHEDULE_ROUNDS);
    if (geodesics) *geodesics = total;
    if (rounds) *rounds = nr;
    return FOORT_OK;
}

}  // extern "C"
