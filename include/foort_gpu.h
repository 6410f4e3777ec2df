/*
 * foort_gpu.h -- C ABI of the GB300 geodesic-integration engine.
 *
 * The engine replaces the integration stage of a FOORT run: the OpenMP pixel loop
 * FOORT/Main.cpp:327-414 and everything it calls (ViewScreen initial conditions,
 * Geodesic::Reset/Update, the RK4/Verlet integrators, Metric::getChristoffel_udd,
 * the Terminations and the Diagnostics). One null geodesic per pixel is integrated
 * backward from the camera until a termination fires.
 *
 * Conventions (plain C, no C++ types or exceptions cross this boundary):
 *   - every function returns FOORT_OK (0) or a negative FOORT_E_* code;
 *   - buffers are owned by the caller;
 *   - one context per host thread; a context is not reentrant;
 *   - foort_gpu_last_error() gives a human-readable message for the last failure.
 *
 * The enum values, bitflags and termination codes are numerically identical to the
 * reference's, so a FOORT host that already holds TermBitflag / DiagBitflag values can
 * pass them through unchanged:
 *   Terminations.h:29-33 (TermBitflag), Terminations.h:48-67 (enum class Term),
 *   Diagnostics.h:33-37 (DiagBitflag).
 */
#ifndef FOORT_GPU_H
#define FOORT_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- return codes ---------------------------------------------------------------- */
#define FOORT_OK 0
#define FOORT_E_BADARG (-1)      /* invalid descriptor, pointer or size               */
#define FOORT_E_CUDA (-2)        /* a CUDA runtime call failed                         */
#define FOORT_E_BUDGET (-3)      /* the global step budget ran out; results partial   */
#define FOORT_E_NUMERIC (-4)     /* at least one geodesic hit a non-finite state       */
#define FOORT_E_CANCELLED (-5)   /* foort_gpu_cancel() stopped the launch             */
#define FOORT_E_UNSUPPORTED (-6) /* option combination this build does not implement  */
#define FOORT_E_IO (-7)          /* an output file could not be opened or written      */

/* ---- plugin ids ------------------------------------------------------------------ */
/* Metric classes of Metric.h:78-189; the names follow Config.cpp:153-290. */
#define FOORT_METRIC_KERR 0           /* params: a                                   */
#define FOORT_METRIC_FLAT 1           /* params: none                                */
#define FOORT_METRIC_RASHEED_LARSEN 2 /* params: m, a, p, q                          */
#define FOORT_METRIC_JOHANNSEN 3      /* params: a, alpha13, alpha22, alpha52, eps3  */
#define FOORT_METRIC_MANKO_NOVIKOV 4  /* params: a, alpha3                           */

/* GeodesicIntegratorFunc choices, Integrators.h:240-248 */
#define FOORT_INTEGRATOR_RK4 0
#define FOORT_INTEGRATOR_VERLET 1

/* Arithmetic of the integration kernel */
#define FOORT_PREC_FP64 0  /* every operation in FP64, finite-difference Christoffels   */
#define FOORT_PREC_MIXED 1 /* FP32 bulk with compensated state, FP64 where needed       */
/* Every step in FP64 with the analytic derivatives of the mixed kernel (its step_fp64):
 * the all-FP64 reference of the mixed kernel's own formulation, against which its
 * rounding error is measured. The reference's finite differences (FOORT_PREC_FP64,
 * Metric.cpp:14-55, h = 1e-7) lose digits where the metric is nearly constant: at
 * r ~ 100 a central difference of g_tt ~ -1 + 2/r keeps ~6 of its 16 digits. Engine
 * extension; no counterpart in the reference. */
#define FOORT_PREC_FP64_ANALYTIC 2

/* Options of the mixed-precision kernel (engine extension). By default its decisions
 * (terminations, equator crossings, closest radius) are taken by float-float
 * comparisons of its compensated (48-bit) state, which agree with FP64 comparisons
 * except within 2^-48 (relative) of a threshold. */
#define FOORT_MIXED_FP64_DECISIONS 0x1u    /* take them in FP64 on the exact double value  */
#define FOORT_MIXED_FP64_NEAR_HORIZON 0x2u /* whole steps in FP64 inside r_+ + margin       */
/* whole steps in FP64 near turning points of r and theta: where |dr/dlambda| is below
 * 5 % of r times the angular speed |u^theta| + |sin(theta) u^phi|, or |u^theta| below 5 %
 * of |sin(theta) u^phi| */
#define FOORT_MIXED_FP64_TURNING_POINTS 0x4u

/* TermBitflag, Terminations.h:29-33 */
#define FOORT_TERM_BOUNDARY_SPHERE 0x1u
#define FOORT_TERM_TIMEOUT 0x2u
#define FOORT_TERM_HORIZON 0x4u
#define FOORT_TERM_THETA_SINGULARITY 0x8u

/* DiagBitflag, Diagnostics.h:33-37 */
#define FOORT_DIAG_GEODESIC_POSITION 0x1u
#define FOORT_DIAG_FOUR_COLOR_SCREEN 0x2u
#define FOORT_DIAG_EQUATORIAL_PASSES 0x4u
#define FOORT_DIAG_CLOSEST_RADIUS 0x8u

/* enum class Term, Terminations.h:48-67 */
#define FOORT_TERMCODE_CONTINUE 0
#define FOORT_TERMCODE_HORIZON 1
#define FOORT_TERMCODE_BOUNDARY_SPHERE 2
#define FOORT_TERMCODE_TIMEOUT 3
#define FOORT_TERMCODE_THETA_SINGULARITY 4

/* Per-geodesic error bits (engine extension; the reference has no such report). */
#define FOORT_ERR_NONFINITE 0x1u   /* state became NaN/Inf; integration stopped      */
#define FOORT_ERR_VERLET_ITER 0x2u /* Verlet velocity iteration hit its cap           */
#define FOORT_ERR_BUDGET 0x4u      /* stopped by the global step budget (term = 0)    */
#define FOORT_ERR_CANCELLED 0x8u   /* stopped by foort_gpu_cancel (term = 0)          */
#define FOORT_ERR_UNFINISHED 0x10u /* never started (launch stopped before it)        */
#define FOORT_ERR_BADPIXEL 0x20u   /* image index out of range or grid < 2; skipped   */

/* Diagnostic update cadence, Diagnostics.h:50-55 (UpdateFrequency). */
typedef struct foort_update_freq {
    uint64_t every_n; /* >0: update every n steps; 0: only at start and/or finish */
    int32_t at_start;
    int32_t at_finish;
} foort_update_freq;

/* One image: a metric instance plus a camera (ViewScreen.h:44-51). */
typedef struct foort_image_desc {
    double metric_params[6]; /* see FOORT_METRIC_* for the order                    */
    double cam_pos[4];       /* (t, r, theta, phi); r is the ordinary radius         */
    double cam_dir[4];       /* only {0,-1,0,0} is supported, as in the reference     */
    double screen_size[2];
    double screen_center[2];
    double horizon_eps;      /* > 0: this image's Epsilon_Horizon, else the run's     */
} foort_image_desc;

/*
 * Everything the reference holds in process globals during a round (Main.cpp:211-235,
 * Config.cpp:11-28, Integrators.h:31-57), as one POD descriptor.
 */
typedef struct foort_run_desc {
    int32_t metric_id;     /* FOORT_METRIC_*                                         */
    int32_t rlog;          /* RLogScale: integrate u = ln r (Metric.cpp:134)         */
    int32_t integrator_id; /* FOORT_INTEGRATOR_*                                      */
    int32_t precision;     /* FOORT_PREC_*                                            */

    double epsilon;        /* Integrators::epsilon, default 0.03                     */
    double derivative_h;   /* Integrators::Derivative_hval, default 1e-7             */
    double smallest_step;  /* Integrators::SmallestPossibleStepsize, default 1e-12   */
    double verlet_tol;     /* Integrators::VerletVelocityTolerance, default 0.001    */

    uint32_t term_flags;   /* FOORT_TERM_* bitflag                                    */
    uint32_t diag_flags;   /* FOORT_DIAG_* bitflag                                    */
    uint32_t value_diag;   /* the one diagnostic whose value feeds the Mesh           */
    uint32_t mixed_options; /* FOORT_MIXED_* bits (mixed precision only)             */

    double horizon_eps;          /* HorizonTermOptions::AtHorizonEps (relative)      */
    uint64_t horizon_every;      /* UpdateEveryNSteps                                 */
    double boundary_radius;      /* BoundarySphereTermOptions::SphereRadius          */
    uint64_t boundary_every;
    uint64_t timeout_max_steps;  /* TimeOutTermOptions::MaxSteps                     */
    uint64_t timeout_every;
    double theta_eps;            /* ThetaSingularityTermOptions::ThetaSingEpsilon    */
    uint64_t theta_every;

    foort_update_freq equat_freq;     /* EquatorialPassesOptions                      */
    double equat_threshold;
    foort_update_freq closest_freq;   /* ClosestRadiusOptions                         */
    foort_update_freq geopos_freq;    /* GeodesicPositionOptions                      */
    uint64_t geopos_output_steps;

    double mixed_fp64_margin;        /* with FOORT_MIXED_FP64_NEAR_HORIZON: lanes with
                                        r < r_+ + margin take the whole step in FP64    */

    uint32_t n_images;               /* >= 1                                          */
    uint32_t reserved1;
    const foort_image_desc* images;  /* host array of n_images entries                */
} foort_run_desc;

/* One pixel to integrate. Unit screen point = (row, col) / (grid - 1)
 * (Mesh.cpp:49 SimpleSquareMesh, Mesh.cpp:671-672 SquareSubdivisionMeshV2). */
typedef struct foort_pixel {
    uint32_t image;
    uint32_t reserved;
    uint64_t row;
    uint64_t col;
    uint64_t grid;
} foort_pixel;

/* Per-geodesic result: the state Geodesic.h:114-122 ends with plus every diagnostic. */
typedef struct foort_result {
    int32_t term;          /* FOORT_TERMCODE_*                                       */
    uint32_t err;          /* FOORT_ERR_* bits                                       */
    uint64_t steps;        /* Geodesic::Update calls                                 */
    double lambda;         /* final affine parameter                                 */
    double pos[4];
    double vel[4];
    int32_t quadrant;      /* FourColorScreen (Diagnostics.cpp:159-200)              */
    int32_t equat_passes;  /* EquatorialPasses (Diagnostics.cpp:351-380)             */
    double closest_r;      /* ClosestRadius (Diagnostics.cpp:427-446)                */
} foort_result;

/* Counters of the last launch. */
typedef struct foort_stats {
    uint64_t geodesics;      /* geodesics finished                                  */
    uint64_t steps;          /* integration steps summed over geodesics             */
    uint64_t rhs_evals;      /* right-hand-side evaluations (Verlet iterations incl.) */
    uint64_t fp64_steps;     /* mixed kernel: steps taken on the FP64 path           */
    double kernel_ms;        /* device time of the last launch (CUDA events)         */
    uint32_t status;         /* FOORT_OK or the launch's FOORT_E_* code             */
    uint32_t n_blocks;
    uint32_t block_size;
    uint32_t lanes_per_geodesic; /* 1, or 2 where two lanes integrated each geodesic   */
    uint32_t refill_steps;   /* the launch's regrouping cadence (foort_launch_shape)   */
    uint32_t poll_steps;     /* its steps between budget / cancel polls               */
} foort_stats;

typedef struct foort_ctx foort_ctx;

/* Fill a descriptor with the reference's defaults (Config.cpp:127-1071): Kerr a=0.5,
 * RK4 eps=0.03, h=1e-7, hmin=1e-12, Verlet tol 1e-3, Boundary 1000 + TimeOut 1e4,
 * FourColorScreen as value diagnostic. `images` must be set by the caller. */
void foort_gpu_default_desc(foort_run_desc* desc);

/* Validate the descriptor, build the per-image camera frames (ViewScreen.cpp:10-73)
 * and the device-side constants. Replaces the object construction of Main.cpp:211-235. */
int foort_gpu_create(const foort_run_desc* desc, foort_ctx** out_ctx);

/* Integrate n pixels held in HOST memory and write n results to HOST memory.
 * Synchronous. Replaces one round of Main.cpp:348-402 (SetNewInitialConditions,
 * Geodesic::Reset, the Update loop, getDiagnosticFinalValue/getAllOutputStr). */
int foort_gpu_integrate(foort_ctx* ctx, const foort_pixel* px, uint64_t n, foort_result* out);

/* Same with DEVICE buffers, enqueued on `cuda_stream` (a cudaStream_t, 0 = legacy).
 * Returns once the launch is enqueued; foort_gpu_sync() waits and reports status. */
int foort_gpu_integrate_async(foort_ctx* ctx, const foort_pixel* d_px, uint64_t n,
                              foort_result* d_out, void* cuda_stream);

/* Allocation-free integration. No counterpart in the reference, which has no device code.
 *
 * For callers that may not allocate device memory: a plugin inside an application whose
 * pool allocator owns all of the GPU's memory and hands its plugins buffers rather than
 * the right to call cudaMalloc, or a pipeline that cannot take the device-wide
 * synchronisation that cudaMalloc / cudaFree may cause. foort_gpu_create() allocates its
 * image constants and launch counters with cudaMalloc; this call keeps them instead in
 * one fixed array of device memory that the library declares statically, of
 * FOORT_NOALLOC_SCRATCH_BYTES (room for FOORT_NOALLOC_MAX_IMAGES images). Every GPU on
 * which the library's device code is loaded holds that array until the process exits.
 *
 * The same kernels as foort_gpu_integrate_async() integrate n pixels from the DEVICE
 * buffer d_px into the DEVICE buffer d_out (both the caller's), on `cuda_stream`
 * (a cudaStream_t, 0 = legacy). The call allocates nothing on the device: no cudaMalloc,
 * cudaFree or allocating library routine. It copies the image constants into the array
 * and zeroes the counters on the stream before the launch.
 *   - More than FOORT_NOALLOC_MAX_IMAGES images: FOORT_E_BADARG, and nothing is launched.
 *   - The first call on a device, made with that device current, looks up the array's
 *     device address (cudaGetSymbolAddress) and keeps it. Make that first call before
 *     any stream capture.
 *   - All calls share the one array, which keeps the last call's contents. Calls whose
 *     work overlaps on the GPU (different streams, or other host threads) race on it
 *     and give wrong results. Calls in sequence on one stream are safe.
 *   - stats == NULL: the call returns once the work is enqueued. Per-geodesic outcomes
 *     are in d_out[i].err.
 *   - stats != NULL: the call waits for the stream. It fills stats (kernel_ms = 0: no
 *     events are recorded) and returns the launch status, as foort_gpu_sync() does.
 * There is no cancel flag; the step budget follows foort_gpu_integrate()'s default.
 * Errors are reported through foort_gpu_last_error(NULL). */
#define FOORT_NOALLOC_MAX_IMAGES 256u
#define FOORT_NOALLOC_SCRATCH_BYTES (256u + 672u * FOORT_NOALLOC_MAX_IMAGES) /* 172,288 */
int foort_gpu_integrate_noalloc(const foort_run_desc* desc, const foort_pixel* d_px, uint64_t n,
                                foort_result* d_out, void* cuda_stream, foort_stats* stats);

/* GeodesicPosition (Diagnostics.cpp:246-284): the saved positions of each geodesic, after
 * the reference's decimation to OutputSteps. `first` holds the results of the pixels'
 * foort_gpu_integrate call (pass 1, same context); this call integrates them once more
 * and records the kept positions. counts[i] receives the number of positions of
 * geodesic i; points (host, 4 doubles per position: t, x1, theta, phi, with x1 = ln r in
 * log-r mode as the reference stores it) receives them geodesic after geodesic. With
 * points == NULL only counts and *total_points are filled (to size the buffer).
 * FOORT_E_NUMERIC if the second pass did not retrace the first. */
int foort_gpu_positions(foort_ctx* ctx, const foort_pixel* px, uint64_t n, const foort_result* first, uint64_t* counts,
                        double* points, uint64_t cap_points, uint64_t* total_points);

/* Number of GeodesicPosition samples of a geodesic of `steps` steps that ended with
 * termination `term`, and how many of them the reference keeps. */
int foort_geopos_count(const foort_run_desc* desc, uint64_t steps, int32_t term, uint64_t* samples, uint64_t* kept);

/* Wait for the last async launch of this context and return its status. */
int foort_gpu_sync(foort_ctx* ctx);

/* Global budget of integration steps per launch (0 = unlimited). When it runs out the
 * kernel stops every lane, marks unfinished results with FOORT_ERR_BUDGET and the
 * launch returns FOORT_E_BUDGET. The reference has only the per-geodesic TimeOut
 * (Terminations.cpp:159-186). */
int foort_gpu_set_budget(foort_ctx* ctx, uint64_t max_total_steps);

/* Ask the running launch to stop (host flag in mapped pinned memory, polled by the
 * kernel every few hundred steps). Safe to call from another host thread. */
int foort_gpu_cancel(foort_ctx* ctx);

/* Launch shape override: CTA size (a multiple of 32, at most 128) and a cap on resident
 * CTAs per SM; 0 leaves each to the autotuner's cached shape for the launch, or to the
 * built-in rule (128 threads, as many CTAs as fit) where the cache has none. */
int foort_gpu_set_launch(foort_ctx* ctx, uint32_t block_size, uint32_t blocks_per_sm);

/* Lanes per geodesic in mixed precision with RK4 and the Kerr or flat metric: 0 chooses
 * per launch (two lanes when the launch's geodesics, at two lanes each, fit on the GPU's
 * resident lanes: a step's latency then sets the pace, and two lanes halve the metric
 * work on it), 1 or 2 force the choice; other configurations always use one. Results
 * are the same either way. No counterpart in the reference (one OpenMP thread per
 * geodesic, Main.cpp:327-414). */
int foort_gpu_set_lanes(foort_ctx* ctx, uint32_t lanes_per_geodesic);

/* ---- launch shapes and the autotuner --------------------------------------------------
 * A launch shape is the CTA size, a cap on resident CTAs per SM, the lanes per geodesic,
 * the regrouping cadence -- how many steps a warp integrates before it refills lanes whose
 * geodesics ended -- and how many steps pass between polls of the step budget and the
 * cancel flag. Results do not depend on the shape: every geodesic goes through the same
 * arithmetic wherever it runs. Only the time does, and the autotuner measures it.
 * Engine extension: the reference's round loop is an OpenMP for with the static schedule
 * (Main.cpp:348). */
typedef struct foort_launch_shape {
    uint32_t block_size;    /* threads per CTA: 32, 64, 96 or 128                      */
    uint32_t blocks_per_sm; /* cap on resident CTAs per SM (0 = as many as fit)        */
    uint32_t lanes;         /* lanes per geodesic: 1, or 2 where the kernel has two    */
    uint32_t refill_steps;  /* >= 1: steps a warp runs between refills of idle lanes   */
    uint32_t poll_steps;    /* >= 1: steps between budget / cancel polls               */
    uint32_t reserved;
    double ms;              /* the search's measured time for this shape (0: none)     */
} foort_launch_shape;

/* Autotune the launch of n pixels held in DEVICE memory: time candidate shapes with CUDA
 * events on `cuda_stream` (lanes x CTA size, then the regrouping cadence and the poll
 * interval around the best), on all n pixels or, for launches of more than
 * FOORT_TUNE_SAMPLE_LANES_X times the resident lanes, on a prefix of that many. The
 * fastest goes into the launch-shape cache under this context's key for n (see
 * foort_tune_key) and into *best (may be NULL). The call ends with a launch of all n
 * pixels in the best shape, so d_out holds their results as after
 * foort_gpu_integrate_async. Synchronous. */
#define FOORT_TUNE_SAMPLE_LANES_X 4u
int foort_gpu_autotune(foort_ctx* ctx, const foort_pixel* d_px, uint64_t n, foort_result* d_out,
                       void* cuda_stream, foort_launch_shape* best);

/* on = 1: a launch whose key has no cache entry first runs the search (that launch waits
 * for its stream and takes several times longer); on = 0 (default): launches use the
 * cached shape where there is one and the built-in rule elsewhere. */
int foort_gpu_set_autotune(foort_ctx* ctx, int32_t on);

/* The shape a launch of n pixels would use now (cache, overrides, built-in rule). */
int foort_gpu_launch_shape(foort_ctx* ctx, uint64_t n, foort_launch_shape* shape);

/* The launch-shape cache: one table per process, shared by every context. A key names
 * the GPU's SM count, the kernel variant (metric, integrator, precision, log-r, FP64
 * decisions, FP64 steps by radius or at turning points) and the size bucket
 * floor(log2 n) of the launch.
 * save / load write and read one text line per entry (load adds to the table). */
uint32_t foort_tune_bucket(uint64_t n);
int foort_tune_key(const foort_run_desc* desc, int32_t num_sms, uint64_t n, char* buf, uint64_t cap);
int foort_tune_put(const char* key, const foort_launch_shape* shape);
int foort_tune_get(const char* key, foort_launch_shape* shape); /* FOORT_E_BADARG: no entry */
uint64_t foort_tune_count(void);
void foort_tune_clear(void);
int foort_tune_save(const char* path);
int foort_tune_load(const char* path);

int foort_gpu_get_stats(const foort_ctx* ctx, foort_stats* stats);

/* The context's run descriptor (its images point to the context's own copy). */
int foort_gpu_get_desc(const foort_ctx* ctx, foort_run_desc* desc);

void foort_gpu_destroy(foort_ctx* ctx);

/* Message of the last failure of this context (or of the last failed create when
 * ctx is NULL). Never NULL. */
const char* foort_gpu_last_error(const foort_ctx* ctx);

/* Horizon radius the reference gives the metric (Metric.cpp:113, 250, 385, 496);
 * 0 for flat space. */
double foort_horizon_radius(int32_t metric_id, const double* metric_params);

/* 1 if this build has a kernel for (metric, integrator, precision), else 0. The
 * reference selects these at run time through Config::GetMetric / GetGeodesicIntegrator
 * (Config.cpp:123-323, 985-1071). */
int foort_gpu_has_kernel(int32_t metric_id, int32_t integrator_id, int32_t precision);

/* Christoffel symbols gamma[16*mu + 4*nu + rho] at the point x (integration
 * coordinates: x[1] = ln r when rlog) from the analytic metric derivatives the
 * mixed-precision kernel uses, evaluated in FP64 on the host. Replaces
 * Metric::getChristoffel_udd (Metric.cpp:14-55), which differentiates numerically.
 * FOORT_E_UNSUPPORTED for an unknown metric_id. */
int foort_metric_christoffel(int32_t metric_id, const double* metric_params, int32_t rlog, const double* x,
                             double* gamma);

/* sizeof() of the ABI structs, for binding checks: 0 foort_pixel, 1 foort_result,
 * 2 foort_run_desc, 3 foort_image_desc, 4 foort_stats, 5 foort_output_desc,
 * 6 foort_config; 0 otherwise. Engine extension. */
uint64_t foort_abi_size(int32_t which);

/* Measured FP32 and FP64 FMA throughput of the current GPU in TFLOP/s (an FMA counts as
 * two operations): the denominators of the engine's ALU roofline. Engine extension. */
int foort_measure_peaks(double* fp32_tflops, double* fp64_tflops);

/* ---- meshes: which pixels each integration round gets --------------------------------
 * Host-side counterparts of the reference's Mesh plugins (Mesh.h:24-61). A FOORT run is
 *     while (!is_finished) { get_pixels; integrate; set_results; end_current_loop; }
 * (Main.cpp:313-419). The adaptive mesh hands out exactly the reference's pixels, in the
 * reference's order. */
typedef struct foort_mesh foort_mesh;

/* SimpleSquareMesh(totalPixels, valdiag), Mesh.h:73-82. diag_flags / value_diag are the
 * run's (they select the value each geodesic reports to the mesh). */
int foort_mesh_create_simple(uint64_t total_pixels, uint32_t diag_flags, uint32_t value_diag, foort_mesh** out);

/* SquareSubdivisionMeshV2(maxPixels, initialPixels, maxSubdivide, iterationPixels,
 * initialSubToFinal, valdiag), Mesh.h:301-315. */
int foort_mesh_create_v2(uint64_t max_pixels, uint64_t initial_pixels, int32_t max_subdivide,
                         uint64_t iteration_pixels, int32_t initial_sub_to_final, uint32_t diag_flags,
                         uint32_t value_diag, foort_mesh** out);

/* Mesh::IsFinished (1 / 0), Mesh::getCurNrGeodesics, the grid size R of the unit
 * screen point (row, col) / (R - 1), and the number of completed rounds. */
int foort_mesh_is_finished(const foort_mesh* mesh);
uint64_t foort_mesh_cur_nr_geodesics(const foort_mesh* mesh);
uint64_t foort_mesh_grid(const foort_mesh* mesh);
uint64_t foort_mesh_rounds(const foort_mesh* mesh);

/* Mesh::getNewInitConds for every index of the current round, as pixels of `image`. */
int foort_mesh_get_pixels(const foort_mesh* mesh, uint32_t image, foort_pixel* out);

/* Mesh::GeodesicFinished(index, values) (Mesh.h:44-46). */
int foort_mesh_geodesic_finished(foort_mesh* mesh, uint64_t index, const double* values, uint32_t n_values);

/* GeodesicFinished for the whole round from the integration results: each geodesic's
 * value is Geodesic::getDiagnosticFinalValue() (Geodesic.cpp:141-149). */
int foort_mesh_set_results(foort_mesh* mesh, const foort_result* results, uint64_t n);

/* Mesh::EndCurrentLoop: weights, ordering and subdivision of the next round. */
int foort_mesh_end_current_loop(foort_mesh* mesh);

void foort_mesh_destroy(foort_mesh* mesh);

/* The mesh's level waves: a new, unstarted mesh with the same parameters but unlimited
 * IterationPixels and MaxPixels, whose rounds subdivide every square of positive weight,
 * so that its round k hands out the pixels of subdivision level k. For a
 * SquareSubdivisionMeshV2 with unlimited MaxPixels (0) the reference's rounds go on until
 * no square of positive weight is left, so both meshes hand out the same pixels, the
 * waves in max_subdivide rounds or fewer; with a finite MaxPixels the mesh hands out at
 * most that many of the waves' pixels (the cut depends on the round order). A
 * SimpleSquareMesh is its own single wave. FOORT_E_UNSUPPORTED for a mesh that has ended
 * a round. Engine extension: the reference has no such schedule. */
int foort_mesh_create_waves(const foort_mesh* mesh, foort_mesh** out);

/* The most pixels the mesh hands out over a run: MaxPixels of a V2 mesh (0: unlimited),
 * the grid's pixel count of a SimpleSquareMesh. */
uint64_t foort_mesh_max_pixels(const foort_mesh* mesh);

/* FOORT_MESH_SIMPLE or FOORT_MESH_SUBDIVISION_V2. */
#define FOORT_MESH_SIMPLE 0
#define FOORT_MESH_SUBDIVISION_V2 1
int foort_mesh_kind(const foort_mesh* mesh);

/* The pixels that the squares whose weight the end of this round decides can add: the top
 * and left edge midpoints, the centre and the right and bottom edge midpoints of each, as
 * pixels of `image` in row-major order (V2 meshes; none for a SimpleSquareMesh). In a mesh
 * of level waves (foort_mesh_create_waves), where every square of positive weight is
 * subdivided in the next round, the next round hands out a subset of them. *n receives the
 * count; with out == NULL only the count, otherwise cap must hold it. Engine extension. */
int foort_mesh_lookahead(const foort_mesh* mesh, uint32_t image, foort_pixel* out, uint64_t cap, uint64_t* n);

/* The mesh's Mesh::getFullDescriptionStr() (Mesh.cpp:69-73, 697-707) into buf. */
int foort_mesh_description(const foort_mesh* mesh, char* buf, uint64_t cap);

/* ---- device-resident adaptive mesh ----------------------------------------------------
 * SquareSubdivisionMeshV2 (Mesh.h:285-423, Mesh.cpp:660-1186) with its grid, values and
 * pixel lists in DEVICE memory: a round's pixels go from the mesh to
 * foort_gpu_integrate_async and the results back to the mesh without a host copy.
 * Engine extension: the reference's mesh is host code.
 *
 * Ordering of the active squares (EndCurrentLoop, Mesh.cpp:1137-1148; std::sort, which is
 * not stable, by weight then level):
 *   FOORT_DMESH_ORDER_REFERENCE  a host copy of the active list (24 bytes per square) is
 *       sorted with libstdc++'s std::sort in the reference's sequence: every round hands
 *       out the reference's pixels, in the reference's order. Per round the new squares
 *       come to the host and the squares to subdivide go back.
 *   FOORT_DMESH_ORDER_DEVICE  the list stays on the device and is sorted there with the
 *       grid cell as the last key. The rounds agree with the reference's where no two
 *       squares of equal weight and level fall on either side of the IterationPixels cut.
 * All calls are stream-ordered on `cuda_stream` (a cudaStream_t, 0 = legacy); create and
 * end_current_loop wait for it. The grid takes 16 bytes per cell (R^2 cells, R as
 * foort_mesh_grid), at most FOORT_DMESH_MAX_CELLS cells. The value diagnostic may not be
 * GeodesicPosition (FOORT_E_UNSUPPORTED). */
typedef struct foort_dmesh foort_dmesh;
#define FOORT_DMESH_ORDER_REFERENCE 0u
#define FOORT_DMESH_ORDER_DEVICE 1u
#define FOORT_DMESH_MAX_CELLS (1ull << 29)

/* SquareSubdivisionMeshV2(maxPixels, initialPixels, maxSubdivide, iterationPixels,
 * initialSubToFinal, valdiag) whose pixels belong to image `image` of the run. */
int foort_dmesh_create_v2(uint64_t max_pixels, uint64_t initial_pixels, int32_t max_subdivide,
                          uint64_t iteration_pixels, int32_t initial_sub_to_final, uint32_t diag_flags,
                          uint32_t value_diag, uint32_t image, uint32_t order, void* cuda_stream,
                          foort_dmesh** out);
int foort_dmesh_is_finished(const foort_dmesh* mesh);
uint64_t foort_dmesh_cur_nr_geodesics(const foort_dmesh* mesh);
uint64_t foort_dmesh_grid(const foort_dmesh* mesh);
uint64_t foort_dmesh_rounds(const foort_dmesh* mesh);
/* Squares with a positive weight not yet subdivided. */
uint64_t foort_dmesh_active(const foort_dmesh* mesh);
/* The current round's pixels: a DEVICE array of foort_dmesh_cur_nr_geodesics entries,
 * valid until the next foort_dmesh_end_current_loop. */
const foort_pixel* foort_dmesh_pixels(const foort_dmesh* mesh);
/* The same copied to HOST memory (out: foort_dmesh_cur_nr_geodesics entries). */
int foort_dmesh_get_pixels(foort_dmesh* mesh, foort_pixel* out);
/* The round's values from DEVICE results (Geodesic::getDiagnosticFinalValue,
 * Geodesic.cpp:141-149), or directly as one DEVICE double per pixel. n must be the
 * round's pixel count. */
int foort_dmesh_set_results(foort_dmesh* mesh, const foort_result* d_res, uint64_t n);
int foort_dmesh_set_values(foort_dmesh* mesh, const double* d_values, uint64_t n);
/* Mesh::EndCurrentLoop: weights, ordering and subdivision of the next round. */
int foort_dmesh_end_current_loop(foort_dmesh* mesh);
const char* foort_dmesh_last_error(const foort_dmesh* mesh);
void foort_dmesh_destroy(foort_dmesh* mesh);

/* A whole run on one device mesh: the round loop of Main.cpp:313-419. Each round's
 * pixels are integrated into the DEVICE buffer d_out (room for cap_out results), then
 * on_round (may be NULL) sees the round's DEVICE pixels and results (its non-zero return
 * ends the run with that code), then the mesh takes the results and ends the round.
 * Optional geodesics / rounds receive the totals. */
typedef int (*foort_dmesh_round_fn)(void* user, const foort_pixel* d_px, const foort_result* d_res, uint64_t n,
                                    uint32_t round);
int foort_gpu_run_dmesh(foort_ctx* ctx, foort_dmesh* mesh, foort_result* d_out, uint64_t cap_out,
                        foort_dmesh_round_fn on_round, void* user, uint64_t* geodesics, uint32_t* rounds);

/* ---- Output files (GeodesicOutputHandler, InputOutput.h:40-110) -------------------------
 * Writes a run's results as FOORT does, byte for byte: one file per diagnostic, named
 * prefix_[timestamp_]Name[_n].ext, each starting with the first-line description, then
 * "row col  value" per geodesic; outputs are cached up to outputs_to_cache geodesics and
 * split over files of geodesics_per_file lines (InputOutput.cpp:95-330). */
typedef struct foort_output_desc {
    const char* prefix;          /* FilePrefix (may contain directories; created)         */
    const char* timestamp;       /* "" or NULL for none                                   */
    const char* extension;       /* e.g. "dat"; "" or NULL for none                       */
    const char* first_line;      /* first line of every file; "" or NULL for none         */
    uint64_t outputs_to_cache;   /* GeodesicOutputHandler's nroutputstocache              */
    uint64_t geodesics_per_file; /* geodperfile (> 0; 0 is console output: unsupported)   */
    uint32_t diag_flags;         /* the run's diagnostics and value diagnostic: they set  */
    uint32_t value_diag;         /* the files' order (CreateDiagnosticVector)             */
} foort_output_desc;

typedef struct foort_output foort_output;

/* Utilities::GetFirstLineInfoString (Utilities.cpp:52-84) for image `image` of the
 * descriptor and its mesh, into buf (NUL-terminated). */
int foort_first_line_info(const foort_run_desc* desc, uint32_t image, const foort_mesh* mesh, char* buf,
                          uint64_t cap);
int foort_output_create(const foort_output_desc* desc, foort_output** out);
/* One round's results (host arrays, pixel order): PrepareForOutput(n) and n
 * NewGeodesicOutput calls (Main.cpp:334, :400). FOORT_E_IO on a file error. */
int foort_output_round(foort_output* out, const foort_pixel* px, const foort_result* res, uint64_t n);
/* The same with the GeodesicPosition diagnostic: counts / points as foort_gpu_positions
 * returns them (its line: "row col  count ;; t x1 theta phi ...", Diagnostics.cpp:286-302). */
int foort_output_round_positions(foort_output* out, const foort_pixel* px, const foort_result* res, uint64_t n,
                                 const uint64_t* counts, const double* points);
/* OutputFinished (InputOutput.cpp:123-127): write what is cached. */
int foort_output_finish(foort_output* out);
void foort_output_destroy(foort_output* out);

/* ---- FOORT configuration files (Main.cpp:161-200, Config.cpp:94-1155) --------------------
 * Reads a .cfg file as the reference does (libconfig syntax, typed lookups without
 * automatic conversion, the reference's defaults and fallbacks) into the descriptors of
 * one run. `notes` receives the reference's default-setting messages, one per line. */
#define FOORT_CONFIG_MESH_SIMPLE 0         /* SimpleSquareMesh                              */
#define FOORT_CONFIG_MESH_SUBDIVISION_V2 1 /* SquareSubdivisionMeshV2                       */
#define FOORT_CONFIG_MESH_SUBDIVISION 2    /* SquareSubdivisionMesh (V1): not in the engine */
#define FOORT_CONFIG_MESH_INPUT_PIXELS 3   /* InputCertainPixelsMesh: not in the engine     */
typedef struct foort_config {
    foort_run_desc run;           /* n_images = 1; set run.images = &image before use   */
    foort_image_desc image;       /* metric parameters, camera, screen                  */
    int32_t mesh_kind;            /* FOORT_CONFIG_MESH_*                                 */
    int32_t max_subdivide;
    uint64_t total_pixels;        /* SimpleSquareMesh / InputCertainPixelsMesh          */
    uint64_t initial_pixels, max_pixels, iteration_pixels;
    int32_t initial_sub_to_final;
    int32_t timestamp;            /* Output.TimeStamp: prefix_timestamp_ file names     */
    uint64_t outputs_to_cache;    /* Output.GeodesicsToCache                            */
    uint64_t geodesics_per_file;  /* Output.GeodesicsPerFile (0 read as unlimited)      */
    int32_t first_line_info;      /* Output.FirstLineInfo                               */
    int32_t screen_output_level;  /* Output.ScreenOutputLevel, 0..4                     */
    uint64_t loop_message_frequency;
    char file_prefix[1024];       /* Output.FilePrefix; "" = console output             */
    char file_extension[64];
} foort_config;
int foort_config_load(const char* path, foort_config* cfg, char* notes, uint64_t cap);
int foort_config_parse(const char* text, foort_config* cfg, char* notes, uint64_t cap);
/* The configured mesh (FOORT_E_UNSUPPORTED for the V1 and input-pixels meshes). */
int foort_config_create_mesh(const foort_config* cfg, foort_mesh** mesh);
/* Utilities::GetTimeStampString (Utilities.cpp:28-36): local time, %y%m%d-%H%M%S. */
int foort_timestamp_string(char* buf, uint64_t cap);

/* A whole run: the round loop of Main.cpp:313-419. meshes[i] (and, unless NULL,
 * outputs[i]) belong to image i of the context's descriptor. Each round integrates the
 * pixels of every unfinished mesh in one launch (foort_gpu_integrate), passes the
 * results to the meshes (Main.cpp:399) and output files (Main.cpp:400), and ends the
 * meshes' rounds (Main.cpp:410); the outputs are finished at the end. Optional
 * geodesics / rounds receive the totals. The context keeps pinned host buffers for the
 * pixels and results of its largest launch (136 bytes per geodesic) until
 * foort_gpu_destroy. */
int foort_gpu_run(foort_ctx* ctx, foort_mesh* const* meshes, foort_output* const* outputs, uint32_t n_images,
                  uint64_t* geodesics, uint32_t* rounds);

/* Schedule of foort_gpu_run's launches. Engine extension: the reference integrates
 * round after round (Main.cpp:313-419).
 *   FOORT_SCHEDULE_WAVES (default): where a mesh is a SquareSubdivisionMeshV2, no step
 *     budget is set and GeodesicPosition is off, the run integrates the meshes' level
 *     waves (foort_mesh_create_waves) -- one
 *     launch per subdivision level, over all images -- and then replays the meshes'
 *     rounds from the stored results. The meshes, the output files and the returned
 *     counts see the reference's rounds in the reference's order, and each result is the
 *     one the round's own launch would give (a geodesic's result does not depend on the
 *     launch it runs in). An image's waves stop before the one that would take its
 *     pixels past foort_mesh_max_pixels. A pixel of a round that no wave held is
 *     integrated then, in one launch per such round. Elsewhere the run goes round by round.
 *   FOORT_SCHEDULE_ROUNDS: one launch per round.
 * foort_gpu_run_info reports the last run's launch count and the schedule it used. */
#define FOORT_SCHEDULE_WAVES 0u
#define FOORT_SCHEDULE_ROUNDS 1u
int foort_gpu_set_schedule(foort_ctx* ctx, uint32_t schedule);
int foort_gpu_run_info(const foort_ctx* ctx, uint32_t* launches, uint32_t* schedule);

/* Lookahead of the wave schedule. A launch lasts about as long as its slowest geodesic
 * while the GPU has idle lanes, so the launch of a wave may also take the next wave's
 * candidates (foort_mesh_lookahead: a superset of the next wave) as long as the launch
 * then holds at most max_geodesics geodesics; the next wave then needs no launch of its
 * own. Candidates the run does not use are integrated and dropped: they reach neither
 * the meshes nor the files. 0 = off; FOORT_LOOKAHEAD_AUTO (default) = 128 x the GPU's SM
 * count (19,456 on GB300): at two lanes each, two warps per SM sub-partition, up to which
 * a launch of such geodesics takes little longer than its longest geodesic alone. */
#define FOORT_LOOKAHEAD_AUTO UINT64_MAX
int foort_gpu_set_lookahead(foort_ctx* ctx, uint64_t max_geodesics);

/* on = 1: foort_gpu_run keeps the pixel list of each launch of the run (the last run's
 * only); foort_gpu_run_launch copies launch k's list to out (count in *n; out == NULL:
 * count only). For benchmarks that replay a run's launches from device memory. */
int foort_gpu_set_record_launches(foort_ctx* ctx, int32_t on);
int foort_gpu_run_launch(const foort_ctx* ctx, uint32_t k, foort_pixel* out, uint64_t cap, uint64_t* n);

#ifdef __cplusplus
}
#endif

#endif /* FOORT_GPU_H */
