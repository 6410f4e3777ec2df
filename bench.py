"""Benchmark of the GB300 geodesic engine (one JSON line on rank 0).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl engine|reference]
                    [--workload c2|c1|c3|c4|c5] [--no-fp64] [--iteration-pixels P]

Metric: geodesics/s on one GB300 of the mixed-precision kernel on the workload (default
C2: Kerr a=0.99 seen at 60 deg, 12 M half-width screen, SquareSubdivisionMeshV2 from a
128^2 seed, MaxSubdivide 3, seed round + 4 refinement rounds), next to the plain FP64
kernel on the same pixels and the endpoint error between the two.

One step = one whole run of the workload (every geodesic of its mesh once):
  value  the run's launches with their pixel lists resident in HBM, one persistent-kernel
         launch each through foort_gpu_integrate_async on one stream; CUDA events on that
         stream around each step; L2 flushed (256 MB write) between steps; the launch
         shape of each launch chosen by the engine's autotuner (foort_gpu_autotune) in
         the first warm-up step. The launches are the schedule's (--schedule): those
         foort_gpu_run makes by default, the meshes' level waves with lookahead (one
         launch per subdivision level, a launch also taking the next level's candidates
         while it stays small enough; C2: 2 launches of 16,384 and 14,367 geodesics for
         the reference's 5 rounds of 26,547), or one per round. value counts the run's
         geodesics only;
  e2e    the whole run through the public C ABI, foort_gpu_run: host meshes, H2D of each
         launch's pixels, kernel, D2H of its results, and the meshes' rounds replayed in
         the reference's order. e2e_per_round_api: the same run through the per-round
         call from pinned host memory (host mesh -> foort_gpu_integrate ->
         foort_mesh_set_results -> foort_mesh_end_current_loop, every round);
         rounds_schedule: the device-resident leg with one launch per round;
         device_mesh: the run through foort_gpu_run_dmesh (mesh on the GPU).
Accuracy (N = 1): the plain FP64 kernel (the reference's finite differences) on the same
rounds, timed for the speed-up; the FP64-analytic oracle (every step in FP64 with the
mixed kernel's derivatives) on all pixels; per-pixel condition numbers from two shifted
launches; error reports of mixed and plain FP64 against the oracle (foort_gb300.accuracy).
N > 1 (torchrun): every rank integrates its own copy of the workload (weak scaling,
no collective on the data path); times are the max over ranks. The FP64 and CPU legs
run at N = 1 only. --shard: one run split over the ranks instead, each round gathered
before the mesh picks the next (strong scaling).
--impl reference: the reference's algorithm on the host cores (the oracle's
restatement built with the reference's -Ofast flags; the reference itself only builds
where its sources are), on a bounded seeded sample of the pixels the reference's own
complete C2 run integrates (tests/golden/c2_run.npz; other workloads: of their grid).
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "geodesics/sec on 1 GB300: mixed-FP32 batched vs FP64 plain, at ≤1e-6 rel. error"
UNIT = "geodesics/s"

# Canonical algorithmic operation counts per integration step (reference formulation:
# finite-difference Christoffels, 5 metric evaluations per right-hand side; 1 op = one
# add/sub/mul/div/sqrt, FMA = 2; sin/cos pairs counted separately).
OPS_PER_STEP = {("kerr", "rk4"): 1130, ("johannsen", "rk4"): 1650, ("johannsen", "verlet"): 830}
SINCOS_PER_STEP = {("kerr", "rk4"): 20, ("johannsen", "rk4"): 20, ("johannsen", "verlet"): 10}
OPS_PER_EXTRA_VERLET_RHS = 380
# DRAM traffic per geodesic of the mixed kernel: dram__bytes_read.sum + dram__bytes_write.sum
# of one ncu capture of the two-lane kernel on a 6,000-pixel sample of the C2 grid, divided
# by its geodesics
DRAM_BYTES_PER_GEODESIC = {("kerr", "rk4"): 120.4}
# Executed thread instructions per geodesic step of the mixed kernel (ncu
# smsp__inst_executed x 32 / steps): two lanes of ~929 each and one lane of 1,270 on a
# 6,000-pixel sample of the C2 grid; Johannsen Verlet (one lane) 1,754 on 20,000 pixels
# of C4's. With the GPU's issue rate (one warp instruction per cycle on each of its
# 4 x 152 sub-partitions) they give the fraction of issue slots the path fills.
EXEC_INSTR_PER_STEP = {("kerr", "rk4", 2): 1857, ("kerr", "rk4", 1): 1270, ("johannsen", "verlet", 1): 1754}
SUBPARTITIONS = 4
# runs of more geodesics take the FP64 legs on a seeded sample (1 %, at least 20,000)
FP64_SAMPLE_ABOVE = 60000
FP64_SAMPLE_SEED = 20261203


from foort_gb300.multirank import dist_env  # noqa: E402


def log(*a):
    print(*a, file=sys.stderr, flush=True)


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for n, v in zip(names, f[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "samples": len(sm), "reasons": sorted(reasons)}


def workload(name, precision, iteration_pixels=None):
    from foort_gb300 import workloads
    if name == "c1":
        return workloads.c1(precision)
    if name == "c2":
        return workloads.c2(precision, iteration_pixels=iteration_pixels)
    if name == "c3":
        return workloads.c3(precision)
    if name == "c4":
        return workloads.c4(precision)
    if name == "c5":
        return workloads.c5(precision)
    raise SystemExit(f"unknown workload {name}")


def kind_of(wl):
    from foort_gb300 import abi
    m = "kerr" if wl.desc.metric_id == abi.METRIC_KERR else "johannsen"
    i = "rk4" if wl.desc.integrator_id == abi.INTEGRATOR_RK4 else "verlet"
    return m, i


def adaptive_rounds(eng_mod, wl, results_out=None, waves=False):
    """The pixel list of every round of the workload (one run with the engine), or of
    every level wave (waves=True)."""
    px_rounds = []
    with eng_mod.Engine(wl.desc) as e:
        def keep(px, res):
            px_rounds.append(px.copy())
            if results_out is not None:
                results_out.append(res.copy())
        eng_mod.run_rounds(wl.mesh, wl.desc, e.integrate, keep, waves=waves)
    return px_rounds


def cpu_sample_rate(wl, px_all, target_seconds, nthreads, use_ref=False):
    """Geodesics/s on the host cores on a seeded sample of px_all: the reference itself
    (use_ref, where it was built from its sources) or the oracle's restatement, both
    with the reference's -Ofast flags."""
    import oracle

    def run(px):
        if use_ref:
            return oracle.ref_integrate(wl.desc, px, nthreads=nthreads)
        return oracle.integrate(wl.desc, px, fast=True, nthreads=nthreads)

    rng = np.random.default_rng(20261203)
    order = rng.permutation(len(px_all))
    probe = px_all[order[:max(64, 4 * nthreads)]]
    t0 = time.perf_counter()
    run(probe)
    dt = time.perf_counter() - t0
    per = dt / len(probe)
    n = int(min(len(px_all), max(len(probe), target_seconds / max(per, 1e-9))))
    sample = px_all[order[:n]]
    t0 = time.perf_counter()
    res = run(sample)
    dt = time.perf_counter() - t0
    return n / dt, n, dt, res


def reference_run_pixels(args):
    """The pixels of the reference's own complete C2 run (tests/golden/c2_run.npz:
    26,547 pixels of the 509^2 grid, in its order) when the workload is C2 with its
    default IterationPixels; None otherwise."""
    from foort_gb300 import abi, workloads
    fn = os.path.join(ROOT, "tests", "golden", "c2_run.npz")
    if args.workload != "c2" or args.iteration_pixels not in (None, workloads.C2_ITERATION_PIXELS) \
            or not os.path.exists(fn):
        return None
    f = np.load(fn)
    px = np.zeros(len(f["row"]), dtype=abi.PIXEL_DTYPE)
    px["row"], px["col"], px["grid"] = f["row"], f["col"], 509
    return px


def run_reference(args, rank):
    """--impl reference: the reference's algorithm on the host cores."""
    if rank != 0:
        return 0
    import oracle
    from foort_gb300 import abi
    oracle.build()
    wl = workload(args.workload, abi.PREC_FP64, args.iteration_pixels)
    side = None
    kind, spec = wl.mesh[0]
    if kind == "simple":
        side = spec
    else:
        side = int((math.sqrt(spec["initial_pixels"]) - 1) * 2 ** (spec["max_subdivide"] - 1) + 1)
    grid = reference_run_pixels(args)
    run_px = grid is not None  # the pixel set of the reference's complete C2 run (5 rounds)
    where = f"of the reference's own complete run ({len(grid)} pixels of the {side}^2 grid)" if grid is not None \
        else f"of the {side}^2 grid"
    if grid is None:
        grid = abi.square_pixels(side)
    nthreads = os.cpu_count() or 1
    # a few seconds of all host threads per step: shorter samples measure the one
    # slowest geodesic of the sample more than the throughput
    per_step = max(4.0, (args.cpu_seconds or 40.0) / max(1, args.steps + args.warmup))
    use_ref = oracle.have_ref()
    kind_name = "reference" if use_ref else "port"
    rates = []
    for i in range(args.warmup + args.steps):
        rate, n, dt, _ = cpu_sample_rate(wl, grid, per_step, nthreads, use_ref=use_ref)
        if i >= args.warmup:
            rates.append((rate, n, dt))
    rate = sum(r[1] for r in rates) / sum(r[2] for r in rates)
    line = {
        "metric": METRIC, "value": rate, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(r[2] for r in rates) / len(rates),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config_block(wl, args, side=side, rounds=5 if run_px else None,
                               geod=len(grid) if run_px else None),
        "cpu_baseline": {"value": rate, "unit": UNIT, "cores": nthreads, "kind": kind_name,
                         "sample": f"{rates[-1][1]} seeded-random pixels {where} per step; "
                                   + ("the reference compiled from its sources with its own -Ofast -fopenmp flags"
                                      if use_ref else "the oracle's restatement built with the reference's "
                                                      "-Ofast -fopenmp flags")},
        "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_sharded(args, rank, world, local):
    """--shard: ONE run of the workload split over the ranks (strong scaling). Every rank
    holds the same mesh; each launch of the schedule (a level wave, or a round), each rank
    integrates its contiguous slice through the C ABI from host memory and the slices are
    gathered before the mesh goes on (foort_gb300.multirank.sharded_run). value = the run's
    geodesics / the slowest rank's time per run."""
    import torch
    import foort_gb300
    from foort_gb300 import abi, multirank
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    wl = workload(args.workload, abi.PREC_MIXED, args.iteration_pixels)
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    with foort_gb300.Engine(wl.desc) as e:
        def one_run():
            n = [0, 0, 0]

            def count(px, res):
                n[0] += len(px)
                n[1] += 1

            def integrate(px):
                n[2] += 1
                return e.integrate(px)
            # each rank's slice of a launch is held to foort_gpu_run's default lookahead cap
            multirank.sharded_run(wl.mesh, wl.desc, integrate, rank, world, dist, on_round=count,
                                  waves=args.schedule == "waves", lookahead=128 * sms * world)
            return n
        for _ in range(args.warmup):
            n_geod, n_rounds, n_launch = one_run()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            one_run()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        t = multirank.max_over_ranks((time.perf_counter() - t0) / args.steps, dist, device="cuda")
    value = n_geod / t
    if rank == 0:
        print(json.dumps({
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "strong",
            "vs_baseline": None, "dtype": "mixed-f32", "data": "synthetic", "mode": "sharded",
            "config": dict(config_block(wl, args, rounds=n_rounds, geod=n_geod), parallelism=f"shard{world}"),
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": n_geod * abi.PIXEL_DTYPE.itemsize,
                    "d2h_bytes_per_step": n_geod * abi.RESULT_DTYPE.itemsize},
            "schedule": args.schedule, "gpu_launches": args.steps * n_launch}), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def run_profile_case(args):
    """One warm-up and one measured launch per precision on a seeded sample of the grid."""
    import foort_gb300
    from foort_gb300 import abi
    out = {}
    for prec, name in ((abi.PREC_MIXED, "mixed"), (abi.PREC_FP64, "fp64")):
        if args.profile_precision not in ("both", name):
            continue
        wl = workload(args.workload, prec, args.iteration_pixels)
        kind, spec = wl.mesh[0]
        side = spec if kind == "simple" else int((math.sqrt(spec["initial_pixels"]) - 1) * 2 ** (spec["max_subdivide"] - 1) + 1)
        rng = np.random.default_rng(5)
        idx = np.sort(rng.choice(side * side, min(args.profile, side * side), replace=False))
        px = np.zeros(len(idx), dtype=abi.PIXEL_DTYPE)
        px["row"], px["col"], px["grid"] = idx // side, idx % side, side
        with foort_gb300.Engine(wl.desc) as e:
            e.set_lanes(args.lanes)
            e.integrate(px[:512])
            res = e.integrate(px)
            st = e.stats()
        out[name] = {"pixels": len(px), "kernel_ms": st["kernel_ms"], "steps": st["steps"],
                     "rhs_evals": st["rhs_evals"], "blocks": st["n_blocks"], "block_size": st["block_size"],
                     "lanes_per_geodesic": st["lanes_per_geodesic"],
                     "geodesics": int(st["geodesics"]), "mean_steps": float(res["steps"].mean())}
    print(json.dumps({"profile_case": args.workload, **out}), flush=True)
    return 0


def pixel_index(have, want):
    """Index into `have` of each pixel of `want` (both PIXEL_DTYPE arrays; every pixel of
    `want` must be in `have`)."""
    def key(p):
        return (p["image"].astype(np.int64) << 42) | (p["row"].astype(np.int64) * p["grid"].astype(np.int64)
                                                     + p["col"].astype(np.int64))
    kh, kw = key(have), key(want)
    order = np.argsort(kh, kind="stable")
    i = order[np.searchsorted(kh[order], kw)]
    assert np.array_equal(kh[i], kw)
    return i


def config_block(wl, args, side=None, rounds=None, geod=None):
    c = {"workload": wl.name, "model": None, "global_batch": geod, "rounds": rounds,
         "metric_params": list(wl.images[0].metric_params)[:2], "iteration_pixels": None,
         "l2": "flushed between timed steps (256 MB write); inputs ~3 MB"}
    kind, spec = wl.mesh[0]
    if kind == "v2":
        c["iteration_pixels"] = spec["iteration_pixels"]
        c["mesh"] = f"SquareSubdivisionMeshV2 {int(math.isqrt(spec['initial_pixels']))}^2 seed, " \
                    f"MaxSubdivide {spec['max_subdivide']}"
    else:
        c["mesh"] = f"SimpleSquareMesh x{len(wl.mesh)} images"
    c.pop("model")
    return c


def accuracy_legs(fg, args, wl, px_all, mixed_all, res64_all):
    """Endpoint errors against the FP64-analytic oracle (every step in FP64 with the mixed
    kernel's analytic derivatives): of the mixed kernel, and of the plain FP64 kernel (the
    reference's finite differences); and of the mixed kernel against the plain FP64 kernel.
    Every pixel counts (a discrete disagreement as an infinite error); each report splits
    off the well-conditioned pixels and gives the backward error err / kappa, with the
    condition numbers kappa from two launches of the mixed kernel at screen points shifted
    by ~1e-6 (foort_gb300.accuracy)."""
    from foort_gb300 import abi, accuracy
    rlog = bool(wl.desc.rlog)
    wla = workload(args.workload, abi.PREC_FP64_ANALYTIC, args.iteration_pixels)
    with fg.Engine(wla.desc) as e:
        e.integrate(px_all[:128])
        resa = e.integrate(px_all)
        ta = e.stats()["kernel_ms"]
    grids = px_all["grid"].astype(np.int64)
    K, _ = accuracy.shift_refinement(int(grids.max()))
    step = 1.0 / (K * (grids - 1))
    with fg.Engine(wl.desc) as e:
        shifted = [e.integrate(accuracy.shifted_pixels(px_all, K, ax)) for ax in (0, 1)]
    kappa = accuracy.condition_numbers(mixed_all, shifted, step, rlog=rlog)
    rep = {
        "oracle": "FP64-analytic: every step in FP64 with the mixed kernel's analytic derivatives "
                  f"({len(px_all)} pixels in one launch, {ta:.0f} ms)",
        "kappa": f"endpoint change per unit screen shift, from shifts of {float(np.median(step)):.2e} of the screen; "
                 f"well-conditioned: kappa <= {accuracy.KAPPA_WELL:g}",
        "mixed_vs_fp64_analytic": accuracy.error_report(accuracy.endpoint_err_all(mixed_all, resa, rlog), kappa),
        "fp64_vs_fp64_analytic": accuracy.error_report(accuracy.endpoint_err_all(res64_all, resa, rlog), kappa),
        "mixed_vs_fp64": accuracy.error_report(accuracy.endpoint_err_all(mixed_all, res64_all, rlog), kappa),
    }
    return rep


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--workload", default="c2", choices=["c1", "c2", "c3", "c4", "c5"])
    ap.add_argument("--iteration-pixels", type=int, default=None)
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 comparison leg")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--shard", action="store_true",
                    help="one run split over the ranks, gathered each round (strong scaling) instead of one "
                         "independent run per rank")
    ap.add_argument("--schedule", default="waves", choices=["waves", "rounds"],
                    help="launches of a run: the meshes' level waves (foort_gpu_run's default) or one per round")
    ap.add_argument("--no-tune", action="store_true",
                    help="use the built-in launch rule instead of autotuning each round in the first warm-up step")
    ap.add_argument("--cpu-seconds", type=float, default=None,
                    help="host-core seconds of the CPU legs (default: 15 for cpu_baseline, 40 for --impl reference)")
    ap.add_argument("--profile-precision", default="both", choices=["both", "mixed", "fp64"])
    ap.add_argument("--lanes", type=int, default=0, choices=[0, 1, 2],
                    help="lanes per geodesic of the mixed kernel: 0 chosen per launch (default), 1 or 2")
    ap.add_argument("--profile", type=int, default=0, metavar="N",
                    help="profiling case: one launch of the mixed and one of the FP64 kernel on N pixels of "
                         "the workload's grid (after one warm-up launch each), then exit")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "engine" else args.warmup
    rank, world, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, rank)
    if args.profile:
        return run_profile_case(args)
    if args.shard:
        return run_sharded(args, rank, world, local)

    import torch
    import foort_gb300
    from foort_gb300 import abi, multirank
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    def max_over_ranks(x):
        return multirank.max_over_ranks(x, dist, device="cuda")

    # ---- prepare: the workload's pixel lists (one adaptive run with the mixed kernel): the
    # reference's rounds, and the launches of the schedule (the level waves: one launch per
    # subdivision level, the same pixels; or the rounds themselves)
    wl = workload(args.workload, abi.PREC_MIXED, args.iteration_pixels)
    mkind = kind_of(wl)
    t0 = time.perf_counter()
    rounds = adaptive_rounds(foort_gb300, wl)
    launches_px = rounds
    if args.schedule == "waves":  # the launches foort_gpu_run makes (waves with lookahead)
        with foort_gb300.Engine(wl.desc) as e:
            e.set_record_launches(True)
            meshes = [foort_gb300.Mesh.from_spec(spec, wl.desc.diag_flags, wl.desc.value_diag) for spec in wl.mesh]
            e.run(meshes)
            for m in meshes:
                m.close()
            launches_px = e.run_launches()
    log(f"[bench] {wl.name}: {len(rounds)} rounds, sizes {[len(r) for r in rounds]}; {args.schedule}: "
        f"{[len(r) for r in launches_px]}; prepare {time.perf_counter() - t0:.1f}s")
    n_geod = sum(len(r) for r in rounds)
    n_launched = sum(len(r) for r in launches_px)
    stream = torch.cuda.Stream()

    def to_device(lists):
        return ([torch.from_numpy(r.view(np.uint8)).to("cuda") for r in lists],
                [torch.empty(len(r) * abi.RESULT_DTYPE.itemsize, dtype=torch.uint8, device="cuda") for r in lists])

    d_px, d_out = to_device(launches_px)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")

    rhs_per_round = [0] * len(launches_px)
    lanes_per_round = [1] * len(launches_px)
    shapes = [None] * len(launches_px)

    def device_step(e, tune=False, lists=None):
        kms = []
        dpx, dout, lst = lists if lists else (d_px, d_out, launches_px)
        with torch.cuda.stream(stream):
            for i, (dp, do, r) in enumerate(zip(dpx, dout, lst)):
                if tune:  # the project autotuner: search, cache, and integrate in the best shape
                    e.autotune(dp.data_ptr(), len(r), do.data_ptr(), stream.cuda_stream)
                else:
                    e.integrate_async(dp.data_ptr(), len(r), do.data_ptr(), stream.cuda_stream)
                    e.sync()
                st = e.stats()
                kms.append(st["kernel_ms"])
                if lists:
                    continue
                shapes[i] = {"geodesics": len(r), "block_size": st["block_size"], "lanes": st["lanes_per_geodesic"],
                             "refill_steps": st["refill_steps"], "poll_steps": st["poll_steps"]}
                rhs_per_round[i] = st["rhs_evals"]
                lanes_per_round[i] = st["lanes_per_geodesic"]
        return kms

    def timed_steps(e, lists=None):
        ms, kms_all = [], []
        for _ in range(args.steps):
            flush.fill_(1)
            torch.cuda.synchronize()
            ev0 = torch.cuda.Event(enable_timing=True)
            ev1 = torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
            kms = device_step(e, lists=lists)
            ev1.record(stream)
            ev1.synchronize()
            ms.append(ev0.elapsed_time(ev1))
            kms_all.extend(kms)
        return ms, kms_all

    # ---- value: device-resident inputs
    peaks = foort_gb300.measure_peaks()
    with foort_gb300.Engine(wl.desc) as e:
        e.set_lanes(args.lanes)
        t0 = time.perf_counter()
        for w in range(args.warmup):
            device_step(e, tune=(w == 0 and not args.no_tune))
            if w == 0:
                log(f"[bench] first warm-up step{' (autotuning every round)' if not args.no_tune else ''}: "
                    f"{time.perf_counter() - t0:.1f}s; shapes {shapes}")
        barrier()
        tuned_shapes = [dict(sh) for sh in shapes]  # the FP64 leg reuses device_step
        clocks = ClockSampler(local)
        clocks.start()
        step_ms, launch_ms = timed_steps(e)
        barrier()
        clk = clocks.stop()
        mixed_res = [np.frombuffer(do.cpu().numpy().tobytes(), dtype=abi.RESULT_DTYPE) for do in d_out]
        mixed_rhs, mixed_lanes = list(rhs_per_round), list(lanes_per_round)  # the FP64 leg reuses device_step
    t_step = max_over_ranks(sum(step_ms) / len(step_ms))
    value = world * n_geod / (t_step * 1e-3)
    steps_total = sum(int(r["steps"].sum()) for r in mixed_res)

    # ---- the same pixels launched round by round (the reference's rounds), device-resident;
    # sizes the search has not seen are tuned in the warm-up
    rounds_leg = None
    if [len(r) for r in launches_px] != [len(r) for r in rounds]:
        r_lists = to_device(rounds) + (rounds,)
        with foort_gb300.Engine(wl.desc) as e:
            e.set_lanes(args.lanes)
            e.set_autotune(not args.no_tune)
            for _ in range(args.warmup):
                device_step(e, lists=r_lists)
            barrier()
            r_ms, _ = timed_steps(e, lists=r_lists)
            barrier()
        t_r = max_over_ranks(sum(r_ms) / len(r_ms))
        rounds_leg = {"value": world * n_geod / (t_r * 1e-3), "unit": UNIT, "ms_per_step": t_r,
                      "launches_per_step": len(rounds),
                      "scope": "the same pixels, one launch per round of the reference's mesh, device-resident"}
        del r_lists

    # ---- e2e: a whole run through the public C ABI (foort_gpu_run: host mesh, H2D of each
    # launch's pixels, kernel, D2H of its results, mesh rounds), and the same run through
    # the per-round call (foort_gpu_integrate from pinned host memory, round after round:
    # what a binding inside the reference's own round loop does)
    def new_meshes():
        return [foort_gb300.Mesh.from_spec(spec, wl.desc.diag_flags, wl.desc.value_diag) for spec in wl.mesh]

    run_launches = []

    def e2e_run(e):
        meshes = new_meshes()
        try:
            g, _ = e.run(meshes)
        finally:
            for m in meshes:
                m.close()
        run_launches.append(e.run_info() + (g,))

    with foort_gb300.Engine(wl.desc) as e:
        e.set_lanes(args.lanes)
        e.set_schedule(abi.SCHEDULE_WAVES if args.schedule == "waves" else abi.SCHEDULE_ROUNDS)
        for _ in range(args.warmup):
            e2e_run(e)
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_run(e)
        barrier()
        t_e2e = max_over_ranks((time.perf_counter() - t0) / args.steps)
    n_launch_run, sched_used, g_run = run_launches[-1]
    # each launched pixel goes up once and its result comes back once: the launches are
    # the recorded ones (checked, and reported)
    e2e = {"value": world * n_geod / t_e2e, "unit": UNIT, "h2d_bytes_per_step": n_launched * abi.PIXEL_DTYPE.itemsize,
           "d2h_bytes_per_step": n_launched * abi.RESULT_DTYPE.itemsize, "ms_per_step": t_e2e * 1e3,
           "api": "foort_gpu_run", "launches_per_step": n_launch_run,
           "launches_as_recorded": n_launch_run == len(launches_px) and g_run == n_geod,
           "schedule": "level waves" if sched_used == abi.SCHEDULE_WAVES else "rounds"}

    h2d = d2h = 0
    pin_px = [torch.empty(len(r) * abi.PIXEL_DTYPE.itemsize, dtype=torch.uint8).pin_memory() for r in rounds]
    pin_out = [torch.empty(len(r) * abi.RESULT_DTYPE.itemsize, dtype=torch.uint8).pin_memory() for r in rounds]

    def e2e_step(e):
        nonlocal h2d, d2h
        h2d = d2h = 0
        state = {"r": 0}

        def integrate(px):
            nonlocal h2d, d2h
            k = min(state["r"], len(pin_px) - 1)
            n = len(px)
            if pin_px[k].numel() < n * abi.PIXEL_DTYPE.itemsize:
                pin_px[k] = torch.empty(n * abi.PIXEL_DTYPE.itemsize, dtype=torch.uint8).pin_memory()
                pin_out[k] = torch.empty(n * abi.RESULT_DTYPE.itemsize, dtype=torch.uint8).pin_memory()
            pv = pin_px[k].numpy().view(abi.PIXEL_DTYPE)[:n]
            ov = pin_out[k].numpy().view(abi.RESULT_DTYPE)[:n]
            pv[:] = px
            e.integrate_ptr(pv.ctypes.data, n, ov.ctypes.data)
            h2d += n * abi.PIXEL_DTYPE.itemsize
            d2h += n * abi.RESULT_DTYPE.itemsize
            state["r"] += 1
            return ov

        foort_gb300.run_rounds(wl.mesh, wl.desc, integrate)

    with foort_gb300.Engine(wl.desc) as e:
        e.set_lanes(args.lanes)
        for _ in range(args.warmup):
            e2e_step(e)
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_step(e)
        barrier()
        t_e2e_r = max_over_ranks((time.perf_counter() - t0) / args.steps)
    e2e_rounds = {"value": world * n_geod / t_e2e_r, "unit": UNIT, "h2d_bytes_per_step": h2d,
                  "d2h_bytes_per_step": d2h, "ms_per_step": t_e2e_r * 1e3, "api": "foort_gpu_integrate per round",
                  "launches_per_step": len(rounds)}

    # ---- device-resident mesh: the same run through foort_gpu_run_dmesh, mesh state and
    # results in device memory (one V2 mesh). The warm-up run checks every round's pixels
    # against the host mesh's.
    dmesh = None
    if len(wl.mesh) == 1 and wl.mesh[0][0] == "v2":
        cap = max(len(r) for r in rounds)
        d_res = torch.empty(cap * abi.RESULT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
        same = []

        def new_mesh():
            return foort_gb300.DeviceMesh.from_spec(wl.mesh[0], wl.desc.diag_flags, wl.desc.value_diag)

        with foort_gb300.Engine(wl.desc) as e:
            e.set_lanes(args.lanes)
            e.set_schedule(abi.SCHEDULE_WAVES if args.schedule == "waves" else abi.SCHEDULE_ROUNDS)
            dm = new_mesh()
            g_dm, r_dm = dm.run(e, d_res.data_ptr(), cap, lambda d_px, d_r, n, k: same.append(
                k < len(rounds) and np.array_equal(dm.pixels(), rounds[k])))
            dm.close()
            dm_launches, _ = e.run_info()
            barrier()
            t0 = time.perf_counter()
            for _ in range(args.steps):
                dm = new_mesh()
                dm.run(e, d_res.data_ptr(), cap)
                dm.close()
            barrier()
            t_dm = max_over_ranks((time.perf_counter() - t0) / args.steps)
        dmesh = {"value": world * n_geod / t_dm, "unit": UNIT, "ms_per_step": t_dm * 1e3, "geodesics": g_dm,
                 "rounds": r_dm, "launches_per_step": dm_launches,
                 "same_pixels_as_host_mesh": len(same) == len(rounds) and all(same),
                 "scope": "whole run, device-resident V2 mesh (reference order) and the same schedule on the "
                          "device, results left in device memory"}

    # ---- FP64 plain kernel on the same pixels (N = 1 only: under torchrun the other GPUs
    # would wait for it). Runs of more than FP64_SAMPLE_ABOVE geodesics (C3, C4, C5) take
    # the FP64 legs on a seeded sample of their pixels instead: 1 %, at least 20,000.
    fp64 = None
    acc = None
    if not args.no_fp64 and world == 1 and n_geod > FP64_SAMPLE_ABOVE:
        run_px = np.concatenate(rounds)
        rng = np.random.default_rng(FP64_SAMPLE_SEED)
        n_s = min(n_geod, max(20000, n_geod // 100))
        sample = run_px[np.sort(rng.choice(n_geod, n_s, replace=False))]
        rates, res_s = {}, {}
        for prec in (abi.PREC_MIXED, abi.PREC_FP64):
            wls = workload(args.workload, prec, args.iteration_pixels)
            with foort_gb300.Engine(wls.desc) as e:
                e.set_lanes(args.lanes)
                e.integrate(sample[:256])  # warm-up
                res_s[prec] = e.integrate(sample)
                st = e.stats()
            rates[prec] = (n_s / (st["kernel_ms"] * 1e-3), st["kernel_ms"], st["steps"])
        r64, t64, steps64 = rates[abi.PREC_FP64]
        fp64 = {"value": r64, "unit": UNIT, "ms_per_step": t64, "steps_per_s": steps64 / (t64 * 1e-3),
                "sample": f"{n_s} seeded-random pixels of the run's {n_geod}, one launch per kernel",
                "mixed_on_sample": rates[abi.PREC_MIXED][0],
                "roofline_fp64": {"achieved": steps64 * OPS_PER_STEP.get(mkind, 1130) / (t64 * 1e-3) / 1e12,
                                  "peak": peaks[1], "unit": "TFLOP/s",
                                  "frac": steps64 * OPS_PER_STEP.get(mkind, 1130) / (t64 * 1e-3) / 1e12 / peaks[1]}}
        acc = accuracy_legs(foort_gb300, args, wl, sample, res_s[abi.PREC_MIXED], res_s[abi.PREC_FP64])
    elif not args.no_fp64 and world == 1:
        wl64 = workload(args.workload, abi.PREC_FP64, args.iteration_pixels)
        with foort_gb300.Engine(wl64.desc) as e:
            e.integrate(rounds[-1][:256])  # warm-up
            ev0 = torch.cuda.Event(enable_timing=True)
            ev1 = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            ev0.record(stream)
            kms = device_step(e)
            ev1.record(stream)
            ev1.synchronize()
            t64 = ev0.elapsed_time(ev1)
            res64 = [np.frombuffer(do.cpu().numpy().tobytes(), dtype=abi.RESULT_DTYPE) for do in d_out]
        steps64 = sum(int(r["steps"].sum()) for r in res64)
        fp64 = {"value": n_geod / (t64 * 1e-3), "unit": UNIT, "ms_per_step": t64, "launch_ms": kms,
                "steps_per_s": steps64 / (t64 * 1e-3),
                "roofline_fp64": {"achieved": steps64 * OPS_PER_STEP.get(mkind, 1130) / (t64 * 1e-3) / 1e12,
                                  "peak": peaks[1], "unit": "TFLOP/s",
                                  "frac": steps64 * OPS_PER_STEP.get(mkind, 1130) / (t64 * 1e-3) / 1e12 / peaks[1]}}
        run_px = np.concatenate(rounds)  # the run's own pixels (no looked-ahead ones)
        try:
            pick = pixel_index(np.concatenate(launches_px), run_px)
            acc = accuracy_legs(foort_gb300, args, wl, run_px, np.concatenate(mixed_res)[pick],
                                np.concatenate(res64)[pick])
        except (AssertionError, IndexError) as exc:  # reported, so that the line is still printed
            acc = {"error": f"accuracy legs failed: {exc!r}"}

    # ---- roofline of the dominant kernel: the mixed kernel over all launches of a step
    # (each round is one launch of it), and its largest launch alone
    n_launch = len(launches_px)
    per_launch_ms = [launch_ms[i::n_launch] for i in range(n_launch)]
    ops = OPS_PER_STEP.get(mkind, 1130)

    def launch_ops(i):
        st = int(mixed_res[i]["steps"].sum())
        o = st * ops
        if mkind[1] == "verlet":  # every velocity iteration beyond the two base evaluations
            o += OPS_PER_EXTRA_VERLET_RHS * max(0, mixed_rhs[i] - 2 * st)
        return o, st

    tot_ops = sum(launch_ops(i)[0] for i in range(n_launch))
    tot_ms = sum(statistics.mean(m) for m in per_launch_ms)
    achieved = tot_ops / (tot_ms * 1e-3) / 1e12
    big = int(np.argmax([len(r) for r in launches_px]))
    big_ms = statistics.mean(per_launch_ms[big])
    big_ops, big_steps = launch_ops(big)
    # executed instructions: the issue-slot fraction of the whole step
    instr = sum(int(mixed_res[i]["steps"].sum()) * EXEC_INSTR_PER_STEP.get(mkind + (mixed_lanes[i],), 0)
                for i in range(n_launch))
    clock_mhz = (clk or {}).get("sm_mhz") or 2070.0
    issue_peak = SUBPARTITIONS * torch.cuda.get_device_properties(local).multi_processor_count * clock_mhz * 1e6
    issue = instr / 32 / (tot_ms * 1e-3)
    # DRAM bytes (read + write) of one launch, from ncu's per-geodesic figure scaled to the
    # launch's geodesics (the capture is a 6,000-geodesic sample of the same grid)
    tpg = DRAM_BYTES_PER_GEODESIC.get(mkind)
    traffic = tpg * len(launches_px[big]) if tpg else None
    roofline = {"bound": "alu-fp32", "achieved": achieved, "peak": peaks[0], "unit": "TFLOP/s",
                "frac": achieved / peaks[0], "traffic": traffic, "traffic_unit": "bytes per launch (largest launch)",
                "scope": f"all {n_launch} launches of a step: {tot_ops:.4g} reference-formulation operations in "
                         f"{tot_ms:.1f} ms of kernel time",
                "ops_per_step": ops, "sincos_per_step": SINCOS_PER_STEP.get(mkind, 20),
                "peak_source": "FP32 FMA microbenchmark on this GPU (foort_measure_peaks); MEASURED_PEAKS.json "
                               "has no FP32/FP64 entry",
                "kernel": "integrate_mixed_pair_kernel" if mixed_lanes[big] == 2 else "integrate_mixed_kernel",
                "lanes_per_geodesic": mixed_lanes,
                "largest_launch": {"geodesics": len(launches_px[big]), "launch_ms": big_ms, "steps": big_steps,
                                   "achieved": big_ops / (big_ms * 1e-3) / 1e12,
                                   "frac": big_ops / (big_ms * 1e-3) / 1e12 / peaks[0]},
                "executed": {"thread_instructions_per_step": {f"{k[2]}-lane": v for k, v in EXEC_INSTR_PER_STEP.items()
                                                              if k[:2] == mkind},
                             "warp_instructions_per_s": issue, "issue_peak_per_s": issue_peak,
                             "issue_frac": issue / issue_peak if instr else None,
                             "source": "instructions per step from ncu captures (C2: 6,000-pixel sample; "
                                       "Johannsen Verlet: 20,000 C4 pixels); issue peak = 4 x SMs x median SM clock"},
                "fp64_peak_tflops": peaks[1]}

    # ---- CPU baseline: oracle restatement (-Ofast, all host threads) on a sample (N = 1 only)
    cpu = None
    if not args.no_cpu and world == 1:
        nthreads = os.cpu_count() or 1
        wl_cpu = workload(args.workload, abi.PREC_FP64, args.iteration_pixels)
        rate, n, dt, _ = cpu_sample_rate(wl_cpu, np.concatenate(rounds), args.cpu_seconds or 15.0, nthreads)
        cpu = {"value": rate, "unit": UNIT, "cores": nthreads, "kind": "port",
               "sample": f"{n} seeded-random pixels of this run's pixel set, {dt:.1f} s; oracle restatement "
                         f"built with the reference's -Ofast -fopenmp flags"}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "mixed-f32 (FP32 right-hand side; float-float state and decisions)", "data": "synthetic",
        "config": dict(config_block(wl, args, rounds=len(rounds), geod=n_geod),
                       schedule=("level waves with lookahead (foort_gpu_run's launches): one launch per "
                                 "subdivision level, a launch also taking the next level's candidates while it "
                                 "holds at most 128 x SMs geodesics; the reference's rounds replayed from the "
                                 "results; value counts the run's geodesics only"
                                 if launches_px is not rounds else "one launch per round"),
                       autotuned=not args.no_tune, launch_shapes=tuned_shapes),
        "geodesics_per_step": world * n_geod, "steps_per_s": world * steps_total / (t_step * 1e-3),
        "gpu_launches": args.steps * len(launches_px),
        "e2e": e2e, "e2e_per_round_api": e2e_rounds, "rounds_schedule": rounds_leg, "device_mesh": dmesh,
        "roofline": roofline, "cpu_baseline": cpu, "clocks": clk,
        "fp64": fp64,
        "speedup_vs_fp64": ((fp64["mixed_on_sample"] if "sample" in fp64 else value / world) / fp64["value"])
        if fp64 else None,
        "accuracy": acc,
        "round_sizes": [len(r) for r in rounds],
        "launch_sizes": [len(r) for r in launches_px],
        "geodesics_launched_per_step": world * n_launched,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
