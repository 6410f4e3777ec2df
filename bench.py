"""Benchmark of the GB300 geodesic engine (one JSON line on rank 0).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl engine|reference]
                    [--workload c2|c1|c3|c4|c5] [--no-fp64] [--iteration-pixels P]

Metric: geodesics/s on one GB300 of the mixed-precision kernel on the workload (default
C2: Kerr a=0.99 seen at 60 deg, 12 M half-width screen, SquareSubdivisionMeshV2 from a
128^2 seed, MaxSubdivide 3, seed round + 4 refinement rounds), next to the plain FP64
kernel on the same pixels and the endpoint error between the two.

One step = every round of the workload:
  value  pixel lists of all rounds resident in HBM, one persistent-kernel launch per
         round through foort_gpu_integrate_async on one stream; CUDA events on that
         stream around each step; L2 flushed (256 MB write) between steps;
  e2e    the full run through the public C ABI from pinned host memory: host mesh ->
         foort_gpu_integrate (H2D of the pixels, kernel, D2H of the results) ->
         foort_mesh_set_results -> foort_mesh_end_current_loop, every round.
N > 1 (torchrun): every rank integrates its own copy of the workload (weak scaling,
no collective on the data path); times are the max over ranks. The FP64 and CPU legs
run at N = 1 only.
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
# DRAM traffic per geodesic of the mixed kernel (dram__bytes_read.sum + dram__bytes_write.sum
# of one ncu capture divided by its geodesics; profiles/integrate_mixed_pair_kernel_c2.md)
DRAM_BYTES_PER_GEODESIC = {("kerr", "rk4"): 121.1}


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


def run_meshes(eng_mod, e, wl, integrate, on_round=None):
    """One FOORT run (Main.cpp:313-419) of every image of the workload, the images'
    meshes advancing in lockstep so that each round is one launch over all images.
    integrate(px) -> results; on_round(px, res) is called after each round."""
    meshes = [eng_mod.Mesh.from_spec(spec, wl.desc.diag_flags, wl.desc.value_diag) for spec in wl.mesh]
    n_rounds = 0
    while True:
        live = [(i, m) for i, m in enumerate(meshes) if not m.finished()]
        if not live:
            break
        parts = [m.pixels(image=i) for i, m in live]
        px = np.concatenate(parts)
        res = integrate(px)
        k = 0
        for (i, m), p in zip(live, parts):
            m.set_results(res[k:k + len(p)])
            m.end_round()
            k += len(p)
        if on_round:
            on_round(px, res)
        n_rounds += 1
    for m in meshes:
        m.close()
    return n_rounds


def adaptive_rounds(eng_mod, wl, results_out=None):
    """The pixel list of every round of the workload (one run with the engine)."""
    px_rounds = []
    with eng_mod.Engine(wl.desc) as e:
        def keep(px, res):
            px_rounds.append(px.copy())
            if results_out is not None:
                results_out.append(res.copy())
        run_meshes(eng_mod, e, wl, e.integrate, keep)
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


def endpoint_stats(mixed, fp64, rlog):
    from foort_gb300 import accuracy
    mism = accuracy.discrete_mismatch(mixed, fp64)
    same = (~mism) & (mixed["steps"] == fp64["steps"])
    err = accuracy.endpoint_rel_err(mixed[same], fp64[same], rlog=rlog)
    s = accuracy.summarize(err)
    s["frac_le_1e-6"] = float(np.mean(err <= 1e-6)) if len(err) else None
    s["discrete_agreement"] = float(1.0 - mism.mean())
    s["same_step_count"] = float(same.mean())
    return s


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

    # ---- prepare: the workload's pixel lists (one adaptive run with the mixed kernel)
    wl = workload(args.workload, abi.PREC_MIXED, args.iteration_pixels)
    mkind = kind_of(wl)
    t0 = time.perf_counter()
    prep_results = []
    rounds = adaptive_rounds(foort_gb300, wl, prep_results)
    log(f"[bench] {wl.name}: {len(rounds)} rounds, sizes {[len(r) for r in rounds]}, prepare {time.perf_counter() - t0:.1f}s")
    n_geod = sum(len(r) for r in rounds)
    stream = torch.cuda.Stream()
    d_px = [torch.from_numpy(r.view(np.uint8)).to("cuda") for r in rounds]
    d_out = [torch.empty(len(r) * abi.RESULT_DTYPE.itemsize, dtype=torch.uint8, device="cuda") for r in rounds]
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")

    rhs_per_round = [0] * len(rounds)
    lanes_per_round = [1] * len(rounds)

    def device_step(e):
        kms = []
        with torch.cuda.stream(stream):
            for i, (dp, do, r) in enumerate(zip(d_px, d_out, rounds)):
                e.integrate_async(dp.data_ptr(), len(r), do.data_ptr(), stream.cuda_stream)
                e.sync()
                st = e.stats()
                kms.append(st["kernel_ms"])
                rhs_per_round[i] = st["rhs_evals"]
                lanes_per_round[i] = st["lanes_per_geodesic"]
        return kms

    # ---- value: device-resident inputs
    peaks = foort_gb300.measure_peaks()
    with foort_gb300.Engine(wl.desc) as e:
        e.set_lanes(args.lanes)
        for _ in range(args.warmup):
            device_step(e)
        barrier()
        clocks = ClockSampler(local)
        clocks.start()
        step_ms, launch_ms, steps_per_launch = [], [], []
        for _ in range(args.steps):
            flush.fill_(1)
            torch.cuda.synchronize()
            ev0 = torch.cuda.Event(enable_timing=True)
            ev1 = torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
            kms = device_step(e)
            ev1.record(stream)
            ev1.synchronize()
            step_ms.append(ev0.elapsed_time(ev1))
            launch_ms.extend(kms)
        barrier()
        clk = clocks.stop()
        mixed_res = [np.frombuffer(do.cpu().numpy().tobytes(), dtype=abi.RESULT_DTYPE) for do in d_out]
        mixed_rhs, mixed_lanes = list(rhs_per_round), list(lanes_per_round)  # the FP64 leg reuses device_step
    t_step = max_over_ranks(sum(step_ms) / len(step_ms))
    value = world * n_geod / (t_step * 1e-3)
    steps_total = sum(int(r["steps"].sum()) for r in mixed_res)

    # ---- e2e: public C ABI from pinned host memory, host mesh in the loop
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

        run_meshes(foort_gb300, e, wl, integrate)

    with foort_gb300.Engine(wl.desc) as e:
        e.set_lanes(args.lanes)
        for _ in range(args.warmup):
            e2e_step(e)
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_step(e)
        barrier()
        t_e2e = max_over_ranks((time.perf_counter() - t0) / args.steps)
    e2e = {"value": world * n_geod / t_e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
           "ms_per_step": t_e2e * 1e3}

    # ---- FP64 plain kernel on the same pixels (N = 1 only: under torchrun the other GPUs
    # would wait for it)
    fp64 = None
    acc = None
    if not args.no_fp64 and world == 1:
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
        acc = endpoint_stats(np.concatenate(mixed_res), np.concatenate(res64), rlog=bool(wl.desc.rlog))

    # ---- roofline of the dominant kernel (the mixed kernel's largest launch)
    n_launch = len(rounds)
    per_launch_ms = [launch_ms[i::n_launch] for i in range(n_launch)]
    big = int(np.argmax([len(r) for r in rounds]))
    big_ms = statistics.mean(per_launch_ms[big])
    big_rhs = mixed_rhs[big]
    big_steps = int(mixed_res[big]["steps"].sum())
    ops = OPS_PER_STEP.get(mkind, 1130)
    big_ops = big_steps * ops
    if mkind[1] == "verlet":  # every velocity iteration beyond the two base evaluations
        big_ops += OPS_PER_EXTRA_VERLET_RHS * max(0, big_rhs - 2 * big_steps)
    achieved = big_ops / (big_ms * 1e-3) / 1e12
    # DRAM bytes (read + write) of one launch, from ncu's per-geodesic figure scaled to the
    # launch's geodesics (the capture is a 6,000-geodesic sample of the same grid)
    tpg = DRAM_BYTES_PER_GEODESIC.get(mkind)
    traffic = tpg * len(rounds[big]) if tpg else None
    roofline = {"bound": "alu-fp32", "achieved": achieved, "peak": peaks[0], "unit": "TFLOP/s",
                "frac": achieved / peaks[0], "traffic": traffic, "traffic_unit": "bytes per launch",
                "ops_per_step": ops, "sincos_per_step": SINCOS_PER_STEP.get(mkind, 20),
                "peak_source": "FP32 FMA microbenchmark on this GPU (foort_measure_peaks); MEASURED_PEAKS.json "
                               "has no FP32/FP64 entry",
                "kernel": "integrate_mixed_pair_kernel" if mixed_lanes[big] == 2 else "integrate_mixed_kernel",
                "lanes_per_geodesic": mixed_lanes[big],
                "launch_ms": big_ms, "steps_per_launch": big_steps,
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
        "config": config_block(wl, args, rounds=len(rounds), geod=n_geod),
        "geodesics_per_step": world * n_geod, "steps_per_s": world * steps_total / (t_step * 1e-3),
        "gpu_launches": args.steps * len(rounds),
        "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu, "clocks": clk,
        "fp64": fp64, "speedup_vs_fp64": (value / world / fp64["value"]) if fp64 else None,
        "endpoint_error_vs_fp64": acc,
        "round_sizes": [len(r) for r in rounds],
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
