"""GPU parity of the mixed-precision kernel (-m gpu), through the C ABI.

Against the reference (shipped golden files and reference fixtures): the discrete
outputs, with the rules of foort_gb300/accuracy.py (>= 99.9 % agreement, every
disagreement on a decision boundary). Against the FP64 kernel on the same pixels: the
relative endpoint error e (accuracy.endpoint_rel_err) on pixels with the same discrete
outputs and step count, bounded per workload by the tolerances below.
"""
import os

import numpy as np
import pytest

import parity
from conftest import GOLDEN
from foort_gb300 import abi, workloads

pytestmark = pytest.mark.gpu

# Endpoint error of the mixed kernel against the FP64 kernel (median, p90). The FP32
# right-hand side has ~1e-7 relative error per evaluation; compensated state and
# unbiased step arithmetic keep the accumulated endpoint error near that level.
MIXED_MEDIAN_TOL = 1e-6
MIXED_P90_TOL = 1e-5


@pytest.fixture(scope="module")
def eng():
    import foort_gb300
    from foort_gb300 import build as engine_build
    engine_build.build()
    foort_gb300.check_layout()
    if not foort_gb300.mixed_available():
        pytest.fail("the mixed-precision kernels are missing from this build")
    return foort_gb300


def run(eng, desc, px, precision, options=0):
    desc.precision = precision
    desc.mixed_options = options
    with eng.Engine(desc) as e:
        r = e.integrate(px)
        return r, e.stats()


@pytest.mark.parametrize("name", ["test", "debug"])
@pytest.mark.parametrize("options", [0, abi.MIXED_FP64_DECISIONS])
def test_mixed_reproduces_shipped_golden(eng, oracle_mod, name, options):
    """FOORT/Output/{Test,debug}_*.dat: Johannsen, log-r, Verlet / RK4, 62,500 pixels."""
    g = np.load(os.path.join(GOLDEN, f"johannsen_{name}.npz"))
    wl = workloads.johannsen_golden(name == "test")
    px = abi.square_pixels(250)
    res, st = run(eng, wl.desc, px, abi.PREC_MIXED, options)
    mism = (res["quadrant"] != g["quadrant"]) | (res["equat_passes"] != g["passes"])
    agree = 1.0 - mism.mean()
    print(f"{name} options={options}: agreement {agree:.6f} ({mism.sum()} differ), {st['kernel_ms']:.1f} ms")
    assert agree >= parity.MIN_DISCRETE_AGREEMENT
    wl.desc.precision = abi.PREC_FP64
    ref = oracle_mod.integrate(wl.desc, px[mism], fast=True)
    real = np.zeros(len(px), dtype=bool)
    real[np.nonzero(mism)[0]] = parity.discrete_mismatch(res[mism], ref)
    unexplained = parity.explain_mismatches(oracle_mod, wl.desc, px, res, real)
    assert len(unexplained) == 0, unexplained


CASES = {"c1": lambda: workloads.c1(), "c2": lambda: workloads.c2(), "c3": lambda: workloads.c3(n_images=64),
         "c4": lambda: workloads.c4(), "c5": lambda: workloads.c5(),
         "debug_sample": lambda: workloads.johannsen_golden(False)}


@pytest.mark.parametrize("case", sorted(CASES))
def test_mixed_vs_reference_and_fp64(eng, oracle_mod, case):
    f = np.load(os.path.join(GOLDEN, f"ref_{case}.npz"))
    wl = CASES[case]()
    if case in ("c2", "c4"):
        wl.desc.value_diag = abi.DIAG_CLOSEST_RADIUS
    px, ref = f["px"], f["fast"]
    res, _ = run(eng, wl.desc, px, abi.PREC_MIXED)
    r64, _ = run(eng, wl.desc, px, abi.PREC_FP64)
    wl.desc.precision = abi.PREC_FP64
    mism = parity.discrete_mismatch(res, ref)
    unexplained = parity.explain_mismatches(oracle_mod, wl.desc, px, res, mism)
    print(f"{case}: agreement with the reference {1 - mism.mean():.4f}")
    assert len(unexplained) == 0, unexplained
    m64 = parity.discrete_mismatch(res, r64)
    same = (~m64) & (res["steps"] == r64["steps"])
    s = parity.summarize(parity.endpoint_rel_err(res[same], r64[same], rlog=bool(wl.desc.rlog)))
    print(f"{case}: vs FP64 kernel: agreement {1 - m64.mean():.4f}, same steps {same.mean():.4f}, endpoint {s}")
    assert s["median"] < MIXED_MEDIAN_TOL and s["p90"] < MIXED_P90_TOL, s


def oracle_report(eng, desc, px):
    """Mixed and plain FP64 (the reference's finite differences) against the FP64-analytic
    oracle: per-pixel errors, condition numbers from two shifted mixed launches, and the
    accuracy reports of both."""
    from foort_gb300 import accuracy
    rlog = bool(desc.rlog)
    out = {}
    keep = desc.precision
    for prec in (abi.PREC_MIXED, abi.PREC_FP64_ANALYTIC, abi.PREC_FP64):
        desc.precision = prec
        with eng.Engine(desc) as e:
            out[prec] = e.integrate(px)
    desc.precision = abi.PREC_MIXED
    K, _ = accuracy.shift_refinement(int(px["grid"].max()))
    step = 1.0 / (K * (px["grid"].astype(np.int64) - 1))
    with eng.Engine(desc) as e:
        shifted = [e.integrate(accuracy.shifted_pixels(px, K, ax)) for ax in (0, 1)]
    desc.precision = keep
    kappa = accuracy.condition_numbers(out[abi.PREC_MIXED], shifted, step, rlog=rlog)
    ora = out[abi.PREC_FP64_ANALYTIC]
    em = accuracy.endpoint_err_all(out[abi.PREC_MIXED], ora, rlog)
    ef = accuracy.endpoint_err_all(out[abi.PREC_FP64], ora, rlog)
    return accuracy.error_report(em, kappa), accuracy.error_report(ef, kappa)


def c2_sample(n=8000, seed=11):
    rng = np.random.default_rng(seed)
    idx = np.sort(rng.choice(509 * 509, n, replace=False))
    px = np.zeros(len(idx), dtype=abi.PIXEL_DTYPE)
    px["row"], px["col"], px["grid"] = idx // 509, idx % 509, 509
    return px


# Against the FP64-analytic oracle (every step in FP64 with the mixed kernel's
# derivatives), plain r: on well-conditioned pixels (kappa <= 10) the p99 of the endpoint
# error within 1e-6 (at least 98 % of end points within it) and the median within 1e-7;
# a backward error (error / kappa, in units of the screen) with p99 within 1e-6 and a
# median no larger than that of the plain FP64 kernel, whose finite differences
# (h = 1e-7) keep fewer digits where the metric is nearly flat. In log-r mode the backward error is as small as in plain r, but the reference's
# finite differences are far better there (h = 1e-7 in ln r is a relative step) and the
# shipped log-r view is mostly ill-conditioned pixels: there the median within 1e-6, 80 %
# of well-conditioned pixels within 1e-6 and the backward error's p99 within 1e-6.
ORACLE_CASES = dict(CASES, c2_sample8000=None)


@pytest.mark.parametrize("case", sorted(ORACLE_CASES))
def test_mixed_against_the_fp64_analytic_oracle(eng, case):
    if case == "c2_sample8000":
        wl, px = workloads.c2(), c2_sample()
    else:
        wl, px = CASES[case](), np.load(os.path.join(GOLDEN, f"ref_{case}.npz"))["px"]
    if case in ("c2", "c4"):
        wl.desc.value_diag = abi.DIAG_CLOSEST_RADIUS
    rm, rf = oracle_report(eng, wl.desc, px)
    print(f"{case}: mixed {rm}\n{case}: plain FP64 {rf}")
    mism = rm["all"]["mismatched_or_nonfinite"]
    assert mism <= max(1, len(px) // 1000), rm["all"]
    w, b, bf = rm["well_conditioned"], rm["backward_error"], rf["backward_error"]
    assert b["p99"] <= 1e-6, b
    if wl.desc.rlog:
        assert rm["all"]["median"] <= 1e-6 and w["frac_le_1e-6"] >= 0.8, (rm["all"], w)
    else:
        assert w["p99"] <= 1e-6 and w["frac_le_1e-6"] >= 0.98 and w["median"] <= 1e-7, w
        assert b["median"] <= bf["median"], (b, bf)


def test_mixed_large_sample_vs_fp64(eng):
    """8,000 pixels of the C2 grid: the statistic the benchmark reports."""
    wl = workloads.c2()
    rng = np.random.default_rng(11)
    idx = np.sort(rng.choice(509 * 509, 8000, replace=False))
    px = np.zeros(len(idx), dtype=abi.PIXEL_DTYPE)
    px["row"], px["col"], px["grid"] = idx // 509, idx % 509, 509
    res, sm = run(eng, wl.desc, px, abi.PREC_MIXED)
    r64, s64 = run(eng, wl.desc, px, abi.PREC_FP64)
    m64 = parity.discrete_mismatch(res, r64)
    same = (~m64) & (res["steps"] == r64["steps"])
    err = parity.endpoint_rel_err(res[same], r64[same])
    s = parity.summarize(err)
    print(f"C2 sample: agreement {1 - m64.mean():.5f}; endpoint {s}; <=1e-6: {np.mean(err <= 1e-6):.4f}; "
          f"speed-up {s64['kernel_ms'] / sm['kernel_ms']:.1f}x")
    assert 1 - m64.mean() >= parity.MIN_DISCRETE_AGREEMENT
    assert s["median"] < MIXED_MEDIAN_TOL and s["p90"] < MIXED_P90_TOL


@pytest.mark.parametrize("case", ["c2", "c1"])
def test_two_lanes_per_geodesic_give_the_one_lane_results(eng, case):
    """The two-lane kernel (foort_gpu_set_lanes) does step()'s arithmetic on the same
    values, split over two lanes: every field of every record must be identical."""
    wl = workloads.c2() if case == "c2" else workloads.c1()
    wl.desc.precision = abi.PREC_MIXED
    rng = np.random.default_rng(3)
    side = 509 if case == "c2" else 100
    idx = np.sort(rng.choice(side * side, 3000, replace=False))
    px = np.zeros(len(idx), dtype=abi.PIXEL_DTYPE)
    px["row"], px["col"], px["grid"] = idx // side, idx % side, side
    out = {}
    with eng.Engine(wl.desc) as e:
        for lanes in (1, 2, 0):
            e.set_lanes(lanes)
            out[lanes] = e.integrate(px)
            st = e.stats()
            assert st["lanes_per_geodesic"] == (lanes or 2), st  # 3,000 geodesics: two lanes fit
            assert st["geodesics"] == len(px)
    for name in abi.RESULT_DTYPE.names:
        np.testing.assert_array_equal(out[2][name], out[1][name], err_msg=name)
        np.testing.assert_array_equal(out[0][name], out[1][name], err_msg=name)


# Rasheed-Larsen parameter sets (m, a, p, q): "Lorenzo" and the extremal "M1" of the
# reference's Test.cfg, and the reference's defaults
RL_SETS = {"lorenzo": (0.3556562853309941, 0.2969060968239216, 3.057664971085168, 0.942335028914832),
           "m1": (0.0000292676523070559347272298622578, 0.0000292676523070559347272298622578,
                  3.15470053516341633378322799917, 0.84529946483658456162619604143),
           "default": (1.0, 0.5, 2.0, 2.0)}


# screens: (inclination, half-width). 63 deg and 12 M mostly see weakly bent rays; 80 deg
# and 5 M put most pixels on the strongly lensed rays around the shadow.
VIEWS = {"wide": (1.1, 12.0), "shadow": (1.3962634016, 5.0)}


@pytest.mark.parametrize("name,rlog,integ,view", [("lorenzo", 0, abi.INTEGRATOR_RK4, "wide"),
                                                  ("lorenzo", 1, abi.INTEGRATOR_RK4, "wide"),
                                                  ("m1", 0, abi.INTEGRATOR_RK4, "wide"),
                                                  ("default", 0, abi.INTEGRATOR_RK4, "wide"),
                                                  ("lorenzo", 0, abi.INTEGRATOR_VERLET, "wide"),
                                                  ("lorenzo", 0, abi.INTEGRATOR_RK4, "shadow")])
def test_mixed_rasheed_larsen(eng, oracle_mod, name, rlog, integ, view):
    """Rasheed-Larsen on a 48^2 screen: the mixed kernel's discrete outcomes against the
    FP64 kernel (disagreements explained by the oracle), and its endpoint error against
    the FP64 kernel within the mixed tolerances."""
    d = workloads.base_desc()
    d.metric_id, d.rlog, d.integrator_id = abi.METRIC_RASHEED_LARSEN, rlog, integ
    d.term_flags |= abi.TERM_THETA_SINGULARITY
    d.timeout_max_steps = 20000
    d.diag_flags = abi.DIAG_FOUR_COLOR_SCREEN | abi.DIAG_EQUATORIAL_PASSES | abi.DIAG_CLOSEST_RADIUS
    inc, hw = VIEWS[view]
    keep = abi.attach_images(d, [abi.make_image(RL_SETS[name], r=1000.0, theta=inc, half_width=hw)])
    px = abi.square_pixels(48)
    res, sm = run(eng, d, px, abi.PREC_MIXED)
    r64, s64 = run(eng, d, px, abi.PREC_FP64)
    d.precision = abi.PREC_FP64
    mism = parity.discrete_mismatch(res, r64)
    unexplained = parity.explain_mismatches(oracle_mod, d, px, res, mism)
    same = (~mism) & (res["steps"] == r64["steps"])
    s = parity.summarize(parity.endpoint_rel_err(res[same], r64[same], rlog=bool(rlog)))
    print(f"RL {name} rlog={rlog} integrator={integ} {view}: agreement {1 - mism.mean():.4f}, same steps "
          f"{same.mean():.4f}, endpoint {s}, speed-up {s64['kernel_ms'] / sm['kernel_ms']:.1f}x")
    assert len(unexplained) == 0, unexplained
    assert 1 - mism.mean() >= parity.MIN_DISCRETE_AGREEMENT
    assert s["median"] < MIXED_MEDIAN_TOL and s["p90"] < MIXED_P90_TOL, s
    del keep


def test_mixed_budget_and_cancel_paths(eng):
    wl = workloads.c1(precision=abi.PREC_MIXED)
    px = abi.square_pixels(60)
    with eng.Engine(wl.desc) as e:
        e.set_budget(100000)
        res = e.integrate(px, allow=(abi.FOORT_E_BUDGET,))
        assert e.stats()["status"] != 0
    assert np.any(res["err"] & (abi.ERR_BUDGET | abi.ERR_UNFINISHED))


def test_integrate_async_returns_before_the_launch_ends(eng):
    """foort_gpu_integrate_async returns once the launch is enqueued: on a launch of about
    0.1 s (2,048 of the C2 run's pixels, ~66k steps each) the call takes a small part of
    it, and foort_gpu_sync then waits for results equal to the synchronous call's."""
    import time
    import torch
    f = np.load(os.path.join(GOLDEN, "c2_run.npz"))
    px = np.zeros(2048, dtype=abi.PIXEL_DTYPE)
    px["row"], px["col"], px["grid"] = f["row"][:2048], f["col"][:2048], 509
    wl = workloads.c2(abi.PREC_MIXED)
    with eng.Engine(wl.desc) as e:
        ref = e.integrate(px)
        d_px = torch.from_numpy(px.view(np.uint8).copy()).cuda()
        d_out = torch.zeros(len(px) * abi.RESULT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e.integrate_async(d_px.data_ptr(), len(px), d_out.data_ptr())
        t_call = time.perf_counter() - t0
        e.sync()
        t_all = time.perf_counter() - t0
        got = np.frombuffer(d_out.cpu().numpy().tobytes(), dtype=abi.RESULT_DTYPE)
    print(f"call {t_call * 1e3:.2f} ms, launch {t_all * 1e3:.1f} ms")
    assert t_all > 0.03 and t_call < 0.25 * t_all, (t_call, t_all)
    for name in abi.RESULT_DTYPE.names:
        np.testing.assert_array_equal(got[name], ref[name], err_msg=name)


# Manko-Novikov (a, alpha3): the reference's Test.cfg value alpha3 = 13, its default 5,
# and a mild 1
MN_SETS = {"alpha3_13": (0.94, 13.0), "alpha3_5": (0.9, 5.0), "alpha3_1": (0.7, 1.0)}


@pytest.mark.parametrize("name,integ,view", [("alpha3_13", abi.INTEGRATOR_RK4, "wide"),
                                             ("alpha3_5", abi.INTEGRATOR_RK4, "wide"),
                                             ("alpha3_1", abi.INTEGRATOR_RK4, "wide"),
                                             ("alpha3_5", abi.INTEGRATOR_VERLET, "wide"),
                                             ("alpha3_13", abi.INTEGRATOR_RK4, "shadow")])
def test_mixed_manko_novikov(eng, oracle_mod, name, integ, view):
    """Manko-Novikov on a 48^2 screen: the mixed kernel (FP32 outside the radius where the
    metric's exponents exceed 8, FP64 inside) against the FP64 kernel, as for the other
    metrics."""
    d = workloads.base_desc()
    d.metric_id, d.integrator_id = abi.METRIC_MANKO_NOVIKOV, integ
    d.term_flags |= abi.TERM_THETA_SINGULARITY
    d.timeout_max_steps = 20000
    d.diag_flags = abi.DIAG_FOUR_COLOR_SCREEN | abi.DIAG_EQUATORIAL_PASSES | abi.DIAG_CLOSEST_RADIUS
    inc, hw = VIEWS[view]
    keep = abi.attach_images(d, [abi.make_image(MN_SETS[name], r=1000.0, theta=inc, half_width=hw)])
    px = abi.square_pixels(48)
    res, sm = run(eng, d, px, abi.PREC_MIXED)
    r64, s64 = run(eng, d, px, abi.PREC_FP64)
    d.precision = abi.PREC_FP64
    mism = parity.discrete_mismatch(res, r64)
    unexplained = parity.explain_mismatches(oracle_mod, d, px, res, mism)
    same = (~mism) & (res["steps"] == r64["steps"])
    s = parity.summarize(parity.endpoint_rel_err(res[same], r64[same]))
    print(f"MN {name} integrator={integ} {view}: agreement {1 - mism.mean():.4f}, same steps {same.mean():.4f}, "
          f"endpoint {s}, FP64 share of right-hand sides {sm['fp64_steps'] / max(1, sm['rhs_evals']):.3f}, "
          f"speed-up {s64['kernel_ms'] / sm['kernel_ms']:.1f}x")
    assert len(unexplained) == 0, unexplained
    assert 1 - mism.mean() >= parity.MIN_DISCRETE_AGREEMENT
    assert s["median"] < MIXED_MEDIAN_TOL and s["p90"] < MIXED_P90_TOL, s
    del keep
