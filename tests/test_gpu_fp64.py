"""GPU parity of the FP64 kernel against the reference and the oracle (-m gpu).

Every call goes through the C ABI (libfoort_gpu.so). The rules are in tests/parity.py:
>= 99.9 % discrete agreement with every disagreement on a decision boundary, and the
endpoint error stated per case.
"""
import ctypes as C
import os

import numpy as np
import pytest

import parity
from conftest import GOLDEN
from foort_gb300 import abi, workloads

pytestmark = pytest.mark.gpu

# Endpoint tolerance of the FP64 kernel against the reference's FP64 CPU result, on
# pixels with the same discrete outputs and step count. Both follow the same algorithm
# in FP64; they differ in the libm (CUDA vs glibc), FMA contraction and the reference's
# -Ofast, and the finite-difference Christoffels amplify last-bit differences of the
# metric by 1/h = 1e7, so agreement is to ~1e-9 for most pixels rather than bit for bit.
FP64_MEDIAN_TOL = 1e-7
FP64_P90_TOL = 1e-5


@pytest.fixture(scope="module")
def eng():
    import foort_gb300
    from foort_gb300 import build as engine_build
    engine_build.build()
    foort_gb300.check_layout()
    return foort_gb300


def run(eng, wl, px):
    with eng.Engine(wl.desc) as e:
        return e.integrate(px)


@pytest.mark.parametrize("name", ["test", "debug"])
def test_fp64_reproduces_shipped_golden(eng, oracle_mod, name):
    """All 62,500 pixels of FOORT/Output/{Test,debug}_*.dat."""
    g = np.load(os.path.join(GOLDEN, f"johannsen_{name}.npz"))
    wl = workloads.johannsen_golden(name == "test")
    px = abi.square_pixels(250)
    res = run(eng, wl, px)
    assert np.all(res["err"] == 0)
    mism = (res["quadrant"] != g["quadrant"]) | (res["equat_passes"] != g["passes"])
    agree = 1.0 - mism.mean()
    print(f"{name}: agreement {agree:.6f} ({mism.sum()} pixels differ)")
    assert agree >= parity.MIN_DISCRETE_AGREEMENT
    ref = oracle_mod.integrate(wl.desc, px[mism], fast=True)
    ref_mism = np.zeros(len(px), dtype=bool)
    ref_mism[np.nonzero(mism)[0]] = parity.discrete_mismatch(res[mism], ref)
    unexplained = parity.explain_mismatches(oracle_mod, wl.desc, px, res, ref_mism)
    assert len(unexplained) == 0, unexplained


def _fixture_case(case):
    wl = {"c1": workloads.c1, "c2": workloads.c2, "c4": workloads.c4, "c5": workloads.c5,
          "debug_sample": lambda: workloads.johannsen_golden(False),
          "c3": lambda: workloads.c3(precision=abi.PREC_FP64)}[case]()
    if case in ("c2", "c4"):
        wl.desc.value_diag = abi.DIAG_CLOSEST_RADIUS
    wl.desc.precision = abi.PREC_FP64
    return wl


@pytest.mark.parametrize("case", ["c1", "c2", "c3", "c4", "c5", "debug_sample"])
def test_fp64_vs_reference_fixture(eng, oracle_mod, case):
    f = np.load(os.path.join(GOLDEN, f"ref_{case}.npz"))
    wl = _fixture_case(case)
    px, ref = f["px"], f["fast"]
    res = run(eng, wl, px)
    mism = parity.discrete_mismatch(res, ref)
    agree = 1.0 - mism.mean()
    unexplained = parity.explain_mismatches(oracle_mod, wl.desc, px, res, mism)
    same = (~mism) & (res["steps"] == ref["steps"])
    err = parity.endpoint_rel_err(res[same], ref[same], rlog=bool(wl.desc.rlog))
    s = parity.summarize(err)
    print(f"{case}: agreement {agree:.4f}, same-steps {same.mean():.3f}, endpoint {s}")
    assert len(unexplained) == 0, unexplained
    assert agree >= 0.99
    assert s["median"] < FP64_MEDIAN_TOL and s["p90"] < FP64_P90_TOL
    if wl.desc.diag_flags & abi.DIAG_CLOSEST_RADIUS:
        # The closest radius is a minimum over the step points; orbits that pass close
        # to the photon sphere amplify last-bit differences (the reference's own -Ofast
        # and strict builds differ by up to 2e-6 there), so the bound is statistical.
        ok = ~mism & (ref["term"] != abi.TERMCODE_HORIZON)
        rel = np.abs(res["closest_r"][ok] - ref["closest_r"][ok]) / np.abs(ref["closest_r"][ok])
        print(f"{case}: closest radius rel. diff median {np.median(rel):.2e}, max {rel.max():.2e}")
        assert np.median(rel) < 1e-8 and np.quantile(rel, 0.99) < 1e-5


def test_fp64_vs_oracle_random_metrics(eng, oracle_mod):
    """Every metric plugin and both integrators on a small screen."""
    cases = [(abi.METRIC_KERR, (0.9,), 0, abi.INTEGRATOR_RK4),
             (abi.METRIC_KERR, (0.3,), 1, abi.INTEGRATOR_VERLET),
             (abi.METRIC_JOHANNSEN, (0.8, 1.0, 0.5, 0.2, 0.1), 1, abi.INTEGRATOR_RK4),
             (abi.METRIC_RASHEED_LARSEN, (0.3556562853309941, 0.2969060968239216, 3.057664971085168,
                                          0.942335028914832), 1, abi.INTEGRATOR_RK4),
             (abi.METRIC_MANKO_NOVIKOV, (0.94, 13.0), 1, abi.INTEGRATOR_RK4),
             (abi.METRIC_FLAT, (), 0, abi.INTEGRATOR_VERLET)]
    for metric, params, rlog, integ in cases:
        d = workloads.base_desc()
        d.metric_id, d.rlog, d.integrator_id = metric, rlog, integ
        d.term_flags |= abi.TERM_THETA_SINGULARITY
        d.timeout_max_steps = 20000
        d.diag_flags = abi.DIAG_FOUR_COLOR_SCREEN | abi.DIAG_EQUATORIAL_PASSES | abi.DIAG_CLOSEST_RADIUS
        keep = abi.attach_images(d, [abi.make_image(params, r=1000.0, theta=1.1, half_width=12.0)])
        px = abi.square_pixels(24)
        with eng.Engine(d) as e:
            res = e.integrate(px)
        ref = oracle_mod.integrate(d, px)
        mism = parity.discrete_mismatch(res, ref)
        unexplained = parity.explain_mismatches(oracle_mod, d, px, res, mism)
        same = (~mism) & (res["steps"] == ref["steps"])
        s = parity.summarize(parity.endpoint_rel_err(res[same], ref[same], rlog=bool(rlog)))
        print(metric, integ, f"agreement {1 - mism.mean():.4f}", s)
        assert len(unexplained) == 0, (metric, unexplained)
        assert s["median"] < FP64_MEDIAN_TOL, (metric, s)
        del keep


def test_budget_stops_every_lane(eng):
    wl = workloads.c1()
    px = abi.square_pixels(40)
    with eng.Engine(wl.desc) as e:
        e.set_budget(200000)
        res = e.integrate(px, allow=(abi.FOORT_E_BUDGET,))
        st = e.stats()
    assert st["status"] == abi.FOORT_E_BUDGET & 0xFFFFFFFF or st["status"] == abi.FOORT_E_BUDGET
    unfinished = res["term"] == abi.TERMCODE_CONTINUE
    assert unfinished.sum() > 0
    assert np.all(res["err"][unfinished] & (abi.ERR_BUDGET | abi.ERR_UNFINISHED))
    # the counter may overshoot by at most one poll interval per warp
    assert st["steps"] < 200000 + 512 * 32 * st["n_blocks"] * 4


def test_cancel_from_host(eng):
    """C1 in FP64 (10,000 geodesics of ~60,000 steps) takes ~5 s on a GB300: a cancel
    from another host thread after 0.3 s must stop it, mark the geodesics in flight
    FOORT_ERR_CANCELLED and the unstarted ones FOORT_ERR_UNFINISHED."""
    import threading
    import time
    wl = workloads.c1()
    px = abi.square_pixels(100)
    with eng.Engine(wl.desc) as e:
        t = threading.Timer(0.3, e.cancel)
        t.start()
        t0 = time.time()
        res = e.integrate(px, allow=(0, abi.FOORT_E_CANCELLED))
        dt = time.time() - t0
        t.join()
        st = e.stats()
    print(f"cancelled after {dt:.2f} s: {st['geodesics']} of {len(px)} geodesics finished")
    status = C.c_int32(st["status"]).value  # foort_stats.status holds the FOORT_E_* code in a uint32
    assert status == abi.FOORT_E_CANCELLED, f"the launch ended ({dt:.2f} s) without seeing the cancel flag"
    assert dt < 3.0
    assert np.any(res["err"] & abi.ERR_CANCELLED)
    stopped = (res["err"] & (abi.ERR_CANCELLED | abi.ERR_UNFINISHED)) != 0
    assert np.all(res["term"][stopped] == abi.TERMCODE_CONTINUE)
    assert np.all(res["term"][~stopped] != abi.TERMCODE_CONTINUE)


def test_empty_and_bad_pixels(eng):
    wl = workloads.c1()
    with eng.Engine(wl.desc) as e:
        assert len(e.integrate(abi.square_pixels(1)[:0])) == 0
        px = abi.square_pixels(3)
        px["image"][1] = 5
        with pytest.raises(eng.FoortError) as err:
            e.integrate(px)
        assert err.value.code == abi.FOORT_E_BADARG


def test_nonfinite_state_is_flagged_and_times_out_like_the_reference(eng, oracle_mod):
    """A camera on the axis (theta = 0) gives a NaN frame (1 / sin(theta)); the reference
    integrates the NaN state until TimeOut fires, and so does the engine, with
    FOORT_ERR_NONFINITE set."""
    d = workloads.base_desc()
    d.timeout_max_steps = 50
    keep = abi.attach_images(d, [abi.make_image((0.5,), r=1000.0, theta=0.0)])
    px = abi.square_pixels(4)
    with eng.Engine(d) as e:
        res = e.integrate(px)
    ref = oracle_mod.integrate(d, px)
    assert np.all(res["term"] == abi.TERMCODE_TIMEOUT) and np.all(ref["term"] == abi.TERMCODE_TIMEOUT)
    assert np.all(res["steps"] == ref["steps"])
    assert np.all(res["err"] & abi.ERR_NONFINITE) and np.all(ref["err"] & abi.ERR_NONFINITE)
    del keep
