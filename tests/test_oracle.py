"""The oracle (CPU restatement) pinned against the reference.

* the shipped golden outputs FOORT/Output/{Test,debug}_*.dat (all 62,500 pixels each);
* fixtures produced by the reference itself (tests/golden/ref_*.npz): the strict-IEEE
  build of the restatement must equal the strict-IEEE build of the reference bit for bit,
  and the restatement built with the reference's -Ofast flags must give the same discrete
  outputs as the reference's own -Ofast build;
* where the reference sources are present, a live comparison on fresh pixels.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from foort_gb300 import abi, workloads

FIELDS = ("term", "steps", "lam", "pos", "vel", "quadrant", "equat_passes", "closest_r")


@pytest.mark.parametrize("name", ["test", "debug"])
@pytest.mark.parametrize("fast", [False, True])
def test_oracle_reproduces_shipped_dat(oracle_mod, name, fast):
    g = np.load(os.path.join(GOLDEN, f"johannsen_{name}.npz"))
    wl = workloads.johannsen_golden(name == "test")
    px = abi.square_pixels(250)
    res = oracle_mod.integrate(wl.desc, px, fast=fast)
    assert np.array_equal(res["quadrant"], g["quadrant"].astype(np.int32))
    assert np.array_equal(res["equat_passes"], g["passes"].astype(np.int32))


@pytest.mark.parametrize("case", ["c1", "c2", "c3", "c4", "c5", "debug_sample"])
def test_oracle_bit_exact_vs_reference_strict(oracle_mod, case):
    f = np.load(os.path.join(GOLDEN, f"ref_{case}.npz"))
    wl = _workload(case)
    res = oracle_mod.integrate(wl.desc, f["px"])
    ref = f["strict"]
    for k in FIELDS:
        if k == "closest_r" and not (wl.desc.diag_flags & abi.DIAG_CLOSEST_RADIUS):
            continue
        assert np.array_equal(res[k], ref[k]), k


@pytest.mark.parametrize("case", ["c1", "c2", "c3", "c4", "c5", "debug_sample"])
def test_oracle_fast_vs_reference_fast(oracle_mod, case):
    f = np.load(os.path.join(GOLDEN, f"ref_{case}.npz"))
    wl = _workload(case)
    res = oracle_mod.integrate(wl.desc, f["px"], fast=True)
    ref = f["fast"]
    for k in ("term", "quadrant", "equat_passes"):
        assert np.array_equal(res[k], ref[k]), k


def _workload(case):
    if case == "c1":
        return workloads.c1()
    if case == "c2":
        wl = workloads.c2()
        wl.desc.value_diag = abi.DIAG_CLOSEST_RADIUS
        return wl
    if case == "c3":
        return workloads.c3(n_images=64)
    if case == "c4":
        wl = workloads.c4()
        wl.desc.value_diag = abi.DIAG_CLOSEST_RADIUS
        return wl
    if case == "c5":
        return workloads.c5()
    if case == "debug_sample":
        return workloads.johannsen_golden(False)
    raise KeyError(case)


def test_oracle_live_vs_reference(oracle_mod):
    """Fresh pixels and a metric no fixture covers, against the reference run live."""
    if not oracle_mod.have_ref(strict=True):
        pytest.skip("reference sources not present")
    for metric, params, rlog in ((abi.METRIC_RASHEED_LARSEN, (0.3556562853309941, 0.2969060968239216,
                                                              3.057664971085168, 0.942335028914832), 1),
                                 (abi.METRIC_MANKO_NOVIKOV, (0.94, 13.0), 1),
                                 (abi.METRIC_FLAT, (), 0),
                                 (abi.METRIC_KERR, (0.94,), 1)):
        d = workloads.base_desc()
        d.metric_id = metric
        d.rlog = rlog
        d.term_flags |= abi.TERM_THETA_SINGULARITY
        d.timeout_max_steps = 20000
        d.diag_flags = abi.DIAG_FOUR_COLOR_SCREEN | abi.DIAG_EQUATORIAL_PASSES | abi.DIAG_CLOSEST_RADIUS
        d.value_diag = abi.DIAG_CLOSEST_RADIUS
        d.integrator_id = abi.INTEGRATOR_VERLET if metric == abi.METRIC_FLAT else abi.INTEGRATOR_RK4
        keep = abi.attach_images(d, [abi.make_image(params, r=1000.0, theta=1.2, half_width=12.0)])
        px = abi.square_pixels(23)[::11]
        a = oracle_mod.integrate(d, px)
        b = oracle_mod.ref_integrate(d, px, strict=True)
        for k in FIELDS[:-1]:
            assert np.array_equal(a[k], b[k]), (metric, k)
        # With FourColor + EquatorialPasses + ClosestRadius (value) the reference's
        # diagnostic vector is [EquatorialPasses, ClosestRadius, FourColor]
        # (Diagnostics.cpp:28-75 rotates left by one), so ClosestRadius is read back from
        # its std::to_string text, six decimals.
        assert np.allclose(a["closest_r"], b["closest_r"], rtol=0, atol=5.01e-7)
        del keep


def test_mt19937_64_known_answer():
    # The C++ standard requires the 10000th output of a default-constructed
    # std::mt19937_64 (seed 5489) to be 9981545732273789042.
    g = workloads.MT19937_64(5489)
    for _ in range(9999):
        g.next_u64()
    assert g.next_u64() == 9981545732273789042
