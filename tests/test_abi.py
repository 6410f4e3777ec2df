"""The C-ABI library: it loads, exports every declared symbol, and its struct layouts
match the ctypes mirror. No GPU is needed (no compute call is made)."""
import ctypes as C
import os
import re

import pytest

from conftest import ROOT
from foort_gb300 import abi


def declared_functions(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(foort_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol(engine_lib):
    names = declared_functions("foort_gpu.h")
    assert "foort_gpu_create" in names and "foort_gpu_integrate" in names
    missing = [n for n in names if not hasattr(engine_lib, n)]
    assert not missing, missing


def test_struct_layouts(engine_lib):
    import foort_gb300
    foort_gb300.check_layout()


def test_default_desc_matches_reference_defaults(engine_lib):
    d = abi.RunDesc()
    engine_lib.foort_gpu_default_desc(C.byref(d))
    # Config.cpp:989-1071 (integrator), :690-724 (terminations), Integrators.h:34-57
    assert d.epsilon == 0.03 and d.derivative_h == 1e-7 and d.smallest_step == 1e-12
    assert d.verlet_tol == 0.001 and d.boundary_radius == 1000.0 and d.timeout_max_steps == 10000
    assert d.term_flags == abi.TERM_BOUNDARY_SPHERE | abi.TERM_TIMEOUT
    assert d.value_diag == abi.DIAG_FOUR_COLOR_SCREEN
    ref = abi.default_desc()
    for f, _ in abi.RunDesc._fields_:
        if f in ("images", "n_images"):
            continue
        a, b = getattr(d, f), getattr(ref, f)
        if isinstance(a, abi.UpdateFreq):
            assert (a.every_n, a.at_start, a.at_finish) == (b.every_n, b.at_start, b.at_finish), f
        else:
            assert a == b, f


@pytest.mark.parametrize("metric,params,want", [
    (abi.METRIC_KERR, (0.5,), 1 + (1 - 0.25) ** 0.5),
    (abi.METRIC_JOHANNSEN, (0.9, 0.3, 0, 0, 0), 1 + (1 - 0.81) ** 0.5),
    (abi.METRIC_FLAT, (), 0.0),
])
def test_horizon_radius(engine_lib, metric, params, want):
    import foort_gb300
    assert foort_gb300.horizon_radius(metric, params) == pytest.approx(want, rel=1e-15)


def test_create_rejects_bad_descriptors_without_touching_the_gpu(engine_lib):
    import foort_gb300
    d = abi.default_desc()  # no images
    with pytest.raises(foort_gb300.FoortError) as e:
        foort_gb300.Engine(d)
    assert e.value.code == abi.FOORT_E_BADARG
    keep = abi.attach_images(d, [abi.make_image()])
    d.metric_id = 9
    with pytest.raises(foort_gb300.FoortError) as e:
        foort_gb300.Engine(d)
    assert e.value.code == abi.FOORT_E_BADARG
    d.metric_id = abi.METRIC_KERR
    d.diag_flags |= 0x100  # no such diagnostic
    with pytest.raises(foort_gb300.FoortError) as e:
        foort_gb300.Engine(d)
    assert e.value.code == abi.FOORT_E_BADARG
    d.diag_flags = abi.DIAG_FOUR_COLOR_SCREEN
    d.term_flags = 0  # no termination
    with pytest.raises(foort_gb300.FoortError) as e:
        foort_gb300.Engine(d)
    assert e.value.code == abi.FOORT_E_BADARG
    del keep


def test_kernel_registry(engine_lib):
    """Every metric has FP64 and mixed-precision kernels for both integrators. Host-only
    query."""
    for metric in (abi.METRIC_KERR, abi.METRIC_FLAT, abi.METRIC_RASHEED_LARSEN, abi.METRIC_JOHANNSEN,
                   abi.METRIC_MANKO_NOVIKOV):
        for integ in (abi.INTEGRATOR_RK4, abi.INTEGRATOR_VERLET):
            assert engine_lib.foort_gpu_has_kernel(metric, integ, abi.PREC_FP64) == 1
            assert engine_lib.foort_gpu_has_kernel(metric, integ, abi.PREC_MIXED) == 1, (metric, integ)
    assert engine_lib.foort_gpu_has_kernel(5, abi.INTEGRATOR_RK4, abi.PREC_FP64) == 0
    assert engine_lib.foort_gpu_has_kernel(abi.METRIC_KERR, 2, abi.PREC_FP64) == 0
