"""The device-resident V2 mesh's argument checks (include/foort_gpu.h foort_dmesh_*),
which return before any CUDA call; its rounds are tested on the GPU in
test_gpu_dmesh.py."""
import ctypes as C

import pytest

from foort_gb300 import abi


def create(lib, **kw):
    a = dict(max_pixels=0, initial_pixels=81, max_subdivide=3, iteration_pixels=10, initial_sub_to_final=0,
             diag_flags=abi.DIAG_FOUR_COLOR_SCREEN, value_diag=abi.DIAG_FOUR_COLOR_SCREEN, image=0,
             order=abi.DMESH_ORDER_REFERENCE)
    a.update(kw)
    out = C.c_void_p()
    rc = lib.foort_dmesh_create_v2(a["max_pixels"], a["initial_pixels"], a["max_subdivide"], a["iteration_pixels"],
                                   a["initial_sub_to_final"], a["diag_flags"], a["value_diag"], a["image"],
                                   a["order"], None, C.byref(out))
    return rc, out


@pytest.mark.parametrize("kw,code", [
    (dict(max_subdivide=0), abi.FOORT_E_BADARG),
    (dict(initial_pixels=3), abi.FOORT_E_BADARG),
    (dict(order=2), abi.FOORT_E_BADARG),
    # 2^30 seed pixels at MaxSubdivide 3: over FOORT_DMESH_MAX_CELLS grid cells
    (dict(initial_pixels=1 << 30), abi.FOORT_E_BADARG),
    (dict(diag_flags=abi.DIAG_GEODESIC_POSITION, value_diag=abi.DIAG_GEODESIC_POSITION), abi.FOORT_E_UNSUPPORTED),
    # [FourColor, GeodesicPosition, EquatorialPasses] rotated by the value diagnostic
    # EquatorialPasses starts with GeodesicPosition
    (dict(diag_flags=abi.DIAG_FOUR_COLOR_SCREEN | abi.DIAG_GEODESIC_POSITION | abi.DIAG_EQUATORIAL_PASSES,
          value_diag=abi.DIAG_EQUATORIAL_PASSES), abi.FOORT_E_UNSUPPORTED),
    (dict(diag_flags=0, value_diag=0), abi.FOORT_E_UNSUPPORTED),
])
def test_create_rejects_bad_arguments_before_touching_the_gpu(engine_lib, kw, code):
    rc, out = create(engine_lib, **kw)
    assert rc == code and not out.value


def test_null_mesh_is_rejected(engine_lib):
    lib = engine_lib
    assert lib.foort_dmesh_is_finished(None) == abi.FOORT_E_BADARG
    assert lib.foort_dmesh_cur_nr_geodesics(None) == 0
    assert lib.foort_dmesh_end_current_loop(None) == abi.FOORT_E_BADARG
    assert lib.foort_dmesh_set_values(None, None, 0) == abi.FOORT_E_BADARG
    assert lib.foort_dmesh_get_pixels(None, None) == abi.FOORT_E_BADARG
    assert lib.foort_dmesh_last_error(None) == b"mesh is NULL"
    lib.foort_dmesh_destroy(None)
