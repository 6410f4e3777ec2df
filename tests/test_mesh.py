"""Host meshes against the reference's own meshes (tests/golden/mesh_traces.npz, produced
by driving SimpleSquareMesh / SquareSubdivisionMeshV2 of the reference with synthetic
values). Index work: the pixel sequences must be identical."""
import os

import numpy as np
import pytest

import oracle
from conftest import GOLDEN
from foort_gb300 import abi

TRACES = np.load(os.path.join(GOLDEN, "mesh_traces.npz"))
CASES = sorted({k.rsplit("_", 1)[0] for k in TRACES.files if k.endswith("_spec")})


@pytest.mark.parametrize("case", CASES)
def test_mesh_matches_reference_trace(engine_lib, case):
    import foort_gb300
    kind, init, maxsub, iterpix, maxpix, stf, vd, vk = [int(v) for v in TRACES[case + "_spec"]]
    rows, cols, rnd = TRACES[case + "_rows"], TRACES[case + "_cols"], TRACES[case + "_round"]
    if kind == 0:
        mesh = foort_gb300.Mesh("simple", int(vd), int(vd), total_pixels=init)
    else:
        mesh = foort_gb300.Mesh("v2", int(vd), int(vd), max_pixels=maxpix, initial_pixels=init, max_subdivide=maxsub,
                                iteration_pixels=iterpix, initial_sub_to_final=stf)
    grid = mesh.grid()
    k, r = 0, 0
    while not mesh.finished():
        px = mesh.pixels()
        n = len(px)
        assert np.array_equal(px["row"], rows[k:k + n]), (case, r)
        assert np.array_equal(px["col"], cols[k:k + n]), (case, r)
        assert np.all(rnd[k:k + n] == r)
        assert np.all(px["grid"] == grid)
        mesh.set_values([oracle.synth_value(vk, a, b, grid) for a, b in zip(px["row"], px["col"])])
        mesh.end_round()
        k += n
        r += 1
    assert k == len(rows)
    assert r == int(rnd[-1]) + 1


def test_value_vector_follows_the_rotated_diagnostic_order(engine_lib):
    """FourColor + EquatorialPasses + ClosestRadius with ClosestRadius as value
    diagnostic: the reference's vector is [EquatorialPasses, ClosestRadius, FourColor]
    (Diagnostics.cpp:28-75), so the mesh receives pass counts."""
    import foort_gb300
    flags = abi.DIAG_FOUR_COLOR_SCREEN | abi.DIAG_EQUATORIAL_PASSES | abi.DIAG_CLOSEST_RADIUS
    m1 = foort_gb300.Mesh("v2", flags, abi.DIAG_CLOSEST_RADIUS, initial_pixels=9, max_subdivide=2, iteration_pixels=10)
    m2 = foort_gb300.Mesh("v2", flags, abi.DIAG_CLOSEST_RADIUS, initial_pixels=9, max_subdivide=2, iteration_pixels=10)
    px = m1.pixels()
    res = np.zeros(len(px), dtype=abi.RESULT_DTYPE)
    res["equat_passes"] = np.arange(len(px)) % 2   # differ between neighbours
    res["closest_r"] = 5.0                            # all equal
    m1.set_results(res)
    m1.end_round()
    m2.set_values([5.0] * len(px))
    m2.end_round()
    assert m1.size() > 0 and m2.size() == 0
