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


def c2_run_fixture():
    """The reference's complete C2 run (tests/golden/c2_run.npz, make_golden.py part
    "c2run"): per geodesic in hand-out order its pixel, quadrant and closest radius."""
    f = np.load(os.path.join(GOLDEN, "c2_run.npz"))
    return {k: f[k] for k in f.files}


def test_v2_mesh_hands_out_the_reference_c2_run(engine_lib):
    """Given the reference's own quadrant of every pixel, the host V2 mesh of the C2
    workload (128^2 seed, MaxSubdivide 3, IterationPixels 800) hands out the reference
    run's 26,547 pixels in the same order, over the same five rounds."""
    import foort_gb300
    from foort_gb300 import workloads
    f = c2_run_fixture()
    rows, cols = f["row"].astype(np.int64), f["col"].astype(np.int64)
    wl = workloads.c2()
    mesh = foort_gb300.Mesh.from_spec(wl.mesh[0], wl.desc.diag_flags, wl.desc.value_diag)
    grid = mesh.grid()
    assert grid == 509
    quad = np.full((grid, grid), -1, np.int64)
    quad[rows, cols] = f["quadrant"]
    assert len(np.unique(rows * grid + cols)) == len(rows)  # every pixel once
    k, r = 0, 0
    while not mesh.finished():
        px = mesh.pixels()
        n = len(px)
        assert np.array_equal(px["row"], rows[k:k + n]), r
        assert np.array_equal(px["col"], cols[k:k + n]), r
        mesh.set_values(quad[px["row"].astype(np.int64), px["col"].astype(np.int64)])
        mesh.end_round()
        k += n
        r += 1
    mesh.close()
    assert k == len(rows) == 26547
    assert r == int(f["rounds"]) == 5


def drive_values(mesh, value_of):
    rounds = []
    while not mesh.finished():
        px = mesh.pixels()
        rounds.append(px)
        mesh.set_values(value_of(px["row"].astype(np.int64), px["col"].astype(np.int64)))
        mesh.end_round()
    return rounds


def cells(rounds, grid):
    allpx = np.concatenate(rounds)
    return np.sort(allpx["row"].astype(np.int64) * grid + allpx["col"].astype(np.int64))


@pytest.mark.parametrize("case", [c for c in CASES if c.startswith("v2")])
def test_level_waves_hand_out_the_reference_pixel_set(engine_lib, case):
    """foort_mesh_create_waves: with unlimited MaxPixels the waves hand out exactly the
    pixels of the reference's rounds (each once), in at most MaxSubdivide waves; with a
    finite MaxPixels the reference's pixels are among the waves'."""
    import foort_gb300
    kind, init, maxsub, iterpix, maxpix, stf, vd, vk = [int(v) for v in TRACES[case + "_spec"]]
    mesh = foort_gb300.Mesh("v2", int(vd), int(vd), max_pixels=maxpix, initial_pixels=init, max_subdivide=maxsub,
                            iteration_pixels=iterpix, initial_sub_to_final=stf)
    grid = mesh.grid()
    assert mesh.max_pixels() == maxpix
    waves = mesh.waves()
    assert waves.grid() == grid and waves.max_pixels() == 0
    got = drive_values(waves, lambda r, c: np.array([oracle.synth_value(vk, a, b, grid) for a, b in zip(r, c)]))
    want = np.sort(TRACES[case + "_rows"].astype(np.int64) * grid + TRACES[case + "_cols"].astype(np.int64))
    if maxpix:
        assert len(want) <= maxpix and np.isin(want, cells(got, grid)).all()
    else:
        assert np.array_equal(cells(got, grid), want)
    assert len(got) <= maxsub
    # a mesh that has ended a round has no waves
    mesh.set_values([0.0] * mesh.size())
    mesh.end_round()
    with pytest.raises(foort_gb300.FoortError):
        mesh.waves()


def test_level_waves_of_the_reference_c2_run(engine_lib):
    """The C2 mesh's waves given the reference run's quadrants: the run's 26,547 pixels in
    three waves (the reference takes five rounds)."""
    import foort_gb300
    from foort_gb300 import workloads
    f = c2_run_fixture()
    rows, cols = f["row"].astype(np.int64), f["col"].astype(np.int64)
    wl = workloads.c2()
    mesh = foort_gb300.Mesh.from_spec(wl.mesh[0], wl.desc.diag_flags, wl.desc.value_diag)
    quad = np.full((509, 509), -1.0)
    quad[rows, cols] = f["quadrant"]
    got = drive_values(mesh.waves(), lambda r, c: quad[r, c])
    assert [len(w) for w in got] == [16384, 3125, 7038]
    assert np.array_equal(cells(got, 509), np.sort(rows * 509 + cols))


@pytest.mark.parametrize("case", [c for c in CASES if c.startswith("v2")])
def test_lookahead_holds_the_next_wave(engine_lib, case):
    """foort_mesh_lookahead on a mesh of level waves: each round's candidates hold every
    pixel of the next round, and none of them has been handed out before."""
    import foort_gb300
    kind, init, maxsub, iterpix, maxpix, stf, vd, vk = [int(v) for v in TRACES[case + "_spec"]]
    mesh = foort_gb300.Mesh("v2", int(vd), int(vd), max_pixels=maxpix, initial_pixels=init, max_subdivide=maxsub,
                            iteration_pixels=iterpix, initial_sub_to_final=stf)
    grid = mesh.grid()
    waves = mesh.waves()
    seen = set()
    cand = None
    while not waves.finished():
        px = waves.pixels()
        got = set((px["row"].astype(np.int64) * grid + px["col"].astype(np.int64)).tolist())
        if cand is not None:
            assert got <= cand
        assert not (got & seen)
        seen |= got
        la = waves.lookahead()
        cand = set((la["row"].astype(np.int64) * grid + la["col"].astype(np.int64)).tolist())
        assert len(cand) == len(la) and np.all(la["grid"] == grid)
        waves.set_values([oracle.synth_value(vk, a, b, grid) for a, b in zip(px["row"], px["col"])])
        waves.end_round()


def test_mesh_kind_and_pixel_cap(engine_lib):
    """foort_mesh_kind and foort_mesh_max_pixels; a SimpleSquareMesh is its own single wave
    with no lookahead candidates."""
    import foort_gb300
    simple = foort_gb300.Mesh("simple", abi.DIAG_FOUR_COLOR_SCREEN, abi.DIAG_FOUR_COLOR_SCREEN, total_pixels=40 * 40)
    v2 = foort_gb300.Mesh("v2", abi.DIAG_FOUR_COLOR_SCREEN, abi.DIAG_FOUR_COLOR_SCREEN, max_pixels=500,
                          initial_pixels=81, max_subdivide=3, iteration_pixels=10)
    assert (simple.kind(), v2.kind()) == (abi.MESH_SIMPLE, abi.MESH_SUBDIVISION_V2)
    assert (simple.max_pixels(), v2.max_pixels()) == (1600, 500)
    assert engine_lib.foort_mesh_kind(None) == abi.FOORT_E_BADARG
    w = simple.waves()
    assert w.kind() == abi.MESH_SIMPLE and w.size() == 1600 and len(w.lookahead()) == 0
    w.set_values([0.0] * 1600)
    w.end_round()
    assert w.finished()


@pytest.mark.parametrize("init,maxsub,vk", [(9, 9, 0), (25, 6, 2), (129 * 129, 2, 0)])
def test_lookahead_ascending_on_sparse_and_dense_grids(engine_lib, init, maxsub, vk):
    """The candidates come out in ascending cell order, each once, whether the grid is much
    larger than the candidate list (a 3 x 3 seed on a 513-cell side: the early rounds sort
    the list) or not (the later rounds, the 129 x 129 seed: a bitmap of the grid), and every
    round's candidates hold the next round's pixels."""
    import foort_gb300
    mesh = foort_gb300.Mesh("v2", abi.DIAG_FOUR_COLOR_SCREEN, abi.DIAG_FOUR_COLOR_SCREEN, max_pixels=0,
                            initial_pixels=init, max_subdivide=maxsub, iteration_pixels=1000, initial_sub_to_final=0)
    grid = mesh.grid()
    waves = mesh.waves()
    mesh.close()
    cand, sizes, rounds = None, [], 0
    while not waves.finished() and rounds < 6:
        px = waves.pixels()
        cells = px["row"].astype(np.int64) * grid + px["col"].astype(np.int64)
        if cand is not None:
            assert np.isin(cells, cand).all()
        la = waves.lookahead()
        cand = la["row"].astype(np.int64) * grid + la["col"].astype(np.int64)
        assert np.all(np.diff(cand) > 0)
        sizes.append(len(cand))
        waves.set_values([oracle.synth_value(vk, a, b, grid) for a, b in zip(px["row"], px["col"])])
        waves.end_round()
        rounds += 1
    waves.close()
    assert rounds >= 2 and max(sizes) > 0
