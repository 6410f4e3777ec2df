"""Output files and first-line descriptions, byte for byte against the reference.

The golden files (tests/golden/dat/, first_lines.json) were written by the reference's
own GeodesicOutputHandler and Utilities::GetFirstLineInfoString (tests/golden/make_golden.py).
Here the writer is fed the reference's values read back from those files, so the files
it writes must be identical: names, first lines, line format, caching and file splits.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN
from foort_gb300 import abi, workloads

DAT = os.path.join(GOLDEN, "dat")
# the two complete runs of the Test.cfg configuration (make_golden.dat_runs)
RUNS = {
    "simple40": dict(mesh=("simple", 40), cache=1000, per_file=700),
    "v2_17": dict(mesh=("v2", dict(initial_pixels=17 * 17, max_subdivide=3, iteration_pixels=150)), cache=1 << 40,
                  per_file=1 << 40),
}


def read_files(name, diag):
    """The reference's files of one diagnostic of a run, in order: (first line, rows)."""
    lines, first, k = [], None, 1
    while True:
        fn = os.path.join(DAT, f"{name}_{diag}.dat" if k == 1 else f"{name}_{diag}_{k}.dat")
        if not os.path.exists(fn):
            break
        with open(fn) as f:
            part = f.read().splitlines()
        first = part[0]
        lines += part[1:]
        k += 1
    rows = [ln.split() for ln in lines]
    return first, np.array([[int(r[0]), int(r[1]), int(r[2])] for r in rows])


def reference_results(name):
    first, eq = read_files(name, "EquatPasses")
    _, fc = read_files(name, "FourColorScreen")
    assert (eq[:, :2] == fc[:, :2]).all()
    px = np.zeros(len(eq), dtype=abi.PIXEL_DTYPE)
    px["row"], px["col"] = eq[:, 0], eq[:, 1]
    res = np.zeros(len(eq), dtype=abi.RESULT_DTYPE)
    res["equat_passes"], res["quadrant"] = eq[:, 2], fc[:, 2]
    return first, px, res


def compare_dirs(out_dir, name):
    want = sorted(f for f in os.listdir(DAT) if f.startswith(name + "_"))
    got = sorted(f for f in os.listdir(out_dir) if f.startswith(name + "_"))
    assert got == want
    for f in want:
        with open(os.path.join(DAT, f), "rb") as a, open(os.path.join(out_dir, f), "rb") as b:
            assert a.read() == b.read(), f


def test_first_line_matches_reference(engine_lib):
    import foort_gb300
    golden = json.load(open(os.path.join(GOLDEN, "first_lines.json")))
    cases = {
        "c1": (workloads.c1(), ("simple", 100)),
        # the fixture was recorded with IterationPixels 3000
        "c2": (workloads.c2(iteration_pixels=3000), ("v2", dict(initial_pixels=128 * 128, max_subdivide=3,
                                                                 iteration_pixels=3000))),
        "c4": (workloads.c4(side=1024), ("simple", 1024)),
        "test": (workloads.johannsen_golden(True), ("simple", 250)),
        "debug": (workloads.johannsen_golden(False), ("simple", 250)),
    }
    for name, (wl, spec) in cases.items():
        m = foort_gb300.Mesh.from_spec(spec, wl.desc.diag_flags, wl.desc.value_diag)
        assert m.first_line_info(wl.desc) == golden[name], name
        m.close()
    for name, run in RUNS.items():  # first lines of the golden files
        wl = workloads.johannsen_golden(True)
        m = foort_gb300.Mesh.from_spec(run["mesh"], wl.desc.diag_flags, wl.desc.value_diag)
        assert m.first_line_info(wl.desc) == read_files(name, "EquatPasses")[0], name
        m.close()


@pytest.mark.parametrize("name", sorted(RUNS))
def test_writer_reproduces_reference_files(engine_lib, tmp_path, name):
    import foort_gb300
    first, px, res = reference_results(name)
    wl = workloads.johannsen_golden(True)
    run = RUNS[name]
    with foort_gb300.Output(str(tmp_path / name), wl.desc.diag_flags, wl.desc.value_diag, first_line=first,
                            outputs_to_cache=run["cache"], geodesics_per_file=run["per_file"]) as out:
        out.round(px, res)
        out.finish()
    compare_dirs(tmp_path, name)


def test_cache_flushes_between_rounds_give_the_same_files(engine_lib, tmp_path):
    """Rounds of 600, 600, 400 with a 1000-geodesic cache: the second round flushes the
    first to file 1, the end writes the rest across files 1-3 (700 / 700 / 200 lines),
    as one round of 1600 does (InputOutput.cpp:95-269)."""
    import foort_gb300
    first, px, res = reference_results("simple40")
    wl = workloads.johannsen_golden(True)
    with foort_gb300.Output(str(tmp_path / "simple40"), wl.desc.diag_flags, wl.desc.value_diag, first_line=first,
                            outputs_to_cache=1000, geodesics_per_file=700) as out:
        for a, b in ((0, 600), (600, 1200), (1200, 1600)):
            out.round(px[a:b], res[a:b])
        out.finish()
    compare_dirs(tmp_path, "simple40")


def test_closest_radius_lines_and_file_names(engine_lib, tmp_path):
    import foort_gb300
    px = np.zeros(3, dtype=abi.PIXEL_DTYPE)
    px["row"], px["col"] = [0, 1, 2], [5, 6, 7]
    res = np.zeros(3, dtype=abi.RESULT_DTYPE)
    res["closest_r"] = [4.5, 0.0, 1234.5678905]
    res["quadrant"] = [1, 2, 3]
    flags = abi.DIAG_FOUR_COLOR_SCREEN | abi.DIAG_CLOSEST_RADIUS
    with foort_gb300.Output(str(tmp_path / "sub" / "run"), flags, abi.DIAG_CLOSEST_RADIUS, timestamp="T1",
                            extension="txt") as out:
        out.round(px, res)
        out.finish()
    assert sorted(os.listdir(tmp_path / "sub")) == ["run_T1_ClosestRadius.txt", "run_T1_FourColorScreen.txt"]
    text = (tmp_path / "sub" / "run_T1_ClosestRadius.txt").read_text()
    assert text == "0 5  4.500000\n1 6  0.000000\n2 7  1234.567890\n"


def test_writer_errors(engine_lib, tmp_path):
    import foort_gb300
    with pytest.raises(foort_gb300.FoortError) as e:
        foort_gb300.Output("", abi.DIAG_FOUR_COLOR_SCREEN, abi.DIAG_FOUR_COLOR_SCREEN)
    assert e.value.code == abi.FOORT_E_UNSUPPORTED  # console output
    out = foort_gb300.Output(str(tmp_path / "x"), abi.DIAG_GEODESIC_POSITION, abi.DIAG_GEODESIC_POSITION)
    with pytest.raises(foort_gb300.FoortError) as e:  # GeodesicPosition needs its positions
        out.round(np.zeros(1, dtype=abi.PIXEL_DTYPE), np.zeros(1, dtype=abi.RESULT_DTYPE))
    assert e.value.code == abi.FOORT_E_BADARG
    out.close()
    blocker = tmp_path / "file"
    blocker.write_text("")
    out = foort_gb300.Output(str(blocker / "run"), abi.DIAG_FOUR_COLOR_SCREEN, abi.DIAG_FOUR_COLOR_SCREEN)
    out.round(np.zeros(1, dtype=abi.PIXEL_DTYPE), np.zeros(1, dtype=abi.RESULT_DTYPE))
    with pytest.raises(foort_gb300.FoortError) as e:
        out.finish()
    assert e.value.code == abi.FOORT_E_IO
    out.close()


# ---- GeodesicPosition ---------------------------------------------------------------
def geopos_workload(every, output_steps, value_geopos):
    """The configuration of tests/golden/make_golden.py geopos_workload."""
    wl = workloads.c2(abi.PREC_FP64)
    d = wl.desc
    d.diag_flags = abi.DIAG_GEODESIC_POSITION | (abi.DIAG_EQUATORIAL_PASSES if value_geopos else abi.DIAG_FOUR_COLOR_SCREEN)
    d.value_diag = abi.DIAG_GEODESIC_POSITION if value_geopos else abi.DIAG_FOUR_COLOR_SCREEN
    d.geopos_freq = abi.UpdateFreq(every, 0, 1)
    d.geopos_output_steps = output_steps
    return wl


GEOPOS = {"geopos12": (1, 40, False, ("simple", 12)), "geopos12f3": (3, 25, True, ("simple", 12)),
          "geoposv2": (1, 8, True, ("v2", dict(initial_pixels=81, max_subdivide=2, iteration_pixels=30)))}


def read_geopos(name):
    """(first line, px, counts, points) of a reference GeodesicPosition file."""
    with open(os.path.join(DAT, f"{name}_GeodesicPosition.dat")) as f:
        lines = f.read().splitlines()
    px = np.zeros(len(lines) - 1, dtype=abi.PIXEL_DTYPE)
    counts = np.zeros(len(px), dtype=np.uint64)
    pts = []
    for i, ln in enumerate(lines[1:]):
        head, tail = ln.split(" ;; ")
        row, col, k = (int(x) for x in head.split())
        px["row"][i], px["col"][i], counts[i] = row, col, k
        vals = [float(x) for x in tail.split()]
        assert len(vals) == 4 * k
        pts.append(np.array(vals).reshape(-1, 4))
    return lines[0], px, counts, np.concatenate(pts)


def test_geopos_counts_follow_the_step_counts(oracle_mod, engine_lib):
    """Kept positions per geodesic from its step count (foort_geopos_count) against the
    reference's files; the steps come from the strict oracle, which retraces the strict
    reference the files were written with."""
    import ctypes as C
    for name in ("geopos12", "geopos12f3"):
        every, steps, val, mesh = GEOPOS[name]
        wl = geopos_workload(every, steps, val)
        _, px, counts, _ = read_geopos(name)
        px["grid"] = mesh[1]
        res = oracle_mod.integrate(wl.desc, px, fast=False)
        for i in range(len(px)):
            s, k = C.c_uint64(), C.c_uint64()
            assert engine_lib.foort_geopos_count(C.byref(wl.desc), int(res["steps"][i]), int(res["term"][i]),
                                                 C.byref(s), C.byref(k)) == 0
            assert k.value == counts[i], (name, i, int(res["steps"][i]), k.value, counts[i])


@pytest.mark.parametrize("name", sorted(GEOPOS))
def test_writer_reproduces_reference_geopos_files(engine_lib, tmp_path, name):
    import foort_gb300
    every, steps, val, _ = GEOPOS[name]
    wl = geopos_workload(every, steps, val)
    first, px, counts, points = read_geopos(name)
    other = "EquatPasses" if val else "FourColorScreen"
    _, vals = read_files(name, other)
    assert (vals[:, 0] == px["row"]).all() and (vals[:, 1] == px["col"]).all()
    res = np.zeros(len(px), dtype=abi.RESULT_DTYPE)
    res["equat_passes" if val else "quadrant"] = vals[:, 2]
    with foort_gb300.Output(str(tmp_path / name), wl.desc.diag_flags, wl.desc.value_diag, first_line=first) as out:
        out.round(px, res, counts, points)
        out.finish()
    compare_dirs(tmp_path, name)


def test_v2_mesh_driven_by_positions_follows_the_reference(oracle_mod, engine_lib):
    """SquareSubdivisionMeshV2 with GeodesicPosition as its value diagnostic: the mesh
    driven by the strict oracle's final (theta, phi) (the last position, which the
    reference's getFinalDataVal returns at UpdateFrequency 1) hands out exactly the
    reference's pixels, round after round. The great-circle distances are continuous, so
    arithmetic that differs in the last bits may order near-equal weights differently:
    the GPU tests compare such runs pixel by pixel instead."""
    import ctypes as C
    import foort_gb300
    every, steps, val, spec = GEOPOS["geoposv2"]
    wl = geopos_workload(every, steps, val)
    m = foort_gb300.Mesh.from_spec(spec, wl.desc.diag_flags, wl.desc.value_diag)
    order = []
    while not m.finished():
        px = m.pixels()
        res = oracle_mod.integrate(wl.desc, px, fast=False)
        for i in range(len(px)):
            v = (C.c_double * 2)(res["pos"][i][2], res["pos"][i][3])
            assert m._lib.foort_mesh_geodesic_finished(m._m, i, v, 2) == 0
        m.end_round()
        order += list(zip(px["row"].tolist(), px["col"].tolist()))
    m.close()
    _, ref_px, _, _ = read_geopos("geoposv2")
    assert order == list(zip(ref_px["row"].tolist(), ref_px["col"].tolist()))
