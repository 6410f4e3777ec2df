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
    with pytest.raises(foort_gb300.FoortError) as e:
        foort_gb300.Output(str(tmp_path / "x"), abi.DIAG_GEODESIC_POSITION, abi.DIAG_GEODESIC_POSITION)
    assert e.value.code == abi.FOORT_E_UNSUPPORTED
    blocker = tmp_path / "file"
    blocker.write_text("")
    out = foort_gb300.Output(str(blocker / "run"), abi.DIAG_FOUR_COLOR_SCREEN, abi.DIAG_FOUR_COLOR_SCREEN)
    out.round(np.zeros(1, dtype=abi.PIXEL_DTYPE), np.zeros(1, dtype=abi.RESULT_DTYPE))
    with pytest.raises(foort_gb300.FoortError) as e:
        out.finish()
    assert e.value.code == abi.FOORT_E_IO
    out.close()
