"""A complete FOORT run on the GPU (foort_gpu_run: engine, mesh, output files) writes
the reference's files byte for byte (-m gpu).

The two runs of the Test.cfg configuration (Johannsen, log-r, Verlet) of
tests/golden/dat: a 40^2 SimpleSquareMesh with a 1000-geodesic cache and 700 geodesics
per file, and a SquareSubdivisionMeshV2 from a 17^2 seed, whose rounds depend on the
values of the previous ones. Both kernels must reproduce every quadrant and pass count.
"""
import os

import numpy as np
import pytest

from foort_gb300 import abi, workloads
from test_output import DAT, GEOPOS, RUNS, compare_dirs, geopos_workload

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("schedule,lookahead", [(abi.SCHEDULE_WAVES, None), (abi.SCHEDULE_WAVES, 0),
                                                (abi.SCHEDULE_ROUNDS, None)])
@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_MIXED])
@pytest.mark.parametrize("name", sorted(RUNS))
def test_run_writes_the_reference_files(engine_lib, tmp_path, name, precision, schedule, lookahead):
    """Every schedule of foort_gpu_run: the V2 run's level waves take at most three
    launches for the reference's rounds (fewer with lookahead), and the files are the
    reference's either way."""
    import foort_gb300
    foort_gb300.check_layout()
    wl = workloads.johannsen_golden(True, precision=precision)
    run = RUNS[name]
    mesh = foort_gb300.Mesh.from_spec(run["mesh"], wl.desc.diag_flags, wl.desc.value_diag)
    out = foort_gb300.Output(str(tmp_path / name), wl.desc.diag_flags, wl.desc.value_diag,
                             first_line=mesh.first_line_info(wl.desc), outputs_to_cache=run["cache"],
                             geodesics_per_file=run["per_file"])
    with foort_gb300.Engine(wl.desc) as e:
        e.set_schedule(schedule)
        e.set_lookahead(lookahead)
        e.set_record_launches(True)
        geodesics, rounds = e.run([mesh], [out])
        launches, used = e.run_info()
        launched = e.run_launches()
    out.close()
    mesh.close()
    print(f"{name}: {geodesics} geodesics in {rounds} rounds, {launches} launches")
    # a SimpleSquareMesh is its own single wave: the run goes by rounds
    assert used == (schedule if name.startswith("v2") else abi.SCHEDULE_ROUNDS) and len(launched) == launches
    if schedule == abi.SCHEDULE_ROUNDS or name.startswith("simple"):
        assert launches == rounds
        assert sum(len(p) for p in launched) == geodesics
    else:
        assert launches <= min(3 if lookahead == 0 else 2, rounds)  # MaxSubdivide 3
        assert sum(len(p) for p in launched) >= geodesics
        if lookahead == 0:
            assert sum(len(p) for p in launched) == geodesics
    compare_dirs(tmp_path, name)


def parse_geopos(path):
    """{(row, col): (count, positions)} and the first line of a GeodesicPosition file."""
    with open(path) as f:
        lines = f.read().splitlines()
    out = {}
    order = []
    for ln in lines[1:]:
        head, tail = ln.split(" ;; ")
        row, col, k = (int(x) for x in head.split())
        out[(row, col)] = (k, np.array([float(x) for x in tail.split()]))
        order.append((row, col))
    return lines[0], out, order


@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_MIXED])
@pytest.mark.parametrize("name", sorted(GEOPOS))
def test_run_records_the_reference_positions(engine_lib, tmp_path, name, precision):
    """GeodesicPosition through foort_gpu_run (two passes) against the strict reference:
    same first line, same pixels, same number of kept positions, and positions equal to
    the printed precision (FP64; the mixed kernel to its endpoint tolerance)."""
    import foort_gb300
    every, steps, val, spec = GEOPOS[name]
    wl = geopos_workload(every, steps, val)
    wl.desc.precision = precision
    mesh = foort_gb300.Mesh.from_spec(spec, wl.desc.diag_flags, wl.desc.value_diag)
    out = foort_gb300.Output(str(tmp_path / name), wl.desc.diag_flags, wl.desc.value_diag,
                             first_line=mesh.first_line_info(wl.desc))
    with foort_gb300.Engine(wl.desc) as e:
        e.run([mesh], [out])
    out.close()
    mesh.close()
    ref_first, ref, ref_order = parse_geopos(os.path.join(DAT, f"{name}_GeodesicPosition.dat"))
    first, got, order = parse_geopos(str(tmp_path / f"{name}_GeodesicPosition.dat"))
    assert first == ref_first
    common = [p for p in ref_order if p in got]
    if spec[0] == "v2":
        # positions drive the mesh: near-equal weights may be ordered differently than
        # in the reference's arithmetic (the mesh itself is pinned on the CPU against the
        # strict oracle), so the runs are compared on the pixels they share
        assert len(common) >= 0.95 * len(ref_order)
        # The 17-wide grid has a row on the screen's alpha = 0 line (row 8): at 60 deg
        # those rays pass over the rotation axis, where phi is singular, and the
        # reference's own -Ofast and strict-IEEE builds already differ there (all 15 such
        # rays of this run: other step counts, positions 1e-6 - 2e-5 apart, against 1e-9
        # for the next row). They are left out of the comparison.
        common = [p for p in common if p[0] != 8]
    else:
        assert order == ref_order
    same = [p for p in common if got[p][0] == ref[p][0]]
    assert len(same) >= (0.99 if precision == abi.PREC_FP64 else 0.95) * len(common), (len(same), len(common))
    # per geodesic: do all its kept positions agree (relative, to the printed precision
    # for FP64; to the mixed kernel's endpoint tolerance)?
    tol = 2e-6 if precision == abi.PREC_FP64 else 1e-4
    ok = np.array([np.all(np.abs(got[p][1] - ref[p][1]) <= tol * np.maximum(1.0, np.abs(ref[p][1]))) for p in same])
    frac = 1.0 if precision == abi.PREC_FP64 else 0.99
    print(f"{name}: {len(same)}/{len(ref_order)} same counts, {ok.mean():.5f} of those geodesics within {tol}")
    assert ok.mean() >= frac


@pytest.mark.parametrize("max_pixels", [400, 700, 100000])
def test_wave_schedule_under_a_pixel_budget_writes_the_round_files(engine_lib, tmp_path, max_pixels):
    """A V2 run (17^2 seed, MaxSubdivide 3, IterationPixels 150) whose MaxPixels cuts the
    rounds (400, 700) or never does (100000): the wave schedule, which stops an image's
    waves at its budget and integrates what the rounds then miss, writes the same files as
    the round-by-round schedule, byte for byte."""
    import foort_gb300
    wl = workloads.johannsen_golden(True, precision=abi.PREC_MIXED)
    spec = ("v2", dict(max_pixels=max_pixels, initial_pixels=17 * 17, max_subdivide=3, iteration_pixels=150))
    files, counts = {}, {}
    for schedule in (abi.SCHEDULE_ROUNDS, abi.SCHEDULE_WAVES):
        d = tmp_path / str(schedule)
        d.mkdir()
        mesh = foort_gb300.Mesh.from_spec(spec, wl.desc.diag_flags, wl.desc.value_diag)
        out = foort_gb300.Output(str(d / "run"), wl.desc.diag_flags, wl.desc.value_diag,
                                 first_line=mesh.first_line_info(wl.desc))
        with foort_gb300.Engine(wl.desc) as e:
            e.set_schedule(schedule)
            counts[schedule] = e.run([mesh], [out]) + e.run_info()
        out.close()
        mesh.close()
        files[schedule] = {f.name: f.read_bytes() for f in sorted(d.iterdir())}
    assert files[abi.SCHEDULE_WAVES] == files[abi.SCHEDULE_ROUNDS] and files[abi.SCHEDULE_ROUNDS]
    g_r, r_r, l_r, s_r = counts[abi.SCHEDULE_ROUNDS]
    g_w, r_w, l_w, s_w = counts[abi.SCHEDULE_WAVES]
    assert (g_w, r_w) == (g_r, r_r) and g_r <= max_pixels
    assert (s_r, s_w) == (abi.SCHEDULE_ROUNDS, abi.SCHEDULE_WAVES) and l_r == r_r
    if max_pixels == 100000:
        assert l_w < l_r


def test_wave_schedule_over_two_images_writes_the_round_files(engine_lib, tmp_path):
    """Two Kerr images in one run, each with its own V2 mesh (17^2 seed, MaxSubdivide 3,
    IterationPixels 100), the first under a MaxPixels budget that cuts its rounds and the
    second unlimited: the wave schedule (per-image waves, lookahead and budgets, one launch
    per wave over both images) writes each image's files as the round-by-round schedule
    does, byte for byte."""
    import foort_gb300
    wl = workloads.c2(abi.PREC_MIXED)
    d = wl.desc
    keep = abi.attach_images(d, [abi.make_image((0.99,), r=1000.0, theta=np.radians(60), half_width=12.0),
                                 abi.make_image((0.7,), r=1000.0, theta=np.radians(35), half_width=10.0)])
    specs = [("v2", dict(max_pixels=700, initial_pixels=17 * 17, max_subdivide=3, iteration_pixels=100)),
             ("v2", dict(max_pixels=0, initial_pixels=17 * 17, max_subdivide=3, iteration_pixels=100))]
    files, info = {}, {}
    for schedule in (abi.SCHEDULE_ROUNDS, abi.SCHEDULE_WAVES):
        meshes = [foort_gb300.Mesh.from_spec(sp, d.diag_flags, d.value_diag) for sp in specs]
        outs = []
        for i, m in enumerate(meshes):
            od = tmp_path / f"s{schedule}_{i}"
            od.mkdir()
            outs.append(foort_gb300.Output(str(od / "run"), d.diag_flags, d.value_diag,
                                           first_line=m.first_line_info(d, image=i)))
        with foort_gb300.Engine(d) as e:
            e.set_schedule(schedule)
            info[schedule] = e.run(meshes, outs) + e.run_info()
        for o in outs:
            o.close()
        for m in meshes:
            m.close()
        files[schedule] = {(i, f.name): f.read_bytes() for i in range(2)
                           for f in sorted((tmp_path / f"s{schedule}_{i}").iterdir())}
    del keep
    assert files[abi.SCHEDULE_WAVES] == files[abi.SCHEDULE_ROUNDS] and len(files[abi.SCHEDULE_ROUNDS]) >= 4
    g_r, r_r, l_r, s_r = info[abi.SCHEDULE_ROUNDS]
    g_w, r_w, l_w, s_w = info[abi.SCHEDULE_WAVES]
    assert (g_w, r_w) == (g_r, r_r) and (s_r, s_w) == (abi.SCHEDULE_ROUNDS, abi.SCHEDULE_WAVES)
    assert l_w <= l_r == r_r  # the budgeted image's later rounds may each take a launch
