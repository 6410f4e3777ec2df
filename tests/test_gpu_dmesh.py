"""The device-resident V2 mesh (include/foort_gpu.h foort_dmesh_*) against the
reference's own meshes: with FOORT_DMESH_ORDER_REFERENCE its rounds hand out the
pixel sequences of tests/golden/mesh_traces.npz and of the reference's C2 run
(tests/golden/c2_run.npz) exactly; with FOORT_DMESH_ORDER_DEVICE they do wherever the
weights have no ties, and the mesh stays a valid subdivision where they do. A whole run
through foort_gpu_run_dmesh gives the host loop's pixels and results bit for bit.
Index work: every comparison is exact."""
import os

import numpy as np
import pytest

import oracle
from conftest import GOLDEN
from foort_gb300 import abi, workloads

pytestmark = pytest.mark.gpu

TRACES = np.load(os.path.join(GOLDEN, "mesh_traces.npz"))
V2_CASES = sorted({k.rsplit("_", 1)[0] for k in TRACES.files if k.endswith("_spec")} - {"simple_37"})


@pytest.fixture(scope="module")
def eng():
    import foort_gb300
    from foort_gb300 import build as engine_build
    engine_build.build()
    foort_gb300.check_layout()
    return foort_gb300


def device_values(values):
    import torch
    return torch.tensor(np.asarray(values, dtype=np.float64), device="cuda")


def drive(mesh, value_of, max_rounds=10_000):
    """Run a host or device mesh with values value_of(rows, cols) -> array; returns the
    rounds' pixels."""
    import torch
    rounds = []
    while not mesh.finished():
        px = mesh.pixels()
        rounds.append(px)
        vals = value_of(px["row"].astype(np.int64), px["col"].astype(np.int64))
        if hasattr(mesh, "set_values_ptr"):
            t = device_values(vals)
            mesh.set_values_ptr(t.data_ptr(), len(px))
            mesh.end_round()
            torch.cuda.synchronize()
        else:
            mesh.set_values(vals)
            mesh.end_round()
        assert len(rounds) < max_rounds
    return rounds


def synth(kind, grid):
    return lambda rows, cols: np.array([oracle.synth_value(kind, a, b, grid) for a, b in zip(rows, cols)])


@pytest.mark.parametrize("case", V2_CASES)
def test_device_mesh_matches_reference_trace(eng, case):
    _, init, maxsub, iterpix, maxpix, stf, vd, vk = [int(v) for v in TRACES[case + "_spec"]]
    rows, cols, rnd = TRACES[case + "_rows"], TRACES[case + "_cols"], TRACES[case + "_round"]
    mesh = eng.DeviceMesh(vd, vd, max_pixels=maxpix, initial_pixels=init, max_subdivide=maxsub,
                          iteration_pixels=iterpix, initial_sub_to_final=stf)
    grid = mesh.grid()
    got = drive(mesh, synth(vk, grid))
    k = 0
    for r, px in enumerate(got):
        n = len(px)
        assert np.array_equal(px["row"], rows[k:k + n]), (case, r)
        assert np.array_equal(px["col"], cols[k:k + n]), (case, r)
        assert np.all(rnd[k:k + n] == r)
        assert np.all(px["grid"] == grid) and np.all(px["image"] == 0)
        k += n
    assert k == len(rows)
    assert len(got) == int(rnd[-1]) + 1 == mesh.rounds()
    mesh.close()


def test_device_mesh_hands_out_the_reference_c2_run(eng):
    """The C2 workload's mesh (128^2 seed, MaxSubdivide 3, IterationPixels 800) given the
    reference run's quadrants: its 26,547 pixels in the reference's order, five rounds."""
    f = np.load(os.path.join(GOLDEN, "c2_run.npz"))
    rows, cols = f["row"].astype(np.int64), f["col"].astype(np.int64)
    wl = workloads.c2()
    mesh = eng.DeviceMesh.from_spec(wl.mesh[0], wl.desc.diag_flags, wl.desc.value_diag)
    grid = mesh.grid()
    assert grid == 509
    quad = np.full((grid, grid), -1.0)
    quad[rows, cols] = f["quadrant"]
    got = drive(mesh, lambda r, c: quad[r, c])
    seq = np.concatenate(got)
    assert np.array_equal(seq["row"], rows) and np.array_equal(seq["col"], cols)
    assert len(got) == int(f["rounds"]) == 5


def tie_free(grid, seed):
    """Continuous values without equal differences: no two squares share a weight."""
    rng = np.random.default_rng(seed)
    v = rng.random((grid, grid)) + np.linspace(0, 3, grid)[:, None] ** 2
    return lambda r, c: v[r, c]


@pytest.mark.parametrize("init,maxsub,iterpix,maxpix", [(81, 4, 37, 0), (17 * 17, 3, 200, 0), (12, 5, 40, 900),
                                                         (33 * 33, 5, 1 << 20, 0)])
def test_device_order_without_ties_is_the_reference_order(eng, init, maxsub, iterpix, maxpix):
    vd = abi.DIAG_CLOSEST_RADIUS
    spec = dict(max_pixels=maxpix, initial_pixels=init, max_subdivide=maxsub, iteration_pixels=iterpix)
    host = eng.Mesh("v2", vd, vd, **spec)
    dev = eng.DeviceMesh(vd, vd, order=abi.DMESH_ORDER_DEVICE, **spec)
    assert host.grid() == dev.grid()
    f = tie_free(host.grid(), init)
    a, b = drive(host, f), drive(dev, f)
    assert len(a) == len(b) and len(a) > 2
    for r, (x, y) in enumerate(zip(a, b)):
        assert np.array_equal(x, y), r
    if iterpix == 1 << 20 and not maxpix:
        assert dev.active() == 0


def test_device_order_with_ties_is_a_valid_subdivision(eng):
    """FourColorScreen values (weights 0 or 1): the device sort may pick other squares
    among equal ones, but every pixel is handed out once, the seed round is the
    reference's, and the rounds stop where the reference's do when every square with a
    colour change has been subdivided to the end (IterationPixels above the square count)."""
    vd = abi.DIAG_FOUR_COLOR_SCREEN
    for iterpix in (25, 1 << 20):
        spec = dict(initial_pixels=17 * 17, max_subdivide=4, iteration_pixels=iterpix)
        host = eng.Mesh("v2", vd, vd, **spec)
        dev = eng.DeviceMesh(vd, vd, order=abi.DMESH_ORDER_DEVICE, **spec)
        grid = host.grid()
        f = synth(0, grid)
        a, b = drive(host, f), drive(dev, f)
        sa, sb = np.concatenate(a), np.concatenate(b)
        cells = sb["row"].astype(np.int64) * grid + sb["col"].astype(np.int64)
        assert len(np.unique(cells)) == len(cells)
        assert np.all(sb["row"] < grid) and np.all(sb["col"] < grid)
        assert np.array_equal(a[0], b[0])
        if iterpix == 1 << 20:
            # everything subdivided every round: no choice, the same pixels
            ca = sa["row"].astype(np.int64) * grid + sa["col"].astype(np.int64)
            assert len(a) == len(b)
            for x, y in zip(a, b):
                assert np.array_equal(np.sort(x["row"] * grid + x["col"]), np.sort(y["row"] * grid + y["col"]))
            assert np.array_equal(np.sort(ca), np.sort(cells))


@pytest.mark.parametrize("schedule,lookahead", [(abi.SCHEDULE_WAVES, None), (abi.SCHEDULE_WAVES, 0),
                                                (abi.SCHEDULE_ROUNDS, None)])
def test_run_dmesh_matches_the_host_round_loop(eng, schedule, lookahead):
    """foort_gpu_run_dmesh over a Kerr a = 0.99 V2 run (33^2 seed, MaxSubdivide 3,
    IterationPixels 150): each round's pixels and results equal those of the host loop
    (host mesh, foort_gpu_integrate) bit for bit, whether the device run launches round by
    round or by level waves (at most three launches, fewer with lookahead)."""
    import torch
    wl = workloads.c2(abi.PREC_MIXED)
    spec = dict(max_pixels=0, initial_pixels=33 * 33, max_subdivide=3, iteration_pixels=150,
                initial_sub_to_final=0)
    d = wl.desc
    host_rounds = []
    with eng.Engine(d) as e:
        mesh = eng.Mesh("v2", d.diag_flags, d.value_diag, **spec)
        while not mesh.finished():
            px = mesh.pixels()
            res = e.integrate(px)
            host_rounds.append((px, res))
            mesh.set_results(res)
            mesh.end_round()
        dev_rounds = []
        dmesh = eng.DeviceMesh(d.diag_flags, d.value_diag, **spec)
        cap = 5 * 150 + 33 * 33
        out = torch.zeros(cap * abi.RESULT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")

        def on_round(d_px, d_res, n, rnd):
            res = np.frombuffer(out[:n * abi.RESULT_DTYPE.itemsize].cpu().numpy().tobytes(),
                                dtype=abi.RESULT_DTYPE)
            dev_rounds.append((dmesh.pixels(), res))
            assert d_res == out.data_ptr() and d_px == dmesh.pixels_ptr() and rnd == len(dev_rounds) - 1

        e.set_schedule(schedule)
        e.set_lookahead(lookahead)
        g, r = dmesh.run(e, out.data_ptr(), cap, on_round)
        launches, used = e.run_info()
    assert r == len(host_rounds) == len(dev_rounds) >= 3
    assert used == schedule
    if schedule == abi.SCHEDULE_ROUNDS:
        assert launches == r
    else:  # three levels; with lookahead the second launch also holds the third level
        assert launches <= (3 if lookahead == 0 else 2)
    assert g == sum(len(p) for p, _ in host_rounds)
    for k, ((hp, hr), (dp, dr)) in enumerate(zip(host_rounds, dev_rounds)):
        assert np.array_equal(hp, dp), k
        for name in abi.RESULT_DTYPE.names:
            np.testing.assert_array_equal(hr[name], dr[name], err_msg=f"round {k}: {name}")


def test_run_dmesh_rejects_a_small_result_buffer(eng):
    import torch
    wl = workloads.c2(abi.PREC_MIXED)
    d = wl.desc
    with eng.Engine(d) as e:
        dmesh = eng.DeviceMesh(d.diag_flags, d.value_diag, initial_pixels=81, max_subdivide=2, iteration_pixels=10)
        out = torch.zeros(80 * abi.RESULT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
        with pytest.raises(eng.FoortError) as ei:
            dmesh.run(e, out.data_ptr(), 80)
        assert ei.value.code == abi.FOORT_E_BADARG and "80" in str(ei.value)


@pytest.mark.parametrize("value_diag,max_pixels", [(abi.DIAG_EQUATORIAL_PASSES, 0), (abi.DIAG_CLOSEST_RADIUS, 0),
                                                   (abi.DIAG_FOUR_COLOR_SCREEN, 1500)])
def test_run_dmesh_other_values_and_a_pixel_budget(eng, value_diag, max_pixels):
    """foort_gpu_run_dmesh with EquatorialPasses or ClosestRadius as the mesh's value (the
    device scatters the value the reference's vector starts with) and with a finite
    MaxPixels (the device mesh then goes round by round, cutting the last round as the
    reference does): the host loop's pixels and results, bit for bit."""
    import torch
    wl = workloads.c2(abi.PREC_MIXED)
    d = wl.desc
    d.diag_flags = abi.DIAG_FOUR_COLOR_SCREEN | abi.DIAG_EQUATORIAL_PASSES | abi.DIAG_CLOSEST_RADIUS
    d.value_diag = value_diag
    spec = dict(max_pixels=max_pixels, initial_pixels=25 * 25, max_subdivide=3, iteration_pixels=120,
                initial_sub_to_final=0)
    host_rounds = []
    with eng.Engine(d) as e:
        mesh = eng.Mesh("v2", d.diag_flags, d.value_diag, **spec)
        while not mesh.finished():
            px = mesh.pixels()
            res = e.integrate(px)
            host_rounds.append((px, res))
            mesh.set_results(res)
            mesh.end_round()
        dev_rounds = []
        dmesh = eng.DeviceMesh(d.diag_flags, d.value_diag, **spec)
        cap = 5 * 120 + 25 * 25
        out = torch.zeros(cap * abi.RESULT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")

        def on_round(d_px, d_res, n, rnd):
            dev_rounds.append((dmesh.pixels(), np.frombuffer(out[:n * abi.RESULT_DTYPE.itemsize].cpu().numpy().tobytes(),
                                                             dtype=abi.RESULT_DTYPE)))

        g, r = dmesh.run(e, out.data_ptr(), cap, on_round)
        _, used = e.run_info()
    assert r == len(host_rounds) == len(dev_rounds) >= 2
    assert used == (abi.SCHEDULE_ROUNDS if max_pixels else abi.SCHEDULE_WAVES)
    if max_pixels:
        assert g <= max_pixels
    for k, ((hp, hr), (dp, dr)) in enumerate(zip(host_rounds, dev_rounds)):
        assert np.array_equal(hp, dp), k
        for name in abi.RESULT_DTYPE.names:
            np.testing.assert_array_equal(hr[name], dr[name], err_msg=f"round {k}: {name}")
