"""foort_gpu_run's schedules on the CPU (csrc/run.cpp, Main.cpp:313-419).

run.cpp, mesh.cpp and output.cpp are compiled here with tests/fake_engine.cpp, which
stands in for the engine's launch calls: a pixel's result is a pure function of its
cell, as an integration's is. Whole runs then go through foort_gpu_run one launch per
round and by level waves (with and without lookahead, with the rounds replayed while a
launch is in flight), and must write the same output files and return the same counts,
in no more launches (fewer with lookahead).
"""
import ctypes as C
import filecmp
import os
import subprocess

import pytest

from foort_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "foort_gb300", "csrc")
INCLUDE = os.path.join(HERE, "..", "include")

FC, EP, CR = abi.DIAG_FOUR_COLOR_SCREEN, abi.DIAG_EQUATORIAL_PASSES, abi.DIAG_CLOSEST_RADIUS


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("fake_engine") / "libfake_run.so")
    srcs = [os.path.join(HERE, "fake_engine.cpp")] + [os.path.join(CSRC, f) for f in ("run.cpp", "mesh.cpp", "output.cpp")]
    subprocess.run(["g++", "-std=c++17", "-O1", "-fPIC", "-shared", "-I" + INCLUDE, "-o", out] + srcs, check=True)
    L = C.CDLL(out)
    vp, u32, u64 = C.c_void_p, C.c_uint32, C.c_uint64
    L.fake_ctx_create.restype = vp
    L.fake_ctx_create.argtypes = [u32, u32, u32, u64]
    L.fake_ctx_destroy.argtypes = [vp]
    for f in ("fake_ctx_launches", "fake_ctx_launch_size"):
        getattr(L, f).restype = u64
    L.fake_ctx_launches.argtypes = [vp]
    L.fake_ctx_launch_size.argtypes = [vp, u64]
    for f in ("fake_ctx_run_schedule", "fake_ctx_run_launches"):
        getattr(L, f).restype = u32
        getattr(L, f).argtypes = [vp]
    L.fake_ctx_fail_at.argtypes = [vp, C.c_int64, C.c_int]
    L.foort_mesh_create_v2.argtypes = [u64, u64, C.c_int32, u64, C.c_int32, u32, u32, C.POINTER(vp)]
    L.foort_mesh_create_simple.argtypes = [u64, u32, u32, C.POINTER(vp)]
    L.foort_mesh_destroy.argtypes = [vp]
    L.foort_output_create.argtypes = [C.POINTER(abi.OutputDesc), C.POINTER(vp)]
    L.foort_output_destroy.argtypes = [vp]
    L.foort_gpu_run.argtypes = [vp, C.POINTER(vp), C.POINTER(vp), u32, C.POINTER(u64), C.POINTER(u32)]
    return L


def run(L, meshes, diag, value, schedule, lookahead, outdir, fail=None):
    """One foort_gpu_run over fresh meshes built from `meshes` ((kind, args) per image),
    with each image's files under outdir. Returns (geodesics, rounds, launch sizes, the
    schedule it used); with fail = (launch, code), that launch reports the error code and
    the run's return code is returned instead."""
    ctx = L.fake_ctx_create(diag, value, schedule, lookahead)
    if fail:
        L.fake_ctx_fail_at(ctx, *fail)
    ms, outs = [], []
    try:
        for i, (kind, args) in enumerate(meshes):
            m = C.c_void_p()
            if kind == "v2":
                rc = L.foort_mesh_create_v2(*args, diag, value, C.byref(m))
            else:
                rc = L.foort_mesh_create_simple(*args, diag, value, C.byref(m))
            assert rc == 0
            ms.append(m)
            d = abi.OutputDesc(os.path.join(str(outdir), f"img{i}", "run").encode(), b"", b"dat", b"first line",
                               1000, 50000, diag, value)
            o = C.c_void_p()
            assert L.foort_output_create(C.byref(d), C.byref(o)) == 0
            outs.append(o)
        n = len(meshes)
        g, r = C.c_uint64(), C.c_uint32()
        rc = L.foort_gpu_run(ctx, (C.c_void_p * n)(*[m.value for m in ms]), (C.c_void_p * n)(*[o.value for o in outs]),
                             n, C.byref(g), C.byref(r))
        if fail:
            return rc, L.fake_ctx_run_launches(ctx)
        assert rc == 0, rc
        sizes = [L.fake_ctx_launch_size(ctx, k) for k in range(L.fake_ctx_launches(ctx))]
        assert L.fake_ctx_run_launches(ctx) == len(sizes)
        return g.value, r.value, sizes, L.fake_ctx_run_schedule(ctx)
    finally:
        for o in outs:
            L.foort_output_destroy(o)
        for m in ms:
            L.foort_mesh_destroy(m)
        L.fake_ctx_destroy(ctx)


def same_tree(a, b):
    files = sorted(os.path.relpath(os.path.join(d, f), a) for d, _, fs in os.walk(a) for f in fs)
    assert files and files == sorted(os.path.relpath(os.path.join(d, f), b) for d, _, fs in os.walk(b) for f in fs)
    match, mismatch, errors = filecmp.cmpfiles(a, b, files, shallow=False)
    assert not mismatch and not errors, (mismatch, errors)


# (mesh list, value diagnostic): V2 meshes are (max_pixels, initial_pixels, max_subdivide,
# iteration_pixels, initial_sub_to_final); simple ones (total_pixels,)
CASES = {
    "v2_fourcolor": ([("v2", (0, 33 * 33, 4, 300, 0))], FC),
    "v2_budget": ([("v2", (2500, 33 * 33, 4, 300, 0))], FC),
    "v2_budget_in_the_seed_wave": ([("v2", (700, 25 * 25, 3, 40, 0))], FC),
    "v2_passes": ([("v2", (0, 17 * 17, 5, 150, 1))], EP),
    "v2_closest": ([("v2", (0, 21 * 21, 4, 1000000, 0))], CR),
    "v2_and_simple": ([("v2", (0, 25 * 25, 4, 200, 0)), ("simple", (40 * 40,))], FC),
    "two_v2": ([("v2", (0, 25 * 25, 4, 200, 0)), ("v2", (3000, 17 * 17, 5, 100, 0))], FC),
    "simple_only": ([("simple", (30 * 30,)), ("simple", (20 * 20,))], FC),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_waves_write_the_round_by_round_files(lib, tmp_path, case):
    meshes, value = CASES[case]
    diag = FC | EP | CR
    ref = run(lib, meshes, diag, value, abi.SCHEDULE_ROUNDS, 0, tmp_path / "rounds")
    g, r, sizes, used = ref
    assert used == abi.SCHEDULE_ROUNDS and len(sizes) == r and sum(sizes) == g
    adaptive = any(kind == "v2" for kind, _ in meshes)
    for name, la in (("waves", 0), ("waves_lookahead", 4000), ("waves_small_cap", 50)):
        got = run(lib, meshes, diag, value, abi.SCHEDULE_WAVES, la, tmp_path / name)
        assert got[:2] == (g, r), (name, got, ref)
        same_tree(str(tmp_path / "rounds"), str(tmp_path / name))
        if adaptive:
            # never more launches than rounds; fewer with lookahead where every V2 mesh is
            # unlimited (a budget can leave rounds whose pixels no wave held, one launch
            # each, and without lookahead a mesh whose rounds are its levels keeps them)
            assert got[3] == abi.SCHEDULE_WAVES
            assert len(got[2]) <= r, (name, got[2], sizes)
            unlimited = all(kind != "v2" or args[0] == 0 for kind, args in meshes)
            if unlimited and la >= 4000 and r > 2:
                assert len(got[2]) < r, (name, got[2], sizes)
        else:
            assert got[3] == abi.SCHEDULE_ROUNDS and got[2] == sizes


@pytest.mark.parametrize("schedule,lookahead", [(abi.SCHEDULE_ROUNDS, 0), (abi.SCHEDULE_WAVES, 0),
                                                (abi.SCHEDULE_WAVES, 4000)])
@pytest.mark.parametrize("at", [0, 1, 2])
def test_a_failing_launch_ends_the_run_with_its_code(lib, tmp_path, schedule, lookahead, at):
    """A launch that reports an error (a stand-in for a CUDA failure, made on the host)
    ends foort_gpu_run with that code under every schedule, including a launch whose host
    side was replaying stored rounds meanwhile; the launches counted stop there."""
    meshes, value = CASES["v2_fourcolor"]
    rc, launches = run(lib, meshes, FC | EP | CR, value, schedule, lookahead, tmp_path / "out",
                       fail=(at, abi.FOORT_E_CUDA))
    ok = run(lib, meshes, FC | EP | CR, value, schedule, lookahead, tmp_path / "ok")
    if at < len(ok[2]):
        assert rc == abi.FOORT_E_CUDA and launches == at + 1, (rc, launches, ok[2])
    else:
        assert rc == 0
