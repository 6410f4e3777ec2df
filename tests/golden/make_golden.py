"""Generate the golden fixtures of tests/golden/ from the reference.

Run here, where the reference sources exist (they are not on the GPU machines):

    python tests/golden/make_golden.py

Inputs:
* the golden outputs shipped with the reference, FOORT/Output/{Test,debug}_*.dat
  (FOORT/Test.cfg and its RK4 variant, Johannsen a=0.7, alpha13=2, log-r, 250^2);
* the reference itself, compiled from its own sources by oracle/Makefile, run through
  oracle/ref_driver.cpp on sampled pixels of the benchmark workloads, with the
  reference's own flags (-Ofast, "fast") and with strict IEEE flags ("strict").

Outputs (.npz of numpy arrays, a few hundred KB in total):
* johannsen_{test,debug}.npz   quadrant / passes per pixel of the shipped .dat files
                               and their first lines;
* ref_<name>.npz               pixels + per-pixel results of the reference (fast, strict);
* mesh_traces.npz              SquareSubdivisionMeshV2 / SimpleSquareMesh pixel sequences
                               driven by synthetic values;
* first_lines.json             Utilities::GetFirstLineInfoString for several runs;
* dat/*.dat                    output files of small complete runs (GeodesicOutputHandler);
* c2_run.npz                   the reference's complete C2 run: pixel order, quadrant and
                               closest radius of its 26,547 geodesics (part "c2run").
"""
import ctypes as C
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from foort_gb300 import abi, workloads  # noqa: E402

OUTDIR = os.path.join(oracle.REF_SRC, "Output")


def shipped_dat():
    for name, test in (("test", True), ("debug", False)):
        arrs = {}
        for diag, key in (("EquatPasses", "passes"), ("FourColorScreen", "quadrant")):
            fn = os.path.join(OUTDIR, f"{'Test' if test else 'debug'}_{diag}.dat")
            lines = open(fn).read().split("\n")
            rows = np.array([[int(t) for t in l.split()] for l in lines[1:] if l.strip()], dtype=np.int64)
            assert len(rows) == 62500
            assert np.array_equal(rows[:, 0] * 250 + rows[:, 1], np.arange(62500))
            arrs[key] = rows[:, 2].astype(np.int8)
            arrs[key + "_header"] = np.array(lines[0])
        np.savez_compressed(os.path.join(HERE, f"johannsen_{name}.npz"), **arrs)
        print("wrote", name, {k: v.shape for k, v in arrs.items()})


def sample_pixels(side, n, seed, image=0):
    rng = np.random.default_rng(seed)
    idx = np.sort(rng.choice(side * side, size=min(n, side * side), replace=False))
    px = np.zeros(len(idx), dtype=abi.PIXEL_DTYPE)
    px["image"] = image
    px["row"] = idx // side
    px["col"] = idx % side
    px["grid"] = side
    return px


def ref_case(name, wl, px, value_diag=None):
    d = wl.desc
    if value_diag is not None:
        d.value_diag = value_diag
    fast = oracle.ref_integrate(d, px, strict=False)
    strict = oracle.ref_integrate(d, px, strict=True)
    np.savez_compressed(os.path.join(HERE, f"ref_{name}.npz"), px=px, fast=fast, strict=strict)
    print("wrote", name, len(px), "pixels; mean steps", fast["steps"].mean())


def mesh_traces():
    lib = oracle.ref_lib()
    out = {}
    cases = [
        # name, kind, initial, maxsub, iterpix, maxpixels, sub_to_final, value_diag, value_kind
        ("v2_fc_9_4_60", 1, 81, 4, 60, 0, 0, abi.DIAG_FOUR_COLOR_SCREEN, 0),
        ("v2_fc_17_3_1000", 1, 289, 3, 1000, 0, 0, abi.DIAG_FOUR_COLOR_SCREEN, 0),
        ("v2_ep_16_4_25", 1, 256, 4, 25, 0, 0, abi.DIAG_EQUATORIAL_PASSES, 1),
        ("v2_cr_12_5_40_max", 1, 144, 5, 40, 900, 0, abi.DIAG_CLOSEST_RADIUS, 2),
        ("v2_fc_33_3_big", 1, 1089, 3, 1 << 16, 0, 0, abi.DIAG_FOUR_COLOR_SCREEN, 0),
        ("simple_37", 0, 37 * 37, 1, 0, 0, 0, abi.DIAG_FOUR_COLOR_SCREEN, 0),
    ]
    for name, kind, init, maxsub, iterpix, maxpix, stf, vd, vk in cases:
        spec = oracle.RefMeshSpec(kind, maxsub, init, maxpix, init, iterpix, stf, 0)
        cap = 1 << 20
        rows = np.zeros(cap, np.uint64)
        cols = np.zeros(cap, np.uint64)
        rnd = np.zeros(cap, np.uint32)
        n = C.c_uint64()
        nr = C.c_uint32()
        rc = lib.ref_mesh_trace(C.byref(spec), vd, vk, rows.ctypes.data, cols.ctypes.data, rnd.ctypes.data, cap,
                                C.byref(n), C.byref(nr))
        assert rc == 0
        k = n.value
        out[name + "_rows"] = rows[:k]
        out[name + "_cols"] = cols[:k]
        out[name + "_round"] = rnd[:k]
        out[name + "_spec"] = np.array([kind, init, maxsub, iterpix, maxpix, stf, vd, vk], dtype=np.uint64)
        print("mesh", name, k, "pixels", nr.value, "rounds")
    np.savez_compressed(os.path.join(HERE, "mesh_traces.npz"), **out)


def first_lines():
    lib = oracle.ref_lib()
    res = {}
    cases = {
        "c1": (workloads.c1(), oracle.RefMeshSpec(0, 1, 100 * 100, 0, 0, 0, 0, 0)),
        "c2": (workloads.c2(), oracle.RefMeshSpec(1, 3, 0, 0, 128 * 128, workloads.C2_ITERATION_PIXELS, 0, 0)),
        "c4": (workloads.c4(side=1024), oracle.RefMeshSpec(0, 1, 1024 * 1024, 0, 0, 0, 0, 0)),
        "test": (workloads.johannsen_golden(True), oracle.RefMeshSpec(0, 1, 62500, 0, 0, 0, 0, 0)),
        "debug": (workloads.johannsen_golden(False), oracle.RefMeshSpec(0, 1, 62500, 0, 0, 0, 0, 0)),
    }
    for name, (wl, spec) in cases.items():
        buf = C.create_string_buffer(4096)
        assert lib.ref_first_line(C.byref(wl.desc), C.byref(spec), buf, 4096) == 0
        res[name] = buf.value.decode()
    json.dump(res, open(os.path.join(HERE, "first_lines.json"), "w"), indent=1)
    print("first lines", list(res))


def dat_runs():
    lib = oracle.ref_lib()
    os.makedirs(os.path.join(HERE, "dat"), exist_ok=True)
    wl = workloads.johannsen_golden(True)
    d = wl.desc
    runs = [
        ("simple40", oracle.RefMeshSpec(0, 1, 40 * 40, 0, 0, 0, 0, 0), 1000, 700),
        ("v2_17", oracle.RefMeshSpec(1, 3, 0, 0, 17 * 17, 150, 0, 0), 0, 0),
    ]
    for name, spec, cache, per_file in runs:
        prefix = os.path.join(HERE, "dat", name).encode()
        n = C.c_uint64()
        nr = C.c_uint32()
        sec = C.c_double()
        rc = lib.ref_run(C.byref(d), C.byref(spec), prefix, b"", b"dat", cache or (1 << 40), per_file or (1 << 40),
                         1, 0, C.byref(n), C.byref(nr), C.byref(sec))
        assert rc == 0
        print("dat run", name, n.value, "geodesics", nr.value, "rounds")


def geopos_workload(every, output_steps, value_geopos):
    """Kerr a = 0.99 at 60 deg (the C2 view) with the GeodesicPosition diagnostic."""
    wl = workloads.c2(abi.PREC_FP64)
    d = wl.desc
    d.diag_flags = abi.DIAG_GEODESIC_POSITION | (abi.DIAG_EQUATORIAL_PASSES if value_geopos else abi.DIAG_FOUR_COLOR_SCREEN)
    d.value_diag = abi.DIAG_GEODESIC_POSITION if value_geopos else abi.DIAG_FOUR_COLOR_SCREEN
    d.geopos_freq = abi.UpdateFreq(every, 0, 1)
    d.geopos_output_steps = output_steps
    return wl


GEOPOS_RUNS = {
    # name: (UpdateFrequency, OutputSteps, GeodesicPosition drives the mesh, mesh)
    "geopos12": (1, 40, False, oracle.RefMeshSpec(0, 1, 12 * 12, 0, 0, 0, 0, 0)),
    "geopos12f3": (3, 25, True, oracle.RefMeshSpec(0, 1, 12 * 12, 0, 0, 0, 0, 0)),
    "geoposv2": (1, 8, True, oracle.RefMeshSpec(1, 2, 0, 0, 9 * 9, 30, 0, 0)),
}


def geopos_runs():
    """Complete runs with GeodesicPosition, written by the reference built with strict
    IEEE flags (so that the strict oracle retraces them step for step)."""
    lib = oracle.ref_lib(strict=True)
    for name, (every, steps, val, spec) in GEOPOS_RUNS.items():
        wl = geopos_workload(every, steps, val)
        prefix = os.path.join(HERE, "dat", name).encode()
        n = C.c_uint64()
        nr = C.c_uint32()
        sec = C.c_double()
        rc = lib.ref_run(C.byref(wl.desc), C.byref(spec), prefix, b"", b"dat", 1 << 40, 1 << 40, 1, 0, C.byref(n),
                         C.byref(nr), C.byref(sec))
        assert rc == 0
        print("geopos run", name, n.value, "geodesics", nr.value, "rounds")


def read_dat(fn):
    """First line and (row, col, value text) rows of one reference output file."""
    lines = open(fn).read().split("\n")
    rows = [l.split() for l in lines[1:] if l.strip()]
    return lines[0], rows


def c2_run():
    """The reference's complete C2 run (Kerr a = 0.99 at 60 deg, SquareSubdivisionMeshV2
    from a 128^2 seed, MaxSubdivide 3, IterationPixels 800), the reference's own -Ofast
    build on all host threads (about 8 minutes on 8 cores). c2_run.npz keeps the order
    in which the run handed out its pixels, the quadrant and closest radius of each, and
    the files' first line."""
    lib = oracle.ref_lib()
    wl = workloads.c2(abi.PREC_FP64)
    spec = oracle.RefMeshSpec(1, 3, 0, 0, 128 * 128, workloads.C2_ITERATION_PIXELS, 0, 0)
    tmp = os.path.join(HERE, "_c2run_tmp")
    os.makedirs(tmp, exist_ok=True)
    prefix = os.path.join(tmp, "c2")
    n, nr, sec = C.c_uint64(), C.c_uint32(), C.c_double()
    rc = lib.ref_run(C.byref(wl.desc), C.byref(spec), prefix.encode(), b"", b"dat", 1 << 40, 1 << 40, 1, 0,
                     C.byref(n), C.byref(nr), C.byref(sec))
    assert rc == 0
    head_q, quad = read_dat(prefix + "_FourColorScreen.dat")
    head_c, clos = read_dat(prefix + "_ClosestRadius.dat")
    assert head_q == head_c and len(quad) == len(clos) == n.value
    assert all(a[:2] == b[:2] for a, b in zip(quad, clos))
    np.savez_compressed(os.path.join(HERE, "c2_run.npz"),
                        row=np.array([int(t[0]) for t in quad], np.uint16),
                        col=np.array([int(t[1]) for t in quad], np.uint16),
                        quadrant=np.array([int(t[2]) for t in quad], np.int8),
                        closest_r=np.array([float(t[2]) for t in clos]),
                        rounds=np.array(nr.value), seconds=np.array(sec.value), header=np.array(head_q))
    for f in os.listdir(tmp):
        os.remove(os.path.join(tmp, f))
    os.rmdir(tmp)
    print("c2 run", n.value, "geodesics", nr.value, "rounds", f"{sec.value:.0f} s")


def main(parts):
    oracle.build(with_ref=True)
    if "c2run" in parts:
        c2_run()
    if "geopos" in parts:
        geopos_runs()
    if "c5" in parts or "ref" in parts:
        ref_case("c5", workloads.c5(abi.PREC_FP64), sample_pixels(4097, 300, 6))
    if "mesh" in parts:
        mesh_traces()
        first_lines()
        dat_runs()
    if "ref" not in parts:
        return
    shipped_dat()
    wl = workloads.c1()
    ref_case("c1", wl, sample_pixels(100, 400, 1))
    wl = workloads.c2()
    ref_case("c2", wl, sample_pixels(509, 400, 2), value_diag=abi.DIAG_CLOSEST_RADIUS)
    wl = workloads.c4(side=1024)
    ref_case("c4", wl, sample_pixels(1024, 300, 4), value_diag=abi.DIAG_CLOSEST_RADIUS)
    wl = workloads.c3(n_images=64)
    parts = []
    for im in range(0, 64, 8):
        parts.append(sample_pixels(wl.mesh[im][1], 40, 100 + im, image=im))
    ref_case("c3", wl, np.concatenate(parts))
    wl = workloads.johannsen_golden(False)
    ref_case("debug_sample", wl, sample_pixels(250, 500, 5))


if __name__ == "__main__":
    main(sys.argv[1:] or ["ref", "mesh"])
