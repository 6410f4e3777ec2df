"""ORACLE -- TEST INFRASTRUCTURE ONLY.

Python loader for the CPU checkers of the geodesic engine:

* ``liboracle.so`` / ``liboracle_fast.so``: the restatement in foort_oracle.cpp
  (strict IEEE / reference flags);
* ``_ref/libfoort_ref.so`` / ``_ref/libfoort_ref_strict.so``: the reference itself,
  compiled from its own sources by the Makefile here (only where they exist).

Only tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py use this.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from foort_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
# The reference's FOORT source directory (its .cpp / .h files and Output/), for the `ref`
# targets of the Makefile and the fixtures; FOORT_REFERENCE_SRC overrides the default.
REF_SRC = os.environ.get("FOORT_REFERENCE_SRC", "/root/reference/FOORT")

_LIBS = {}


def build(with_ref=None, quiet=True):
    """Compile the restatement (and the reference, when its sources are present)."""
    if with_ref is None:
        with_ref = os.path.isdir(REF_SRC)
    targets = ["all"] + (["ref"] if with_ref else [])
    out = subprocess.run(["make", "-j8", "-C", HERE, f"REF={REF_SRC}"] + targets, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout[-3000:] + out.stderr[-3000:])
    return out


def have_ref(strict=False):
    name = "libfoort_ref_strict.so" if strict else "libfoort_ref.so"
    return os.path.exists(os.path.join(HERE, "_ref", name))


def _load(name):
    if name not in _LIBS:
        path = os.path.join(HERE, name)
        if not os.path.exists(path):
            build(with_ref=name.startswith("_ref"))
        lib = C.CDLL(path)
        if name.startswith("liboracle"):
            lib.oracle_integrate.argtypes = [C.POINTER(abi.RunDesc), C.c_void_p, C.c_uint64, C.c_void_p, C.c_int]
            lib.oracle_integrate_offset.argtypes = [C.POINTER(abi.RunDesc), C.c_void_p, C.c_uint64, C.c_double,
                                                    C.c_double, C.c_void_p, C.c_int, C.c_uint64]
            lib.oracle_metric.argtypes = [C.c_int32, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]
            lib.oracle_christoffel.argtypes = [C.c_int32, C.c_void_p, C.c_int32, C.c_double, C.c_void_p, C.c_void_p]
            lib.oracle_camera.argtypes = [C.POINTER(abi.RunDesc), C.c_uint32, C.c_void_p, C.c_void_p]
            lib.oracle_initial_conditions.argtypes = [C.POINTER(abi.RunDesc), C.c_void_p, C.c_void_p, C.c_void_p]
            lib.oracle_horizon_radius.argtypes = [C.c_int32, C.c_void_p]
            lib.oracle_horizon_radius.restype = C.c_double
        else:
            lib.ref_integrate.argtypes = [C.POINTER(abi.RunDesc), C.c_void_p, C.c_uint64, C.c_void_p, C.c_int,
                                          C.c_char_p, C.c_uint64]
            lib.ref_run.argtypes = [C.POINTER(abi.RunDesc), C.c_void_p, C.c_char_p, C.c_char_p, C.c_char_p,
                                    C.c_uint64, C.c_uint64, C.c_int32, C.c_int, C.POINTER(C.c_uint64),
                                    C.POINTER(C.c_uint32), C.POINTER(C.c_double)]
            lib.ref_first_line.argtypes = [C.POINTER(abi.RunDesc), C.c_void_p, C.c_char_p, C.c_uint64]
            lib.ref_mesh_trace.argtypes = [C.c_void_p, C.c_uint32, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p,
                                           C.c_uint64, C.POINTER(C.c_uint64), C.POINTER(C.c_uint32)]
        _LIBS[name] = lib
    return _LIBS[name]


def oracle_lib(fast=False):
    return _load("liboracle_fast.so" if fast else "liboracle.so")


def ref_lib(strict=False):
    return _load(os.path.join("_ref", "libfoort_ref_strict.so" if strict else "libfoort_ref.so"))


def integrate(desc, px, fast=False, nthreads=0, offset=(0.0, 0.0), max_steps_guard=0):
    """Run the restatement on a PIXEL_DTYPE array; returns a RESULT_DTYPE array."""
    px = np.ascontiguousarray(px, dtype=abi.PIXEL_DTYPE)
    out = np.zeros(len(px), dtype=abi.RESULT_DTYPE)
    lib = oracle_lib(fast)
    if offset == (0.0, 0.0) and max_steps_guard == 0:
        rc = lib.oracle_integrate(C.byref(desc), px.ctypes.data, len(px), out.ctypes.data, nthreads)
    else:
        rc = lib.oracle_integrate_offset(C.byref(desc), px.ctypes.data, len(px), offset[0], offset[1],
                                         out.ctypes.data, nthreads, max_steps_guard)
    if rc != 0:
        raise RuntimeError(f"oracle_integrate failed: {rc}")
    return out


def ref_integrate(desc, px, strict=False, nthreads=0, lines=False, line_stride=64):
    """Run the reference itself on a PIXEL_DTYPE array (only where it was built)."""
    px = np.ascontiguousarray(px, dtype=abi.PIXEL_DTYPE)
    out = np.zeros(len(px), dtype=abi.RESULT_DTYPE)
    buf = C.create_string_buffer(len(px) * line_stride) if lines else None
    rc = ref_lib(strict).ref_integrate(C.byref(desc), px.ctypes.data, len(px), out.ctypes.data, nthreads,
                                       buf, line_stride if lines else 0)
    if rc != 0:
        raise RuntimeError(f"ref_integrate failed: {rc}")
    if lines:
        raw = buf.raw
        txt = [raw[i * line_stride:(i + 1) * line_stride].split(b"\0", 1)[0].decode() for i in range(len(px))]
        return out, txt
    return out


class RefMeshSpec(C.Structure):
    _fields_ = [("kind", C.c_int32), ("max_subdivide", C.c_int32), ("total_pixels", C.c_uint64),
                ("max_pixels", C.c_uint64), ("initial_pixels", C.c_uint64), ("iteration_pixels", C.c_uint64),
                ("initial_sub_to_final", C.c_int32), ("reserved", C.c_int32)]


def synth_value(kind, row, col, grid):
    """Same pure function as synth_value() in ref_driver.cpp."""
    R = int(grid)
    row, col = int(row), int(col)
    dr, dc = 2 * row - R, 2 * col - R
    if kind == 0:
        if dr * dr + 3 * dc * dc < (R * R) // 3:
            return 0.0
        return float(1 + (0 if row < col else 1) + (0 if row + col < R else 2))
    if kind == 1:
        w = R // 8 + 1
        v = (row * 31 + col * 17) // w
        return float(v % 6 - 2)
    h = (row * 7919 + col * 104729) % 1009
    return 1.5 + float(h) * 0.0009765625 * float((row + col) % 3)
