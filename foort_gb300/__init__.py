"""GB300 geodesic-integration engine for FOORT runs.

The compute path is the C-ABI library ``libfoort_gpu.so`` (hand-written sm_103a CUDA
kernels plus a C++ host layer; see include/foort_gpu.h). This package loads it with
ctypes and offers a thin Python view used by tests and benchmarks. There is no CPU
fallback: without the compiled library every entry point raises.
"""
import ctypes as C
import os

import numpy as np

from . import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfoort_gpu.so")

_LIB = None

# foort_dmesh_round_fn: (user, d_px, d_res, n, round) -> int
DMESH_ROUND_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.c_uint32)


class FoortError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"FOORT error {code}: {msg}")
        self.code = code


def load():
    """Load libfoort_gpu.so (raises if it has not been built)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        raise FoortError(abi.FOORT_E_CUDA, f"{LIB_PATH} is missing: build it with foort_gb300.build.build()")
    lib = C.CDLL(LIB_PATH)
    vp, u64, i32, u32 = C.c_void_p, C.c_uint64, C.c_int32, C.c_uint32
    lib.foort_gpu_default_desc.argtypes = [C.POINTER(abi.RunDesc)]
    lib.foort_gpu_default_desc.restype = None
    lib.foort_gpu_create.argtypes = [C.POINTER(abi.RunDesc), C.POINTER(vp)]
    lib.foort_gpu_integrate.argtypes = [vp, vp, u64, vp]
    lib.foort_gpu_integrate_async.argtypes = [vp, vp, u64, vp, vp]
    lib.foort_gpu_integrate_noalloc.argtypes = [C.POINTER(abi.RunDesc), vp, u64, vp, vp, C.POINTER(abi.Stats)]
    lib.foort_gpu_sync.argtypes = [vp]
    lib.foort_gpu_set_budget.argtypes = [vp, u64]
    lib.foort_gpu_cancel.argtypes = [vp]
    lib.foort_gpu_set_launch.argtypes = [vp, u32, u32]
    lib.foort_gpu_set_lanes.argtypes = [vp, u32]
    lib.foort_gpu_get_stats.argtypes = [vp, C.POINTER(abi.Stats)]
    lib.foort_gpu_destroy.argtypes = [vp]
    lib.foort_gpu_destroy.restype = None
    lib.foort_gpu_last_error.argtypes = [vp]
    lib.foort_gpu_last_error.restype = C.c_char_p
    lib.foort_horizon_radius.argtypes = [i32, vp]
    lib.foort_horizon_radius.restype = C.c_double
    lib.foort_abi_size.argtypes = [i32]
    lib.foort_abi_size.restype = u64
    lib.foort_measure_peaks.argtypes = [C.POINTER(C.c_double), C.POINTER(C.c_double)]
    lib.foort_gpu_has_kernel.argtypes = [i32, i32, i32]
    lib.foort_metric_christoffel.argtypes = [i32, vp, i32, vp, vp]
    lib.foort_mesh_create_simple.argtypes = [u64, u32, u32, C.POINTER(vp)]
    lib.foort_mesh_create_v2.argtypes = [u64, u64, i32, u64, i32, u32, u32, C.POINTER(vp)]
    lib.foort_mesh_is_finished.argtypes = [vp]
    lib.foort_mesh_cur_nr_geodesics.argtypes = [vp]
    lib.foort_mesh_cur_nr_geodesics.restype = u64
    lib.foort_mesh_grid.argtypes = [vp]
    lib.foort_mesh_grid.restype = u64
    lib.foort_mesh_rounds.argtypes = [vp]
    lib.foort_mesh_rounds.restype = u64
    lib.foort_mesh_get_pixels.argtypes = [vp, u32, vp]
    lib.foort_mesh_geodesic_finished.argtypes = [vp, u64, vp, u32]
    lib.foort_mesh_set_results.argtypes = [vp, vp, u64]
    lib.foort_mesh_end_current_loop.argtypes = [vp]
    lib.foort_mesh_destroy.argtypes = [vp]
    lib.foort_mesh_destroy.restype = None
    lib.foort_mesh_description.argtypes = [vp, C.c_char_p, u64]
    lib.foort_first_line_info.argtypes = [C.POINTER(abi.RunDesc), u32, vp, C.c_char_p, u64]
    lib.foort_output_create.argtypes = [C.POINTER(abi.OutputDesc), C.POINTER(vp)]
    lib.foort_output_round.argtypes = [vp, vp, vp, u64]
    lib.foort_output_finish.argtypes = [vp]
    lib.foort_output_destroy.argtypes = [vp]
    lib.foort_output_destroy.restype = None
    lib.foort_gpu_run.argtypes = [vp, C.POINTER(vp), C.POINTER(vp), u32, C.POINTER(u64), C.POINTER(u32)]
    lib.foort_config_load.argtypes = [C.c_char_p, C.POINTER(abi.Config), C.c_char_p, u64]
    lib.foort_config_parse.argtypes = [C.c_char_p, C.POINTER(abi.Config), C.c_char_p, u64]
    lib.foort_config_create_mesh.argtypes = [C.POINTER(abi.Config), C.POINTER(vp)]
    lib.foort_timestamp_string.argtypes = [C.c_char_p, u64]
    lib.foort_gpu_positions.argtypes = [vp, vp, u64, vp, vp, vp, u64, C.POINTER(u64)]
    lib.foort_geopos_count.argtypes = [C.POINTER(abi.RunDesc), u64, i32, C.POINTER(u64), C.POINTER(u64)]
    lib.foort_output_round_positions.argtypes = [vp, vp, vp, u64, vp, vp]
    lib.foort_gpu_get_desc.argtypes = [vp, C.POINTER(abi.RunDesc)]
    lib.foort_gpu_autotune.argtypes = [vp, vp, u64, vp, vp, C.POINTER(abi.LaunchShape)]
    lib.foort_gpu_set_autotune.argtypes = [vp, i32]
    lib.foort_gpu_launch_shape.argtypes = [vp, u64, C.POINTER(abi.LaunchShape)]
    lib.foort_tune_bucket.argtypes = [u64]
    lib.foort_tune_bucket.restype = u32
    lib.foort_tune_key.argtypes = [C.POINTER(abi.RunDesc), i32, u64, C.c_char_p, u64]
    lib.foort_tune_put.argtypes = [C.c_char_p, C.POINTER(abi.LaunchShape)]
    lib.foort_tune_get.argtypes = [C.c_char_p, C.POINTER(abi.LaunchShape)]
    lib.foort_tune_count.argtypes = []
    lib.foort_tune_count.restype = u64
    lib.foort_tune_clear.argtypes = []
    lib.foort_tune_clear.restype = None
    lib.foort_tune_save.argtypes = [C.c_char_p]
    lib.foort_tune_load.argtypes = [C.c_char_p]
    lib.foort_mesh_create_waves.argtypes = [vp, C.POINTER(vp)]
    lib.foort_mesh_lookahead.argtypes = [vp, u32, vp, u64, C.POINTER(u64)]
    lib.foort_mesh_max_pixels.argtypes = [vp]
    lib.foort_mesh_max_pixels.restype = u64
    lib.foort_mesh_kind.argtypes = [vp]
    lib.foort_gpu_set_lookahead.argtypes = [vp, u64]
    lib.foort_gpu_set_record_launches.argtypes = [vp, i32]
    lib.foort_gpu_run_launch.argtypes = [vp, u32, vp, u64, C.POINTER(u64)]
    lib.foort_gpu_set_schedule.argtypes = [vp, u32]
    lib.foort_gpu_run_info.argtypes = [vp, C.POINTER(u32), C.POINTER(u32)]
    lib.foort_dmesh_create_v2.argtypes = [u64, u64, i32, u64, i32, u32, u32, u32, u32, vp, C.POINTER(vp)]
    lib.foort_dmesh_is_finished.argtypes = [vp]
    for f in ("cur_nr_geodesics", "grid", "rounds", "active"):
        getattr(lib, "foort_dmesh_" + f).argtypes = [vp]
        getattr(lib, "foort_dmesh_" + f).restype = u64
    lib.foort_dmesh_pixels.argtypes = [vp]
    lib.foort_dmesh_pixels.restype = vp
    lib.foort_dmesh_get_pixels.argtypes = [vp, vp]
    lib.foort_dmesh_set_results.argtypes = [vp, vp, u64]
    lib.foort_dmesh_set_values.argtypes = [vp, vp, u64]
    lib.foort_dmesh_end_current_loop.argtypes = [vp]
    lib.foort_dmesh_last_error.argtypes = [vp]
    lib.foort_dmesh_last_error.restype = C.c_char_p
    lib.foort_dmesh_destroy.argtypes = [vp]
    lib.foort_dmesh_destroy.restype = None
    lib.foort_gpu_run_dmesh.argtypes = [vp, vp, vp, u64, DMESH_ROUND_FN, vp, C.POINTER(u64), C.POINTER(u32)]
    _LIB = lib
    return lib


def check_layout():
    """Compare the ctypes layouts with the compiled library's struct sizes."""
    lib = load()
    want = [C.sizeof(abi.Pixel), C.sizeof(abi.Result), C.sizeof(abi.RunDesc), C.sizeof(abi.ImageDesc),
            C.sizeof(abi.Stats), C.sizeof(abi.OutputDesc), C.sizeof(abi.Config)]
    got = [lib.foort_abi_size(i) for i in range(len(want))]
    if want != got:
        raise FoortError(abi.FOORT_E_BADARG, f"ABI layout mismatch: python {want} vs library {got}")
    return got


def mixed_available(metric_id=abi.METRIC_KERR, integrator=abi.INTEGRATOR_RK4):
    """True when this build has a mixed-precision kernel for the metric / integrator."""
    return bool(load().foort_gpu_has_kernel(metric_id, integrator, abi.PREC_MIXED))


def measure_peaks():
    """Measured FP32 / FP64 FMA throughput of the current GPU in TFLOP/s."""
    a, b = C.c_double(), C.c_double()
    rc = load().foort_measure_peaks(C.byref(a), C.byref(b))
    if rc != 0:
        raise FoortError(rc, "peak measurement failed")
    return a.value, b.value


class Engine:
    """One engine context (include/foort_gpu.h: foort_gpu_create ... foort_gpu_destroy)."""

    def __init__(self, desc):
        self._lib = load()
        self._desc = desc
        self._ctx = C.c_void_p()
        rc = self._lib.foort_gpu_create(C.byref(desc), C.byref(self._ctx))
        if rc != 0:
            raise FoortError(rc, self._lib.foort_gpu_last_error(None).decode())

    def _check(self, rc, ok=(0,)):
        if rc not in ok:
            raise FoortError(rc, self._lib.foort_gpu_last_error(self._ctx).decode())
        return rc

    def integrate(self, px, out=None, allow=(0,)):
        """Host pixels (PIXEL_DTYPE array) -> host results (RESULT_DTYPE array)."""
        px = np.ascontiguousarray(px, dtype=abi.PIXEL_DTYPE)
        if out is None:
            out = np.zeros(len(px), dtype=abi.RESULT_DTYPE)
        rc = self._lib.foort_gpu_integrate(self._ctx, px.ctypes.data, len(px), out.ctypes.data)
        self._check(rc, allow)
        return out

    def integrate_ptr(self, px_ptr, n, out_ptr, allow=(0,)):
        """Same with raw host pointers (e.g. pinned buffers)."""
        rc = self._lib.foort_gpu_integrate(self._ctx, C.c_void_p(px_ptr), n, C.c_void_p(out_ptr))
        return self._check(rc, allow)

    def integrate_async(self, d_px, n, d_out, stream=0):
        """Device pointers; enqueued on `stream` (a cudaStream_t as int)."""
        rc = self._lib.foort_gpu_integrate_async(self._ctx, C.c_void_p(d_px), n, C.c_void_p(d_out),
                                                 C.c_void_p(stream))
        return self._check(rc)

    def sync(self, allow=(0,)):
        return self._check(self._lib.foort_gpu_sync(self._ctx), allow)

    def set_budget(self, steps):
        self._check(self._lib.foort_gpu_set_budget(self._ctx, steps))

    def cancel(self):
        self._check(self._lib.foort_gpu_cancel(self._ctx))

    def set_launch(self, block_size=0, blocks_per_sm=0):
        self._check(self._lib.foort_gpu_set_launch(self._ctx, block_size, blocks_per_sm))

    def set_lanes(self, lanes_per_geodesic=0):
        """0: chosen per launch; 1 or 2 lanes per geodesic where the kernel has both."""
        self._check(self._lib.foort_gpu_set_lanes(self._ctx, lanes_per_geodesic))

    def autotune(self, d_px, n, d_out, stream=0):
        """Search launch shapes for n device pixels (foort_gpu_autotune); returns the
        fastest shape as a dict. d_out then holds the pixels' results."""
        best = abi.LaunchShape()
        self._check(self._lib.foort_gpu_autotune(self._ctx, C.c_void_p(d_px), n, C.c_void_p(d_out),
                                                 C.c_void_p(stream), C.byref(best)))
        return best.as_dict()

    def set_autotune(self, on=True):
        self._check(self._lib.foort_gpu_set_autotune(self._ctx, 1 if on else 0))

    def launch_shape(self, n):
        """The shape a launch of n pixels would use now."""
        s = abi.LaunchShape()
        self._check(self._lib.foort_gpu_launch_shape(self._ctx, n, C.byref(s)))
        return s.as_dict()

    def positions(self, px, first):
        """GeodesicPosition of the pixels whose first-pass results are `first`
        (foort_gpu_positions). Returns (counts, points): points is (total, 4)."""
        px = np.ascontiguousarray(px, dtype=abi.PIXEL_DTYPE)
        first = np.ascontiguousarray(first, dtype=abi.RESULT_DTYPE)
        n = len(px)
        counts = np.zeros(n, dtype=np.uint64)
        total = C.c_uint64()
        self._check(self._lib.foort_gpu_positions(self._ctx, px.ctypes.data, n, first.ctypes.data,
                                                  counts.ctypes.data, None, 0, C.byref(total)))
        points = np.zeros((max(total.value, 1), 4))
        self._check(self._lib.foort_gpu_positions(self._ctx, px.ctypes.data, n, first.ctypes.data,
                                                  counts.ctypes.data, points.ctypes.data, total.value,
                                                  C.byref(total)))
        return counts, points[:total.value]

    def run(self, meshes, outputs=None):
        """A whole run over one mesh (and optional Output) per image (foort_gpu_run).
        Returns (geodesics, rounds)."""
        n = len(meshes)
        ms = (C.c_void_p * n)(*[m._m for m in meshes])
        os_ = (C.c_void_p * n)(*[(o._o if o is not None else None) for o in (outputs or [None] * n)])
        g, r = C.c_uint64(), C.c_uint32()
        self._check(self._lib.foort_gpu_run(self._ctx, ms, os_, n, C.byref(g), C.byref(r)))
        return g.value, r.value

    def set_schedule(self, schedule=abi.SCHEDULE_WAVES):
        """foort_gpu_run's launches: level waves where they apply, or one per round."""
        self._check(self._lib.foort_gpu_set_schedule(self._ctx, schedule))

    def set_lookahead(self, max_geodesics=None):
        """Cap of a wave launch that also takes the next wave's candidates (None: the
        default, 128 x the SM count; 0: off)."""
        self._check(self._lib.foort_gpu_set_lookahead(self._ctx, (1 << 64) - 1 if max_geodesics is None
                                                      else max_geodesics))

    def set_record_launches(self, on=True):
        self._check(self._lib.foort_gpu_set_record_launches(self._ctx, 1 if on else 0))

    def run_launches(self):
        """The pixel lists of the last run's launches (set_record_launches)."""
        out, k = [], 0
        n = C.c_uint64()
        while self._lib.foort_gpu_run_launch(self._ctx, k, None, 0, C.byref(n)) == 0:
            a = np.zeros(n.value, dtype=abi.PIXEL_DTYPE)
            if n.value:
                self._check(self._lib.foort_gpu_run_launch(self._ctx, k, a.ctypes.data, n.value, C.byref(n)))
            out.append(a)
            k += 1
        return out

    def run_info(self):
        """(launches, schedule) of the last foort_gpu_run."""
        n, sch = C.c_uint32(), C.c_uint32()
        self._check(self._lib.foort_gpu_run_info(self._ctx, C.byref(n), C.byref(sch)))
        return n.value, sch.value

    def stats(self):
        s = abi.Stats()
        self._lib.foort_gpu_get_stats(self._ctx, C.byref(s))
        return {k: getattr(s, k) for k, _ in abi.Stats._fields_}

    def last_error(self):
        return self._lib.foort_gpu_last_error(self._ctx).decode()

    def close(self):
        if self._ctx:
            self._lib.foort_gpu_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def tune_key(desc, num_sms, n):
    """The launch-shape cache key of a launch of n pixels (foort_tune_key)."""
    buf = C.create_string_buffer(160)
    rc = load().foort_tune_key(C.byref(desc), num_sms, n, buf, len(buf))
    if rc != 0:
        raise FoortError(rc, "tune key")
    return buf.value.decode()


def tune_get(key):
    s = abi.LaunchShape()
    return s.as_dict() if load().foort_tune_get(key.encode(), C.byref(s)) == 0 else None


def tune_put(key, **shape):
    s = abi.LaunchShape(**shape)
    rc = load().foort_tune_put(key.encode(), C.byref(s))
    if rc != 0:
        raise FoortError(rc, "invalid launch shape or key")


def tune_save(path):
    rc = load().foort_tune_save(os.fsencode(path))
    if rc != 0:
        raise FoortError(rc, f"cannot write {path}")


def tune_load(path):
    rc = load().foort_tune_load(os.fsencode(path))
    if rc != 0:
        raise FoortError(rc, f"cannot read {path}")


def tune_clear():
    load().foort_tune_clear()


def tune_count():
    return load().foort_tune_count()


def horizon_radius(metric_id, params):
    arr = (C.c_double * 6)(*([float(p) for p in params] + [0.0] * (6 - len(params))))
    return load().foort_horizon_radius(metric_id, C.cast(arr, C.c_void_p))


class Mesh:
    """A host mesh (include/foort_gpu.h foort_mesh_*): SimpleSquareMesh or
    SquareSubdivisionMeshV2 with the reference's constructor arguments."""

    def __init__(self, kind, diag_flags, value_diag, total_pixels=0, max_pixels=0, initial_pixels=0,
                 max_subdivide=1, iteration_pixels=0, initial_sub_to_final=0):
        self._lib = load()
        self._m = C.c_void_p()
        if kind == "simple":
            rc = self._lib.foort_mesh_create_simple(total_pixels, diag_flags, value_diag, C.byref(self._m))
        else:
            rc = self._lib.foort_mesh_create_v2(max_pixels, initial_pixels, max_subdivide, iteration_pixels,
                                                initial_sub_to_final, diag_flags, value_diag, C.byref(self._m))
        if rc != 0:
            raise FoortError(rc, "mesh creation failed")

    @classmethod
    def from_spec(cls, spec, diag_flags, value_diag):
        kind, args = spec
        if kind == "simple":
            return cls("simple", diag_flags, value_diag, total_pixels=args * args)
        return cls("v2", diag_flags, value_diag, **args)

    def finished(self):
        return bool(self._lib.foort_mesh_is_finished(self._m))

    def size(self):
        return self._lib.foort_mesh_cur_nr_geodesics(self._m)

    def grid(self):
        return self._lib.foort_mesh_grid(self._m)

    def rounds(self):
        return self._lib.foort_mesh_rounds(self._m)

    def pixels(self, image=0, out=None):
        n = self.size()
        if out is None:
            out = np.zeros(n, dtype=abi.PIXEL_DTYPE)
        rc = self._lib.foort_mesh_get_pixels(self._m, image, out.ctypes.data)
        if rc != 0:
            raise FoortError(rc, "get_pixels failed")
        return out[:n]

    def set_values(self, values):
        for i, v in enumerate(values):
            arr = (C.c_double * 1)(float(v))
            self._lib.foort_mesh_geodesic_finished(self._m, i, arr, 1)

    def set_results(self, results):
        rc = self._lib.foort_mesh_set_results(self._m, results.ctypes.data, len(results))
        if rc != 0:
            raise FoortError(rc, "set_results failed")

    def end_round(self):
        self._lib.foort_mesh_end_current_loop(self._m)

    def max_pixels(self):
        """Most pixels the mesh hands out over a run (0: no limit)."""
        return self._lib.foort_mesh_max_pixels(self._m)

    def kind(self):
        """abi.MESH_SIMPLE or abi.MESH_SUBDIVISION_V2."""
        return self._lib.foort_mesh_kind(self._m)

    def lookahead(self, image=0):
        """foort_mesh_lookahead: candidates of the next round of a mesh of level waves."""
        n = C.c_uint64()
        rc = self._lib.foort_mesh_lookahead(self._m, image, None, 0, C.byref(n))
        if rc != 0:
            raise FoortError(rc, "lookahead failed")
        out = np.zeros(n.value, dtype=abi.PIXEL_DTYPE)
        if n.value:
            self._lib.foort_mesh_lookahead(self._m, image, out.ctypes.data, n.value, C.byref(n))
        return out

    def waves(self):
        """The mesh's level waves (foort_mesh_create_waves) as a new Mesh."""
        w = Mesh.__new__(Mesh)
        w._lib = self._lib
        w._m = C.c_void_p()
        rc = self._lib.foort_mesh_create_waves(self._m, C.byref(w._m))
        if rc != 0:
            raise FoortError(rc, "this mesh has no level waves")
        return w

    def description(self):
        buf = C.create_string_buffer(1024)
        if self._lib.foort_mesh_description(self._m, buf, len(buf)) != 0:
            raise FoortError(abi.FOORT_E_BADARG, "mesh description failed")
        return buf.value.decode()

    def first_line_info(self, desc, image=0):
        """Utilities::GetFirstLineInfoString for image `image` of desc run on this mesh."""
        buf = C.create_string_buffer(8192)
        rc = self._lib.foort_first_line_info(C.byref(desc), image, self._m, buf, len(buf))
        if rc != 0:
            raise FoortError(rc, "first-line description failed")
        return buf.value.decode()

    def close(self):
        if self._m:
            self._lib.foort_mesh_destroy(self._m)
            self._m = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DeviceMesh:
    """SquareSubdivisionMeshV2 held in device memory (include/foort_gpu.h foort_dmesh_*).
    order: abi.DMESH_ORDER_REFERENCE (the reference's pixel order) or
    abi.DMESH_ORDER_DEVICE. stream: a cudaStream_t as int (0 = legacy)."""

    def __init__(self, diag_flags, value_diag, max_pixels=0, initial_pixels=0, max_subdivide=1,
                 iteration_pixels=0, initial_sub_to_final=0, image=0, order=abi.DMESH_ORDER_REFERENCE, stream=0):
        self._lib = load()
        self._m = C.c_void_p()
        rc = self._lib.foort_dmesh_create_v2(max_pixels, initial_pixels, max_subdivide, iteration_pixels,
                                             initial_sub_to_final, diag_flags, value_diag, image, order,
                                             C.c_void_p(stream), C.byref(self._m))
        if rc != 0:
            raise FoortError(rc, "device mesh creation failed")

    @classmethod
    def from_spec(cls, spec, diag_flags, value_diag, **kw):
        kind, args = spec
        if kind != "v2":
            raise FoortError(abi.FOORT_E_UNSUPPORTED, "the device mesh is SquareSubdivisionMeshV2")
        return cls(diag_flags, value_diag, **args, **kw)

    def _check(self, rc, what):
        if rc != 0:
            raise FoortError(rc, f"{what}: {self._lib.foort_dmesh_last_error(self._m).decode()}")

    def finished(self):
        return bool(self._lib.foort_dmesh_is_finished(self._m))

    def size(self):
        return self._lib.foort_dmesh_cur_nr_geodesics(self._m)

    def grid(self):
        return self._lib.foort_dmesh_grid(self._m)

    def rounds(self):
        return self._lib.foort_dmesh_rounds(self._m)

    def active(self):
        return self._lib.foort_dmesh_active(self._m)

    def pixels_ptr(self):
        """Device address of the round's pixels."""
        return self._lib.foort_dmesh_pixels(self._m) or 0

    def pixels(self):
        """The round's pixels copied to the host."""
        out = np.zeros(self.size(), dtype=abi.PIXEL_DTYPE)
        self._check(self._lib.foort_dmesh_get_pixels(self._m, out.ctypes.data if len(out) else None), "get_pixels")
        return out

    def set_results_ptr(self, d_res, n):
        self._check(self._lib.foort_dmesh_set_results(self._m, C.c_void_p(d_res), n), "set_results")

    def set_values_ptr(self, d_values, n):
        """n doubles in device memory, one per pixel of the round."""
        self._check(self._lib.foort_dmesh_set_values(self._m, C.c_void_p(d_values), n), "set_values")

    def end_round(self):
        self._check(self._lib.foort_dmesh_end_current_loop(self._m), "end_current_loop")

    def run(self, engine, d_out, cap_out, on_round=None):
        """foort_gpu_run_dmesh with `engine`; on_round(d_px, d_res, n, round) is called
        after each round's integration. Returns (geodesics, rounds)."""
        err = []

        def cb(_user, d_px, d_res, n, rnd):
            try:
                on_round(d_px or 0, d_res or 0, n, rnd)
                return 0
            except Exception as e:  # noqa: BLE001 -- reported after the run
                err.append(e)
                return abi.FOORT_E_BADARG

        fn = DMESH_ROUND_FN(cb) if on_round else C.cast(None, DMESH_ROUND_FN)
        g, r = C.c_uint64(), C.c_uint32()
        rc = self._lib.foort_gpu_run_dmesh(engine._ctx, self._m, C.c_void_p(d_out), cap_out, fn, None, C.byref(g),
                                           C.byref(r))
        if err:
            raise err[0]
        if rc != 0:
            msg = self._lib.foort_dmesh_last_error(self._m).decode() or engine.last_error()
            raise FoortError(rc, f"run_dmesh: {msg}")
        return g.value, r.value

    def close(self):
        if self._m:
            self._lib.foort_dmesh_destroy(self._m)
            self._m = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Output:
    """Output files of a run as FOORT writes them (include/foort_gpu.h foort_output_*)."""

    def __init__(self, prefix, diag_flags, value_diag, first_line="", extension="dat", timestamp="",
                 outputs_to_cache=1 << 40, geodesics_per_file=1 << 40):
        self._lib = load()
        self._o = C.c_void_p()
        d = abi.OutputDesc()
        d.prefix, d.timestamp, d.extension = prefix.encode(), timestamp.encode(), extension.encode()
        d.first_line = first_line.encode()
        d.outputs_to_cache, d.geodesics_per_file = outputs_to_cache, geodesics_per_file
        d.diag_flags, d.value_diag = diag_flags, value_diag
        rc = self._lib.foort_output_create(C.byref(d), C.byref(self._o))
        if rc != 0:
            raise FoortError(rc, "output creation failed")

    def round(self, px, res, counts=None, points=None):
        """One round's results; counts / points (Engine.positions) with GeodesicPosition."""
        px = np.ascontiguousarray(px, dtype=abi.PIXEL_DTYPE)
        res = np.ascontiguousarray(res, dtype=abi.RESULT_DTYPE)
        if counts is None:
            rc = self._lib.foort_output_round(self._o, px.ctypes.data, res.ctypes.data, len(px))
        else:
            counts = np.ascontiguousarray(counts, dtype=np.uint64)
            points = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 4)
            if len(points) == 0:
                points = np.zeros((1, 4))
            rc = self._lib.foort_output_round_positions(self._o, px.ctypes.data, res.ctypes.data, len(px),
                                                        counts.ctypes.data, points.ctypes.data)
        if rc != 0:
            raise FoortError(rc, "writing output failed")

    def finish(self):
        rc = self._lib.foort_output_finish(self._o)
        if rc != 0:
            raise FoortError(rc, "writing output failed")

    def close(self):
        if self._o:
            self._lib.foort_output_destroy(self._o)
            self._o = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def load_config(path=None, text=None):
    """A FOORT .cfg file (or its text) read as the reference reads it
    (foort_config_load). Returns (config, notes): config.run has its image attached."""
    lib = load()
    cfg = abi.Config()
    notes = C.create_string_buffer(1 << 16)
    if text is not None:
        rc = lib.foort_config_parse(text.encode(), C.byref(cfg), notes, len(notes))
    else:
        rc = lib.foort_config_load(os.fsencode(path), C.byref(cfg), notes, len(notes))
    if rc != 0:
        raise FoortError(rc, notes.value.decode())
    cfg.run.images = C.pointer(cfg.image)
    cfg.run.n_images = 1
    return cfg, [ln for ln in notes.value.decode().splitlines() if ln]


def config_mesh(cfg):
    """The mesh a configuration asks for (a Mesh object)."""
    m = Mesh.__new__(Mesh)
    m._lib = load()
    m._m = C.c_void_p()
    rc = m._lib.foort_config_create_mesh(C.byref(cfg), C.byref(m._m))
    if rc != 0:
        raise FoortError(rc, "this mesh type is not available in the engine")
    return m


def run_rounds(mesh_specs, desc, integrate, on_round=None, waves=False):
    """One FOORT run (the round loop of Main.cpp:313-419) over one mesh per image, the
    images' meshes advancing in lockstep so that each round is one integrate() call over
    the pixels of every unfinished image. mesh_specs: Mesh.from_spec specs; integrate(px)
    -> results; on_round(px, res) after each round. waves: the meshes' level waves
    (Mesh.waves) instead of their rounds. Returns the number of rounds."""
    meshes = [Mesh.from_spec(spec, desc.diag_flags, desc.value_diag) for spec in mesh_specs]
    if waves:
        base, meshes = meshes, []
        for m in base:
            meshes.append(m.waves())
            m.close()
    n_rounds = 0
    try:
        while True:
            live = [(i, m) for i, m in enumerate(meshes) if not m.finished()]
            if not live:
                break
            parts = [m.pixels(image=i) for i, m in live]
            px = np.concatenate(parts)
            res = integrate(px)
            k = 0
            for (i, m), p in zip(live, parts):
                m.set_results(res[k:k + len(p)])
                m.end_round()
                k += len(p)
            if on_round:
                on_round(px, res)
            n_rounds += 1
    finally:
        for m in meshes:
            m.close()
    return n_rounds


def _pixel_keys(px):
    return (px["image"].astype(np.int64) << 42) | (px["row"].astype(np.int64) * px["grid"].astype(np.int64)
                                                 + px["col"].astype(np.int64))


class _ResultStore:
    """Results by pixel key (image, grid cell), kept sorted for lookups."""

    def __init__(self):
        self.k = np.zeros(0, np.int64)
        self.r = np.zeros(0, abi.RESULT_DTYPE)

    def add(self, px, res):
        k = np.concatenate([self.k, _pixel_keys(px)])
        r = np.concatenate([self.r, res])
        order = np.argsort(k, kind="stable")
        self.k, self.r = k[order], r[order]

    def find(self, px):
        q = _pixel_keys(px)
        if not len(self.k):
            return np.zeros(len(q), bool), np.zeros(len(q), abi.RESULT_DTYPE)
        i = np.minimum(np.searchsorted(self.k, q), len(self.k) - 1)
        return self.k[i] == q, self.r[i].copy()


def run_by_waves(mesh_specs, desc, integrate, on_round=None, lookahead=0):
    """foort_gpu_run's level-wave schedule with any integrate(px) -> results: the meshes'
    level waves (Mesh.waves) are integrated first, one integrate() call per wave, an
    image's waves stopping before the one that would take them past its mesh's
    max_pixels; a call also takes the next wave's candidates (Mesh.lookahead) while it then
    holds at most `lookahead` pixels (0: never). The meshes' rounds are then replayed from
    the stored results, so on_round(px, res) sees the reference's rounds; a round's pixels
    that no wave held go to integrate() then. Returns (rounds, integrate calls)."""
    store = _ResultStore()
    meshes = [Mesh.from_spec(spec, desc.diag_flags, desc.value_diag) for spec in mesh_specs]
    waves = []
    for m in meshes:
        waves.append(m.waves())
        budget = m.max_pixels()
        waves[-1].budget = budget if budget else float("inf")
        waves[-1].handed = 0
        m.close()
    calls = 0
    try:
        while True:
            live = []
            for i, w in enumerate(waves):
                if w.finished() or w.size() > w.budget - w.handed:
                    continue
                live.append((i, w))
            if not live:
                break
            parts = [w.pixels(image=i) for i, w in live]
            for (i, w), p in zip(live, parts):
                w.handed += len(p)
            px = np.concatenate(parts)
            found, _ = store.find(px)
            todo = px[~found]
            if len(todo):
                if lookahead > len(todo):
                    cand = [w.lookahead(image=i) for i, w in live]
                    if all(len(c) <= w.budget - w.handed for c, (i, w) in zip(cand, live)):
                        cand = np.concatenate(cand)
                        known, _ = store.find(cand)
                        cand = cand[~known & ~np.isin(_pixel_keys(cand), _pixel_keys(todo))]
                        if len(todo) + len(cand) <= lookahead:
                            todo = np.concatenate([todo, cand])
                store.add(todo, integrate(todo))
                calls += 1
            _, res = store.find(px)
            k = 0
            for (i, w), p in zip(live, parts):
                w.set_results(res[k:k + len(p)])
                w.end_round()
                k += len(p)
    finally:
        for w in waves:
            w.close()
    extra = [0]

    def lookup(px):
        found, res = store.find(px)
        if not found.all():
            res[~found] = integrate(px[~found])
            extra[0] += 1
        return res

    rounds = run_rounds(mesh_specs, desc, lookup, on_round)
    return rounds, calls + extra[0]


def run_config(path, precision=abi.PREC_MIXED, output_dir=None):
    """A whole FOORT run from a .cfg file: the configured metric, diagnostics,
    terminations, view screen, mesh, integrator and output files (Main.cpp:161-424), on
    the GPU in the given precision. Relative output prefixes are taken from output_dir
    (default: the working directory). Returns (geodesics, rounds, notes)."""
    cfg, notes = load_config(path)
    cfg.run.precision = precision
    mesh = config_mesh(cfg)
    out = None
    prefix = cfg.file_prefix.decode()
    if prefix:
        if output_dir and not os.path.isabs(prefix):
            prefix = os.path.join(output_dir, prefix)
        ts = ""
        if cfg.timestamp:
            buf = C.create_string_buffer(32)
            load().foort_timestamp_string(buf, len(buf))
            ts = buf.value.decode()
        first = mesh.first_line_info(cfg.run) if cfg.first_line_info else ""
        out = Output(prefix, cfg.run.diag_flags, cfg.run.value_diag, first_line=first,
                     extension=cfg.file_extension.decode(), timestamp=ts,
                     outputs_to_cache=cfg.outputs_to_cache, geodesics_per_file=cfg.geodesics_per_file)
    else:
        notes.append("no output file prefix: results are not written (console output is not provided)")
    with Engine(cfg.run) as e:
        geodesics, rounds = e.run([mesh], [out])
    if out is not None:
        out.close()
    mesh.close()
    return geodesics, rounds, notes
