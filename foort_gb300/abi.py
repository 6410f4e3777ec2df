"""ctypes mirror of include/foort_gpu.h.

The layouts below must stay byte-identical to the C structs; `check_layout()` compares
them with the sizes the compiled library reports (foort_abi_sizes).
"""
import ctypes as C

import numpy as np

# Return codes
FOORT_OK = 0
FOORT_E_BADARG = -1
FOORT_E_CUDA = -2
FOORT_E_BUDGET = -3
FOORT_E_NUMERIC = -4
FOORT_E_CANCELLED = -5
FOORT_E_UNSUPPORTED = -6
FOORT_E_IO = -7

# Metrics (Metric.h:78-189)
METRIC_KERR = 0
METRIC_FLAT = 1
METRIC_RASHEED_LARSEN = 2
METRIC_JOHANNSEN = 3
METRIC_MANKO_NOVIKOV = 4

INTEGRATOR_RK4 = 0
INTEGRATOR_VERLET = 1

PREC_FP64 = 0
PREC_MIXED = 1
PREC_FP64_ANALYTIC = 2  # every step in FP64 with the mixed kernel's analytic derivatives

# mesh kinds (foort_mesh_kind)
MESH_SIMPLE = 0
MESH_SUBDIVISION_V2 = 1

# foort_gpu_run's schedule (include/foort_gpu.h)
SCHEDULE_WAVES = 0
SCHEDULE_ROUNDS = 1

# device-resident mesh: order of the active squares (include/foort_gpu.h)
DMESH_ORDER_REFERENCE = 0
DMESH_ORDER_DEVICE = 1
DMESH_MAX_CELLS = 1 << 29

MIXED_FP64_DECISIONS = 0x1
MIXED_FP64_NEAR_HORIZON = 0x2
MIXED_FP64_TURNING_POINTS = 0x4

# foort_gpu_integrate_noalloc: images its static device array has room for
NOALLOC_MAX_IMAGES = 256

# TermBitflag (Terminations.h:29-33)
TERM_BOUNDARY_SPHERE = 0x1
TERM_TIMEOUT = 0x2
TERM_HORIZON = 0x4
TERM_THETA_SINGULARITY = 0x8

# DiagBitflag (Diagnostics.h:33-37)
DIAG_GEODESIC_POSITION = 0x1
DIAG_FOUR_COLOR_SCREEN = 0x2
DIAG_EQUATORIAL_PASSES = 0x4
DIAG_CLOSEST_RADIUS = 0x8

# enum class Term (Terminations.h:48-67)
TERMCODE_CONTINUE = 0
TERMCODE_HORIZON = 1
TERMCODE_BOUNDARY_SPHERE = 2
TERMCODE_TIMEOUT = 3
TERMCODE_THETA_SINGULARITY = 4

ERR_NONFINITE = 0x1
ERR_VERLET_ITER = 0x2
ERR_BUDGET = 0x4
ERR_CANCELLED = 0x8
ERR_UNFINISHED = 0x10
ERR_BADPIXEL = 0x20


class UpdateFreq(C.Structure):
    _fields_ = [("every_n", C.c_uint64), ("at_start", C.c_int32), ("at_finish", C.c_int32)]


class ImageDesc(C.Structure):
    _fields_ = [
        ("metric_params", C.c_double * 6),
        ("cam_pos", C.c_double * 4),
        ("cam_dir", C.c_double * 4),
        ("screen_size", C.c_double * 2),
        ("screen_center", C.c_double * 2),
        ("horizon_eps", C.c_double),
    ]


class RunDesc(C.Structure):
    _fields_ = [
        ("metric_id", C.c_int32),
        ("rlog", C.c_int32),
        ("integrator_id", C.c_int32),
        ("precision", C.c_int32),
        ("epsilon", C.c_double),
        ("derivative_h", C.c_double),
        ("smallest_step", C.c_double),
        ("verlet_tol", C.c_double),
        ("term_flags", C.c_uint32),
        ("diag_flags", C.c_uint32),
        ("value_diag", C.c_uint32),
        ("mixed_options", C.c_uint32),
        ("horizon_eps", C.c_double),
        ("horizon_every", C.c_uint64),
        ("boundary_radius", C.c_double),
        ("boundary_every", C.c_uint64),
        ("timeout_max_steps", C.c_uint64),
        ("timeout_every", C.c_uint64),
        ("theta_eps", C.c_double),
        ("theta_every", C.c_uint64),
        ("equat_freq", UpdateFreq),
        ("equat_threshold", C.c_double),
        ("closest_freq", UpdateFreq),
        ("geopos_freq", UpdateFreq),
        ("geopos_output_steps", C.c_uint64),
        ("mixed_fp64_margin", C.c_double),
        ("n_images", C.c_uint32),
        ("reserved1", C.c_uint32),
        ("images", C.POINTER(ImageDesc)),
    ]


class Pixel(C.Structure):
    _fields_ = [
        ("image", C.c_uint32),
        ("reserved", C.c_uint32),
        ("row", C.c_uint64),
        ("col", C.c_uint64),
        ("grid", C.c_uint64),
    ]


class Result(C.Structure):
    _fields_ = [
        ("term", C.c_int32),
        ("err", C.c_uint32),
        ("steps", C.c_uint64),
        ("lam", C.c_double),
        ("pos", C.c_double * 4),
        ("vel", C.c_double * 4),
        ("quadrant", C.c_int32),
        ("equat_passes", C.c_int32),
        ("closest_r", C.c_double),
    ]


class Stats(C.Structure):
    _fields_ = [
        ("geodesics", C.c_uint64),
        ("steps", C.c_uint64),
        ("rhs_evals", C.c_uint64),
        ("fp64_steps", C.c_uint64),
        ("kernel_ms", C.c_double),
        ("status", C.c_uint32),
        ("n_blocks", C.c_uint32),
        ("block_size", C.c_uint32),
        ("lanes_per_geodesic", C.c_uint32),
        ("refill_steps", C.c_uint32),
        ("poll_steps", C.c_uint32),
    ]


class LaunchShape(C.Structure):
    """foort_launch_shape: CTA size, CTA cap per SM, lanes per geodesic, regrouping
    cadence, poll interval, and the autotuner's measured time."""
    _fields_ = [
        ("block_size", C.c_uint32),
        ("blocks_per_sm", C.c_uint32),
        ("lanes", C.c_uint32),
        ("refill_steps", C.c_uint32),
        ("poll_steps", C.c_uint32),
        ("reserved", C.c_uint32),
        ("ms", C.c_double),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


CONFIG_MESH_SIMPLE = 0
CONFIG_MESH_SUBDIVISION_V2 = 1
CONFIG_MESH_SUBDIVISION = 2
CONFIG_MESH_INPUT_PIXELS = 3


class Config(C.Structure):
    _fields_ = [
        ("run", RunDesc),
        ("image", ImageDesc),
        ("mesh_kind", C.c_int32),
        ("max_subdivide", C.c_int32),
        ("total_pixels", C.c_uint64),
        ("initial_pixels", C.c_uint64),
        ("max_pixels", C.c_uint64),
        ("iteration_pixels", C.c_uint64),
        ("initial_sub_to_final", C.c_int32),
        ("timestamp", C.c_int32),
        ("outputs_to_cache", C.c_uint64),
        ("geodesics_per_file", C.c_uint64),
        ("first_line_info", C.c_int32),
        ("screen_output_level", C.c_int32),
        ("loop_message_frequency", C.c_uint64),
        ("file_prefix", C.c_char * 1024),
        ("file_extension", C.c_char * 64),
    ]


class OutputDesc(C.Structure):
    _fields_ = [
        ("prefix", C.c_char_p),
        ("timestamp", C.c_char_p),
        ("extension", C.c_char_p),
        ("first_line", C.c_char_p),
        ("outputs_to_cache", C.c_uint64),
        ("geodesics_per_file", C.c_uint64),
        ("diag_flags", C.c_uint32),
        ("value_diag", C.c_uint32),
    ]


# numpy views of the arrays the C ABI reads and writes
PIXEL_DTYPE = np.dtype([("image", "<u4"), ("reserved", "<u4"), ("row", "<u8"), ("col", "<u8"), ("grid", "<u8")])
RESULT_DTYPE = np.dtype([
    ("term", "<i4"), ("err", "<u4"), ("steps", "<u8"), ("lam", "<f8"), ("pos", "<f8", (4,)), ("vel", "<f8", (4,)),
    ("quadrant", "<i4"), ("equat_passes", "<i4"), ("closest_r", "<f8"),
])
assert PIXEL_DTYPE.itemsize == C.sizeof(Pixel)
assert RESULT_DTYPE.itemsize == C.sizeof(Result)


def make_image(metric_params=(0.5,), r=1000.0, theta=np.pi / 2, phi=0.0, half_width=10.0, center=(0.0, 0.0),
               size=None, horizon_eps=0.0):
    """One image: metric parameters plus a camera at (0, r, theta, phi) looking inward."""
    im = ImageDesc()
    for i, p in enumerate(metric_params):
        im.metric_params[i] = float(p)
    im.cam_pos[:] = [0.0, float(r), float(theta), float(phi)]
    im.cam_dir[:] = [0.0, -1.0, 0.0, 0.0]
    if size is None:
        size = (2.0 * half_width, 2.0 * half_width)
    im.screen_size[:] = [float(size[0]), float(size[1])]
    im.screen_center[:] = [float(center[0]), float(center[1])]
    im.horizon_eps = float(horizon_eps)
    return im


def default_desc():
    """The reference's defaults (Config.cpp:127-1071); images must be attached."""
    d = RunDesc()
    d.metric_id = METRIC_KERR
    d.rlog = 0
    d.integrator_id = INTEGRATOR_RK4
    d.precision = PREC_FP64
    d.epsilon = 0.03
    d.derivative_h = 1e-7
    d.smallest_step = 1e-12
    d.verlet_tol = 0.001
    d.term_flags = TERM_BOUNDARY_SPHERE | TERM_TIMEOUT
    d.diag_flags = DIAG_FOUR_COLOR_SCREEN
    d.value_diag = DIAG_FOUR_COLOR_SCREEN
    d.horizon_eps = 0.01
    d.horizon_every = 1
    d.boundary_radius = 1000.0
    d.boundary_every = 1
    d.timeout_max_steps = 10000
    d.timeout_every = 1
    d.theta_eps = 1e-5
    d.theta_every = 1
    d.equat_freq = UpdateFreq(1, 1, 1)
    d.equat_threshold = 0.01
    d.closest_freq = UpdateFreq(1, 1, 1)
    d.geopos_freq = UpdateFreq(1, 0, 1)
    d.geopos_output_steps = 0
    d.n_images = 0
    d.images = None
    return d


def attach_images(desc, images):
    """Attach a list of ImageDesc; the returned array must outlive every call using desc."""
    arr = (ImageDesc * len(images))(*images)
    desc.images = C.cast(arr, C.POINTER(ImageDesc))
    desc.n_images = len(images)
    return arr


def square_pixels(side, image=0, rows=None):
    """All pixels of a side x side SimpleSquareMesh (Mesh.cpp:31-50), row-major."""
    idx = np.arange(side * side, dtype=np.uint64)
    px = np.zeros(side * side, dtype=PIXEL_DTYPE)
    px["image"] = image
    px["row"] = idx // side
    px["col"] = idx % side
    px["grid"] = side
    if rows is not None:
        px = px[np.isin(px["row"], rows)]
    return px


def ptr(arr, ctype=C.c_void_p):
    return C.cast(arr.ctypes.data, ctype)
