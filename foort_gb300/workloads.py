"""The engine's benchmark workloads as run descriptors.

C1  Kerr a=0.5, observer r=1000 M at 80 deg, 100x100 SimpleSquareMesh of half-width 10 M,
    RK4, Horizon (r < r_+ + 0.01 M), BoundarySphere 1000 M, TimeOut 1e5; FourColorScreen
    (mesh value) + EquatorialPasses.
C2  Kerr a=0.99 at 60 deg, half-width 12 M, SquareSubdivisionMeshV2 from a 128x128 seed with
    MaxSubdivide 3 (grid 509), seed round + 4 refinement rounds; FourColorScreen (mesh
    value) + ClosestRadius.
C3  64 Kerr images in one launch: a ~ U[0, 0.998], inclination ~ U[5, 85] deg, side in
    {64, 128, 256, 512}, half-width ~ U[10, 15] M; FourColorScreen + EquatorialPasses.
C4  Johannsen a=0.9, alpha13 ~ U[-1, 1], normal r, 1024x1024 at 30 deg, half-width 10 M,
    Verlet (tolerance 1e-3); EquatorialPasses (mesh value) + ClosestRadius.
C5  Kerr a=0.998 at 17 deg, half-width 10 M, SquareSubdivisionMeshV2 from 129x129 with
    MaxSubdivide 6 (grid 4097), every active pixel subdivided each round; FourColorScreen
    (mesh value) + EquatorialPasses.

The reference states its horizon tolerance relative to r_+ (Terminations.cpp:109-110), so
"r < r_+ + 0.01 M" is Epsilon_Horizon = 0.01 / r_+.

All random draws come from a 64-bit Mersenne Twister (mt19937_64) seeded with 20261203,
implemented here so that every machine draws the same values.
"""
import math

import numpy as np

from . import abi

SEED = 20261203
DEG = math.pi / 180.0


class MT19937_64:
    """The standard 64-bit Mersenne Twister (Matsumoto & Nishimura, 2004)."""
    NN, MM = 312, 156
    MATRIX_A = 0xB5026F5AA96619E9
    UM, LM = 0xFFFFFFFF80000000, 0x7FFFFFFF
    MASK = (1 << 64) - 1

    def __init__(self, seed):
        self.mt = [0] * self.NN
        self.mt[0] = seed & self.MASK
        for i in range(1, self.NN):
            self.mt[i] = (6364136223846793005 * (self.mt[i - 1] ^ (self.mt[i - 1] >> 62)) + i) & self.MASK
        self.mti = self.NN

    def next_u64(self):
        if self.mti >= self.NN:
            mt, NN, MM = self.mt, self.NN, self.MM
            for i in range(NN):
                x = (mt[i] & self.UM) | (mt[(i + 1) % NN] & self.LM)
                xa = x >> 1
                if x & 1:
                    xa ^= self.MATRIX_A
                mt[i] = mt[(i + MM) % NN] ^ xa
            self.mti = 0
        x = self.mt[self.mti]
        self.mti += 1
        x ^= (x >> 29) & 0x5555555555555555
        x ^= (x << 17) & 0x71D67FFFEDA60000
        x ^= (x << 37) & 0xFFF7EEE000000000
        x ^= x >> 43
        return x & self.MASK

    def uniform(self, lo, hi):
        """Uniform double in [lo, hi) from the top 53 bits."""
        return lo + (hi - lo) * ((self.next_u64() >> 11) * (1.0 / 9007199254740992.0))

    def choice(self, options):
        return options[self.next_u64() % len(options)]


def _kerr_rp(a):
    return 1.0 + math.sqrt(1.0 - a * a)


def base_desc(precision=abi.PREC_FP64):
    d = abi.default_desc()
    d.precision = precision
    d.term_flags = abi.TERM_HORIZON | abi.TERM_BOUNDARY_SPHERE | abi.TERM_TIMEOUT
    d.boundary_radius = 1000.0
    d.timeout_max_steps = 100000
    d.equat_threshold = 0.01
    d.equat_freq = abi.UpdateFreq(1, 1, 1)
    d.closest_freq = abi.UpdateFreq(1, 1, 1)
    return d


class Workload:
    """A descriptor, its images (kept alive here) and how to enumerate its pixels."""

    def __init__(self, name, desc, images, mesh, note=""):
        self.name = name
        self.desc = desc
        self.images = images
        self._keep = abi.attach_images(desc, images)
        self.mesh = mesh  # ("simple", side) per image, or ("v2", dict(...))
        self.note = note

    def simple_pixels(self):
        """Every pixel of every SimpleSquareMesh image, image after image."""
        parts = []
        for i, (kind, side) in enumerate(self.mesh):
            assert kind == "simple"
            parts.append(abi.square_pixels(side, image=i))
        return np.concatenate(parts)


def c1(precision=abi.PREC_FP64, side=100):
    d = base_desc(precision)
    a = 0.5
    d.metric_id = abi.METRIC_KERR
    d.integrator_id = abi.INTEGRATOR_RK4
    d.horizon_eps = 0.01 / _kerr_rp(a)
    d.diag_flags = abi.DIAG_FOUR_COLOR_SCREEN | abi.DIAG_EQUATORIAL_PASSES
    d.value_diag = abi.DIAG_FOUR_COLOR_SCREEN
    im = abi.make_image((a,), r=1000.0, theta=80 * DEG, half_width=10.0)
    return Workload("C1 Kerr a=0.5 80deg 100^2 RK4", d, [im], [("simple", side)])


# IterationPixels of C2: chosen so that the run is the seed round plus exactly four
# refinement rounds.
C2_ITERATION_PIXELS = 800


def c2(precision=abi.PREC_FP64, iteration_pixels=None):
    d = base_desc(precision)
    a = 0.99
    d.metric_id = abi.METRIC_KERR
    d.integrator_id = abi.INTEGRATOR_RK4
    d.horizon_eps = 0.01 / _kerr_rp(a)
    d.diag_flags = abi.DIAG_FOUR_COLOR_SCREEN | abi.DIAG_CLOSEST_RADIUS
    d.value_diag = abi.DIAG_FOUR_COLOR_SCREEN
    im = abi.make_image((a,), r=1000.0, theta=60 * DEG, half_width=12.0)
    mesh = ("v2", dict(max_pixels=0, initial_pixels=128 * 128, max_subdivide=3,
                       iteration_pixels=iteration_pixels or C2_ITERATION_PIXELS, initial_sub_to_final=0))
    return Workload("C2 Kerr a=0.99 60deg V2 128^2 x3", d, [im], [mesh])


def c3_params(n_images=64):
    rng = MT19937_64(SEED)
    out = []
    for _ in range(n_images):
        a = rng.uniform(0.0, 0.998)
        inc = rng.uniform(5.0, 85.0)
        side = rng.choice((64, 128, 256, 512))
        w = rng.uniform(10.0, 15.0)
        out.append(dict(a=a, inclination_deg=inc, side=side, half_width=w))
    return out


def c3(precision=abi.PREC_MIXED, n_images=64):
    d = base_desc(precision)
    d.metric_id = abi.METRIC_KERR
    d.integrator_id = abi.INTEGRATOR_RK4
    # Each image is one FOORT run of its own: its Epsilon_Horizon is 0.01 / r_+(a).
    d.horizon_eps = 0.01 / _kerr_rp(0.5)
    d.diag_flags = abi.DIAG_FOUR_COLOR_SCREEN | abi.DIAG_EQUATORIAL_PASSES
    d.value_diag = abi.DIAG_FOUR_COLOR_SCREEN
    ims, mesh = [], []
    for p in c3_params(n_images):
        ims.append(abi.make_image((p["a"],), r=1000.0, theta=p["inclination_deg"] * DEG, half_width=p["half_width"],
                                  horizon_eps=0.01 / _kerr_rp(p["a"])))
        mesh.append(("simple", p["side"]))
    return Workload(f"C3 {n_images} Kerr images", d, ims, mesh)


def c4_alpha13():
    return MT19937_64(SEED + 4).uniform(-1.0, 1.0)


def c4(precision=abi.PREC_MIXED, side=1024):
    d = base_desc(precision)
    a = 0.9
    d.metric_id = abi.METRIC_JOHANNSEN
    d.integrator_id = abi.INTEGRATOR_VERLET
    d.verlet_tol = 0.001
    d.horizon_eps = 0.01 / _kerr_rp(a)
    d.diag_flags = abi.DIAG_EQUATORIAL_PASSES | abi.DIAG_CLOSEST_RADIUS
    d.value_diag = abi.DIAG_EQUATORIAL_PASSES
    im = abi.make_image((a, c4_alpha13(), 0.0, 0.0, 0.0), r=1000.0, theta=30 * DEG, half_width=10.0)
    return Workload(f"C4 Johannsen a=0.9 30deg {side}^2 Verlet", d, [im], [("simple", side)])


def c5(precision=abi.PREC_MIXED):
    d = base_desc(precision)
    a = 0.998
    d.metric_id = abi.METRIC_KERR
    d.integrator_id = abi.INTEGRATOR_RK4
    d.horizon_eps = 0.01 / _kerr_rp(a)
    d.diag_flags = abi.DIAG_FOUR_COLOR_SCREEN | abi.DIAG_EQUATORIAL_PASSES
    d.value_diag = abi.DIAG_FOUR_COLOR_SCREEN
    im = abi.make_image((a,), r=1000.0, theta=17 * DEG, half_width=10.0)
    # "Every active pixel each round": the reference reserves 5 * IterationPixels queue
    # slots (Mesh.cpp:1154), so the value is the largest count of level-5 pixels, 2048^2,
    # rather than an unbounded number.
    mesh = ("v2", dict(max_pixels=0, initial_pixels=129 * 129, max_subdivide=6,
                       iteration_pixels=(1 << 22), initial_sub_to_final=0))
    return Workload("C5 Kerr a=0.998 17deg V2 129^2 x6", d, [im], [mesh])


def johannsen_golden(test=True, precision=abi.PREC_FP64):
    """The two runs whose outputs ship with the reference (FOORT/Output/Test_*.dat from
    FOORT/Test.cfg, and debug_*.dat): Johannsen a=0.7, alpha13=2, log-r, 250^2."""
    d = abi.default_desc()
    d.precision = precision
    d.metric_id = abi.METRIC_JOHANNSEN
    d.rlog = 1
    d.term_flags = abi.TERM_HORIZON | abi.TERM_BOUNDARY_SPHERE | abi.TERM_TIMEOUT | abi.TERM_THETA_SINGULARITY
    d.diag_flags = abi.DIAG_FOUR_COLOR_SCREEN | abi.DIAG_EQUATORIAL_PASSES
    d.value_diag = abi.DIAG_EQUATORIAL_PASSES
    d.smallest_step = 1e-7
    d.theta_eps = 1e-5
    if test:
        d.integrator_id = abi.INTEGRATOR_VERLET
        d.verlet_tol = -1.0
        d.horizon_eps = 0.3
        d.timeout_max_steps = 10000
        d.equat_threshold = 0.01
        th, w = 0.087266462599716478846, 15.0
    else:
        d.integrator_id = abi.INTEGRATOR_RK4
        d.horizon_eps = 0.001
        d.timeout_max_steps = 1000000
        d.equat_threshold = 1e-4
        th, w = 1.5707963267948966192, 12.0
    im = abi.make_image((0.7, 2.0, 0.0, 0.0, 0.0), r=1000.0, theta=th, size=(w, w))
    return Workload("Test.cfg" if test else "debug", d, [im], [("simple", 250)])
