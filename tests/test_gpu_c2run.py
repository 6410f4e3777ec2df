"""The engine's complete C2 run against the reference's own complete C2 run (-m gpu).

tests/golden/c2_run.npz holds the reference's run of the C2 workload (Kerr a = 0.99 at
60 deg, SquareSubdivisionMeshV2 from a 128^2 seed, MaxSubdivide 3, IterationPixels 800;
26,547 geodesics in five rounds): the pixels in the order the run handed them out, and
the quadrant and closest radius ("%f") its output files give each. The engine runs the
same workload through the host mesh and the C ABI, round by round, with each kernel.

Each round's pixels depend on the quadrants of all earlier rounds, so the two runs
hand out the same pixels exactly as long as every quadrant agreed. The test asserts:
* the first line of the output files is the reference's;
* the pixel sequences are identical up to the first pixel at which they differ, and a
  quadrant that disagrees comes before that point (a sequence that changes without
  one is a mesh error);
* the quadrants of the common part agree on >= 99.9 % of pixels, and every
  disagreement lies on a decision boundary (parity.explain_mismatches) or on a ray
  whose end point the FP64 algorithm itself does not determine: the reference's
  finite-difference FP64 kernel and the all-FP64 analytic kernel disagree on it by more
  than 1e-4 (parity.fp64_ill_posed; the screen row through the rotation axis), at most
  one such pixel per 10,000;
* the closest radii agree with the reference's "%f" text (6 decimals: 3e-8 relative
  at the median radius): FP64 kernel median < 1e-7 and p99 < 1e-6 relative, the level
  at which the reference's own -Ofast and strict builds differ on strongly lensed rays;
  mixed kernel median < 1e-6 and p99 < 1e-5.
"""
import os

import numpy as np
import pytest

import parity
from conftest import GOLDEN
from foort_gb300 import abi, workloads

pytestmark = pytest.mark.gpu


def reference_run():
    f = np.load(os.path.join(GOLDEN, "c2_run.npz"))
    return {k: f[k] for k in f.files}


def engine_run(precision):
    import foort_gb300
    wl = workloads.c2(precision)
    mesh = foort_gb300.Mesh.from_spec(wl.mesh[0], wl.desc.diag_flags, wl.desc.value_diag)
    first = mesh.first_line_info(wl.desc)
    pxs, ress = [], []
    with foort_gb300.Engine(wl.desc) as e:
        while not mesh.finished():
            px = mesh.pixels()
            res = e.integrate(px)
            mesh.set_results(res)
            mesh.end_round()
            pxs.append(px)
            ress.append(res)
    mesh.close()
    return wl, first, np.concatenate(pxs), np.concatenate(ress), len(pxs)


@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_MIXED], ids=["fp64", "mixed"])
def test_c2_run_matches_the_reference_run(engine_lib, oracle_mod, precision):
    ref = reference_run()
    wl, first, px, res, rounds = engine_run(precision)
    assert first == str(ref["header"])
    n = min(len(px), len(ref["row"]))
    same_px = (px["row"][:n] == ref["row"][:n]) & (px["col"][:n] == ref["col"][:n])
    split = n if same_px.all() else int(np.argmin(same_px))
    quad_mism = res["quadrant"][:split] != ref["quadrant"][:split]
    print(f"precision {precision}: {len(px)} geodesics in {rounds} rounds (reference {len(ref['row'])} in "
          f"{int(ref['rounds'])}); identical sequence for {split} pixels; {int(quad_mism.sum())} quadrants differ")
    if split < len(ref["row"]) or len(px) != len(ref["row"]):
        assert quad_mism.any(), "the pixel sequence changed without a differing quadrant"
    else:
        assert rounds == int(ref["rounds"])
    assert 1.0 - quad_mism.mean() >= parity.MIN_DISCRETE_AGREEMENT
    if quad_mism.any():
        wl.desc.precision = abi.PREC_FP64
        unexplained, ill = parity.explain_or_ill_posed(oracle_mod, wl.desc, px[:split], res[:split], quad_mism)
        print(f"{len(ill)} disagreement(s) where the two FP64 kernels disagree by more than "
              f"{parity.FP64_ILL_POSED:g}: {px[:split][ill]}")
        assert len(unexplained) == 0, px[:split][unexplained]
        assert len(ill) <= max(1, split // 10000)

    # closest radius, on the common part where the quadrants agree
    keep = ~quad_mism
    got = res["closest_r"][:split][keep]
    want = ref["closest_r"][:split][keep]
    d = np.abs(got - want)
    rel = d / np.maximum(want, 1e-300)
    within = d <= 5e-7 + 1e-9 * want
    print(f"closest radius: median |d| {np.median(d):.2e}, median rel {np.median(rel):.2e}, p99 rel "
          f"{np.quantile(rel, 0.99):.2e}, max rel {rel.max():.2e}, within print rounding {within.mean():.5f}")
    assert np.array_equal(got == 0.0, want == 0.0)  # Horizon sets it to 0 in both
    if precision == abi.PREC_FP64:
        assert np.median(rel) < 1e-7 and np.quantile(rel, 0.99) < 1e-6
    else:
        assert np.median(rel) < 1e-6 and np.quantile(rel, 0.99) < 1e-5
