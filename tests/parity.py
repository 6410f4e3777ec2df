"""Parity helpers of the GPU tests: the measures of foort_gb300.accuracy, and the
decision-boundary check that explains a discrete disagreement with the CPU oracle."""
import numpy as np

from foort_gb300.accuracy import (BOUNDARY_DELTA, DISCRETE, MIN_DISCRETE_AGREEMENT,  # noqa: F401
                                  discrete_mismatch, endpoint_rel_err, outcome, summarize)


def explain_mismatches(oracle, desc, px, got, mask, deltas=(BOUNDARY_DELTA, 1e-5, 1e-4), report=None):
    """For each pixel in `mask`, check that the oracle reaches `got`'s outcome after a
    shift of the unit screen point by +-delta in row or column, trying the deltas in
    turn (1e-4 of the screen is 5 % of a pixel on a 509-pixel grid). Returns the indices
    of pixels NOT explained that way; `report` (a dict) receives the delta each
    explained pixel needed."""
    idx = np.nonzero(mask)[0]
    if len(idx) == 0:
        return idx
    want = outcome(got[idx])
    explained = np.zeros(len(idx), dtype=bool)
    for delta in deltas:
        todo = ~explained
        if not todo.any():
            break
        sub = px[idx[todo]]
        hit = np.zeros(int(todo.sum()), dtype=bool)
        for off in ((delta, 0.0), (-delta, 0.0), (0.0, delta), (0.0, -delta)):
            r = oracle.integrate(desc, sub, offset=off)
            hit |= np.all(outcome(r) == want[todo], axis=1)
        if report is not None:
            for i in idx[todo][hit]:
                report[int(i)] = delta
        explained[np.nonzero(todo)[0][hit]] = True
    return idx[~explained]


# A pixel whose end point the FP64 algorithm itself does not determine: the reference's
# finite-difference kernel (FOORT_PREC_FP64) and the all-FP64 analytic kernel
# (FOORT_PREC_FP64_ANALYTIC), two FP64 integrations of the same geodesic equation,
# disagree on it by more than this relative endpoint error.
FP64_ILL_POSED = 1e-4


def fp64_ill_posed(desc, px):
    """True for each pixel whose FP64 end point is not determined to FP64_ILL_POSED: the
    two FP64 kernels disagree on its end point by more than that, or on its outcome. Such
    rays pass over a pole of the coordinates (the screen row through the rotation axis)
    or skim the photon orbit; whichever side of a decision they fall on depends on
    rounding, in the reference's own arithmetic as in any other."""
    import foort_gb300
    from foort_gb300 import abi, accuracy
    px = np.ascontiguousarray(px, dtype=abi.PIXEL_DTYPE)
    if len(px) == 0:
        return np.zeros(0, dtype=bool)
    keep = desc.precision
    out = {}
    try:
        for prec in (abi.PREC_FP64, abi.PREC_FP64_ANALYTIC):
            desc.precision = prec
            with foort_gb300.Engine(desc) as e:
                out[prec] = e.integrate(px)
    finally:
        desc.precision = keep
    err = accuracy.endpoint_err_all(out[abi.PREC_FP64], out[abi.PREC_FP64_ANALYTIC], rlog=bool(desc.rlog))
    return err > FP64_ILL_POSED


def explain_or_ill_posed(oracle, desc, px, got, mask, report=None):
    """explain_mismatches, and for what it leaves, fp64_ill_posed on the GPU. Returns
    (unexplained indices, indices explained as FP64-ill-posed)."""
    rest = explain_mismatches(oracle, desc, px, got, mask, report=report)
    if len(rest) == 0:
        return rest, rest
    ill = fp64_ill_posed(desc, px[rest])
    return rest[~ill], rest[ill]
