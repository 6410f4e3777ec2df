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
