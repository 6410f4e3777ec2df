"""Accuracy measures: discrete agreement, decision-boundary explanation, endpoint error.

Parity rules (floating-point path, stated here and asserted by the tests):

* discrete outputs -- termination code, FourColorScreen quadrant, EquatorialPasses count
  -- must agree on at least 99.9 % of pixels (MIN_DISCRETE_AGREEMENT), and every pixel
  that disagrees must lie on a decision boundary: shifting its unit screen point by at
  most 1e-4 of the screen width (BOUNDARY_DELTA = 1e-6 first; 1e-4 is 5 % of a pixel on
  a 509-pixel grid) in one of four directions makes the oracle produce the other side's
  outcome;
* the endpoint (r, theta, phi) is compared with the relative error
      e = max(|dr| / |r|, |dtheta| / pi, |dphi| / max(|phi|, pi))
  on pixels whose discrete outputs and step counts agree (r is exp(x1) in log-r mode).
"""
import numpy as np

MIN_DISCRETE_AGREEMENT = 0.999
BOUNDARY_DELTA = 1e-6
DISCRETE = ("term", "quadrant", "equat_passes")


def outcome(res):
    return np.stack([res["term"], res["quadrant"], res["equat_passes"]], axis=1)


def discrete_mismatch(a, b):
    return np.any(outcome(a) != outcome(b), axis=1)


def endpoint_rel_err(a, b, rlog=False):
    """Relative endpoint error of a against b (per pixel). Pixels whose endpoint is not
    finite on both sides (a NaN state, flagged FOORT_ERR_NONFINITE) are left out."""
    ok = np.all(np.isfinite(a["pos"][:, 1:]), axis=1) & np.all(np.isfinite(b["pos"][:, 1:]), axis=1)
    a, b = a[ok], b[ok]
    ra, rb = a["pos"][:, 1], b["pos"][:, 1]
    if rlog:
        ra, rb = np.exp(ra), np.exp(rb)
    er = np.abs(ra - rb) / np.abs(rb)
    et = np.abs(a["pos"][:, 2] - b["pos"][:, 2]) / np.pi
    ep = np.abs(a["pos"][:, 3] - b["pos"][:, 3]) / np.maximum(np.abs(b["pos"][:, 3]), np.pi)
    return np.maximum(er, np.maximum(et, ep))


def explain_mismatches(oracle, desc, px, got, mask, deltas=(BOUNDARY_DELTA, 1e-5, 1e-4), report=None):
    """(Tests only: `oracle` is the CPU checker module.)
    For each pixel in `mask`, check that the oracle reaches `got`'s outcome after a
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


def summarize(err):
    if len(err) == 0:
        return {"n": 0}
    return {"n": int(len(err)), "median": float(np.median(err)), "p90": float(np.quantile(err, 0.9)),
            "p99": float(np.quantile(err, 0.99)), "max": float(np.max(err))}
