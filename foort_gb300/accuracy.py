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
  on pixels whose discrete outputs agree (r is exp(x1) in log-r mode).

Conditioning. Rays that skim the photon orbit amplify any perturbation: a pixel's
condition number kappa is the endpoint change e per unit shift of its unit screen point
(condition_numbers: shifts of DELTA_KAPPA = 1e-6 along the row and the column, the larger
of the two; infinite where the shift changes the discrete outcome). An error e on a pixel
of condition kappa is what a shift of the screen point by e / kappa would cause: that
"backward error" is the accuracy measure that does not depend on the pixel's chaos.
Well-conditioned pixels (kappa <= KAPPA_WELL) are reported on their own.

The decision-boundary check itself runs the CPU oracle and lives with the tests
(tests/parity.py).
"""
import numpy as np

MIN_DISCRETE_AGREEMENT = 0.999
BOUNDARY_DELTA = 1e-6
DELTA_KAPPA = 1e-6
KAPPA_WELL = 10.0
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


def summarize(err):
    if len(err) == 0:
        return {"n": 0}
    return {"n": int(len(err)), "median": float(np.median(err)), "p90": float(np.quantile(err, 0.9)),
            "p99": float(np.quantile(err, 0.99)), "max": float(np.max(err))}


def endpoint_err_all(a, b, rlog=False):
    """Per-pixel relative endpoint error of a against b for every pixel (inf where an
    endpoint is not finite or the discrete outcomes differ)."""
    ra, rb = a["pos"][:, 1], b["pos"][:, 1]
    if rlog:
        ra, rb = np.exp(ra), np.exp(rb)
    with np.errstate(invalid="ignore", divide="ignore", over="ignore"):
        er = np.abs(ra - rb) / np.abs(rb)
        et = np.abs(a["pos"][:, 2] - b["pos"][:, 2]) / np.pi
        ep = np.abs(a["pos"][:, 3] - b["pos"][:, 3]) / np.maximum(np.abs(b["pos"][:, 3]), np.pi)
        e = np.maximum(er, np.maximum(et, ep))
    e[~np.isfinite(e)] = np.inf
    e[discrete_mismatch(a, b)] = np.inf
    return e


def shift_refinement(grid, delta=DELTA_KAPPA):
    """The refinement K of a pixel grid of size R such that one step of the refined grid
    ((R - 1) K + 1 points) is about delta of the unit screen; and that step."""
    K = max(1, int(round(1.0 / (delta * (int(grid) - 1)))))
    return K, 1.0 / (K * (int(grid) - 1))


def shifted_pixels(px, K, axis):
    """The pixels moved by one step of the K-fold refined grid along the row (axis 0) or
    column (axis 1): pixel (i, j) of grid R becomes (K i +- 1, K j) of grid (R - 1) K + 1,
    the sign chosen to stay on the screen. Same unit screen point up to that step."""
    q = px.copy()
    g = (px["grid"].astype(np.int64) - 1) * K + 1
    row = px["row"].astype(np.int64) * K
    col = px["col"].astype(np.int64) * K
    if axis == 0:
        row = np.where(row + 1 <= g - 1, row + 1, row - 1)
    else:
        col = np.where(col + 1 <= g - 1, col + 1, col - 1)
    q["row"], q["col"], q["grid"] = row, col, g
    return q


def condition_numbers(base, shifted, step, rlog=False):
    """kappa per pixel from the results at the pixels (base) and at the shifted pixels
    (a list of result arrays, one per shift of `step` of the unit screen)."""
    k = np.zeros(len(base))
    for r in shifted:
        k = np.maximum(k, endpoint_err_all(r, base, rlog=rlog) / step)
    return k


def error_report(err, kappa=None, kappa_well=KAPPA_WELL):
    """Summary of per-pixel errors: all pixels (discrete mismatches as inf), the
    well-conditioned class and the backward error err / kappa where kappa is given."""
    def summ(e):
        e = np.asarray(e, dtype=float)
        if len(e) == 0:
            return {"n": 0}
        fin = np.isfinite(e)
        out = {"n": int(len(e)), "median": float(np.median(e)), "p90": float(np.quantile(e, 0.9)),
               "p99": float(np.quantile(e, 0.99)), "max": float(np.max(e)),
               "frac_le_1e-6": float(np.mean(e <= 1e-6)), "mismatched_or_nonfinite": int((~fin).sum())}
        return out
    rep = {"all": summ(err)}
    if kappa is not None:
        well = kappa <= kappa_well
        rep["kappa_well"] = kappa_well
        rep["well_conditioned"] = summ(err[well])
        rep["ill_conditioned_count"] = int((~well).sum())
        fin = np.isfinite(kappa) & np.isfinite(err) & (kappa > 0)
        rep["backward_error"] = summ(err[fin] / kappa[fin])
        rep["kappa_quantiles"] = {q: float(np.quantile(kappa[np.isfinite(kappa)], float(q)))
                                  for q in ("0.5", "0.9", "0.99")} if np.isfinite(kappa).any() else {}
    return rep

