"""Analytic metric plugins of the mixed-precision kernel (CPU).

* In FP64 they must equal the reference's finite-difference Christoffel symbols
  (Metric.cpp:14-55, restated by the oracle) to the finite differences' own accuracy.
* In FP32 (tests/analytic_check.cpp, the same plugin code the kernel runs) the
  geodesic acceleration must keep FP32 accuracy from r_+ + 0.01 to 1000: no overflow
  (Johannsen's expanded numerators would reach r^15), no near-horizon cancellation, and
  for Rasheed-Larsen none on its ergosurface (H3 = 0) or, with near-extremal
  parameters, at small r.
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT

# Rasheed-Larsen: the "Lorenzo" and extremal "M1" parameter sets of the reference's
# Test.cfg, and its defaults (m, a, p, q)
RL_LORENZO = (0.3556562853309941, 0.2969060968239216, 3.057664971085168, 0.942335028914832)
RL_M1 = (0.0000292676523070559347272298622578, 0.0000292676523070559347272298622578,
         3.15470053516341633378322799917, 0.84529946483658456162619604143)
CASES = [(0, (0.99,), 0), (0, (0.7,), 1), (3, (0.9, -0.6, 0, 0, 0), 0), (3, (0.7, 2.0, 0, 0, 0), 1),
         (3, (0.8, 1.0, 0.5, 0.2, 0.1), 0), (1, (), 0), (2, RL_LORENZO, 0), (2, RL_LORENZO, 1), (2, RL_M1, 0),
         (2, (1.0, 0.5, 2.0, 2.0), 0), (4, (0.94, 13.0), 0), (4, (0.9, 5.0), 1), (4, (0.7, 1.0), 0)]


@pytest.mark.parametrize("metric,params,rlog", CASES)
def test_analytic_christoffel_equals_finite_differences(engine_lib, oracle_mod, metric, params, rlog):
    ol = oracle_mod.oracle_lib()
    p = np.zeros(6)
    p[:len(params)] = params
    rng = np.random.default_rng(1)
    worst = 0.0
    for _ in range(300):
        r = 10 ** rng.uniform(0.3, 3)
        th = rng.uniform(0.1, 3.0)
        x = np.array([0.0, np.log(r) if rlog else r, th, 0.3])
        ga, gb = np.zeros(64), np.zeros(64)
        assert engine_lib.foort_metric_christoffel(metric, p.ctypes.data, rlog, x.ctypes.data, ga.ctypes.data) == 0
        ol.oracle_christoffel(metric, p.ctypes.data, rlog, 1e-5, x.ctypes.data, gb.ctypes.data)
        worst = max(worst, np.abs(ga - gb).max() / np.abs(gb).max())
    # Manko-Novikov: the reference's formulas form their exponents' arguments as differences
    # of O(1) terms that cancel to O(1/x^3), ~1e-15 absolute in FP64; central differences at
    # h = 1e-5 turn that into ~3e-7 of the largest Christoffel symbol at r ~ 10^3
    assert worst < (1e-6 if metric == 4 else 1e-7), worst


def test_unknown_metric_has_no_analytic_plugin(engine_lib):
    p = np.array([0.94, 13.0, 0, 0, 0, 0.0])
    x = np.array([0.0, 10.0, 1.0, 0.0])
    g = np.zeros(64)
    assert engine_lib.foort_metric_christoffel(7, p.ctypes.data, 0, x.ctypes.data, g.ctypes.data) == -6


def test_fp32_acceleration_accuracy(tmp_path):
    exe = tmp_path / "analytic_check"
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-o", str(exe),
                    os.path.join(ROOT, "tests", "analytic_check.cpp")], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    for line in out.strip().splitlines():
        name, p50, p90, p99, mx = line.split()
        p50, p99, mx = float(p50), float(p99), float(mx)
        print(line)
        if name.startswith("manko_novikov"):
            # its derivatives of ratios that tend to constants far out (f = e^(2 psi) AA/BB)
            # lose digits in FP32 dual arithmetic where the generated plugins cancel
            # symbolically: a few times the other metrics' error
            assert p50 < 6e-7 and p99 < 1e-5 and mx < 5e-4, line
            continue
        # FP32 has 6e-8 unit roundoff; a few operations deep the acceleration keeps ~1e-7
        assert p50 < 3e-7 and p99 < 3e-6 and mx < 1e-4, line
        if name == "ff_sincos":
            # the mixed kernel's sin/cos: a few roundings, relative, also next to the poles
            assert mx < 5e-7, line


def test_generated_plugins_match_the_generator(tmp_path):
    """gen_christoffel.inc is what foort_gb300/gen/gen_christoffel.py prints: the
    generator's own checks (Rasheed-Larsen's H3 divides the numerators it removes; the
    quotient has the coefficients the constants code assumes) pass, and the file is
    up to date."""
    pytest.importorskip("sympy")
    out = tmp_path / "gen.inc"
    with open(out, "w") as f:
        subprocess.run([sys.executable, os.path.join(ROOT, "foort_gb300", "gen", "gen_christoffel.py")], check=True,
                       stdout=f, cwd=os.path.join(ROOT, "foort_gb300", "gen"), timeout=600)
    with open(os.path.join(ROOT, "foort_gb300", "csrc", "gen_christoffel.inc")) as f:
        committed = f.read()
    assert out.read_text() == committed


def _mn_gdd_mp(mp, a, a3, r, th):
    """Manko-Novikov g_dd (tt, tp, rr, hh, pp) from the reference's formulas
    (Metric.cpp:511-566), in mpmath arithmetic (test-only restatement)."""
    k = mp.sqrt(1 - a * a)
    al = (-1 + mp.sqrt(1 - a * a)) / a
    x, y = (r - 1) / k, mp.cos(th)
    s = mp.sin(th)
    R = mp.sqrt(x * x + y * y - 1)
    t = x * y / R
    P1, P2 = t, (3 * t * t - 1) / 2
    P3, P4 = (5 * t ** 3 - 3 * t) / 2, (35 * t ** 4 - 30 * t * t + 3) / 8
    aa = -al * mp.exp(2 * a3 * (1 - (x - y) * (1 / R + P1 / R ** 2 + P2 / R ** 3 + P3 / R ** 4)))
    bb = al * mp.exp(2 * a3 * (-1 + (x + y) * (1 / R - P1 / R ** 2 + P2 / R ** 3 - P3 / R ** 4)))
    AA = (x * x - 1) * (1 + aa * bb) ** 2 - (1 - y * y) * (bb - aa) ** 2
    BB = (x + 1 + (x - 1) * aa * bb) ** 2 + ((1 + y) * aa + (1 - y) * bb) ** 2
    CC = (x * x - 1) * (1 + aa * bb) * (bb - aa - y * (aa + bb)) + (1 - y * y) * (bb - aa) * (1 + aa * bb + x * (1 - aa * bb))
    psi = a3 * P3 / R ** 4
    gp = 2 * a3 * a3 * (P4 * P4 - P3 * P3) / R ** 8 + 2 * a3 * (-y + x * P1 / R - y * P2 / R ** 2 + x * P3 / R ** 3) / R
    f = mp.exp(2 * psi) * AA / BB
    e2g = mp.exp(2 * gp) * AA / ((x * x - y * y) * (1 - al * al) ** 2)
    om = 2 * k * mp.exp(-2 * psi) * CC / AA - 4 * k * al / (1 - al * al)
    rho2 = (r - 1) ** 2 - k * k * y * y
    de = (r - 1) ** 2 - k * k
    g22 = e2g * rho2 / f
    return [-f, om * f, g22 / de, g22, -f * om * om + de * s * s / f]


def _gdd_mp(mp, metric, q, r, th):
    """g_dd (tt, tp, rr, hh, pp) of Kerr (0), Rasheed-Larsen (2) and Johannsen (3) from the
    reference's formulas (Metric.cpp:131-159, :273-316, :409-440), in mpmath arithmetic;
    Manko-Novikov (4) by _mn_gdd_mp. Test-only restatements."""
    s, c = mp.sin(th), mp.cos(th)
    if metric == 4:
        return _mn_gdd_mp(mp, q[0], q[1], r, th)
    if metric == 0:
        a = q[0]
        sig = r * r + a * a * c * c
        de = r * r + a * a - 2 * r
        A = (r * r + a * a) ** 2 - de * a * a * s * s
        return [-(1 - 2 * r / sig), -2 * a * r * s * s / sig, sig / de, sig, A / sig * s * s]
    if metric == 3:
        a, a13, a22, a52, e3 = q[:5]
        A1, A2, A5 = 1 + a13 / r ** 3, 1 + a22 / r ** 2, 1 + a52 / r ** 2
        rho2 = r * r + a * a * c * c + e3 / r
        de = r * r + a * a - 2 * r
        den = (r * r + a * a) * A1 - a * a * A2 * s * s
        ra = (r * r + a * a) * A1
        return [-rho2 * (de - a * a * A2 * A2 * s * s) / den ** 2,
                -a * ((r * r + a * a) * A1 * A2 - de) * rho2 * s * s / den ** 2,
                rho2 / (de * A5), rho2, rho2 * s * s * (ra * ra - a * a * de * s * s) / den ** 2]
    # Rasheed-Larsen, parameters rescaled to M = 1 (Metric.cpp:244-252)
    m0, a0, p0, q0 = q[:4]
    sc = (p0 + q0) / 4
    m, a, p, qq = m0 / sc, a0 / sc, p0 / sc, q0 / sc
    de = r * r + a * a - 2 * r * m
    H3 = r * r - 2 * r * m + a * a * c * c
    Bp = mp.sqrt(p * qq) * a * s * s * (((p * qq + 4 * m * m) * r - m * (p - 2 * m) * (qq - 2 * m))
                                        / (2 * m * (p + qq) * H3))
    W = mp.sqrt((p * p - 4 * m * m) * (qq * qq - 4 * m * m))
    H1 = r * r + a * a * c * c + r * (p - 2 * m) + p / (p + qq) * ((p - 2 * m) * (qq - 2 * m) / 2) \
        - p / (2 * m * (p + qq)) * W * a * c
    H2 = r * r + a * a * c * c + r * (qq - 2 * m) + qq / (p + qq) * ((p - 2 * m) * (qq - 2 * m) / 2) \
        + qq / (2 * m * (p + qq)) * W * a * c
    S = mp.sqrt(H1 * H2)
    return [-H3 / S, -H3 * Bp / S, S / de, S, -H3 * Bp * Bp / S + S * de * s * s / H3]


NEAR_CASES = [(0, (0.99,)), (0, (0.5,)), (3, (0.9, -0.6, 0, 0, 0)), (3, (0.8, 1.0, 0.5, 0.2, 0.1)),
              (2, RL_LORENZO), (2, RL_M1), (4, (0.94, 13.0)), (4, (0.9, 5.0)), (4, (0.7, 1.0))]


@pytest.mark.parametrize("metric,params", NEAR_CASES)
def test_plugin_derivatives_near_the_horizon(engine_lib, metric, params):
    """The plugins' FP64 Christoffel symbols (foort_metric_christoffel; the mixed kernel's
    FP64 right-hand side uses the same code) against 50-digit central differences of the
    reference's formulas, from r_+ + 0.01 to r_+ + 1.5, where FP64 finite differences
    cannot resolve the derivatives."""
    mp = pytest.importorskip("mpmath").mp
    mp.dps = 50
    p = np.zeros(6)
    p[:len(params)] = params
    rp = engine_lib.foort_horizon_radius(metric, p.ctypes.data)
    qm = [mp.mpf(v) for v in p]
    rng = np.random.default_rng(3)
    worst = 0.0
    checked = 0
    for _ in range(40):
        r = rp + 10 ** rng.uniform(-2, np.log10(1.5))
        th = rng.uniform(0.2, 2.9)
        x = np.array([0.0, r, th, 0.0])
        g = np.zeros(64)
        assert engine_lib.foort_metric_christoffel(metric, p.ctypes.data, 0, x.ctypes.data, g.ctypes.data) == 0
        if not np.all(np.isfinite(g)):
            continue  # the metric itself leaves FP64's range there
        rm, tm = mp.mpf(r), mp.mpf(th)
        gd = _gdd_mp(mp, metric, qm, rm, tm)
        if not all(mp.mpf("1e-290") < abs(v) < mp.mpf("1e290") for v in gd if v != 0):
            continue
        h = mp.mpf("1e-20")
        d_r = [(u - v) / (2 * h) for u, v in zip(_gdd_mp(mp, metric, qm, rm + h, tm), _gdd_mp(mp, metric, qm, rm - h, tm))]
        d_t = [(u - v) / (2 * h) for u, v in zip(_gdd_mp(mp, metric, qm, rm, tm + h), _gdd_mp(mp, metric, qm, rm, tm - h))]
        # inverse of the (t, phi) block; Manko-Novikov's determinant is -Delta sin^2 exactly
        # (as g_tt g_phiphi - g_tphi^2 it cancels beyond even 50 digits where its
        # components are large)
        if metric == 4:
            det = -((rm - 1) ** 2 - (1 - qm[0] ** 2)) * mp.sin(tm) ** 2
        else:
            det = gd[0] * gd[4] - gd[1] * gd[1]
        gu = {"tt": float(gd[4] / det), "tp": float(-gd[1] / det), "pp": float(gd[0] / det),
              "rr": float(1 / gd[2]), "hh": float(1 / gd[3])}
        D = np.zeros((4, 4, 4))  # D[c][i][j] = d_c g_ij
        for cdir, dv in ((1, d_r), (2, d_t)):
            vt, vtp, vr, vh, vp = [float(v) for v in dv]
            D[cdir][0][0], D[cdir][0][3], D[cdir][3][0], D[cdir][1][1], D[cdir][2][2], D[cdir][3][3] = \
                vt, vtp, vtp, vr, vh, vp
        G = np.zeros((4, 4))
        G[0][0], G[0][3], G[3][0], G[3][3], G[1][1], G[2][2] = gu["tt"], gu["tp"], gu["tp"], gu["pp"], gu["rr"], gu["hh"]
        want = np.zeros(64)
        for mu in range(4):
            for nu in range(4):
                for rho in range(4):
                    want[16 * mu + 4 * nu + rho] = 0.5 * sum(
                        G[mu][sg] * (D[nu][rho][sg] + D[rho][nu][sg] - D[sg][nu][rho]) for sg in range(4))
        worst = max(worst, np.abs(g - want).max() / np.abs(want).max())
        checked += 1
    print(f"metric {metric} {params}: {checked} points, worst relative difference {worst:.2e}")
    assert checked >= 20, checked
    assert worst < 1e-10, worst


MN_RADIUS_CHECK = r"""
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include "analytic_metric.cuh"
using namespace foort;
// The first radius, scanning inward with r - r_+ shrinking by 0.99 per step, at which an
// exponent exceeds 8 on a 0.25-degree theta grid; r_+ if none does down to r_+ + 1e-9.
static double fine_radius(const MetricConst& M) {
    const double rp = 1.0 + M.q[3];
    for (double d = 1e4 - rp; d > 1e-9; d *= 0.99)
        if (!(mn_max_exponent(M, rp + d, 720) <= kMnMaxFp32Exponent)) return rp + d;
    return rp;
}
int main(int argc, char** argv) {
    for (int i = 1; i + 1 < argc; i += 2) {
        const double p[6] = {std::atof(argv[i]), std::atof(argv[i + 1]), 0, 0, 0, 0};
        const MetricConst M = make_metric_const(kMankoNovikov, p);
        std::printf("%s %s %.17g %.17g %.17g\n", argv[i], argv[i + 1], 1.0 + M.q[3],
                    mn_fp64_radius(M, kMnMaxFp32Exponent), fine_radius(M));
    }
}
"""


def test_manko_novikov_fp64_radius_covers_a_fine_scan(tmp_path):
    """The mixed kernel takes Manko-Novikov steps in FP64 inside the radius where one of
    the metric's exponents exceeds 8 (mn_fp64_radius: 1-degree theta grid, r - r_+
    shrinking by 0.8 per step, then bisection and a 10 % margin). A coarse scan could
    step over a narrow band where an exponent peaks; the radius must still enclose the
    first such radius that a 0.25-degree grid with 1 % radial steps finds."""
    src = tmp_path / "mn_radius.cpp"
    src.write_text(MN_RADIUS_CHECK)
    exe = tmp_path / "mn_radius"
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "foort_gb300", "csrc"),
                    "-o", str(exe), str(src)], check=True)
    rng = np.random.default_rng(5)
    sets = [(0.94, 13.0), (0.9, 5.0), (0.7, 1.0), (0.5, -3.0), (0.99, 20.0), (0.2, 0.5)]
    sets += [(float(rng.uniform(0.05, 0.99)), float(rng.uniform(-20.0, 20.0))) for _ in range(10)]
    args = [f"{v:.17g}" for s in sets for v in s]
    out = subprocess.run([str(exe)] + args, check=True, capture_output=True, text=True).stdout
    for line in out.strip().splitlines():
        a, a3, rp, coarse, fine = line.split()
        print(f"a={a} alpha3={a3}: r_+ {float(rp):.6f}, FP64 radius {float(coarse):.6f}, fine scan {float(fine):.6f}")
        assert float(coarse) >= float(fine), line
