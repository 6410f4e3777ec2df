"""Generate analytic metric derivatives for the mixed-precision kernel.

For a stationary, axisymmetric metric the geodesic acceleration needs only
    d_r g_ij, d_theta g_ij  (i, j in {tt, tphi, rr, thth, phiphi})  and  g^ij,
combined in Lagrangian form (kernel_mixed.cuh). The reference obtains the derivatives
by central finite differences (Metric.cpp:14-32), which FP32 cannot resolve; here they
are differentiated exactly with sympy from the reference's own g_dd formulas
(Metric.cpp:131-159 Kerr, :218-222 flat, :273-316 Rasheed-Larsen, :409-440 Johannsen),
with g^ij taken from the reference's getMetric_uu formulas.

Numerical conditioning: every metric here has Delta = (r - r_+)(r - r_-) (Kerr,
Johannsen: r^2 - 2r + a^2; Rasheed-Larsen: r^2 - 2mr + a^2). The generated code
receives dp = r - r_+ and dm = r - r_-, computed by the kernel from its compensated
(float-float) radius, and uses Delta = dp * dm, so the near-horizon cancellation of
r^2 - 2r + a^2 never happens in FP32. Numerators are expanded and collected in r so
that no large terms cancel at r ~ 10^3.

Rasheed-Larsen (Metric.cpp:273-362) is rewritten before it is differentiated. Its
g_phiphi = -H3 Bp^2 / S + S Delta sin^2 / H3 and its g^tt both divide by H3, which
vanishes on the ergosurface, and the two terms of each cancel there. The numerator
H1 H2 Delta - (H3 Bp / sin^2)^2 sin^2 is divisible by H3 exactly (rl_quotient() checks
it), so with the quotient polynomial Q(r, cos):
    g_phiphi = sin^2 Q / S,  g^tt = -Q / (S Delta),  g_tphi = -sin^2 (k1 r - k2) / S,
    g^tphi = -(k1 r - k2) / (S Delta),  S = sqrt(H1 H2),
and H3 remains only in numerators. S stays a symbol: d S = d(H1 H2) / (2 S), and even
powers of S in numerators become powers of H1 H2. The host computes the constants
(a^2, m, the coefficients of H1, H2, k1 r - k2 and Q) from the metric's parameters with
the code printed by main().

Usage: python gen_christoffel.py > ../csrc/gen_christoffel.inc
"""
import sympy as sp

r, th, s, c, dp, dm = sp.symbols("r theta s c dp dm", real=True)
COMP = ["tt", "tp", "rr", "hh", "pp"]
# Every denominator is applied as a product of reciprocals of its factors, rcp(x) =
# correctly rounded 1/x (one per distinct factor after common-subexpression
# elimination) instead of an IEEE division per expression: fewer long dependency
# chains, and every rounding stays unbiased.
rcp = sp.Function("rcp")


def with_reciprocals(num, den):
    out = num
    for base, k in sp.factor(den).as_powers_dict().items():
        if base.is_number:
            out = out / base**k
        else:
            out = out * rcp(base)**k
    return out


def kerr():
    a = sp.Symbol("q0")
    sig = r**2 + a**2 * sp.cos(th)**2
    dl = r**2 + a**2 - 2 * r
    A = (r**2 + a**2)**2 - dl * a**2 * sp.sin(th)**2
    gdd = {"tt": -(1 - 2 * r / sig), "tp": -2 * a * r * sp.sin(th)**2 / sig, "rr": sig / dl, "hh": sig,
           "pp": A / sig * sp.sin(th)**2}
    guu = {"tt": -A / (sig * dl), "tp": -2 * a * r / (sig * dl), "rr": dl / sig, "hh": 1 / sig,
           "pp": (dl - a**2 * sp.sin(th)**2) / (sig * dl * sp.sin(th)**2)}
    return gdd, guu, dl


def johannsen():
    a, a13, a22, a52, e3 = sp.symbols("q0 q1 q2 q3 q4")
    S, C = sp.sin(th), sp.cos(th)
    A1 = 1 + a13 / r**3
    A2 = 1 + a22 / r**2
    A5 = 1 + a52 / r**2
    rho2 = r**2 + a**2 * C**2 + e3 / r
    dl = r**2 + a**2 - 2 * r
    den = (r**2 + a**2) * A1 - a**2 * A2 * S**2
    gdd = {"tt": -rho2 * (dl - a**2 * A2**2 * S**2) / den**2,
           "rr": rho2 / (dl * A5), "hh": rho2,
           "pp": rho2 * S**2 * (((r**2 + a**2) * A1)**2 - a**2 * dl * S**2) / den**2,
           "tp": -a * ((r**2 + a**2) * A1 * A2 - dl) * rho2 * S**2 / den**2}
    guu = {"tt": (-((r**2 + a**2) * A1)**2 + a**2 * dl * S**2) / (dl * rho2),
           "rr": dl * A5 / rho2, "hh": 1 / rho2,
           "pp": (-a**2 * A2**2 * S**2 + dl) / (dl * rho2 * S**2),
           "tp": -a * (A2 * A1 * (r**2 + a**2) - dl) / (dl * rho2)}
    return gdd, guu, dl


def flat():
    S = sp.sin(th)
    gdd = {"tt": sp.Integer(-1), "tp": sp.Integer(0), "rr": sp.Integer(1), "hh": r**2, "pp": r**2 * S**2}
    guu = {"tt": sp.Integer(-1), "tp": sp.Integer(0), "rr": sp.Integer(1), "hh": 1 / r**2, "pp": 1 / (r**2 * S**2)}
    return gdd, guu, None


S_ = sp.Symbol("S", positive=True)  # sqrt(H1 H2) of Rasheed-Larsen
# 1 - cos(theta) and 1 + cos(theta), kept as symbols (d/dtheta: +sin, -sin) and formed
# without cancellation near the poles (sin^2 / (1 + cos) where cos > 0)
W1, W2 = sp.symbols("w1 w2", positive=True)


def rl_params():
    """Rasheed-Larsen's parameters after the reference's rescaling to M = 1
    (Metric.cpp:244-252): m, a, p, q."""
    return sp.symbols("m a p qq", positive=True)


def rl_quotient():
    """Q(r, cos) = (H1 H2 Delta - K^2 sin^2 (K1 r - K2)^2 / K3^2) / H3 in the reference's
    parameters, with K = sqrt(p q) a, K1 = p q + 4 m^2, K2 = m (p - 2m)(q - 2m),
    K3 = 2 m (p + q) (Metric.cpp:285-296). Returns {(i, j): coefficient of r^i cos^j}."""
    m, a, p, q = rl_params()
    x = sp.Symbol("x")  # cos(theta)
    W = sp.Symbol("W", positive=True)
    K1, K2, K3 = p * q + 4 * m**2, m * (p - 2 * m) * (q - 2 * m), 2 * m * (p + q)
    dl = r**2 + a**2 - 2 * r * m
    H3 = r**2 - 2 * r * m + a**2 * x**2
    H1 = r**2 + a**2 * x**2 + r * (p - 2 * m) + p / (p + q) * ((p - 2 * m) * (q - 2 * m) / 2) \
        - p / (2 * m * (p + q)) * W * a * x
    H2 = r**2 + a**2 * x**2 + r * (q - 2 * m) + q / (p + q) * ((p - 2 * m) * (q - 2 * m) / 2) \
        + q / (2 * m * (p + q)) * W * a * x
    num = sp.expand(H1 * H2 * dl - p * q * a**2 * (1 - x**2) * (K1 * r - K2)**2 / K3**2)
    num = sp.expand(num.subs(W**2, (p**2 - 4 * m**2) * (q**2 - 4 * m**2)))
    quo, rem = sp.div(sp.Poly(num, r, x), sp.Poly(sp.expand(H3), r, x))
    assert sp.simplify(rem.as_expr()) == 0, "H3 does not divide the numerator"
    return {mon: sp.simplify(cf) for mon, cf in zip(quo.monoms(), quo.coeffs())}, W


# Rasheed-Larsen constant slots: q0 m, q1 a^2,
# q2..q4: H1 = r^2 + a^2 c^2 + q2 r + q3 + q4 (1 - c), q3 = beta1 - gamma1,
# q5..q7: H2 = r^2 + a^2 c^2 + q5 r + q6 + q7 (1 + c), q6 = beta2 - gamma2,
# q8 q9: k1 r - k2, q10..: the coefficients of Q other than r^4 (1), r^2 c^2 (a^2),
# r c^2 (-2 a^2 m) and c^2 (a^4). H1 = ... + beta1 - gamma1 c and H2 = ... + beta2 +
# gamma2 c in the reference; written with 1 -+ c, the near-equal beta and gamma of
# near-extremal parameter sets (m = a, as in the reference's Test.cfg) do not cancel
# in FP32 where r is small.
RL_Q_SLOTS = [(3, 0), (2, 1), (2, 0), (1, 1), (1, 0), (0, 1), (0, 0)]
RL_NQ = 10 + len(RL_Q_SLOTS)


def rasheed_larsen():
    qs = sp.symbols(" ".join(f"q{i}" for i in range(RL_NQ)))
    m, a2 = qs[0], qs[1]
    S, C = sp.sin(th), sp.cos(th)
    dl = r**2 - 2 * m * r + a2
    H3 = r**2 - 2 * m * r + a2 * C**2
    H1 = r**2 + a2 * C**2 + qs[2] * r + qs[3] + qs[4] * W1
    H2 = r**2 + a2 * C**2 + qs[5] * r + qs[6] + qs[7] * W2
    kk = qs[8] * r - qs[9]
    Q = r**4 + a2 * r**2 * C**2 - 2 * a2 * m * r * C**2 + a2**2 * C**2
    for k, (i, j) in enumerate(RL_Q_SLOTS):
        Q += qs[10 + k] * r**i * C**j
    gdd = {"tt": -H3 / S_, "tp": -S**2 * kk / S_, "rr": S_ / dl, "hh": S_, "pp": S**2 * Q / S_}
    guu = {"tt": -Q / (S_ * dl), "tp": -kk / (S_ * dl), "rr": dl / S_, "hh": 1 / S_,
           "pp": H3 / (S_ * dl * S**2)}
    return gdd, guu, dl, H1 * H2


def rl_constants_code():
    """Host C++ (double) for Rasheed-Larsen's constant slots from m, a, p, qq."""
    m, a, p, q = rl_params()
    coeffs, W = rl_quotient()
    K = sp.sqrt(p * q) * a
    K1, K2, K3 = p * q + 4 * m**2, m * (p - 2 * m) * (q - 2 * m), 2 * m * (p + q)
    beta1, gamma1 = p / (p + q) * ((p - 2 * m) * (q - 2 * m) / 2), p / (2 * m * (p + q)) * W * a
    beta2, gamma2 = q / (p + q) * ((p - 2 * m) * (q - 2 * m) / 2), q / (2 * m * (p + q)) * W * a
    vals = [m, a**2, p - 2 * m, beta1 - gamma1, gamma1, q - 2 * m, beta2 - gamma2, gamma2, K * K1 / K3, K * K2 / K3]
    fixed = {(4, 0): 1, (2, 2): a**2, (1, 2): -2 * a**2 * m, (0, 2): a**4}
    for mon, cf in coeffs.items():
        if mon in fixed:
            assert sp.simplify(cf - fixed[mon]) == 0, mon
        else:
            assert mon in RL_Q_SLOTS, mon
    Wsq = sp.sqrt((p**2 - 4 * m**2) * (q**2 - 4 * m**2))
    for mon in RL_Q_SLOTS:
        vals.append(coeffs.get(mon, sp.Integer(0)))
    lines = [f"    out[{i}] = {sp.ccode(sp.sympify(v).subs(W, Wsq).subs(sp.sqrt((p - 2 * m) * (q - 2 * m)) * sp.sqrt(p + 2 * m) * sp.sqrt(q + 2 * m), Wsq))};"
             for i, v in enumerate(vals)]
    return lines


def to_sc(e):
    return e.subs({sp.sin(th): s, sp.cos(th): c})


def reduce_s(num, P):
    """Even powers of S = sqrt(P) in a numerator as powers of P."""
    if P is None or not num.has(S_):
        return num
    pn = sp.Poly(sp.expand(num), S_)
    P = to_sc(P)
    return sum(cf * P**(k // 2) * S_**(k % 2) for (k,), cf in zip(pn.monoms(), pn.coeffs()))


def condition(e, dl, P=None):
    """Put e over a common denominator, expand the numerator as a polynomial in r (so
    that no leading powers of r cancel numerically) and write Delta as dp * dm."""
    e = sp.together(to_sc(e))
    num, den = sp.fraction(e)
    num = sp.expand(reduce_s(num, P))
    # use s^2 + c^2 = 1 to remove c^2 from the numerator where possible
    num = sp.expand(num.subs(c**2, 1 - s**2))
    den = sp.factor(den)
    if dl is not None:
        dls = sp.expand(to_sc(dl))
        den = den.subs(dls, dp * dm)
        den = sp.factor(den).subs(sp.expand(dls), dp * dm)
        # powers of Delta inside the denominator
        q, rem = sp.div(sp.Poly(den, r), sp.Poly(dls, r)) if den.has(r) else (None, None)
        if q is not None and rem.is_zero:
            k = 0
            dd = den
            while True:
                qq, rr = sp.div(sp.Poly(dd, r), sp.Poly(dls, r))
                if not rr.is_zero:
                    break
                dd = qq.as_expr()
                k += 1
            den = dd * (dp * dm)**k
    return with_reciprocals(sp.collect(num, r), den)


u = sp.Symbol("u", positive=True)


def condition_inv(e, dl):
    """Like condition(), in the inverse radius u = 1/r: e = r^k P(u) / Q(u) with P and Q
    polynomials whose terms are O(1) for every r >= r_+, so that FP32 neither overflows
    (Johannsen's expanded numerators reach r^15) nor cancels large terms. A factor
    Delta / r^2 = 1 - 2u + a^2 u^2 of Q is written dp * dm * u^2."""
    e = sp.together(to_sc(e).subs(r, 1 / u))
    num, den = sp.fraction(e)
    num = sp.expand(sp.expand(num).subs(c**2, 1 - s**2))
    den = sp.expand(den)
    # pull the powers of u out of numerator and denominator
    pn = sp.Poly(num, u)
    pd = sp.Poly(den, u)
    kn = min(m[0] for m in pn.monoms())
    kd = min(m[0] for m in pd.monoms())
    num = sp.expand(num / u**kn)
    den = sp.expand(den / u**kd)
    k = kn - kd  # e = u^k * num / den
    dfac = 1
    if dl is not None:
        dlu = sp.expand(to_sc(dl).subs(r, 1 / u) * u**2)  # Delta / r^2 as a polynomial in u
        pdl = sp.Poly(dlu, u)
        while True:
            q, rem = sp.div(sp.Poly(den, u), pdl)
            if not rem.is_zero:
                break
            den = q.as_expr()
            dfac = dfac * (dp * dm * u**2)
    num = sp.horner(sp.collect(num, u), u) if num.has(u) else num
    den = sp.horner(sp.collect(sp.expand(den), u), u) if sp.expand(den).has(u) else den
    return with_reciprocals(u**k * num, den * dfac)


def deriv(e, x, P):
    """d e / d x, with S = sqrt(P) a symbol: d S = d P / (2 S); and w1 = 1 - cos,
    w2 = 1 + cos symbols: d w1 / d theta = sin = -d w2 / d theta."""
    d = sp.diff(e, x)
    if P is not None:
        d += sp.diff(e, S_) * deriv(P, x, None) / (2 * S_)
    if x == th:
        d += (sp.diff(e, W1) - sp.diff(e, W2)) * sp.sin(th)
    return d


def emit(name, gdd, guu, dl, inv=False, P=None):
    if inv:
        assert P is None
        cond = condition_inv
    else:
        def cond(e, dl):
            return condition(e, dl, P)
    exprs = []
    names = []
    for k in COMP:
        exprs.append(cond(deriv(gdd[k], r, P), dl))
        names.append(f"dr.{k}")
    for k in COMP:
        exprs.append(cond(deriv(gdd[k], th, P), dl))
        names.append(f"dh.{k}")
    for k in COMP:
        exprs.append(cond(guu[k], dl))
        names.append(f"gu.{k}")
    exprs.append(cond(gdd["rr"], dl))
    names.append("grr")
    repl, red = sp.cse(exprs, symbols=sp.numbered_symbols("t"), optimizations="basic")
    lines = ["const T u = rcp(r);"] if inv else []
    if P is not None:
        lines.append("const T w1 = (c > T(0)) ? s * s * rcp(T(1) + c) : T(1) - c;")
        lines.append("const T w2 = (c < T(0)) ? s * s * rcp(T(1) - c) : T(1) + c;")
        lines.append(f"const T S = sqrt({ccode(to_sc(P))});")
    # common subexpressions that are powers of u: their negative powers are powers of r
    upow = {sym: int(e.exp) for sym, e in repl if isinstance(e, sp.Pow) and e.base == u and e.exp.is_Integer}
    upow.update({sym: 1 for sym, e in repl if e == u})
    for sym, e in repl:
        lines.append(f"const T {sym} = {ccode(e, upow)};")
    for n, e in zip(names, red):
        lines.append(f"{n} = {ccode(e, upow)};")
    return "\n".join(lines)


def ccode(e, upow=None):
    """C++ for e with every constant and operation in the template type T: integer powers
    become products, negative powers of u = 1/r powers of r, other negative powers
    divisions."""
    r_sym = sp.Symbol("r")
    upow = dict(upow or {})
    upow[u] = 1

    def atom(x):
        if isinstance(x, sp.Symbol):
            n = x.name
            if n.startswith("q") and n[1:].isdigit():
                return f"q[{n[1:]}]"
            return n
        if isinstance(x, (sp.Integer, sp.Rational, sp.Float)):
            v = float(x)
            return f"T({v!r})" if v >= 0 else f"(-T({-v!r}))"
        return None

    def pw(base, n):
        b = p(base)
        if n == 1:
            return b
        if n == 2:
            return f"({b}*{b})"
        if n == 3:
            return f"({b}*{b}*{b})"
        if n == 4:
            return f"(({b}*{b})*({b}*{b}))"
        h = pw(base, n // 2)
        return f"({h}*{h}*{b})" if n % 2 else f"({h}*{h})"

    def p(x):
        a = atom(x)
        if a is not None:
            return a
        if isinstance(x, sp.Add):
            return "(" + " + ".join(p(t) for t in x.args) + ")"
        if isinstance(x, sp.Mul):
            num, den = [], []
            for f in x.args:
                if isinstance(f, sp.Pow) and f.exp.is_Integer and f.exp < 0 and f.base in upow:
                    num.append(pw(r_sym, -int(f.exp) * upow[f.base]))
                elif isinstance(f, sp.Pow) and f.exp.is_Integer and f.exp < 0:
                    den.append(pw(f.base, -int(f.exp)))
                elif isinstance(f, sp.Rational) and not isinstance(f, sp.Integer) and f.p in (1, -1):
                    num.append("T(-1)" if f.p < 0 else "T(1)")
                    den.append(f"T({float(f.q)!r})")
                else:
                    num.append(p(f))
            s_ = "*".join(num) if num else "T(1)"
            if den:
                s_ = f"({s_})/({'*'.join(den)})"
            return f"({s_})"
        if isinstance(x, sp.Function) and x.func == rcp:
            return f"rcp({p(x.args[0])})"
        if isinstance(x, sp.Pow):
            if x.exp.is_Integer:
                n = int(x.exp)
                if n > 0:
                    return pw(x.base, n)
                if x.base in upow:
                    return pw(r_sym, -n * upow[x.base])
                return f"(T(1)/{pw(x.base, -n)})"
            raise RuntimeError(f"non-integer power: {x}")
        raise RuntimeError(f"cannot print {type(x)}: {x}")

    return p(e)


def main():
    print("// Analytic metric derivatives of the mixed-precision kernel.")
    print("// Generated by foort_gb300/gen/gen_christoffel.py -- do not edit.")
    print("// Inputs: q[] metric constants, r, dp = r - r_+, dm = r - r_-, s = sin(theta),")
    print("// c = cos(theta). Outputs: dr = d_r g_dd, dh = d_theta g_dd, gu = g^uu, grr = g_rr.")
    # Kerr's expanded numerators stay below r^8 and are emitted in r; Johannsen's are
    # emitted in u = 1/r.
    for name, fn, inv in (("Kerr", kerr, False), ("Johannsen", johannsen, True), ("Flat", flat, False),
                          ("RasheedLarsen", rasheed_larsen, False)):
        gdd, guu, dl, *P = fn()
        body = emit(name, gdd, guu, dl, inv, P[0] if P else None)
        print(f"#define FOORT_MIXED_BODY_{name.upper()} \\")
        print(" \\\n".join("    " + l for l in body.split("\n")))
        print()
    print(f"// Rasheed-Larsen constant slots q[0..{RL_NQ - 1}] from the rescaled parameters m, a, p, qq.")
    print("#define FOORT_MIXED_CONSTANTS_RASHEEDLARSEN \\")
    print(" \\\n".join(rl_constants_code()))
    print()


if __name__ == "__main__":
    main()
