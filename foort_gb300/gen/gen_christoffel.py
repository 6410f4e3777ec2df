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


def to_sc(e):
    return e.subs({sp.sin(th): s, sp.cos(th): c})


def condition(e, dl):
    """Put e over a common denominator, expand the numerator as a polynomial in r (so
    that no leading powers of r cancel numerically) and write Delta as dp * dm."""
    e = sp.together(to_sc(e))
    num, den = sp.fraction(e)
    num = sp.expand(num)
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


def emit(name, gdd, guu, dl, inv=False):
    cond = condition_inv if inv else condition
    exprs = []
    names = []
    for k in COMP:
        exprs.append(cond(sp.diff(gdd[k], r), dl))
        names.append(f"dr.{k}")
    for k in COMP:
        exprs.append(cond(sp.diff(gdd[k], th), dl))
        names.append(f"dh.{k}")
    for k in COMP:
        exprs.append(cond(guu[k], dl))
        names.append(f"gu.{k}")
    exprs.append(cond(gdd["rr"], dl))
    names.append("grr")
    repl, red = sp.cse(exprs, symbols=sp.numbered_symbols("t"), optimizations="basic")
    lines = ["const T u = rcp(r);"] if inv else []
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
    for name, fn, inv in (("Kerr", kerr, False), ("Johannsen", johannsen, True), ("Flat", flat, False)):
        gdd, guu, dl = fn()
        body = emit(name, gdd, guu, dl, inv)
        print(f"#define FOORT_MIXED_BODY_{name.upper()} \\")
        print(" \\\n".join("    " + l for l in body.split("\n")))
        print()


if __name__ == "__main__":
    main()
