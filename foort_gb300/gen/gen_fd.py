"""Generate the sparse finite-difference Christoffel contraction used by the FP64 kernel.

Metric::getChristoffel_udd (Metric.cpp:14-55) forms
    Gamma[mu][nu][rho] = sum_{sg=0..3} (0.5 * g^{mu sg}) * (dg[nu][rho][sg] + dg[rho][nu][sg] - dg[sg][nu][rho])
densely over 4^4 terms, and geoRHS (Integrators.cpp:60-68) forms
    a[i] = 0 - sum_{j,k} Gamma[i][j][k] * v[j] * v[k]
densely over 4^3 terms. For a stationary, axisymmetric metric (symmetries t and phi,
only g_tt, g_tphi, g_rr, g_thth, g_phiphi non-zero) most terms are exact zeros. Dropping
an exact zero from a sum or a difference does not change the result (x + 0 = x,
x - 0 = x, 0 - x = -x), so the emitted code performs the reference's remaining operations
in the reference's order.

Usage: python gen_fd.py > ../csrc/gen_fd_christoffel.inc
"""

NZ = {(0, 0), (0, 3), (3, 0), (1, 1), (2, 2), (3, 3)}
COMP = {(0, 0): "tt", (0, 3): "tp", (3, 0): "tp", (1, 1): "rr", (2, 2): "hh", (3, 3): "pp"}


def g_nz(i, j):
    return (i, j) in NZ


def dg(c, i, j):
    """Name of d_c g_ij or None when it is an exact zero."""
    if c not in (1, 2) or not g_nz(i, j):
        return None
    return f"{'dr' if c == 1 else 'dh'}.{COMP[(i, j)]}"


def gu(i, j):
    return f"gu.{COMP[(i, j)]}" if g_nz(i, j) else None


def inner(nu, rho, sg):
    a, b, c = dg(nu, rho, sg), dg(rho, nu, sg), dg(sg, nu, rho)
    # (a + b) - c with exact zeros removed
    if a and b:
        s = f"({a} + {b})"
    else:
        s = a or b
    if c:
        s = f"({s} - {c})" if s else f"(-{c})"
    return s


def main():
    lines = []
    emit = lines.append
    emit("// Generated by foort_gb300/gen/gen_fd.py -- do not edit.")
    emit("// In: G5 dr, dh (central differences of g_dd in x1 and x2), G5 gu (g^uu), double v[4].")
    emit("// Out: double acc[4] = -Gamma^i_jk v^j v^k in the reference's order.")
    gam = {}
    for mu in range(4):
        for nu in range(4):
            for rho in range(4):
                key = (mu, min(nu, rho), max(nu, rho))
                if key in gam:
                    gam[(mu, nu, rho)] = gam[key]
                    continue
                acc = None
                for sg in range(4):
                    g = gu(mu, sg)
                    if not g:
                        continue
                    s = inner(nu, rho, sg)
                    if not s:
                        continue
                    term = f"(0.5 * {g}) * {s}"
                    acc = term if acc is None else f"{acc} + {term}"
                if acc is None:
                    gam[(mu, nu, rho)] = None
                    continue
                name = f"G{mu}{nu}{rho}"
                emit(f"const double {name} = {acc};")
                gam[(mu, nu, rho)] = name
    for i in range(4):
        expr = None
        for j in range(4):
            for k in range(4):
                g = gam[(i, j, k)]
                if not g:
                    continue
                t = f"{g} * v[{j}] * v[{k}]"
                expr = f"-({t})" if expr is None else f"{expr} - {t}"
        emit(f"acc[{i}] = {expr if expr else '0.0'};")
    print("\n".join(lines))


if __name__ == "__main__":
    main()
