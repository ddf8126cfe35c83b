"""Generate lgb_d3q19.h: D3Q19 model tables and unrolled mode transforms.

The D3Q19 velocity set, weights and the 19 modes (rho, j, S_ab, chi1, jchi1,
chi2, jchi2, chi3) are those of the reference (src/lb_d3q19.h:26-38,
src/lb_d3q19.c:107-153).  Every matrix entry is computed here as an exact
rational and printed as ``N.0/D.0``, which the compiler rounds once to the
nearest double: the same value as the reference's unrolled constants
(src/collision.c:1965-1985).

Two kinds of transform are emitted:

* ``*_seq`` keep the reference's accumulation order (acc = 0; acc += f_p*c
  for p = 0..18), drop the terms whose coefficient is exactly zero (adding
  +/-0 to a sum that started at +0 leaves it unchanged under round to
  nearest) and write c = +/-1 as an add or subtract.  Used by the FP64 path,
  which must reproduce the reference bit for bit.
* ``*_fast`` factor the transforms through pairwise sums and differences of
  opposite velocities.  Used by the reduced-precision paths.

Run:  python gen_d3q19.py > lgb_d3q19.h
"""

from fractions import Fraction as F

CV = [(0, 0, 0),
      (1, 1, 0), (1, 0, 1), (1, 0, 0),
      (1, 0, -1), (1, -1, 0), (0, 1, 1),
      (0, 1, 0), (0, 1, -1), (0, 0, 1),
      (0, 0, -1), (0, -1, 1), (0, -1, 0),
      (0, -1, -1), (-1, 1, 0), (-1, 0, 1),
      (-1, 0, 0), (-1, 0, -1), (-1, -1, 0)]
W36 = [12, 1, 1, 2, 1, 1, 1, 2, 1, 2, 2, 1, 2, 1, 1, 1, 2, 1, 1]
NVEL = 19
NHYDRO = 10


def mode(m, p):
    cx, cy, cz = CV[p]
    c2 = cx * cx + cy * cy + cz * cz
    chi1 = (2 * c2 - 3) * (3 * cz * cz - c2)
    chi2 = (2 * c2 - 3) * (cy * cy - cx * cx)
    chi3 = 3 * c2 * c2 - 6 * c2 + 1
    t = F(1, 3)
    return [F(1), F(cx), F(cy), F(cz), cx * cx - t, F(cx * cy), F(cx * cz),
            cy * cy - t, F(cy * cz), cz * cz - t, F(chi1), F(chi1 * cx),
            F(chi1 * cy), F(chi1 * cz), F(chi2), F(chi2 * cx), F(chi2 * cy),
            F(chi2 * cz), F(chi3)][m]


MA = [[F(mode(m, p)) for p in range(NVEL)] for m in range(NVEL)]
W = [F(w, 36) for w in W36]
NA = [1 / sum(W[p] * MA[m][p] ** 2 for p in range(NVEL)) for m in range(NVEL)]
MI = [[W[p] * NA[m] * MA[m][p] for m in range(NVEL)] for p in range(NVEL)]

# sanity: MI is the inverse of MA
for i in range(NVEL):
    for j in range(NVEL):
        s = sum(MA[i][k] * MI[k][j] for k in range(NVEL))
        assert s == (1 if i == j else 0)


def lit(c):
    c = F(c)
    if c.denominator == 1:
        return "T(%d.0)" % c.numerator
    return "T(%d.0/%d.0)" % (c.numerator, c.denominator)


def acc_line(target, terms):
    """terms: list of (coef, operand) in order; emit reference-order sum."""
    out = ["  %s = T(0.0);" % target]
    for c, x in terms:
        if c == 0:
            continue
        if c == 1:
            out.append("  %s += %s;" % (target, x))
        elif c == -1:
            out.append("  %s -= %s;" % (target, x))
        else:
            out.append("  %s += %s*%s;" % (target, x, lit(c)))
    return out


def gen_seq():
    lines = []
    lines.append("/* Modes 0..nm-1 of f, reference accumulation order "
                 "(src/collision.c:1990-2398). */")
    lines.append("template <typename T, int NM>")
    lines.append("__device__ __forceinline__ void d3q19_f2mode_seq("
                 "const T * __restrict__ f, T * __restrict__ m) {")
    for mm in range(NVEL):
        lines.append("  if (NM > %d) {" % mm)
        body = acc_line("m[%d]" % mm,
                        [(MA[mm][p], "f[%d]" % p) for p in range(NVEL)])
        lines += ["  " + b for b in body]
        lines.append("  }")
    lines.append("}")
    lines.append("")
    lines.append("/* f from modes 0..nm-1 (modes nm.. are exactly zero), "
                 "reference order")
    lines.append(" * (src/collision.c:2401-2850: ftmp += c*mode[m]). */")
    lines.append("template <typename T, int NM>")
    lines.append("__device__ __forceinline__ void d3q19_mode2f_seq("
                 "const T * __restrict__ m, T * __restrict__ f) {")
    for p in range(NVEL):
        lines.append("  {")
        lines.append("    T acc = T(0.0);")
        for mm in range(NVEL):
            c = MI[p][mm]
            if c == 0:
                continue
            cond = "if (NM > %d) " % mm if mm >= NHYDRO else ""
            if c == 1:
                lines.append("    %sacc += m[%d];" % (cond, mm))
            elif c == -1:
                lines.append("    %sacc -= m[%d];" % (cond, mm))
            else:
                lines.append("    %sacc += %s*m[%d];" % (cond, lit(c), mm))
        lines.append("    f[%d] = acc;" % p)
        lines.append("  }")
    lines.append("}")
    return lines


def gen_tables():
    lines = []
    lines.append("/* Velocity set (src/lb_d3q19.h:26-33) */")
    lines.append("#define LGB_D3Q19_CV { \\")
    rows = ["  {%2d, %2d, %2d}" % c for c in CV]
    lines.append(", \\\n".join(rows) + "}")
    lines.append("")
    lines.append("/* Weights times 36 (src/lb_d3q19.h:35-38) */")
    lines.append("#define LGB_D3Q19_W36 {" + ", ".join(str(w) for w in W36)
                 + "}")
    lines.append("")
    # opposite velocities
    opp = []
    for p in range(NVEL):
        c = tuple(-v for v in CV[p])
        opp.append(CV.index(c))
    lines.append("#define LGB_D3Q19_OPP {" + ", ".join(str(o) for o in opp)
                 + "}")
    return lines


def gen_fast():
    """Factorised transforms for reduced precision.

    Pairs (p, q) with c_q = -c_p give s = f_p + f_q and d = f_p - f_q; every
    even mode (rho, S_ab, ghosts chi1, chi2, chi3) is a combination of the
    sums and every odd mode (j, jchi1, jchi2) of the differences.
    """
    opp = [CV.index(tuple(-v for v in CV[p])) for p in range(NVEL)]
    pairs = []
    seen = set()
    for p in range(1, NVEL):
        if p in seen:
            continue
        q = opp[p]
        seen.add(p)
        seen.add(q)
        pairs.append((p, q))
    lines = []
    lines.append("/* Factorised transforms (reduced precision only). */")
    lines.append("template <typename T, int NM>")
    lines.append("__device__ __forceinline__ void d3q19_f2mode_fast("
                 "const T * __restrict__ f, T * __restrict__ m) {")
    for k, (p, q) in enumerate(pairs):
        lines.append("  const T s%d = f[%d] + f[%d];" % (k, p, q))
        lines.append("  const T d%d = f[%d] - f[%d];" % (k, p, q))
    for mm in range(NVEL):
        terms = []
        odd = mm in (1, 2, 3, 11, 12, 13, 15, 16, 17)
        if not odd and MA[mm][0] != 0:
            terms.append((MA[mm][0], "f[0]"))
        for k, (p, q) in enumerate(pairs):
            c = MA[mm][p]
            if c == 0:
                continue
            terms.append((c, ("d%d" if odd else "s%d") % k))
        # group by coefficient
        groups = {}
        order = []
        for c, x in terms:
            if c not in groups:
                groups[c] = []
                order.append(c)
            groups[c].append(x)
        expr = []
        for c in order:
            s = " + ".join(groups[c])
            if c == 1:
                expr.append("(%s)" % s)
            elif c == -1:
                expr.append("-(%s)" % s)
            else:
                expr.append("%s*(%s)" % (lit(c), s))
        e = " + ".join(expr) if expr else "T(0.0)"
        lines.append("  if (NM > %d) m[%d] = %s;" % (mm, mm, e))
    lines.append("}")
    lines.append("")
    # mode2f fast: f_p = even_part(p) + odd_part(p); f_q = even - odd
    lines.append("template <typename T, int NM>")
    lines.append("__device__ __forceinline__ void d3q19_mode2f_fast("
                 "const T * __restrict__ m, T * __restrict__ f) {")

    def part(p, odd):
        terms = []
        for mm in range(NVEL):
            if (mm in (1, 2, 3, 11, 12, 13, 15, 16, 17)) != odd:
                continue
            c = MI[p][mm]
            if c == 0:
                continue
            cond = mm >= NHYDRO
            terms.append((c, mm, cond))
        return terms

    def grouped(terms):
        groups, order = {}, []
        for c, mm in terms:
            if c not in groups:
                groups[c] = []
                order.append(c)
            groups[c].append("m[%d]" % mm)
        return " + ".join("%s*(%s)" % (lit(c), " + ".join(groups[c]))
                          for c in order)

    def expr_of(terms):
        """Hydrodynamic terms, then the ghost terms as one added part that
        is -0.0 (an exact additive identity, which the compiler drops) when
        the ghost modes are not carried (NM = 10)."""
        hydro = [(c, mm) for c, mm, cond in terms if not cond]
        ghost = [(c, mm) for c, mm, cond in terms if cond]
        h = grouped(hydro) if hydro else "T(0.0)"
        if not ghost:
            return h
        top = max(mm for _, mm in ghost)
        return "%s + (NM > %d ? (%s) : T(-0.0))" % (h, top, grouped(ghost))

    lines.append("  f[0] = %s;" % expr_of(part(0, False)))
    for (p, q) in pairs:
        lines.append("  {")
        lines.append("    const T e = %s;" % expr_of(part(p, False)))
        lines.append("    const T o = %s;" % expr_of(part(p, True)))
        lines.append("    f[%d] = e + o;" % p)
        lines.append("    f[%d] = e - o;" % q)
        lines.append("  }")
    lines.append("}")
    # check parity structure used above
    for (p, q) in pairs:
        for mm in range(NVEL):
            odd = mm in (1, 2, 3, 11, 12, 13, 15, 16, 17)
            if odd:
                assert MI[q][mm] == -MI[p][mm]
            else:
                assert MI[q][mm] == MI[p][mm]
    return lines


def main():
    out = []
    out.append("/* Generated by gen_d3q19.py -- do not edit. */")
    out.append("/* D3Q19 tables and mode transforms; see gen_d3q19.py for "
               "provenance. */")
    out.append("#ifndef LGB_D3Q19_H")
    out.append("#define LGB_D3Q19_H")
    out.append("")
    out += gen_tables()
    out.append("")
    out.append("#ifdef __CUDACC__")
    out += gen_seq()
    out.append("")
    out += gen_fast()
    out.append("#endif /* __CUDACC__ */")
    out.append("")
    out.append("#endif")
    print("\n".join(out))


if __name__ == "__main__":
    main()
