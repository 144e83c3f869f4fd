"""Writes sphcar_tables.h: the matrices T(m, c) that take the coefficients
of normalised real solid harmonic Gaussians (m = 0, 1, -1, 2, -2, ..., the
order of fchk and molden files) to coefficients of individually
normalised Cartesian Gaussians (fchk's Cartesian order; for l = 4 also
molden's), for l = 2, 3, 4.

Derivation (sympy, exact): R_lm = P_l^|m|(z, r) Re/Im[(x + i y)^|m|] with
P_l^m = sum_k (-1)^k 2^-l C(l,k) C(2l-2k,l) (l-2k)!/(l-2k-m)! r^2k z^(l-2k-m)
(Re for m > 0, Im for m < 0, no Condon-Shortley phase); with R = sum_c a_c
x^c, T(m, c) = a_c |x^c| / |R|, where |.|^2 is the angular Gaussian norm
(2a-1)!!(2b-1)!!(2c-1)!! of x^a y^b z^c (common radial factors cancel).
Run from this directory: python gen_sphcar.py
"""
import sympy as sp

x, y, z = sp.symbols("x y z", real=True)

MOLDEN_G = ["xxxx", "yyyy", "zzzz", "xxxy", "xxxz", "xyyy", "yyyz", "xzzz", "yzzz", "xxyy", "xxzz", "yyzz",
            "xxyz", "xyyz", "xyzz"]
FCHK_CART = {
    2: ["xx", "yy", "zz", "xy", "xz", "yz"],
    3: ["xxx", "yyy", "zzz", "xyy", "xxy", "xxz", "xzz", "yzz", "yyz", "xyz"],
    4: ["zzzz", "yzzz", "yyzz", "yyyz", "yyyy", "xzzz", "xyzz", "xyyz", "xyyy", "xxzz", "xxyz",
        "xxyy", "xxxz", "xxxy", "xxxx"],
}


def dfm1(n):  # (n-1)!! for even n >= 0, as used by the Gaussian moments
    r = 1
    k = n - 1
    while k > 1:
        r *= k
        k -= 2
    return r


def moment(e):
    if any(v % 2 for v in e):
        return 0
    return dfm1(e[0]) * dfm1(e[1]) * dfm1(e[2])


def solid(l, m):
    am = abs(m)
    r2 = x ** 2 + y ** 2 + z ** 2
    P = 0
    for k in range((l - am) // 2 + 1):
        P += ((-1) ** k * sp.Rational(1, 2 ** l) * sp.binomial(l, k) * sp.binomial(2 * l - 2 * k, l)
              * sp.factorial(l - 2 * k) / sp.factorial(l - 2 * k - am) * r2 ** k * z ** (l - 2 * k - am))
    c = sp.expand((x + sp.I * y) ** am)
    part = sp.re(c) if m >= 0 else sp.im(c)
    if m == 0:
        part = 1
    return sp.Poly(sp.expand(P * part), x, y, z)


def exps(label):
    return (label.count("x"), label.count("y"), label.count("z"))


def table(l, cart=None):
    ms = [0]
    for k in range(1, l + 1):
        ms += [k, -k]
    rows = []
    for m in ms:
        R = solid(l, m)
        coef = {tuple(mon): c for mon, c in zip(R.monoms(), R.coeffs())}
        n2 = sum(a * b * moment(tuple(p + q for p, q in zip(ea, eb)))
                 for ea, a in coef.items() for eb, b in coef.items())
        row = []
        for lab in (cart or FCHK_CART[l]):
            e = exps(lab)
            a = coef.get(e, 0)
            row.append(sp.nsimplify(a * sp.sqrt(moment(tuple(2 * v for v in e))) / sp.sqrt(n2)))
        rows.append(row)
    return ms, rows


def main():
    out = ["// Generated by gen_sphcar.py: real solid harmonics (fchk order m = 0, 1, -1, ...)",
           "// to normalised Cartesian Gaussians (fchk Cartesian order), T[m][c].",
           "#pragma once", "", "namespace c2g {", ""]
    for l in (2, 3, 4):
        ms, rows = table(l)
        nc = len(FCHK_CART[l])
        out.append(f"// l = {l}: Cartesian order {' '.join(FCHK_CART[l])}")
        out.append(f"constexpr double kSphCar{l}[{2 * l + 1}][{nc}] = {{")
        for m, row in zip(ms, rows):
            out.append("    {" + ", ".join(repr(float(v)) for v in row) + f"}},  // m = {m}")
        out.append("};")
        out.append("")
    ms, rows = table(4, MOLDEN_G)
    out.append(f"// l = 4, molden Cartesian order {' '.join(MOLDEN_G)}")
    out.append("constexpr double kSphCar4Molden[9][15] = {")
    for m, row in zip(ms, rows):
        out.append("    {" + ", ".join(repr(float(v)) for v in row) + f"}},  // m = {m}")
    out.append("};")
    out.append("")
    out += ["}  // namespace c2g", ""]
    open("sphcar_tables.h", "w").write("\n".join(out))


if __name__ == "__main__":
    main()
