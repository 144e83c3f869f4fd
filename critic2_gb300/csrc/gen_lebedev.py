"""Writes lebedev_tables.h: the Lebedev-Laikov angular quadratures of every
size critic2's good_lebedev offers (6 to 5810 points, degrees 3 to 131:
the molecular meshes use 110-770, the basin integrals any of them) as
octahedral orbit representatives.

The rules are taken from scipy.integrate.lebedev_rule (scipy >= 1.15,
which tabulates Lebedev and Laikov's published parameters).  Each orbit is
stored as (a, b, c, w) with a >= b >= c >= 0; the library expands it into
every distinct signed permutation.  Run from this directory:
    python gen_lebedev.py
"""
import itertools

import numpy as np
from scipy.integrate import lebedev_rule

RULES = ((6, 3), (14, 5), (26, 7), (38, 9), (50, 11), (74, 13), (86, 15), (110, 17), (146, 19), (170, 21),
         (194, 23), (230, 25), (266, 27), (302, 29), (350, 31), (434, 35), (590, 41), (770, 47), (974, 53),
         (1202, 59), (1454, 65), (1730, 71), (2030, 77), (2354, 83), (2702, 89), (3074, 95), (3470, 101),
         (3890, 107), (4334, 113), (4802, 119), (5294, 125), (5810, 131))


def orbits(n, deg):
    x, w = lebedev_rule(deg)
    assert x.shape[1] == n
    reps = {}
    for p, wt in zip(x.T, w / (4.0 * np.pi)):
        key = tuple(sorted(np.round(np.abs(p), 13), reverse=True))
        reps.setdefault(key, []).append((np.sort(np.abs(p))[::-1], wt))
    out = []
    for key, lst in reps.items():
        a, wt = lst[0][0], lst[0][1]
        npts = len({tuple(np.round(s * np.array(q), 12)) for q in itertools.permutations(a)
                    for s in itertools.product((1, -1), repeat=3)})
        assert npts == len(lst), (n, key, npts, len(lst))
        out.append((a, wt))
    out.sort(key=lambda t: (-t[0][0], -t[0][1], -t[0][2]))
    assert sum(len({tuple(np.round(s * np.array(q), 12)) for q in itertools.permutations(a)
                    for s in itertools.product((1, -1), repeat=3)}) for a, _ in out) == n
    return out


def main():
    lines = ["// Generated by gen_lebedev.py (Lebedev-Laikov rules from scipy.integrate.lebedev_rule).",
             "// Octahedral orbit representatives (a >= b >= c >= 0) and weights normalised to 1.",
             "#pragma once", "", "namespace c2g {", "",
             "struct LebedevOrbit {", "  double a, b, c, w;", "};", ""]
    index = []
    for n, deg in RULES:
        orb = orbits(n, deg)
        lines.append(f"constexpr LebedevOrbit kLebedev{n}[] = {{")
        for a, wt in orb:
            lines.append(f"    {{{float(a[0])!r}, {float(a[1])!r}, {float(a[2])!r}, {float(wt)!r}}},")
        lines.append("};")
        index.append((n, f"kLebedev{n}", len(orb)))
    lines += ["", "struct LebedevRule {", "  int npts;", "  const LebedevOrbit *orb;", "  int norb;", "};", "",
              "constexpr LebedevRule kLebedevRules[] = {"]
    for n, name, k in index:
        lines.append(f"    {{{n}, {name}, {k}}},")
    lines += ["};", "", "}  // namespace c2g", ""]
    open("lebedev_tables.h", "w").write("\n".join(lines))


if __name__ == "__main__":
    main()
