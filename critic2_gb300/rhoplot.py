"""critic2's POINT and LINE keywords for the wavefunction field, in
critic2's text formats (src/rhoplot@proc.f90:69-185 rhoplot_point, with the
property block of system%propty, src/systemmod@proc.f90:1329-1420; and
:187-380 rhoplot_line).  Coordinates are Cartesian, in angstrom (critic2's
default unit for molecules) or bohr, in the frame of the wavefunction's
atoms.  The values come from the library's FP64 evaluator (field%grd for
the value, gradient, Hessian, its eigenvalues, rank and signature; rho2 for
G and the spin channels; rho2's valence outputs for the valence lines).

Not mirrored: POINT ALL (it adds critic2's promolecular field 0), FIELD
expressions, and crystal (fractional) coordinates."""
from __future__ import annotations

import numpy as np

BOHR_TO_ANG = 0.52917720859  # critic2's bohrtoa (src/param.F90:42)


def fortran_e(x: float, d: int) -> str:
    """Fortran 1p,E(w).(d) of one value, blanks removed (critic2's
    string(x,'e',decimal=d)): d decimals, a two-digit exponent with its
    E, or three digits without the E when |exponent| > 99."""
    s = f"{x:.{d}E}"
    mant, ex = s.split("E")
    e = int(ex)
    if abs(e) > 99:
        return f"{mant}{e:+04d}"
    return s


def fortran_f(x: float, d: int) -> str:
    """Fortran F(w).(d), blanks removed (critic2's string(x,'f',decimal=d))."""
    return f"{x:.{d}f}"


def _to_bohr(x, unit: str) -> np.ndarray:
    x = np.asarray(x, np.float64).reshape(-1, 3)
    if unit == "ang":
        return x / BOHR_TO_ANG
    if unit == "bohr":
        return x.copy()
    raise ValueError("unit must be 'ang' or 'bohr'")


def point_text(w, xyz, unit: str = "ang") -> str:
    """The output of `POINT x y z` for each row of xyz (critic2's text,
    blank line after each block)."""
    x_in = np.asarray(xyz, np.float64).reshape(-1, 3)
    xb = _to_bohr(x_in, unit)
    g = w.grd(xb, 2, "fp64")
    r2 = w.rho2(xb, 2, "fp64")
    rv = w.rho2_valence(xb, 2)
    e9 = lambda v: fortran_e(float(v), 9)
    out = []
    for i in range(len(xb)):
        out.append("* POINT " + "".join(fortran_f(v, 7) + "  " for v in x_in[i]))
        lab = "ang" if unit == "ang" else "bohr"
        out.append(f"  Coordinates ({lab}): " + "".join(fortran_f(v, 7) + "  " for v in x_in[i]))
        out.append("+ Field: 1")
        if g["isnuc"][i]:
            out.append("  Type : nucleus")
        else:
            out.append(f"  Type : ({int(g['r'][i])},{int(g['s'][i])})")
        f, fval = g["f"][i], rv["rho"][i, 0]
        out.append("  Field value (f): " + e9(f))
        out.append("  Field value, valence (fval): " + e9(fval))
        out.append("  Gradient (grad f): " + "".join(e9(v) + "  " for v in g["gf"][i]))
        out.append("  Gradient norm (|grad f|): " + e9(g["gfmod"][i]))
        gval = 0.0 if g["isnuc"][i] else float(np.linalg.norm(rv["grad"][i, 0]))
        out.append("  Gradient norm, valence: " + e9(gval))
        out.append("  Kinetic energy density (G,tau): " + e9(r2["gkin"][i, 0]))
        hf = g["hf"][i]
        out.append("  Laplacian (del2 f): " + e9(np.trace(hf)))
        out.append("  Laplacian, valence (del2 fval): " + e9(np.trace(rv["hess"][i, 0])))
        out.append("  Hessian:")
        for j in range(3):
            out.append("    " + "".join(f"{e9(hf[j, k]):>16}  " for k in range(3)))
        ev = g["hfeval"][i]
        out.append("  Hessian eigenvalues: " + "".join(e9(v) + "  " for v in ev))
        if int(g["r"][i]) == 3 and int(g["s"][i]) == -1 and not g["isnuc"][i]:
            out.append("  Ellipticity (l_1/l_2 - 1): " + e9(ev[0] / ev[1] - 1.0))
        for s, name in ((1, "Spin up  "), (2, "Spin down")):
            fs = r2["rho"][i, s]
            gs = float(np.linalg.norm(r2["grad"][i, s]))
            ls = float(np.trace(r2["hess"][i, s]))
            out.append(f"  {name} field/gradient_norm/laplacian: " + "".join(e9(v) + "  " for v in (fs, gs, ls)))
            out.append(f"  {name} kinetic energy density (G): " + e9(r2["gkin"][i, s]))
        out.append("")
    return "\n".join(out) + "\n"


LINE_PROPS = {"": None, "gx": ("gf", 0), "gy": ("gf", 1), "gz": ("gf", 2), "gmod": ("gfmod", None),
              "hxx": ("hf", (0, 0)), "hxy": ("hf", (0, 1)), "hyx": ("hf", (0, 1)), "hxz": ("hf", (0, 2)),
              "hzx": ("hf", (0, 2)), "hyy": ("hf", (1, 1)), "hyz": ("hf", (1, 2)), "hzy": ("hf", (1, 2)),
              "hzz": ("hf", (2, 2)), "lap": ("lap", None)}


def line_text(w, x0, x1, npts: int, prop: str = "", unit: str = "ang") -> str:
    """The file written by `LINE x0 y0 z0 x1 y1 z1 npts [prop] FILE f`:
    npts (>= 2) points from x0 to x1, columns x, y, z, distance (input
    unit), f and the property (gx gy gz gmod hxx hxy hxz hyy hyz hzz lap)."""
    prop = prop.lower()
    if prop not in LINE_PROPS:
        raise ValueError(f"unknown LINE property {prop!r}")
    npts = max(int(npts), 2)
    a, b = _to_bohr(x0, unit)[0], _to_bohr(x1, unit)[0]
    t = np.arange(npts, dtype=np.float64) / (npts - 1)
    xp = a[None, :] + (b - a)[None, :] * t[:, None]
    nder = 0 if prop == "" else (1 if prop in ("gx", "gy", "gz", "gmod") else 2)
    g = w.grd(xp, nder, "fp64")
    dun = BOHR_TO_ANG if unit == "ang" else 1.0
    lines = ["# Field values (f) along a line (d = distance).",
             "# " + "".join(f"{c:>15}" for c in ("x", "y", "z", "d")) + f"{'f':>20}" + f"{prop:>20}"]
    for i in range(npts):
        dist = float(np.linalg.norm(xp[i] - a)) * dun
        xout = xp[i] * dun
        cols = [fortran_f(v, 13).ljust(18) for v in xout] + [fortran_f(dist, 13).ljust(18),
                                                             fortran_e(float(g["f"][i]), 13).ljust(20)]
        if prop:
            key, sub = LINE_PROPS[prop]
            if key == "lap":
                v = float(np.trace(g["hf"][i]))
            elif sub is None:
                v = float(g[key][i])
            elif isinstance(sub, tuple):
                v = float(g[key][i][sub])
            else:
                v = float(g[key][i][sub])
            cols.append(fortran_e(v, 13).ljust(20))
        lines.append("".join(" " + c for c in cols) + " ")
    return "\n".join(lines) + "\n\n"
