"""Writes sphcar_fchk.json: critic2's spherical -> Cartesian matrices used by
read_fchk and read_molden (dsphcar, fsphcar, gsphcar_fchk, gsphcar;
src/wfn_private@proc.F90:46-167),
parsed from the reference source with its named sqrt constants resolved,
as T[m][c] (m = 0, 1, -1, ...; Cartesian components in fchk order).
Give the reference's source file (src/wfn_private@proc.F90 of a critic2
source tree):
    python make_sphcar.py <reference-root>/src/wfn_private@proc.F90"""
import json
import math
import re
import sys

if len(sys.argv) != 2:
    sys.exit("usage: make_sphcar.py <path of wfn_private@proc.F90>")
src = open(sys.argv[1]).read()
const = {}
for name, expr in re.findall(r"real\*8, parameter :: (\w+) = ([^\n!]+)", src):
    e = expr.strip().replace("d0", "")
    if e.startswith("sqrt("):
        const[name] = math.sqrt(eval(e[5:-1]))
    else:
        try:
            const[name] = float(eval(e))
        except Exception:
            pass


def value(tok):
    tok = tok.strip()
    if tok in const:
        return const[tok]
    neg = tok.startswith("-")
    t = tok[1:] if neg else tok
    v = const[t] if t in const else float(t.replace("d", "e"))
    return -v if neg else v


out = {}
for name, key, nm, nc in (("dsphcar", "2", 5, 6), ("fsphcar", "3", 7, 10), ("gsphcar_fchk", "4", 9, 15),
                          ("gsphcar", "4molden", 9, 15)):
    body = src.split(f"real*8 :: {name}({nm},{nc}) = reshape((/&")[1].split("/),shape")[0]
    nums = []
    for line in body.split("\n"):
        line = line.split("!")[0].replace("&", "")
        nums += [value(t) for t in line.split(",") if t.strip()]
    assert len(nums) == nm * nc, (name, len(nums))
    # Fortran reshape fills column-major: nums[c*nm + m] is (m, c)
    out[key] = [[nums[c * nm + m] for c in range(nc)] for m in range(nm)]
with open("sphcar_fchk.json", "w") as fh:
    json.dump(out, fh, indent=1)
