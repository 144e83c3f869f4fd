"""Extracts the quadrature columns of critic2's SPHEREINTEGRALS regression
test (tests/014_bisect/ref/007_sphereintegrals.cro).

That test integrates spheres around the CPs of a crystal's promolecular
density, so its charges and Laplacians belong to a field this library does
not evaluate.  Two columns do not depend on the field: the radii of the
logarithmic grid r = r0 exp(h (n - 1)) and the volume of each sphere, which
is the angular rule's weight sum times the radial Gauss-Legendre integral
of r^2 (exact with 50 nodes).  So the records pin the radial grid and the
angular rules (GAULEG 2 2, LEBEDEV 6) of the basin integration.

Run from the repository root, giving the root of a critic2 source tree:
    python tests/golden/make_sphere_golden.py <reference-root>
Writes tests/golden/sphere_quadrature.json.
"""
from __future__ import annotations

import json
import os
import re
import sys

if len(sys.argv) != 2:
    sys.exit("usage: make_sphere_golden.py <reference-root>")
SRC = os.path.join(sys.argv[1], "tests", "014_bisect", "ref", "007_sphereintegrals.cro")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "sphere_quadrature.json")

NUM = r"[-+]?\d*\.\d+(?:[EeDd][-+]?\d+)?"


def num(s: str) -> float:
    return float(s.replace("D", "E").replace("d", "e"))


blocks = []
cur = None
for line in open(SRC):
    if line.startswith("* Integration of spheres"):
        cur = {"rows": []}
        blocks.append(cur)
    elif cur is None:
        continue
    elif "Method : Gauss-Legendre" in line and "angular" not in cur:
        cur["angular"] = "gauleg"
    elif "Method : Lebedev" in line:
        cur["angular"] = "lebedev"
    elif "Polar angle (theta) num. of nodes:" in line:
        cur["ntheta"] = int(line.split(":")[1])
    elif "Azimuthal angle (phi) num. of nodes:" in line:
        cur["nphi"] = int(line.split(":")[1])
    elif line.strip().startswith("Number of nodes:"):
        cur["nleb"] = int(line.split(":")[1])
    elif "Initial radius (r0,bohr):" in line:
        cur["r0"] = num(line.split(":")[1])
    elif "Final radius (rend,bohr):" in line:
        cur["rend"] = num(line.split(":")[1])
    elif "Radial points:" in line:
        cur["nr"] = int(line.split(":")[1])
    elif "Logarithmic step h" in line:
        cur["h"] = num(line.split(":")[-1])
    else:
        f = re.findall(NUM, line)
        if len(f) == 5 and re.match(r"\s+" + NUM + r"\s+\d+\s", line):
            r, err, vol, chg, lap = (num(v) for v in f)
            cur["rows"].append({"r": r, "volume": vol})

assert len(blocks) == 2 and all(b["rows"] for b in blocks), blocks
with open(OUT, "w") as fh:
    json.dump({"source": "tests/014_bisect/ref/007_sphereintegrals.cro", "blocks": blocks}, fh, indent=1)
print(f"wrote {OUT}: " + ", ".join(f"{b['angular']} {len(b['rows'])} radii" for b in blocks))
