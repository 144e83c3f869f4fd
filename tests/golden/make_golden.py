"""Extracts golden POINT records from critic2's own test references.

critic2's regression tests print, for a point in a molecular-wavefunction
field, the density, gradient, |gradient|, kinetic energy density,
Laplacian, the Hessian, its eigenvalues, the CP type (rank, signature) and
the spin-resolved density / |gradient| / Laplacian / G
(tests/004_load/ref/*.cro, tests/005_plot/ref/*.cro; compared by the
reference at 1e-10).  The wavefunction files those tests read are not
distributed with the source, so the records pin the field's
post-processing (eigen-solve, rank/signature, |grad|, Laplacian, spin
halves), not the evaluator itself.

Run from the repository root, giving the root of a critic2 source tree:
    python tests/golden/make_golden.py <reference-root>
Writes tests/golden/point_records.json.
"""
from __future__ import annotations

import glob
import json
import os
import re
import sys

if len(sys.argv) != 2:
    sys.exit("usage: make_golden.py <reference-root>")
REF = os.path.join(sys.argv[1], "tests")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "point_records.json")

NUM = r"[-+]?\d*\.\d+(?:[EeDd][-+]?\d+)?"


def nums(s):
    return [float(v.replace("D", "E")) for v in re.findall(NUM, s)]


def parse_file(path):
    lines = open(path, errors="replace").read().splitlines()
    wfn = any("Type: molecular wavefunction" in l for l in lines)
    recs = []
    i = 0
    while i < len(lines):
        if lines[i].startswith("* POINT"):
            rec = {"file": os.path.relpath(path, REF), "line": i + 1, "wavefunction": wfn}
            j = i + 1
            while j < len(lines) and not lines[j].startswith("* ") and lines[j].strip():
                l = lines[j].strip()
                if l.startswith("Type :"):
                    m = re.search(r"\((\d+),\s*(-?\d+)\)", l)
                    if m:
                        rec["r"], rec["s"] = int(m.group(1)), int(m.group(2))
                elif l.startswith("Field value (f):"):
                    rec["f"] = nums(l)[0]
                elif l.startswith("Gradient (grad f):"):
                    rec["grad"] = nums(l)[:3]
                elif l.startswith("Gradient norm (|grad f|):"):
                    rec["gfmod"] = nums(l)[0]
                elif l.startswith("Kinetic energy density (G,tau):"):
                    rec["gkin"] = nums(l)[0]
                elif l.startswith("Laplacian (del2 f):"):
                    rec["lap"] = nums(l)[0]
                elif l.startswith("Hessian:"):
                    rec["hess"] = [nums(lines[j + k])[:3] for k in (1, 2, 3)]
                    j += 3
                elif l.startswith("Hessian eigenvalues:"):
                    rec["hfeval"] = nums(l)[:3]
                elif l.startswith("Spin up   field/gradient_norm/laplacian:"):
                    rec["up"] = nums(l)[:3]
                elif l.startswith("Spin up   kinetic energy density (G):"):
                    rec["up_gkin"] = nums(l)[0]
                elif l.startswith("Spin down field/gradient_norm/laplacian:"):
                    rec["down"] = nums(l)[:3]
                elif l.startswith("Spin down kinetic energy density (G):"):
                    rec["down_gkin"] = nums(l)[0]
                elif l.startswith("+ Field:") and "f" in rec:
                    break  # only the first field of a multi-field POINT
                j += 1
            if "hess" in rec and "hfeval" in rec and "f" in rec:
                recs.append(rec)
            i = j
        else:
            i += 1
    return recs


def main():
    recs = []
    for path in sorted(glob.glob(os.path.join(REF, "*", "ref", "*.cro"))):
        recs.extend(parse_file(path))
    recs = [r for r in recs if r["wavefunction"]]
    with open(OUT, "w") as fh:
        json.dump({"source": "critic2 tests/*/ref/*.cro POINT records (molecular wavefunctions)",
                   "records": recs}, fh, indent=1)
    print(f"{len(recs)} records -> {OUT}")


if __name__ == "__main__":
    main()
