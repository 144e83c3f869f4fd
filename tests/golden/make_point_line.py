"""Writes point_line_benzene.json: critic2's own POINT block and LINE file
for benzene (tests/004_load/ref/002_load-wfx.cro lines of `point 0.1 0.2
0.3`, and 002_load-wfx.line of `line 0 -4 0 0 4 0 101`), the format pins of
critic2_gb300.rhoplot.  Give the root of a critic2 source tree:
    python tests/golden/make_point_line.py <reference-root>
"""
import json
import os
import sys

if len(sys.argv) != 2:
    sys.exit("usage: make_point_line.py <reference-root>")
REF = os.path.join(sys.argv[1], "tests", "004_load", "ref")
HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    cro = open(os.path.join(REF, "002_load-wfx.cro")).read().split("\n")
    i0 = next(i for i, l in enumerate(cro) if l.startswith("* POINT"))
    i1 = next(i for i in range(i0, len(cro)) if cro[i].startswith("  Field 0 "))
    point = cro[i0:i1]
    line = open(os.path.join(REF, "002_load-wfx.line")).read()
    out = {"point": {"xyz_ang": [0.1, 0.2, 0.3], "lines": point},
           "line": {"x0": [0.0, -4.0, 0.0], "x1": [0.0, 4.0, 0.0], "npts": 101, "text": line}}
    with open(os.path.join(HERE, "point_line_benzene.json"), "w") as f:
        json.dump(out, f, indent=0)


if __name__ == "__main__":
    main()
