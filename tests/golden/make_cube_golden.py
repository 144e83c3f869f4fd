"""Extracts text fixtures of critic2's NCI output from the reference's test
references (tests/015_grdplot/ref/007_nciplot_mols-{dens,grad}.cube and
007_nciplot_mols.dat: an H2O dimer from a molden file, 69 x 22 x 29 grid).

The fixture keeps the cube headers' geometry lines, a sample of body lines
at the same positions in both cubes, a sample of .dat lines and the full
line counts, so that the tests can check the number formats (every sampled
line must be reproduced exactly from its parsed numbers), the body layout
and the cutoff pass (s = 100 wherever |sign(lambda2) rho * 100| > 10),
without the reference tree.

    python tests/golden/make_cube_golden.py <reference-root>
"""
import json
import os
import sys

if len(sys.argv) != 2:
    sys.exit("usage: make_cube_golden.py <reference-root>")
REF = sys.argv[1]
D = os.path.join(REF, "tests", "015_grdplot", "ref")
HERE = os.path.dirname(os.path.abspath(__file__))


def read(name):
    with open(os.path.join(D, name)) as f:
        return f.read().split("\n")


def main():
    dens, grad, dat = read("007_nciplot_mols-dens.cube"), read("007_nciplot_mols-grad.cube"), read(
        "007_nciplot_mols.dat")
    natom = int(dens[2].split()[0])
    nstep = [int(dens[3 + c].split()[0]) for c in range(3)]
    body0 = 6 + natom
    nbody = len([l for l in dens[body0:] if l])
    # every 17th body line (the same lines in both cubes)
    pick = list(range(body0, body0 + nbody, 17))
    out = {
        "source": "tests/015_grdplot/ref/007_nciplot_mols-{dens,grad}.cube, 007_nciplot_mols.dat",
        "nstep": nstep,
        "natom_in_header": natom,
        "header_dens": dens[:6],
        "header_grad": grad[:6],
        "body_lines": nbody,
        "lines_per_record": (nstep[2] + 5) // 6,
        "sample_line_index": [i - body0 for i in pick],
        "dens_lines": [dens[i] for i in pick],
        "grad_lines": [grad[i] for i in pick],
        "dat_lines_total": len([l for l in dat if l]),
        "dat_lines": [l for l in dat if l][::29],
    }
    # writegrid_cube's precise cubes (tests/005_plot/ref): header lines and
    # a sample of body lines
    pre = {}
    for name in ("013_cube_simple_07.cube", "016_cube_grid_01.cube"):
        with open(os.path.join(REF, "tests", "005_plot", "ref", name)) as f:
            lines = f.read().split("\n")
        nat = int(lines[2].split()[0])
        body = [l for l in lines[6 + nat:] if l]
        pre[name] = {"header": lines[:6 + nat], "nstep": [int(lines[3 + c].split()[0]) for c in range(3)],
                     "body_lines": len(body), "sample": body[::13]}
    out["precise_cubes"] = pre
    with open(os.path.join(HERE, "nci_cube_text.json"), "w") as f:
        json.dump(out, f, indent=0)
    print("wrote", len(out["dens_lines"]), "body lines per cube and", len(out["dat_lines"]), "dat lines")


if __name__ == "__main__":
    main()
