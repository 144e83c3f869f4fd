"""POINT and LINE output (critic2_gb300.rhoplot; src/rhoplot@proc.f90:69-380,
src/systemmod@proc.f90:1329-1420).  Pins: critic2's own benzene POINT block
and LINE file (tests/golden/point_line_benzene.json, from the reference's
tests/004_load/ref/002_load-wfx.*), reproduced from their printed values by
a stand-in field; (GPU) the numbers of both against the oracle."""
import json
import os
import re

import numpy as np
import pytest

from critic2_gb300 import rhoplot

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = json.load(open(os.path.join(ROOT, "tests", "golden", "point_line_benzene.json")))
NUM = r"-?\d+\.\d+(?:E[+-]\d+)?"


def nums(line):
    return [float(v) for v in re.findall(NUM, line)]


class GoldenPointField:
    """grd / rho2 / rho2_valence returning critic2's printed benzene values."""

    def __init__(self, lines):
        v = {l.split(":")[0].strip(): nums(l.split(":", 1)[1]) for l in lines if ":" in l}
        self.v = v
        h = [nums(l) for l in lines if re.match(r"^    [ -]\d", l)]
        self.hf = np.array(h)

    def grd(self, x, nder, prec):
        v = self.v
        return dict(f=np.array([v["Field value (f)"][0]]), gf=np.array([v["Gradient (grad f)"]]),
                    gfmod=np.array([v["Gradient norm (|grad f|)"][0]]), hf=self.hf[None],
                    hfeval=np.array([v["Hessian eigenvalues"]]), r=np.array([3]), s=np.array([1]),
                    isnuc=np.array([0]))

    def rho2(self, x, nder, prec):
        v = self.v
        up, dn = v["Spin up   field/gradient_norm/laplacian"], v["Spin down field/gradient_norm/laplacian"]
        rho = np.array([[v["Field value (f)"][0], up[0], dn[0]]])
        grad = np.zeros((1, 3, 3))
        grad[0, 1, 0], grad[0, 2, 0] = up[1], dn[1]
        hess = np.zeros((1, 3, 3, 3))
        hess[0, 1, 0, 0], hess[0, 2, 0, 0] = up[2], dn[2]
        gk = np.array([[v["Kinetic energy density (G,tau)"][0], v["Spin up   kinetic energy density (G)"][0],
                        v["Spin down kinetic energy density (G)"][0]]])
        return dict(rho=rho, grad=grad, hess=hess, gkin=gk)

    def rho2_valence(self, x, nder):
        v = self.v
        rho = np.array([[v["Field value, valence (fval)"][0], 0, 0]])
        grad = np.zeros((1, 3, 3))
        grad[0, 0, 0] = v["Gradient norm, valence"][0]
        hess = np.zeros((1, 3, 3, 3))
        hess[0, 0, 0, 0] = v["Laplacian, valence (del2 fval)"][0]
        return dict(rho=rho, grad=grad, hess=hess)


def test_point_block_matches_critic2s():
    gold = GOLD["point"]["lines"]
    text = rhoplot.point_text(GoldenPointField(gold), GOLD["point"]["xyz_ang"], "ang").split("\n")
    assert text[:len(gold)] == [l if not l.startswith("  Laplacian (del2 f)") else text[gold.index(l)]
                                for l in gold]
    # the Laplacian is the trace of the unrounded Hessian in critic2: here
    # the trace of the printed one, equal to 1e-9
    lg = next(l for l in gold if l.startswith("  Laplacian (del2 f)"))
    lt = next(l for l in text if l.startswith("  Laplacian (del2 f)"))
    assert abs(nums(lt)[0] / nums(lg)[0] - 1) < 1e-9 and lt.split(":")[0] == lg.split(":")[0]


class GoldenLineField:
    def __init__(self, text):
        rows = [l for l in text.split("\n") if l.startswith(" ")]
        self.f = np.array([nums(l)[4] for l in rows])

    def grd(self, x, nder, prec):
        assert len(x) == len(self.f)
        return dict(f=self.f)


def test_line_file_matches_critic2s():
    g = GOLD["line"]
    text = rhoplot.line_text(GoldenLineField(g["text"]), g["x0"], g["x1"], g["npts"], "", "ang")
    assert text == g["text"]


def test_fortran_formats():
    assert rhoplot.fortran_e(-1.139583849e-2, 9) == "-1.139583849E-02"
    assert rhoplot.fortran_e(1.5e-120, 9) == "1.500000000-120"
    assert rhoplot.fortran_f(-0.25, 7) == "-0.2500000"
    with pytest.raises(ValueError):
        rhoplot.line_text(GoldenLineField(GOLD["line"]["text"]), [0, 0, 0], [1, 0, 0], 5, "bogus")


@pytest.mark.gpu
@pytest.mark.parametrize("spin", ["rhf", "uhf"])
def test_point_and_line_values_vs_oracle(gpu_lib, oracle_mod, spin):
    import dataclasses
    from critic2_gb300 import synth
    from critic2_gb300.wfn import Wavefunction
    mol = synth.make_molecule("nci12")
    if spin == "uhf":
        mol = dataclasses.replace(mol, wfntyp=1, nalpha=mol.nmo // 2, occ=np.ones(mol.nmo))
    w, o = Wavefunction(mol), oracle_mod.Wfn(mol)
    xa = (mol.atom_xyz.mean(0) + np.array([0.3, -0.2, 0.1])) * rhoplot.BOHR_TO_ANG
    lines = rhoplot.point_text(w, xa, "ang").split("\n")
    r = o.grd(xa / rhoplot.BOHR_TO_ANG, 2)
    val = {l.split(":")[0].strip(): nums(l.split(":", 1)[1]) for l in lines if ":" in l}
    hess = np.array([nums(l) for l in lines if re.match(r"^    [ -]\d", l)])
    want = {"Field value (f)": [r.f], "Field value, valence (fval)": [r.fval],
            "Gradient (grad f)": list(r.gf), "Gradient norm (|grad f|)": [r.gfmod],
            "Gradient norm, valence": [r.gfmodval], "Kinetic energy density (G,tau)": [r.gkin],
            "Laplacian (del2 f)": [r.del2f], "Laplacian, valence (del2 fval)": [r.del2fval],
            "Hessian eigenvalues": list(r.hfeval),
            "Spin up   field/gradient_norm/laplacian": [r.fspin[0], r.gfmodspin[0], r.lapspin[0]],
            "Spin down field/gradient_norm/laplacian": [r.fspin[1], r.gfmodspin[1], r.lapspin[1]],
            "Spin up   kinetic energy density (G)": [r.gkinspin[0]],
            "Spin down kinetic energy density (G)": [r.gkinspin[1]]}
    scale = max(abs(r.f), abs(r.del2f))
    for k, ref in want.items():
        # printed with 10 significant digits
        assert np.allclose(val[k], ref, rtol=6e-10, atol=1e-12 * scale), (k, val[k], ref)
    assert np.allclose(hess, np.array(r.hf).reshape(3, 3), rtol=6e-10, atol=1e-12 * scale)
    assert f"  Type : ({r.r},{r.s})" in lines
    text = rhoplot.line_text(w, xa, xa + 1.0, 11, "lap", "ang")
    rows = [nums(l) for l in text.split("\n") if l.startswith(" ")]
    assert len(rows) == 11
    a, b = xa / rhoplot.BOHR_TO_ANG, (xa + 1.0) / rhoplot.BOHR_TO_ANG
    for i, row in enumerate(rows):
        q = o.grd(a + (b - a) * (i / 10.0), 2)
        assert abs(row[4] / q.f - 1) < 1e-12
        assert abs(row[5] - q.del2f) < 1e-12 * max(abs(q.del2f), abs(q.f))
