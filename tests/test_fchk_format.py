"""Gaussian formatted checkpoint files (read_fchk, src/wfn_private@proc.F90:
1287-1812).  Pins: the library's spherical -> Cartesian matrices, derived
from the real solid harmonics, against critic2's own dsphcar / fsphcar /
gsphcar_fchk (parsed from the reference source into tests/golden); unit
norm of every normalised pure and Cartesian function of the restated
reader; and (GPU) the library's reader against the restatement, and the
integral of a one-function density over a molecular mesh."""
import json
import os
import re

import numpy as np
import pytest

from critic2_gb300 import synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_derived_matrices_equal_critic2s():
    gold = json.load(open(os.path.join(ROOT, "tests", "golden", "sphcar_fchk.json")))
    text = open(os.path.join(ROOT, "critic2_gb300", "csrc", "sphcar_tables.h")).read()
    for name, key in (("kSphCar2[", "2"), ("kSphCar3[", "3"), ("kSphCar4[", "4"), ("kSphCar4Molden[", "4molden")):
        body = text.split(name)[1].split("};")[0]
        T = np.array([[float(v) for v in r.split(",")] for r in re.findall(r"\{([^{}]+)\}", body)])
        assert np.array_equal(T, np.array(gold[key])), key


def dfm1(n):
    r = 1
    for k in range(n - 1, 1, -2):
        r *= k
    return r


def overlap(e1, e2, a1, a2):
    """<x^e1 exp(-a1 r^2) | x^e2 exp(-a2 r^2)> on one centre."""
    e = [p + q for p, q in zip(e1, e2)]
    if any(v % 2 for v in e):
        return 0.0
    L = sum(e) // 2
    return dfm1(e[0]) * dfm1(e[1]) * dfm1(e[2]) * np.pi ** 1.5 / (2 ** L * (a1 + a2) ** (L + 1.5))


@pytest.mark.parametrize("spin", ["rhf", "uhf", "rohf"])
def test_restated_reader_functions_are_normalised(oracle_mod, tmp_path, spin):
    # one atom, one shell of each type, MO k = basis function k: every MO
    # density then integrates to one electron per occupation
    b = synth.make_shell_basis(3, natom=1, spin=spin)
    nb = b.nbas
    b.moa = np.eye(nb)
    if b.mob is not None:
        b.mob = np.eye(nb)
    # every basis function occupied (alpha and beta in UHF, nb MOs in ROHF)
    b.nalpha, b.nbeta = nb, (nb - 3 if spin == "rohf" else nb)
    b.nelec = b.nalpha + b.nbeta
    p = str(tmp_path / "m.fchk")
    synth.write_fchk(b, p)
    r = oracle_mod.read_fchk_text(p)
    LI = synth.LI
    e, t, C = r["e"], r["itype"], r["cmo"]
    for m in range(C.shape[1]):
        nz = np.nonzero(C[:, m])[0]
        s = sum(C[i, m] * C[j, m] * overlap(LI[t[i] - 1], LI[t[j] - 1], e[i], e[j]) for i in nz for j in nz)
        assert abs(s - 1.0) < 1e-7, (m, s)  # E16.8 exponents and coefficients


def test_restated_reader_structure(oracle_mod, tmp_path):
    b = synth.make_shell_basis(1)
    p = str(tmp_path / "m.fchk")
    synth.write_fchk(b, p)
    r = oracle_mod.read_fchk_text(p)
    ncart = {0: 1, 1: 3, -1: 4, 2: 6, -2: 6, 3: 10, -3: 10, 4: 15, -4: 15}
    assert len(r["e"]) == sum(ncart[s[0]] * len(s[2]) for s in b.shells)
    assert r["cmo"].shape[1] == b.nelec // 2 and r["wfntyp"] == 0


@pytest.mark.gpu
@pytest.mark.parametrize("spin", ["rhf", "uhf", "rohf"])
def test_library_reader_vs_restatement(gpu_lib, oracle_mod, tmp_path, spin):
    from critic2_gb300.wfn import Wavefunction
    b = synth.make_shell_basis(2, spin=spin)
    p = str(tmp_path / "m.fchk")
    synth.write_fchk(b, p)
    r = oracle_mod.read_fchk_text(p)
    mol = synth.Molecule(r["atom_xyz"], r["atom_z"], r["icenter"], r["itype"], r["e"], r["occ"],
                         np.ascontiguousarray(r["cmo"]), wfntyp=r["wfntyp"], nalpha=r["nalpha"], name="fchk")
    g1, g2 = Wavefunction.from_fchk(p), Wavefunction(mol)
    assert (g1.natom, g1.npri, g1.nmo, g1.wfntyp, g1.nalpha) == (g2.natom, g2.npri, g2.nmo, g2.wfntyp, g2.nalpha)
    pts = np.random.default_rng(5).uniform(b.atom_xyz.min(0) - 1, b.atom_xyz.max(0) + 1, (128, 3))
    a, c = g1.rho2(pts, 2, "fp64"), g2.rho2(pts, 2, "fp64")
    for k in ("rho", "grad", "hess"):
        assert np.allclose(a[k], c[k], rtol=1e-12, atol=1e-14 * np.abs(c[k]).max())


@pytest.mark.gpu
def test_pure_shell_densities_integrate_to_occupations(gpu_lib, tmp_path):
    """One atom with pure d, f and g shells, one MO per spherical function:
    the integral of rho over the molecular mesh is the electron count."""
    from critic2_gb300.wfn import Wavefunction
    b = synth.make_shell_basis(4, natom=1, types=(-2, -3, -4))
    nb = b.nbas  # 5 + 7 + 9
    b.moa = np.eye(nb)
    b.nelec, b.nalpha, b.nbeta = 2 * nb, nb, nb
    b.atom_z[:] = 8
    p = str(tmp_path / "pure.fchk")
    synth.write_fchk(b, p)
    g = Wavefunction.from_fchk(p)
    r = g.molcalc(("rho",), "franchini", "vgood", "fp64")
    assert abs(r["rho"] / (2 * nb) - 1) < 1e-5
