"""Molecular meshes in the oracle (genmesh_becke / genmesh_franchini,
src/meshmod@proc.f90:79-627) and the Lebedev rules they use.  Pins: the
mesh sizes critic2 reports for benzene (tests/004_load/ref/002_load-wfx.cro:
"Mesh size 219252", Franchini, good; tests/011_mesh/ref/001_meshtype.cro:
55440, Franchini and Becke, small), the exactness of the angular rules,
the library's compressed Lebedev table against the fixture, and the
convergence of the integral of a normalised Gaussian density."""
import itertools
import math
import os
import re

import numpy as np
import pytest

from critic2_gb300 import synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DEG = {110: 17, 194: 23, 302: 29, 590: 41, 770: 47}


def dfact(n):
    r = 1
    while n > 1:
        r *= n
        n -= 2
    return r


def benzene_like(cmo_atom=0, alpha=0.7, c=1.3):
    ang = np.arange(6) * np.pi / 3
    xyz = np.vstack([np.c_[2.64 * np.cos(ang), 2.64 * np.sin(ang), np.zeros(6)],
                     np.c_[4.68 * np.cos(ang), 4.68 * np.sin(ang), np.zeros(6)]])
    z = np.array([6] * 6 + [1] * 6, np.int32)
    cmo = np.zeros((12, 1))
    cmo[cmo_atom, 0] = c
    return synth.Molecule(xyz, z, np.arange(1, 13, dtype=np.int32), np.ones(12, np.int32), np.full(12, alpha),
                          np.array([2.0]), cmo, name="benzene-like")


@pytest.mark.parametrize("n", sorted(DEG))
def test_lebedev_exactness(oracle_mod, n):
    r = oracle_mod.lebedev_rule(n)
    assert r.shape == (n, 4) and np.all(r[:, 3] > 0)
    assert np.allclose(np.linalg.norm(r[:, :3], axis=1), 1.0, atol=1e-14)
    deg = DEG[n]
    rng = np.random.default_rng(n)
    for _ in range(60):  # random monomials up to the rule's degree
        a, b, c = (int(v) for v in rng.integers(0, deg + 1, 3))
        if a + b + c > deg:
            continue
        val = np.sum(r[:, 3] * r[:, 0] ** a * r[:, 1] ** b * r[:, 2] ** c)
        exact = 0.0 if (a % 2 or b % 2 or c % 2) else \
            dfact(a - 1) * dfact(b - 1) * dfact(c - 1) / dfact(a + b + c + 1)
        assert abs(val - exact) < 1e-14


def test_library_table_matches_fixture(oracle_mod):
    text = open(os.path.join(ROOT, "critic2_gb300", "csrc", "lebedev_tables.h")).read()
    for n in DEG:
        body = text.split(f"kLebedev{n}[] = {{")[1].split("};")[0]
        orbs = [tuple(map(float, m)) for m in re.findall(r"\{([^,{}]+), ([^,{}]+), ([^,{}]+), ([^,{}]+)\}", body)]
        pts = set()
        for a, b, c, w in orbs:
            for p in itertools.permutations((a, b, c)):
                for s in itertools.product((1, -1), repeat=3):
                    pts.add(tuple(round(s[k] * p[k] + 0.0, 13) for k in range(3)) + (round(w, 15),))
        ref = {tuple(round(v + 0.0, 13) for v in q[:3]) + (round(q[3], 15),) for q in oracle_mod.lebedev_rule(n)}
        assert pts == ref


def test_mesh_size_of_benzene(oracle_mod):
    # critic2: "Mesh size 219252", Franchini, good, for benzene (6 C, 6 H)
    # (tests/004_load/ref/002_load-wfx.cro), and "Mesh size 55440" for
    # Franchini and Becke, small (tests/011_mesh/ref/001_meshtype.cro)
    w = oracle_mod.Wfn(benzene_like())
    xyz, wt = w.mesh("franchini", "good")
    assert len(wt) == 219252
    for mesh in ("franchini", "becke"):
        assert len(w.mesh(mesh, "small")[1]) == 55440
    assert oracle_mod.lib().o_z2nr(1, 3) == 52 and oracle_mod.lib().o_z2nr(6, 3) == 69


@pytest.mark.parametrize("mesh", ["franchini", "becke"])
def test_gaussian_integral_converges(oracle_mod, mesh):
    exact = 2 * 1.3 ** 2 * (math.pi / (2 * 0.7)) ** 1.5
    errs = {}
    for atom in (0, 8):  # centred on a C and on an H
        w = oracle_mod.Wfn(benzene_like(atom))
        for lvl, tol in (("small", 3e-5), ("normal", 3e-6), ("good", 3e-7)):
            r = w.molcalc(("rho",), mesh, lvl)
            errs[(atom, lvl)] = abs(r["rho"] / exact - 1)
            assert errs[(atom, lvl)] < tol, (atom, lvl, errs[(atom, lvl)])


def test_mesh_order_and_weights(oracle_mod):
    mol = benzene_like()
    w = oracle_mod.Wfn(mol)
    xyz, wt = w.mesh("franchini", "small")
    nang = 110
    # atoms in order, shells of increasing radius, nang points per shell
    r = np.linalg.norm(xyz[:nang * 36] - mol.atom_xyz[0], axis=1).reshape(36, nang)
    assert np.allclose(r, r[:, :1], rtol=1e-13)
    assert np.all(np.diff(r[:, 0]) > 0)
    assert np.all(wt >= 0)
