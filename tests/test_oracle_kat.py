"""Known-answer tests of the oracle's GTO evaluator.

The reference cannot be run here, so the evaluator restatement is pinned by
mathematics: (1) exact symbolic density, gradient and Hessian of small
wavefunctions (sympy), covering every Cartesian type s..h of critic2's li
table (types 1-56); (2) normalisation integrals of normalised primitives by Gauss-Hermite
quadrature (exact for polynomial x Gaussian), which pins the exponent
convention exp(-alpha r^2) and the coefficient layout; (3) finite
differences on a synthetic workload molecule; (4) the primitive cutoff
dran = sqrt(-ln(1e-12)/alpha) and duplicate-primitive pruning.
"""
import math

import numpy as np
import pytest
import sympy as sp

from critic2_gb300 import synth


def tiny_mol(types, alphas, centers, atoms, cmo, occ, wfntyp=0, nalpha=None, z=None):
    atoms = np.asarray(atoms, float)
    return synth.Molecule(atoms, np.asarray(z if z is not None else [8] * len(atoms), np.int32),
                          np.asarray(centers, np.int32), np.asarray(types, np.int32),
                          np.asarray(alphas, float), np.asarray(occ, float),
                          np.ascontiguousarray(np.asarray(cmo, float)), wfntyp=wfntyp,
                          nalpha=len(occ) if nalpha is None else nalpha)


def sym_density(mol):
    x, y, z = sp.symbols("x y z", real=True)
    phis = []
    for m in range(mol.nmo):
        phi = 0
        for i in range(mol.npri):
            lx, ly, lz = (int(v) for v in synth.LI[mol.itype[i] - 1])
            a = mol.atom_xyz[mol.icenter[i] - 1]
            dx, dy, dz = x - a[0], y - a[1], z - a[2]
            phi += mol.cmo[i, m] * dx ** lx * dy ** ly * dz ** lz * sp.exp(-mol.e[i] * (dx ** 2 + dy ** 2 + dz ** 2))
        phis.append(phi)
    rho = sum(mol.occ[m] * phis[m] ** 2 for m in range(mol.nmo))
    X = (x, y, z)
    grad = [sp.diff(rho, v) for v in X]
    hess = [[sp.diff(rho, u, v) for v in X] for u in X]
    return sp.lambdify(X, [rho] + grad + [h for row in hess for h in row], "math")


@pytest.mark.parametrize("types", [[1], [2, 3, 4], list(range(5, 11)), list(range(11, 21)),
                                   [1, 2, 7, 9, 12, 20], list(range(21, 36)), list(range(36, 57))])
def test_symbolic_density(oracle_mod, types):
    rng = np.random.default_rng(len(types))
    n = len(types)
    atoms = [[0.1, -0.2, 0.3], [1.4, 0.5, -0.6]]
    centers = [1 + (i % 2) for i in range(n)]
    alphas = rng.uniform(0.3, 2.0, n)
    cmo = rng.standard_normal((n, 2))
    mol = tiny_mol(types, alphas, centers, atoms, cmo, [2.0, 2.0])
    f = sym_density(mol)
    w = oracle_mod.Wfn(mol)
    for p in rng.uniform(-1.5, 2.0, size=(6, 3)):
        ref = np.array(f(*p))
        out = w.rho2(p, 2)
        got = np.concatenate([[out["rho"][0]], out["grad"][0], out["h"][0].T.reshape(-1)])
        scale = np.abs(ref).max()
        assert np.allclose(got, ref, rtol=1e-11, atol=1e-13 * scale), (p, got - ref)


def gnorm(lx, ly, lz, a):
    """Normalisation of x^l y^m z^n exp(-a r^2)."""
    df = lambda k: 1 if k <= 0 else k * df(k - 2)
    L = lx + ly + lz
    return math.sqrt((2 * a / math.pi) ** 1.5 * (4 * a) ** L / (df(2 * lx - 1) * df(2 * ly - 1) * df(2 * lz - 1)))


@pytest.mark.parametrize("itype", [1, 2, 5, 8, 11, 14, 20])
def test_normalisation_integral(oracle_mod, itype):
    a = 0.8
    lx, ly, lz = (int(v) for v in synth.LI[itype - 1])
    N = gnorm(lx, ly, lz, a)
    mol = tiny_mol([itype], [a], [1], [[0.0, 0.0, 0.0]], [[N]], [2.0])
    w = oracle_mod.Wfn(mol)
    t, wt = np.polynomial.hermite.hermgauss(12)
    s = 1.0 / math.sqrt(2 * a)  # rho ~ exp(-2 a r^2)
    X, Y, Z = np.meshgrid(t * s, t * s, t * s, indexing="ij")
    W = np.einsum("i,j,k->ijk", wt, wt, wt) * s ** 3
    pts = np.stack([X, Y, Z], -1).reshape(-1, 3)
    rho, _, _ = w.rho2_points(pts, 0)
    integral = np.sum(W.reshape(-1) * rho / np.exp(-2 * a * np.sum(pts ** 2, 1)))
    assert math.isclose(integral, 2.0, rel_tol=1e-12)


def test_finite_differences(oracle_mod):
    mol = synth.make_molecule("nci12")
    w = oracle_mod.Wfn(mol)
    rng = np.random.default_rng(5)
    h = 1e-4
    for p in rng.uniform(2.0, 10.0, size=(5, 3)):
        out = w.rho2(p, 2)
        g = out["grad"][0]
        H = out["h"][0].T
        for d in range(3):
            e = np.zeros(3); e[d] = h
            rp, rm = w.rho2(p + e, 1), w.rho2(p - e, 1)
            fd_g = (rp["rho"][0] - rm["rho"][0]) / (2 * h)
            fd_h = (rp["grad"][0] - rm["grad"][0]) / (2 * h)
            assert math.isclose(fd_g, g[d], rel_tol=1e-6, abs_tol=1e-7 * abs(out["rho"][0]))
            assert np.allclose(fd_h, H[:, d], rtol=1e-5, atol=1e-6 * np.abs(H).max())


def test_cutoff_and_pruning(oracle_mod):
    a = 2.0
    dran = math.sqrt(-math.log(1e-12) / a)
    mol = tiny_mol([1], [a], [1], [[0.0, 0.0, 0.0]], [[1.0]], [2.0])
    w = oracle_mod.Wfn(mol)
    inside = w.rho2(np.array([dran * 0.999, 0, 0]), 0)["rho"][0]
    outside = w.rho2(np.array([dran * 1.001, 0, 0]), 0)["rho"][0]
    assert inside > 0 and math.isclose(inside, 2 * math.exp(-2 * a * (dran * 0.999) ** 2), rel_tol=1e-12)
    assert outside == 0.0
    # two identical primitives merge into one with the summed coefficients
    m2 = tiny_mol([1, 1, 2], [a, a, 1.0], [1, 1, 1], [[0.0, 0.0, 0.0]], [[0.3, 1.0], [0.7, -0.5], [0.2, 0.1]], [2.0, 1.0])
    m1 = tiny_mol([1, 2], [a, 1.0], [1, 1], [[0.0, 0.0, 0.0]], [[1.0, 0.5], [0.2, 0.1]], [2.0, 1.0])
    w2, w1 = oracle_mod.Wfn(m2), oracle_mod.Wfn(m1)
    assert w2.npri == 2
    p = np.array([0.3, -0.2, 0.1])
    assert np.allclose(w2.rho2(p, 2)["h"], w1.rho2(p, 2)["h"], rtol=1e-14)


def test_spin_channels_uhf_rohf(oracle_mod):
    rng = np.random.default_rng(9)
    types = [1, 2, 3, 4, 5]
    cmo = rng.standard_normal((5, 3))
    atoms = [[0.0, 0.0, 0.0]]
    p = np.array([0.2, 0.4, -0.1])
    uhf = oracle_mod.Wfn(tiny_mol(types, [1.0] * 5, [1] * 5, atoms, cmo, [1.0, 1.0, 1.0], wfntyp=1, nalpha=2))
    o = uhf.rho2(p, 2)
    assert math.isclose(o["rho"][1] + o["rho"][2], o["rho"][0], rel_tol=1e-14)
    rohf = oracle_mod.Wfn(tiny_mol(types, [1.0] * 5, [1] * 5, atoms, cmo, [2.0, 2.0, 1.0], wfntyp=2, nalpha=2))
    o = rohf.rho2(p, 2)
    assert math.isclose(o["rho"][1], o["rho"][0], rel_tol=1e-14)


def test_nuclear_gradient_rule(oracle_mod):
    """grd zeroes the gradient within 1e-5 bohr of a nucleus."""
    mol = synth.make_molecule("nci12")
    w = oracle_mod.Wfn(mol)
    r = w.grd(mol.atom_xyz[0] + 1e-6, 2)
    assert r.isnuc == 1 and r.gfmod == 0.0
    r = w.grd(mol.atom_xyz[0] + 1e-4, 2)
    assert r.isnuc == 0 and r.gfmod > 0.0
