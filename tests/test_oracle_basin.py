"""Basin integration by bisection (critic2's INTEGRALS, molecules): the
oracle's restatement on a two-center density whose nuclei are its only
maxima, and the library's Lebedev tables for every size critic2's
good_lebedev offers.  No GPU."""
import itertools
import os
import re

import numpy as np
import pytest

from critic2_gb300 import synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# Lebedev-Laikov rule size -> polynomial degree
LEB_DEG = {6: 3, 14: 5, 26: 7, 38: 9, 50: 11, 74: 13, 86: 15, 110: 17, 146: 19, 170: 21, 194: 23, 230: 25,
           266: 27, 302: 29, 350: 31, 434: 35, 590: 41, 770: 47, 974: 53, 1202: 59, 1454: 65, 1730: 71, 2030: 77,
           2354: 83, 2702: 89, 3074: 95, 3470: 101, 3890: 107, 4334: 113, 4802: 119, 5294: 125, 5810: 131}


def dfact(n):
    r = 1
    while n > 1:
        r *= n
        n -= 2
    return r


def library_rule(n):
    """The n-point rule of lebedev_tables.h, expanded from its orbits."""
    text = open(os.path.join(ROOT, "critic2_gb300", "csrc", "lebedev_tables.h")).read()
    body = text.split(f"kLebedev{n}[] = {{")[1].split("};")[0]
    orbs = [tuple(map(float, m)) for m in re.findall(r"\{([^,{}]+), ([^,{}]+), ([^,{}]+), ([^,{}]+)\}", body)]
    pts = {}
    for a, b, c, w in orbs:
        for p in itertools.permutations((a, b, c)):
            for s in itertools.product((1, -1), repeat=3):
                q = tuple(s[k] * p[k] + 0.0 for k in range(3))
                pts[tuple(round(v, 13) for v in q)] = q + (w,)
    return np.array(list(pts.values()))


@pytest.mark.parametrize("n", sorted(LEB_DEG))
def test_library_lebedev_rules(n):
    """Every rule: n distinct unit points, weights summing to 1 (the 74-point
    rule has one negative orbit weight), exact on monomials up to its
    degree (mean over the sphere)."""
    r = library_rule(n)
    assert r.shape == (n, 4) and np.all(r[:, 3] != 0)
    assert abs(r[:, 3].sum() - 1.0) < 1e-13
    assert np.allclose(np.linalg.norm(r[:, :3], axis=1), 1.0, atol=1e-14)
    deg = LEB_DEG[n]
    rng = np.random.default_rng(n)
    for _ in range(40):
        a, b, c = (int(v) for v in rng.integers(0, deg + 1, 3))
        if a + b + c > deg:
            continue
        val = np.sum(r[:, 3] * r[:, 0] ** a * r[:, 1] ** b * r[:, 2] ** c)
        exact = 0.0 if (a % 2 or b % 2 or c % 2) else \
            dfact(a - 1) * dfact(b - 1) * dfact(c - 1) / dfact(a + b + c + 1)
        assert abs(val - exact) < 2e-14


def diatomic(d=2.2):
    """Two centers with a tight and a diffuse s primitive each, two doubly
    occupied MOs: the nuclei are the density's only maxima."""
    xyz = np.array([[0, 0, 0], [0, 0, d]], float)
    e = np.array([6.0, 0.45, 4.0, 0.35])
    cmo = np.array([[0.9, 0.0], [0.35, 0.3], [0.0, 0.8], [0.3, 0.35]])
    return synth.Molecule(xyz, np.array([7, 8], np.int32), np.array([1, 1, 2, 2], np.int32), np.ones(4, np.int32),
                          e, np.array([2.0, 2.0]), cmo, name="diatomic")


def total_density(mol):
    """Integral of rho for s primitives (closed form)."""
    tot = 0.0
    ic = mol.icenter - 1
    for m in range(mol.nmo):
        for i in range(mol.npri):
            for j in range(mol.npri):
                a, b = mol.e[i], mol.e[j]
                r2 = np.sum((mol.atom_xyz[ic[i]] - mol.atom_xyz[ic[j]]) ** 2)
                tot += mol.occ[m] * mol.cmo[i, m] * mol.cmo[j, m] * (np.pi / (a + b)) ** 1.5 * \
                    np.exp(-a * b / (a + b) * r2)
    return tot


def lebedev_rays(oracle_mod, n):
    """Directions rebuilt from (theta, phi) as critic2 does, weights x 4 pi."""
    r = oracle_mod.lebedev_rule(n)
    th, ph = np.arccos(r[:, 2]), np.arctan2(r[:, 1], r[:, 0])
    return np.c_[np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)], r[:, 3] * 4 * np.pi


def gauleg_rays(ntheta, nphi):
    """gauleg_nodes: directions, azimuthal weights, ring index, ring factor."""
    q, wq = np.polynomial.legendre.leggauss(ntheta)
    th, tw = 0.5 * np.pi * (q + 1), 0.5 * np.pi * wq
    u, wa, ring = [], [], []
    for t in range(ntheta):
        npp = int(nphi * abs(np.sin(th[t]))) + 1
        p, wp = np.polynomial.legendre.leggauss(npp)
        for k in range(npp):
            ph = np.pi * (p[k] + 1)
            u.append([np.sin(th[t]) * np.cos(ph), np.sin(th[t]) * np.sin(ph), np.cos(th[t])])
            wa.append(np.pi * wp[k])
            ring.append(t)
    return np.array(u), np.array(wa), np.array(ring, np.int32), np.sin(th) * tw


@pytest.fixture(scope="module")
def di(oracle_mod):
    mol = diatomic()
    w = oracle_mod.Wfn(mol)
    cpx, cpt = mol.atom_xyz.copy(), np.array([-3, -3], np.int32)
    us, ws = lebedev_rays(oracle_mod, 170)
    return mol, w, cpx, cpt, us, ws


def test_basin_populations_add_up(oracle_mod, di):
    """The two basins hold the molecule's density (the angular rule over a
    surface with an edge limits this to ~3e-4) without a beta-sphere
    restart; the surface crosses the bond where the density along it is
    smallest."""
    mol, w, cpx, cpt, us, ws = di
    u, wu = lebedev_rays(oracle_mod, 590)
    r = w.basin_integrals(cpx, cpt, u, wu, us, ws)
    assert list(r["att_cp"]) == [0, 1]
    assert r["nrestart"] == 0
    tot = total_density(mol)
    assert abs(r["props"][:, 0].sum() - tot) < 3e-4 * tot
    # the zero-flux surface between the two centers lies where the
    # density along the axis has its minimum
    z = np.linspace(0.3, 1.9, 4001)
    rho = np.array([w.grd(np.array([0.0, 0.0, zz]), 0).f for zz in z])
    zmin = z[np.argmin(rho)]
    up = np.argmax(u[:, 2])
    assert abs(r["rsurf"][0, up] - zmin) < 2e-3
    assert abs(r["rsurf"][0, up] + r["rsurf"][1, np.argmin(u[:, 2])] - 2.2) < 2e-5


def test_basin_serial_statistics_vs_parallel_tries(oracle_mod, di):
    """critic2's serial bracket statistics against every ray taking the
    first ray's tries.  The inside/outside test along a ray is not monotonic
    everywhere (paths from near the bond saddle can bounce and end away from
    every attractor; where the gradient falls under gradeps, 1e-7, a path
    starts as a "new CP"), so the two brackets can settle on crossings
    ~2e-4 bohr apart; most rays agree to twice the IAS precision, and the
    integrals to 1e-6 (Pop) and 2e-5 (Lap, absolute)."""
    mol, w, cpx, cpt, us, ws = di
    u, wu = lebedev_rays(oracle_mod, 110)
    a = w.basin_integrals(cpx, cpt, u, wu, us, ws, stats=True)
    b = w.basin_integrals(cpx, cpt, u, wu, us, ws, stats=False)
    d = np.abs(a["rsurf"] - b["rsurf"])
    assert np.mean(d <= 2e-5) >= 0.95
    assert d.max() <= 1e-3
    assert np.allclose(a["props"][:, 0], b["props"][:, 0], rtol=1e-6)
    assert np.allclose(a["props"][:, 1], b["props"][:, 1], atol=2e-5)


def test_basin_gauleg_vs_lebedev(oracle_mod, di):
    """GAULEG and LEBEDEV angular rules give the same basins."""
    mol, w, cpx, cpt, us, ws = di
    u, wu = lebedev_rays(oracle_mod, 590)
    a = w.basin_integrals(cpx, cpt, u, wu, us, ws)
    gu, gw, ring, ringw = gauleg_rays(30, 40)
    b = w.basin_integrals(cpx, cpt, gu, gw, us, ws, ring=ring, ringw=ringw)
    assert np.allclose(a["props"][:, 0], b["props"][:, 0], rtol=2e-4)


def test_basin_single_cp(oracle_mod, di):
    mol, w, cpx, cpt, us, ws = di
    u, wu = lebedev_rays(oracle_mod, 110)
    a = w.basin_integrals(cpx, cpt, u, wu, us, ws)
    b = w.basin_integrals(cpx, cpt, u, wu, us, ws, cpid=2)
    assert list(b["att_cp"]) == [1]
    assert np.allclose(b["props"][0], a["props"][1], rtol=1e-12)


def test_sphere_integrals_one_center(oracle_mod):
    """SPHEREINTEGRALS around a lone s-type center, rho = occ c^2 exp(-b r^2)
    (b = 2 alpha): Pop = 4 pi occ c^2 int_0^R r^2 exp(-b r^2) dr (erf form)
    and Lap = 4 pi R^2 rho'(R), the flux through the sphere."""
    from math import erf
    a, c, occ = 0.8, 1.3, 2.0
    mol = synth.Molecule(np.zeros((1, 3)), np.array([6], np.int32), np.array([1], np.int32), np.ones(1, np.int32),
                         np.array([a]), np.array([occ]), np.array([[c]]), name="one")
    w = oracle_mod.Wfn(mol)
    u, wu = lebedev_rays(oracle_mod, 110)
    r = w.sphere_integrals(np.zeros((1, 3)), np.array([-3], np.int32), u, wu, nr=6, r0=0.1, rend=3.0)
    b = 2 * a
    for R, (pop, lap) in zip(r["radii"][0], r["props"][0]):
        ref = 4 * np.pi * occ * c * c * (np.sqrt(np.pi) / (4 * b ** 1.5) * erf(np.sqrt(b) * R)
                                         - R / (2 * b) * np.exp(-b * R * R))
        rho_r = occ * c * c * np.exp(-b * R * R)
        assert abs(pop - ref) <= 1e-10 * abs(ref)
        assert abs(lap - 4 * np.pi * R * R * (-2 * b * R) * rho_r) <= 1e-9 * abs(4 * np.pi * R * R * 2 * b * R * rho_r)
    assert np.allclose(r["radii"][0], 0.1 * np.exp(np.arange(6) * np.log(30.0) / 5), rtol=1e-14)


def test_sphere_quadrature_golden(oracle_mod):
    """critic2's SPHEREINTEGRALS regression output (a crystal field, so only
    its field-independent columns, tests/golden/make_sphere_golden.py): the
    logarithmic radii r0 exp(h (n - 1)) and each sphere's volume, the
    angular rule's weight sum times r^3 / 3, for GAULEG 2 2 and LEBEDEV 6.
    The oracle's radii and this file's GAULEG and Lebedev weights (the ones
    the GPU tests hold the library's rays and integrals to) reproduce them
    to the printed digits."""
    import json
    gold = json.load(open(os.path.join(ROOT, "tests", "golden", "sphere_quadrature.json")))
    mol = diatomic()
    w = oracle_mod.Wfn(mol)
    cpx, cpt = mol.atom_xyz.copy(), np.array([-3, -3], np.int32)
    for b in gold["blocks"]:
        if b["angular"] == "gauleg":
            u, wa, ring, ringw = gauleg_rays(b["ntheta"], b["nphi"])
            wsum = float(np.sum(ringw[ring] * wa))
            kw = dict(ring=ring, ringw=ringw)
        else:
            u, wu = lebedev_rays(oracle_mod, b["nleb"])
            wa, wsum, kw = wu, float(np.sum(wu)), {}
        r = w.sphere_integrals(cpx, cpt, u, wa, cpid=1, nr=b["nr"], r0=b["r0"], rend=b["rend"], **kw)
        radii = r["radii"][0]
        assert abs(np.log(b["rend"] / b["r0"]) / (b["nr"] - 1) - b["h"]) <= 1e-6 * b["h"]
        for row, rr in zip(b["rows"], radii):
            assert abs(rr - row["r"]) <= 1e-6 * row["r"]
            assert abs(wsum * rr ** 3 / 3.0 - row["volume"]) <= 1e-8 * row["volume"]


@pytest.mark.parametrize("n", [6, 14, 26, 110, 170, 194, 302, 590, 770])
def test_library_lebedev_matches_fixture(oracle_mod, n):
    """The library's tables (lebedev_tables.h) and the independently
    generated rules of tests/golden/lebedev_rules.json (the oracle's) hold
    the same points and weights."""
    lib = library_rule(n)
    ref = oracle_mod.lebedev_rule(n)
    d = np.linalg.norm(lib[:, None, :3] - ref[None, :, :3], axis=2)
    j = d.argmin(1)
    assert d.min(1).max() < 1e-13 and len(set(j)) == n
    assert np.allclose(lib[:, 3], ref[j, 3], rtol=1e-12, atol=1e-15)
