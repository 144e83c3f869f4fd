"""EDF core density in the oracle (calculate_edf and its use in rho2,
src/wfn_private@proc.F90:3275-3369, 2626-2677; cutoffs :3750-3776).

The reference's own tests carry no wavefunction with EDF primitives, so the
restatement is pinned by known answers: the analytic value of single EDF
primitives of s, p and d type, central finite differences for the gradient
and Hessian, the spin-channel rules, the cutoff radius sqrt(-ln(1e-12)/a)
and the widening of the atom's environment radius it causes."""
import dataclasses
import math

import numpy as np
import pytest

from critic2_gb300 import synth

THRES = 1e-12


def one_atom(edf_types, edf_e, edf_c, mo_exp=0.8, wfntyp=0):
    """One atom at (0.3, -0.2, 0.1) with a single s MO primitive and the
    given EDF primitives."""
    xyz = np.array([[0.3, -0.2, 0.1]])
    n = len(edf_e)
    occ = np.array([2.0]) if wfntyp == 0 else np.array([1.0])
    return synth.Molecule(xyz, np.array([8], np.int32), np.array([1], np.int32), np.array([1], np.int32),
                          np.array([mo_exp]), occ, np.array([[0.7]]), wfntyp=wfntyp, nalpha=1,
                          name="edf1", edf_icenter=np.ones(n, np.int32),
                          edf_itype=np.array(edf_types, np.int32), edf_e=np.array(edf_e, float),
                          edf_c=np.array(edf_c, float))


def core_analytic(mol, x):
    val = 0.0
    for a, t, e, c in zip(mol.edf_icenter, mol.edf_itype, mol.edf_e, mol.edf_c):
        d = x - mol.atom_xyz[a - 1]
        r = math.sqrt(d @ d)
        if r > math.sqrt(-math.log(THRES) / e):
            continue
        lx, ly, lz = synth.LI[t - 1]
        val += c * d[0] ** lx * d[1] ** ly * d[2] ** lz * math.exp(-e * r * r)
    return val


def no_edf(mol):
    return dataclasses.replace(mol, edf_icenter=None, edf_itype=None, edf_e=None, edf_c=None)


@pytest.mark.parametrize("types", [(1,), (1, 2, 3, 4), (1, 5, 6, 7, 8, 9, 10)])
def test_core_value_known_answer(oracle_mod, types):
    rng = np.random.default_rng(len(types))
    e = list(np.exp(rng.uniform(np.log(1.0), np.log(40.0), len(types))))
    c = list(rng.uniform(-2.0, 5.0, len(types)))
    # d-type EDFs need an atom with MO lmax >= 2 in critic2: give it d MOs
    mol = one_atom(types, e, c)
    if max(max(synth.LI[t - 1]) for t in types) >= 1:
        lm = max(max(synth.LI[t - 1]) for t in types)
        mt = [t for t in range(1, 11) if max(synth.LI[t - 1]) <= lm]
        mol = dataclasses.replace(mol, icenter=np.ones(len(mt), np.int32), itype=np.array(mt, np.int32),
                                  e=np.full(len(mt), 0.8), cmo=np.full((len(mt), 1), 0.7))
    w, w0 = oracle_mod.Wfn(mol), oracle_mod.Wfn(no_edf(mol))
    for k in range(40):
        x = mol.atom_xyz[0] + rng.uniform(-0.8, 0.8, 3)
        core = w.rho2(x, 0)["rho"][0] - w0.rho2(x, 0)["rho"][0]
        ref = core_analytic(mol, x)
        assert abs(core - ref) <= 1e-12 * max(1.0, abs(ref))


def test_core_derivatives_finite_difference(oracle_mod):
    mol = one_atom([1, 1, 2, 5, 8], [3.0, 0.9, 1.7, 2.2, 1.1], [4.0, 1.5, -0.6, 0.8, 0.3])
    mt = list(range(1, 11))
    mol = dataclasses.replace(mol, icenter=np.ones(10, np.int32), itype=np.array(mt, np.int32),
                              e=np.full(10, 0.8), cmo=np.zeros((10, 1)))
    w = oracle_mod.Wfn(mol)  # zero MO coefficients: the density is the core alone
    rng = np.random.default_rng(7)
    h = 1e-4
    for k in range(10):
        x = mol.atom_xyz[0] + rng.uniform(-0.6, 0.6, 3)
        r = w.rho2(x, 2)
        g = np.asarray(r["grad"]).reshape(-1)[:3]
        H = np.asarray(r["h"]).reshape(-1)[:9].reshape(3, 3)
        for j in range(3):
            dx = np.zeros(3)
            dx[j] = h
            rp, rm = w.rho2(x + dx, 2), w.rho2(x - dx, 2)
            fd = (rp["rho"][0] - rm["rho"][0]) / (2 * h)
            assert abs(fd - g[j]) <= 1e-6 * max(1.0, np.abs(g).max())
            fdh = (np.asarray(rp["grad"]).reshape(-1)[:3] - np.asarray(rm["grad"]).reshape(-1)[:3]) / (2 * h)
            assert np.allclose(fdh, H[:, j], rtol=0, atol=1e-5 * max(1.0, np.abs(H).max()))


def test_spin_channels(oracle_mod):
    base = synth.make_molecule("nci12", seed=3)
    mol = synth.add_edf(base, seed=5, lmax=1)
    uhf = dataclasses.replace(mol, wfntyp=1, nalpha=mol.nmo // 2, occ=np.ones(mol.nmo))
    rng = np.random.default_rng(1)
    heavy = np.nonzero(mol.atom_z != 1)[0]
    for m in (mol, uhf):
        w, w0 = oracle_mod.Wfn(m), oracle_mod.Wfn(no_edf(m))
        for k in range(12):
            x = mol.atom_xyz[heavy[k % len(heavy)]] + rng.uniform(-0.5, 0.5, 3)
            r, r0 = w.rho2(x, 2), w0.rho2(x, 2)
            core = r["rho"][0] - r0["rho"][0]
            assert core > 0.0
            # valence fields are the EDF-free ones
            assert np.allclose(r["rhoval"], r0["rhoval"], rtol=1e-14, atol=0)
            for s in (1, 2):
                assert abs((r["rho"][s] - r0["rho"][s]) - 0.5 * core) <= 1e-12 * abs(r["rho"][0])
            gc = np.asarray(r["grad"]).reshape(-1)[:3] - np.asarray(r0["grad"]).reshape(-1)[:3]
            for s in (1, 2):
                gs = np.asarray(r["grad"]).reshape(-1)[3 * s:3 * s + 3] - np.asarray(r0["grad"]).reshape(-1)[3 * s:3 * s + 3]
                assert np.allclose(gs, 0.5 * gc, rtol=1e-10, atol=1e-12 * np.abs(r["grad"]).max())
            # kinetic energy density and stress carry no core part
            assert np.allclose(r["gkin"], r0["gkin"], rtol=1e-14, atol=0)
            assert np.allclose(r["stress"], r0["stress"], rtol=1e-14, atol=0)


def test_cutoff_and_environment_radius(oracle_mod):
    # a diffuse EDF (a = 0.05: dran_edf = 23.5 bohr) beyond the MO cutoff
    # (a = 0.8: 5.88 bohr) still reaches points between the two radii
    a_edf, a_mo = 0.05, 0.8
    mol = one_atom([1], [a_edf], [1.0], mo_exp=a_mo)
    w = oracle_mod.Wfn(mol)
    d_mo = math.sqrt(-math.log(THRES) / a_mo)
    d_edf = math.sqrt(-math.log(THRES) / a_edf)
    for r in (0.5 * d_mo, 0.5 * (d_mo + d_edf), d_edf - 1e-6, d_edf + 1e-6):
        x = mol.atom_xyz[0] + np.array([r, 0.0, 0.0])
        rho = w.rho2(x, 0)
        assert abs(rho["rho"][0] - rho["rhoval"][0] - core_analytic(mol, x)) <= 1e-15
        if r > d_mo:
            assert rho["rhoval"][0] == 0.0
        if r > d_edf:
            assert rho["rho"][0] == 0.0
        else:
            assert rho["rho"][0] > 0.0


def test_set_edf_empty_removes_core(oracle_mod):
    mol = synth.add_edf(synth.make_molecule("nci12", seed=3), seed=5)
    w, w0 = oracle_mod.Wfn(mol), oracle_mod.Wfn(no_edf(mol))
    w.set_edf([], [], [], [])
    x = mol.atom_xyz[np.nonzero(mol.atom_z != 1)[0][0]] + 0.05
    assert w.rho2(x, 2)["rho"][0] == w0.rho2(x, 2)["rho"][0]


def test_wfx_edf_sections(tmp_path):
    mol = synth.add_edf(synth.make_molecule("nci12", seed=3), seed=5, lmax=1)
    p = tmp_path / "edf.wfx"
    synth.write_wfx(mol, str(p))
    text = p.read_text()
    for tag in ("Number of EDF Primitives", "EDF Primitive Centers", "EDF Primitive Types",
                "EDF Primitive Exponents", "EDF Primitive Coefficients"):
        assert f"<{tag}>" in text and f"</{tag}>" in text
    n = int(text.split("<Number of EDF Primitives>")[1].split("<")[0])
    assert n == mol.nedf
    exps = np.array(text.split("<EDF Primitive Exponents>")[1].split("<")[0].split(), float)
    assert np.array_equal(exps, mol.edf_e)
