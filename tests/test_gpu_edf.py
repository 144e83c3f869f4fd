"""EDF core density on the GPU against the oracle: the FP64 evaluator (rho2
records incl. spin channels, grd, NCI grid, Newton), the split-precision
NCI grid against the FP64 one, the wfx EDF sections and c2g_wfn_set_edf.
Bars: FP64 1e-10 relative; the split modes keep the bars of the core-free
split tests (TF32x3 |drho|/rho 1e-6, |ds| 1e-3; BF16x3 5e-5, 1e-2)."""
import dataclasses

import numpy as np
import pytest

from critic2_gb300 import synth

pytestmark = pytest.mark.gpu

REL = 1e-10


def close(a, b, rel=REL, scale=None):
    a, b = np.asarray(a, float), np.asarray(b, float)
    s = np.abs(b).max() if scale is None else scale
    return np.all(np.abs(a - b) <= rel * np.maximum(np.abs(b), 1e-6 * s))


@pytest.fixture(scope="module")
def mol_edf():
    return synth.add_edf(synth.make_molecule("nci12", seed=3), seed=5, lmax=1)


def spin_variant(mol, wfntyp):
    occ = np.full(mol.nmo, 2.0)
    nalpha = mol.nmo // 2 + 1
    if wfntyp == 1:
        occ[:] = 1.0
    elif wfntyp == 2:
        occ[nalpha:] = 1.0
    return dataclasses.replace(mol, wfntyp=wfntyp, nalpha=nalpha, occ=occ)


def near_points(mol, n, seed, spread=0.6):
    rng = np.random.default_rng(seed)
    heavy = np.nonzero(mol.atom_z != 1)[0]
    at = heavy[rng.integers(0, len(heavy), n)]
    return mol.atom_xyz[at] + rng.uniform(-spread, spread, (n, 3))


@pytest.mark.parametrize("wfntyp", [0, 1, 2])
def test_rho2_fp64_with_core(gpu_lib, oracle_mod, mol_edf, wfntyp):
    from critic2_gb300.wfn import Wavefunction
    m = mol_edf if wfntyp == 0 else spin_variant(mol_edf, wfntyp)
    g, o = Wavefunction(m), oracle_mod.Wfn(m)
    pts = np.vstack([near_points(m, 96, wfntyp), np.random.default_rng(9).uniform(
        m.atom_xyz.min(0) - 2, m.atom_xyz.max(0) + 2, (64, 3))])
    for nder in (0, 2):
        out = g.rho2(pts, nder, "fp64")
        for i in range(0, len(pts), 3):
            ref = o.rho2(pts[i], nder)
            assert close(out["rho"][i], ref["rho"])
            if nder > 1:
                assert close(out["grad"][i], ref["grad"])
                assert close(out["hess"][i], ref["h"])
                assert close(out["gkin"][i], ref["gkin"])
                assert close(out["stress"][i], ref["stress"], scale=np.abs(ref["h"]).max())


def test_core_is_present_and_removable(gpu_lib, mol_edf):
    from critic2_gb300.wfn import Wavefunction
    base = dataclasses.replace(mol_edf, edf_icenter=None, edf_itype=None, edf_e=None, edf_c=None)
    g, g0 = Wavefunction(mol_edf), Wavefunction(base)
    pts = near_points(mol_edf, 64, 4)
    r, r0 = g.rho2(pts, 2, "fp64")["rho"][:, 0], g0.rho2(pts, 2, "fp64")["rho"][:, 0]
    assert np.median(np.abs(r - r0)) > 1e-3 * np.median(r0)
    g.set_edf([], [], [], [])
    assert np.array_equal(g.rho2(pts, 2, "fp64")["rho"], g0.rho2(pts, 2, "fp64")["rho"])


def test_grd_fp64_with_core(gpu_lib, oracle_mod, mol_edf):
    from critic2_gb300.wfn import Wavefunction
    g, o = Wavefunction(mol_edf), oracle_mod.Wfn(mol_edf)
    pts = np.vstack([near_points(mol_edf, 48, 11), mol_edf.atom_xyz[:4]])
    out = g.grd(pts, 2, "fp64")
    for i in range(len(pts)):
        ref = o.grd(pts[i], 2)
        assert abs(out["f"][i] - ref.f) <= REL * abs(ref.f)
        assert close(out["gf"][i], np.array(ref.gf), scale=max(1.0, np.abs(ref.gf).max()))
        assert bool(out["isnuc"][i]) == bool(ref.isnuc)


@pytest.fixture(scope="module")
def grid_edf(mol_edf):
    x0 = mol_edf.atom_xyz.min(0) - 0.5
    step = 0.15
    nstep = np.array([32, 28, 24], np.int32)
    return x0, np.diag([step] * 3), nstep


def test_nci_fp64_with_core(gpu_lib, oracle_mod, mol_edf, grid_edf):
    from critic2_gb300.wfn import Wavefunction
    g, o = Wavefunction(mol_edf), oracle_mod.Wfn(mol_edf)
    x0, xmat, nstep = grid_edf
    crho, cgrad = g.nciplot(x0, xmat, nstep, "fp64")[:2]
    ocrho, ocgrad = o.nciplot(x0, xmat, nstep)
    assert np.all(np.abs(np.abs(crho) - np.abs(ocrho)) <= REL * np.abs(ocrho))
    assert np.all(np.abs(cgrad - ocgrad) <= REL * np.abs(ocgrad))
    assert np.mean(np.sign(crho) != np.sign(ocrho)) < 1e-4


# split-precision bars of the core-free tests (|drho|/rho, |ds|)
TOL = {"tf32x3": dict(rho=1e-6, s=1e-3), "bf16x3": dict(rho=5e-5, s=1e-2)}


@pytest.mark.parametrize("prec", ["tf32x3", "bf16x3"])
def test_nci_split_with_core(gpu_lib, mol_edf, grid_edf, prec):
    from critic2_gb300.wfn import Wavefunction
    g = Wavefunction(mol_edf)
    x0, xmat, nstep = grid_edf
    c64, s64 = g.nciplot(x0, xmat, nstep, "fp64")[:2]
    cs, ss = g.nciplot(x0, xmat, nstep, prec)[:2]
    rel = np.abs(np.abs(cs) - np.abs(c64)) / np.maximum(np.abs(c64), 1e-300)
    assert rel.max() <= TOL[prec]["rho"]
    assert np.abs(ss - s64).max() <= TOL[prec]["s"]
    assert int((np.sign(cs) != np.sign(c64)).sum()) <= max(2, int(1e-5 * cs.size))


def test_split_records_with_core(gpu_lib, mol_edf):
    """Split-precision point records (the Newton/POINT path) carry the FP64
    core: near the nuclei the core dominates and the relative error drops."""
    from critic2_gb300.wfn import Wavefunction
    g = Wavefunction(mol_edf)
    pts = near_points(mol_edf, 256, 8, spread=0.4)
    r64 = g.rho2(pts, 2, "fp64")
    r32 = g.rho2(pts, 2, "tf32x3")
    rho64, rho32 = r64["rho"][:, 0], r32["rho"][:, 0]
    assert np.max(np.abs(rho32 - rho64) / rho64) <= TOL["tf32x3"]["rho"]
    gs = np.abs(r64["grad"][:, 0]).max(1) + 1e-3 * rho64
    assert np.max(np.abs(r32["grad"][:, 0] - r64["grad"][:, 0]).max(1) / gs) <= 2e-5


def test_newton_with_core(gpu_lib, oracle_mod, mol_edf):
    from critic2_gb300.wfn import Wavefunction
    g, o = Wavefunction(mol_edf), oracle_mod.Wfn(mol_edf)
    seeds = g.pair_seeds()[::7]
    assert np.array_equal(seeds, o.pair_seeds()[::7])
    xg, ierg = g.newton(seeds, 1e-12, 200, "fp64")
    xo, iero = o.newton_batch(seeds, 1e-12, 200)
    ok = (np.asarray(ierg) == 0) & (np.asarray(iero) == 0)
    assert ok.mean() > 0.5
    # both runs reach the same CP where the density is not a flat tail
    for x1, x2 in zip(np.asarray(xg)[ok], np.asarray(xo)[ok]):
        r = o.grd(x2, 2)
        if r.f > 1e-8:
            lam = np.abs(np.array(r.hfeval[:])).min()
            assert np.linalg.norm(x1 - x2) <= max(1e-6, 4e-12 / max(lam, 1e-300))


def test_wfx_round_trip_with_core(gpu_lib, mol_edf, tmp_path):
    from critic2_gb300.wfn import Wavefunction
    p = tmp_path / "edf.wfx"
    synth.write_wfx(mol_edf, str(p))
    g1, g2 = Wavefunction.from_wfx(str(p)), Wavefunction(mol_edf)
    pts = near_points(mol_edf, 64, 2)
    a, b = g1.rho2(pts, 2, "fp64"), g2.rho2(pts, 2, "fp64")
    for k in ("rho", "grad", "hess"):
        assert close(a[k], b[k], rel=1e-13)


def test_set_edf_rejects_bad_input(gpu_lib, mol_edf):
    from critic2_gb300 import _lib
    from critic2_gb300.wfn import Wavefunction
    g = Wavefunction(mol_edf)
    with pytest.raises(_lib.C2GError):
        g.set_edf([mol_edf.natom + 1], [1], [1.0], [1.0])
    with pytest.raises(_lib.C2GError):
        g.set_edf([1], [57], [1.0], [1.0])
    with pytest.raises(_lib.C2GError):
        g.set_edf([1], [1], [-1.0], [1.0])


@pytest.mark.parametrize("wfntyp", [0, 1])
def test_rho2_valence_leaves_the_core_out(gpu_lib, oracle_mod, mol_edf, wfntyp):
    """c2g_rho2_valence against rho2's rhoval/gradval/hval in the oracle, and
    equal to the full evaluation of the same MOs without EDF primitives."""
    from critic2_gb300.wfn import Wavefunction
    m = mol_edf if wfntyp == 0 else spin_variant(mol_edf, wfntyp)
    bare = dataclasses.replace(m, edf_icenter=None, edf_itype=None, edf_e=None, edf_c=None)
    g = Wavefunction(m)
    pts = near_points(m, 48, 11 + wfntyp)
    v = g.rho2_valence(pts, 2)
    full = g.rho2(pts, 2, "fp64")
    o = oracle_mod.Wfn(m)
    for i in range(0, len(pts), 4):
        r = o.grd(pts[i], 2)
        assert close([v["rho"][i, 0]], [r.fval])
        assert abs(np.trace(v["hess"][i, 0]) - r.del2fval) <= 1e-10 * max(abs(r.del2fval), abs(r.fval))
    assert np.median(full["rho"][:, 0] - v["rho"][:, 0]) > 0  # the core adds density near the nuclei
    vb = Wavefunction(bare).rho2(pts, 2, "fp64")
    assert close(v["rho"], vb["rho"]) and close(v["grad"], vb["grad"]) and close(v["hess"], vb["hess"])
