"""Basin integrals by bisection through the C ABI (c2g_basin_integrals)
against the oracle's restatement on the same rays (every ray on the first
ray's bracket tries, as the library does): surface radii, Pop and Lap."""
import numpy as np
import pytest

from critic2_gb300 import synth
from test_oracle_basin import diatomic, gauleg_rays, lebedev_rays, total_density

pytestmark = pytest.mark.gpu


def matched_weights(oracle_mod, rays, n):
    """The oracle rule's weights (x 4 pi) for the library's ray directions."""
    u, w = lebedev_rays(oracle_mod, n)
    d = np.linalg.norm(rays[:, None, :] - u[None, :, :], axis=2)
    j = d.argmin(1)
    assert d.min(1).max() < 1e-12 and len(set(j)) == len(j)
    return w[j]


def compare(lib, ora):
    """Fraction of rays whose radii agree to 1e-9, and the largest gap."""
    d = np.abs(lib["rsurf"] - ora["rsurf"])
    return float(np.mean(d <= 1e-9)), float(d.max())


def test_basin_diatomic_vs_oracle(gpu_lib, oracle_mod):
    from critic2_gb300.wfn import Wavefunction
    mol = diatomic()
    w, o = Wavefunction(mol), oracle_mod.Wfn(mol)
    cpx, cpt = mol.atom_xyz.copy(), np.array([-3, -3], np.int32)
    g = w.basin_integrals(cpx, cpt, "lebedev", 110)
    assert g["rays"].shape == (110, 3) and list(g["att_cp"]) == [0, 1]
    wu = matched_weights(oracle_mod, g["rays"], 110)
    us, ws = lebedev_rays(oracle_mod, 170)
    r = o.basin_integrals(cpx, cpt, g["rays"], wu, us, ws)
    same, worst = compare(g, r)
    assert same >= 0.99 and worst <= 1e-3
    assert np.allclose(g["rbeta_int"], r["rbeta_int"], rtol=1e-12)
    assert np.allclose(g["props"][:, 0], r["props"][:, 0], rtol=1e-6)
    assert np.allclose(g["props"][:, 1], r["props"][:, 1], atol=2e-5)
    assert np.allclose(g["iaserr"], r["iaserr"], rtol=1e-3, atol=1e-12)
    tot = total_density(mol)
    assert abs(g["props"][:, 0].sum() - tot) < 1e-3 * tot
    assert g["stats"]["nrestart"] == 0 and g["stats"]["npath"] > 110 * 2 * 10


def test_basin_gauleg_vs_oracle(gpu_lib, oracle_mod):
    """GAULEG ntheta nphi: the library's nodes are gauleg_nodes', and the
    rings are summed as gauleg_mquad."""
    from critic2_gb300.wfn import Wavefunction
    mol = diatomic()
    w, o = Wavefunction(mol), oracle_mod.Wfn(mol)
    cpx, cpt = mol.atom_xyz.copy(), np.array([-3, -3], np.int32)
    g = w.basin_integrals(cpx, cpt, "gauleg", 10, nphi=14)
    gu, gw, ring, ringw = gauleg_rays(10, 14)
    assert g["rays"].shape == gu.shape and np.allclose(g["rays"], gu, atol=1e-12)
    us, ws = lebedev_rays(oracle_mod, 170)
    r = o.basin_integrals(cpx, cpt, g["rays"], gw, us, ws, ring=ring, ringw=ringw)
    same, worst = compare(g, r)
    assert same >= 0.98 and worst <= 1e-3
    assert np.allclose(g["props"][:, 0], r["props"][:, 0], rtol=1e-6)


def test_basin_nci12_vs_oracle(gpu_lib, oracle_mod):
    """nci12 (12 atoms, its own FP64 CP list: nuclei, bond, ring, cage and
    non-nuclear maxima), Lebedev 26: the same surfaces on almost every ray
    and the same populations."""
    from critic2_gb300.wfn import Wavefunction
    mol = synth.make_molecule("nci12")
    w, o = Wavefunction(mol), oracle_mod.Wfn(mol)
    ac = w.autocritic(prec="fp64")
    cpx, cpt = ac["xyz"], ac["typ"]
    g = w.basin_integrals(cpx, cpt, "lebedev", 26)
    natt = mol.natom + int(np.sum(cpt[mol.natom:] == -3))
    assert len(g["att_cp"]) == natt
    us, ws = lebedev_rays(oracle_mod, 170)
    # the 26-point rule is not in the oracle's fixture: weights from the
    # library's own table (only the angular sum uses them)
    from test_oracle_basin import library_rule
    lr = library_rule(26)
    th, ph = np.arccos(lr[:, 2]), np.arctan2(lr[:, 1], lr[:, 0])
    lu = np.c_[np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)]
    j = np.linalg.norm(g["rays"][:, None, :] - lu[None, :, :], axis=2).argmin(1)
    wu = lr[j, 3] * 4 * np.pi
    r = o.basin_integrals(cpx, cpt, g["rays"], wu, us, ws)
    same, worst = compare(g, r)
    print(f"\nnci12 basins: {natt} attractors x 26 rays, {same:.3f} identical, worst {worst:.2e}; "
          f"GPU {g['stats']['ms']:.0f} ms, {g['stats']['npath']} paths, {g['stats']['nbatch']} batches")
    assert same >= 0.97
    assert np.allclose(g["props"][:, 0], r["props"][:, 0], rtol=1e-4)


def test_basin_arguments(gpu_lib):
    from critic2_gb300 import _lib
    from critic2_gb300.wfn import Wavefunction
    mol = diatomic()
    w = Wavefunction(mol)
    cpx, cpt = mol.atom_xyz[::-1].copy(), np.array([-3, -3], np.int32)
    with pytest.raises(_lib.C2GError):
        w.basin_integrals(cpx, cpt, "lebedev", 6)  # nuclei not first in atom order
    one = w.basin_integrals(None, None, "lebedev", 6, cpid=2)
    assert list(one["att_cp"]) == [1] and one["rays"].shape == (6, 3)
    assert w.basin_integrals(None, None, "lebedev", 7)["rays"].shape == (14, 3)  # good_lebedev rounds up


def test_sphere_integrals_vs_oracle(gpu_lib, oracle_mod):
    """SPHEREINTEGRALS through the C ABI against the oracle: nci12's first
    nucleus (LEBEDEV 110, 6 radii up to half the nearest-neighbour distance)
    and the diatomic's two (GAULEG 10 14)."""
    from critic2_gb300.wfn import Wavefunction
    mol = synth.make_molecule("nci12")
    w, o = Wavefunction(mol), oracle_mod.Wfn(mol)
    cpx, cpt = mol.atom_xyz.copy(), np.full(mol.natom, -3, np.int32)
    g = w.sphere_integrals(cpx, cpt, "lebedev", 110, cpid=1, nr=6)
    u, wu = lebedev_rays(oracle_mod, 110)
    r = o.sphere_integrals(cpx, cpt, u, wu, cpid=1, nr=6)
    assert list(g["att_cp"]) == [0] and np.allclose(g["radii"], r["radii"], rtol=1e-14)
    assert np.allclose(g["props"], r["props"], rtol=1e-11, atol=1e-14)
    mol = diatomic()
    w, o = Wavefunction(mol), oracle_mod.Wfn(mol)
    cpx, cpt = mol.atom_xyz.copy(), np.array([-3, -3], np.int32)
    g = w.sphere_integrals(cpx, cpt, "gauleg", 10, nphi=14, nr=4, r0=0.05, rend=1.0)
    gu, gw, ring, ringw = gauleg_rays(10, 14)
    r = o.sphere_integrals(cpx, cpt, gu, gw, ring=ring, ringw=ringw, nr=4, r0=0.05, rend=1.0)
    assert np.allclose(g["props"], r["props"], rtol=1e-11, atol=1e-14)


def test_basin_more_than_1024_mos(gpu_lib, oracle_mod):
    """The device path kernels evaluate the field in chunks of 1024 MOs: a
    1100-MO wavefunction (nci12's MOs repeated with distinct scales) gives
    the oracle's surfaces and populations."""
    from critic2_gb300.wfn import Wavefunction
    base = synth.make_molecule("nci12")
    nmo = 1100
    cols = np.arange(nmo) % base.nmo
    cmo = base.cmo[:, cols] * (1.0 + 1e-3 * np.arange(nmo))[None, :]
    mol = synth.Molecule(base.atom_xyz, base.atom_z, base.icenter, base.itype, base.e,
                         np.full(nmo, 2.0 * base.nmo / nmo), np.ascontiguousarray(cmo), name="nci12-1100")
    w, o = Wavefunction(mol), oracle_mod.Wfn(mol)
    g = w.basin_integrals(None, None, "lebedev", 6, cpid=1)
    wu = matched_weights(oracle_mod, g["rays"], 6)
    us, ws = lebedev_rays(oracle_mod, 170)
    r = o.basin_integrals(mol.atom_xyz, np.full(mol.natom, -3, np.int32), g["rays"], wu, us, ws, cpid=1)
    assert np.max(np.abs(g["rsurf"] - r["rsurf"])) < 1e-9
    assert np.allclose(g["props"], r["props"], rtol=1e-9, atol=1e-12)
