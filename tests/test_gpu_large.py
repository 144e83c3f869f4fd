"""The large configurations through the C ABI: prec200 (200 atoms, s/p/d/f,
3992 primitives, 400 MOs: four 128-MO tiles) and large500 (500 atoms,
10003 primitives, 1000 MOs: eight MO tiles, per-tile atom tables in global
memory).  Split precision against the GPU's FP64 form on i-planes of the
real NCI grids (the split precision's bars: |drho|/rho <= 1e-6, |ds| <= 1e-3,
no sign flips), and the FP64 form against the oracle at 1e-10 on an f-shell patch
of prec200 and at scattered points of large500."""
import numpy as np
import pytest

from critic2_gb300 import synth

pytestmark = pytest.mark.gpu


def _planes(w, mol, wl, planes, prec):
    x0, xm, ns = synth.nci_grid(mol, wl.grid, wl.step)
    out = []
    for i in planes:
        nsp = np.array([1, ns[1], ns[2]], np.int32)
        xi = x0 + i * xm[:, 0]
        c64, s64, _ = w.nciplot(xi, xm, nsp, "fp64")
        c, s, _ = w.nciplot(xi, xm, nsp, prec)
        out.append((c64, s64, c, s))
    return out


@pytest.mark.parametrize("name,planes", [("prec200", (40, 128, 200)), ("large500", (100, 160))])
def test_split_planes_vs_fp64(gpu_lib, name, planes):
    from critic2_gb300.wfn import Wavefunction
    wl = synth.WORKLOADS[name]
    mol = synth.make_molecule(name)
    w = Wavefunction(mol)
    worst = 0.0
    for c64, s64, c, s in _planes(w, mol, wl, planes, "tf32x3"):
        r64, r = np.abs(c64), np.abs(c)
        err = np.abs(r - r64) / r64
        worst = max(worst, float(err.max()))
        assert err.max() <= 1e-6
        assert np.abs(s - s64).max() <= 1e-3
        assert np.array_equal(np.sign(c), np.sign(c64))
    print(f"\n{name}: TF32x3 max |drho|/rho {worst:.3e} on {len(planes)} i-planes of the {wl.grid}^3 grid")


def test_prec200_fp64_vs_oracle_f_shells(gpu_lib, oracle_mod):
    """An f-shell patch (24 x 24 points of the central i-plane) of prec200's
    grid: FP64 NCI output against the oracle at 1e-10."""
    from critic2_gb300.wfn import Wavefunction
    wl = synth.WORKLOADS["prec200"]
    mol = synth.make_molecule("prec200")
    w, o = Wavefunction(mol), oracle_mod.Wfn(mol)
    x0, xm, ns = synth.nci_grid(mol, wl.grid, wl.step)
    xp = x0 + xm @ np.array([128, 116, 116])
    nsp = np.array([1, 24, 24], np.int32)
    c, s, _ = w.nciplot(xp, xm, nsp, "fp64")
    oc, os_ = o.nciplot(xp, xm, nsp)
    assert np.allclose(np.abs(c), np.abs(oc), rtol=1e-10, atol=0)
    assert np.array_equal(np.sign(c), np.sign(oc))
    assert np.allclose(s, os_, rtol=1e-10, atol=1e-300)


def test_large500_fp64_points_vs_oracle(gpu_lib, oracle_mod):
    """large500 (1000 MOs, eight MO tiles): rho2 at 200 scattered points in
    FP64 against the oracle at 1e-10, and TF32x3 against FP64 at the
    split precision's density bar (1e-6)."""
    from critic2_gb300.wfn import Wavefunction
    mol = synth.make_molecule("large500")
    w, o = Wavefunction(mol), oracle_mod.Wfn(mol)
    rng = np.random.default_rng(5)
    pts = rng.uniform(mol.atom_xyz.min(0), mol.atom_xyz.max(0), size=(200, 3))
    r64 = w.rho2(pts, 2, "fp64")
    rho_o, g_o, h_o = o.rho2_points(pts, 2)
    assert np.allclose(r64["rho"][:, 0], rho_o, rtol=1e-10, atol=0)
    assert np.allclose(r64["grad"][:, 0, :], g_o, rtol=1e-9, atol=1e-12 * np.abs(g_o).max())
    r32 = w.rho2(pts, 2, "tf32x3")
    e = np.abs(r32["rho"][:, 0] - r64["rho"][:, 0]) / r64["rho"][:, 0]
    assert e.max() <= 1e-6
