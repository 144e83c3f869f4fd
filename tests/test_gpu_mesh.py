"""Molecular meshes and molcalc on the GPU (c2g_mesh_size, c2g_mesh_dev,
c2g_molcalc) against the oracle's restatement of genmesh and fillmesh.
Bars: same size and shell order, the same angular points on each shell;
positions 1e-13 and weights 1e-12 relative or 1e-14 of the largest
weight (FP64 exp/sqrt and contractions on two machines); FP64 integrals 1e-11 relative; TF32x3
integrals 1e-6."""
import math

import numpy as np
import pytest

from critic2_gb300 import synth

pytestmark = pytest.mark.gpu


def gaussian_mol(alpha=0.7, c=1.3):
    ang = np.arange(6) * np.pi / 3
    xyz = np.vstack([np.c_[2.64 * np.cos(ang), 2.64 * np.sin(ang), np.zeros(6)],
                     np.c_[4.68 * np.cos(ang), 4.68 * np.sin(ang), np.zeros(6)]])
    cmo = np.zeros((12, 1))
    cmo[0, 0] = c
    return synth.Molecule(xyz, np.array([6] * 6 + [1] * 6, np.int32), np.arange(1, 13, dtype=np.int32),
                          np.ones(12, np.int32), np.full(12, alpha), np.array([2.0]), cmo, name="gauss")


@pytest.mark.parametrize("mesh", ["franchini", "becke"])
@pytest.mark.parametrize("level", ["small", "good"])
def test_mesh_vs_oracle(gpu_lib, oracle_mod, mesh, level):
    from critic2_gb300.wfn import Wavefunction
    mol = synth.make_molecule("nci12")
    g, o = Wavefunction(mol), oracle_mod.Wfn(mol)
    xg, wg = g.mesh(mesh, level)
    xo, wo = o.mesh(mesh, level)
    assert g.mesh_size(mesh, level) == len(wo) == len(wg)
    # same shells in the same order; within a shell the angular points are
    # the same set (each side expands the Lebedev orbits in its own order)
    nang = {"small": 110, "good": 302}[level]

    def per_shell(x, w):
        x, w = x.reshape(-1, nang, 3), w.reshape(-1, nang)
        key = np.round(x, 9)
        out_x, out_w = np.empty_like(x), np.empty_like(w)
        for s in range(x.shape[0]):
            o = np.lexsort(key[s].T[::-1])
            out_x[s], out_w[s] = x[s][o], w[s][o]
        return out_x, out_w

    xg2, wg2 = per_shell(xg, wg)
    xo2, wo2 = per_shell(xo, wo)
    assert np.allclose(xg2, xo2, rtol=0, atol=1e-13 * np.abs(xo).max())
    # Becke's cutoff products lose digits where (1 - h)/2 cancels (weights
    # far below the largest): absolute bar relative to the largest weight
    assert np.allclose(wg2, wo2, rtol=1e-12, atol=1e-14 * wo.max())


def test_molcalc_gaussian_known_answer(gpu_lib):
    from critic2_gb300.wfn import Wavefunction
    g = Wavefunction(gaussian_mol())
    exact = 2 * 1.3 ** 2 * (math.pi / 1.4) ** 1.5
    r = g.molcalc(("rho",), "franchini", "good")
    assert r["npoints"] == 219252
    assert abs(r["rho"] / exact - 1) < 3e-7
    # critic2's benzene meshes, small level (tests/011_mesh/ref/001_meshtype.cro)
    assert g.mesh_size("franchini", "small") == 55440 and g.mesh_size("becke", "small") == 55440


@pytest.mark.parametrize("mesh", ["franchini", "becke"])
def test_molcalc_vs_oracle(gpu_lib, oracle_mod, mesh):
    from critic2_gb300.wfn import Wavefunction
    mol = synth.make_molecule("nci12")
    g, o = Wavefunction(mol), oracle_mod.Wfn(mol)
    q = ("rho", "gradrho", "volume")
    rg = g.molcalc(q, mesh, "good", "fp64")
    ro = o.molcalc(q, mesh, "good")
    for k in q:
        assert abs(rg[k] - ro[k]) <= 1e-11 * abs(ro[k]), (k, rg[k], ro[k])
    rs = g.molcalc(("rho",), mesh, "good", "tf32x3")
    assert abs(rs["rho"] - ro["rho"]) <= 1e-6 * abs(ro["rho"])
    gk = g.molcalc(("gkin",), mesh, "small", "fp64")["gkin"]
    assert np.isfinite(gk) and gk > 0


def test_molcalc_errors(gpu_lib):
    from critic2_gb300 import _lib
    from critic2_gb300.wfn import Wavefunction
    g = Wavefunction(synth.make_molecule("nci12"))
    with pytest.raises(_lib.C2GError):
        g.molcalc(("gkin",), "franchini", "small", "tf32x3")
    import ctypes
    n = ctypes.c_long(0)
    assert _lib.lib().c2g_mesh_size(g._h, 3, 3, ctypes.byref(n)) == 1  # unknown mesh type
    assert _lib.lib().c2g_mesh_size(g._h, 2, 6, ctypes.byref(n)) == 1  # unknown level
