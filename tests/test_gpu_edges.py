"""Edge cases through the C ABI: empty batches, one-point and ragged grids
in every precision, a molecule too large for the split kernel's shared
memory, a pipeline wait that runs out, and an empty seed list."""
import numpy as np
import pytest

from critic2_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def w12(gpu_lib):
    from critic2_gb300.wfn import Wavefunction
    mol = synth.make_molecule("nci12")
    return mol, Wavefunction(mol)


def test_empty_batches(w12):
    mol, g = w12
    e = np.zeros((0, 3))
    for prec in ("fp64", "tf32x3", "bf16x3"):
        assert g.rho2(e, 2, prec)["rho"].shape == (0, 3)
        assert g.grd(e, 2, prec)["f"].shape == (0,)
    x, ier = g.newton(e)
    assert x.shape == (0, 3) and ier.shape == (0,)
    out = g.cp_graph(e, np.zeros(0, np.int32))
    assert out["ipath"].shape == (0, 2)


@pytest.mark.parametrize("nstep", [(1, 1, 1), (1, 3, 5), (7, 1, 1), (2, 9, 1), (3, 5, 17)])
@pytest.mark.parametrize("prec", ["tf32x3", "bf16x3"])
def test_one_point_and_ragged_grids(w12, oracle_mod, nstep, prec):
    mol, g = w12
    x0 = mol.atom_xyz.mean(0) + np.array([0.013, -0.021, 0.007])
    xm = np.diag([0.17, 0.11, 0.09])
    ns = np.array(nstep, np.int32)
    c64, s64, _ = g.nciplot(x0, xm, ns, "fp64")
    c, s, _ = g.nciplot(x0, xm, ns, prec)
    assert c.shape == tuple(nstep) and s.shape == tuple(nstep)
    tol = 1e-6 if prec == "tf32x3" else 5e-5
    assert np.all(np.abs(np.abs(c) - np.abs(c64)) <= tol * np.abs(c64))
    assert np.all(np.abs(s - s64) <= (1e-3 if prec == "tf32x3" else 1e-2))
    # and the FP64 grid against the oracle on the same ragged shape
    oc, og = oracle_mod.Wfn(mol).nciplot(x0, xm, ns)
    assert np.allclose(np.abs(c64), np.abs(oc), rtol=1e-10, atol=0)
    assert np.allclose(s64, og, rtol=1e-10, atol=1e-300)


def test_split_kernel_800_atoms(gpu_lib):
    """800 atoms: the split kernel's per-tile atom tables no longer fit a
    CTA's shared memory and move to global memory; the split grid matches
    FP64 as for small molecules.  The no-allocation entry refuses such a
    molecule (C2G_ERR_UNSUPPORTED) and the handle keeps working."""
    import torch
    from critic2_gb300 import _lib
    from critic2_gb300.wfn import Wavefunction
    w = synth.Workload("h800", 800, None, 800, False, 16, 0, 0.1, 1, 9)
    mol = synth.build_molecule(w, 9)
    g = Wavefunction(mol)
    x0 = mol.atom_xyz.mean(0) + np.array([0.013, -0.021, 0.007])
    xm = np.eye(3) * 0.17
    ns = np.array([6, 8, 16], np.int32)
    c64, s64, _ = g.nciplot(x0, xm, ns, "fp64")
    c, s, _ = g.nciplot(x0, xm, ns, "tf32x3")
    assert np.all(np.abs(np.abs(c) - np.abs(c64)) <= 1e-6 * np.abs(c64))
    assert np.abs(s - s64).max() <= 1e-3
    n = int(np.prod(ns))
    r = torch.empty(n, dtype=torch.float64, device="cuda")
    q = torch.empty_like(r)
    with pytest.raises(_lib.C2GError) as e:
        g.nciplot_dev_noalloc(x0, xm, ns, "tf32x3", r.data_ptr(), q.data_ptr())
    assert e.value.code == 5
    c2, _, _ = g.nciplot(x0, xm, ns, "tf32x3")
    assert np.array_equal(c, c2)


def test_empty_seed_list_gives_the_nuclei(w12):
    mol, g = w12
    r = g.autocritic(np.zeros((0, 3)), prec="fp64")
    assert r["nseed"] == 0
    assert np.all(r["typ"] == -3) and len(r["typ"]) == mol.natom


@pytest.mark.parametrize("prec", ["tf32x3", "bf16x3"])
def test_pipeline_wait_timeout_is_reported(gpu_lib, prec):
    """A pipeline wait that runs out (C2G_PARAM_WAIT_NS set to 1 ns) stops
    the split kernel cleanly: the call fails with C2G_ERR_CUDA naming the
    timed-out wait, nothing faults, and with the default limit restored the
    same handle gives the FP64-matching grid again."""
    from critic2_gb300 import _lib
    from critic2_gb300.wfn import Wavefunction
    mol = synth.make_molecule("nci12")
    g = Wavefunction(mol)
    x0, xm, ns = synth.nci_grid(mol, 40, 0.2)
    c64, s64, _ = g.nciplot(x0, xm, ns, "fp64")
    g.set_wait_ns(1.0)
    with pytest.raises(_lib.C2GError) as e:
        g.nciplot(x0, xm, ns, prec)
    assert e.value.code == 2 and "pipeline wait timed out" in str(e.value)
    g.set_wait_ns(4e9)
    c, s, _ = g.nciplot(x0, xm, ns, prec)
    tol = 1e-6 if prec == "tf32x3" else 5e-5
    assert np.all(np.abs(np.abs(c) - np.abs(c64)) <= tol * np.abs(c64))
    assert np.abs(s - s64).max() <= (1e-3 if prec == "tf32x3" else 1e-2)
    with pytest.raises(_lib.C2GError):
        g.set_wait_ns(0.0)
