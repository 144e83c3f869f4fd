"""Host logic of the learned CP-seed proposer (no GPU): BF16 rounding of the
stored weights, the coarse grid, the CP labels, the weights file."""
import os

import numpy as np
import pytest

from critic2_gb300 import cpseed, synth


def test_bf16_round_matches_torch():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(0)
    a = (rng.standard_normal(10000) * 10.0 ** rng.uniform(-8, 8, 10000)).astype(np.float32)
    a[:4] = [0.0, -0.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8]  # ties to even
    want = torch.tensor(a).to(torch.bfloat16).float().numpy()
    assert np.array_equal(cpseed.bf16_round(a), want)


def test_coarse_grid_covers_training_molecules():
    for i in range(5):
        mol = synth.training_molecule(i)
        x0, xm, ns = cpseed.coarse_grid(mol.atom_xyz)
        hi = x0 + np.diag(xm) * (ns - 1)
        assert np.all(mol.atom_xyz.min(0) - x0 >= 1.5) and np.all(hi - mol.atom_xyz.max(0) >= 1.5)
    mol = synth.make_molecule("cp100")
    x0, xm, ns = cpseed.coarse_grid(mol.atom_xyz)
    assert tuple(ns) == (64, 64, 64)
    assert np.all(mol.atom_xyz.min(0) - x0 >= 1.0)


def test_cp_labels():
    atoms = np.array([[0.0, 0.0, 0.0], [3.0, 0.0, 0.0]])
    x0, h, S = np.array([-5.0, -5.0, -5.0]), 0.5, 32
    xyz = np.array([[0.0, 0.0, 0.01],   # nucleus (-3 near an atom): skipped
                    [1.5, 0.0, 0.0],    # bond
                    [1.5, 2.0, 0.0],    # ring
                    [1.0, 1.0, 1.0],    # cage
                    [5.0, 5.0, 5.0],    # non-nuclear maximum
                    [50.0, 0.0, 0.0],   # outside the grid: skipped
                    [1.0, 1.0, 2.0]])   # degenerate signature: skipped
    typ = np.array([-3, -1, 1, 3, -3, -1, 0])
    lab = cpseed.cp_labels(xyz, typ, atoms, x0, h, S)
    assert lab.shape == (4, 4)
    assert list(lab[:, 3]) == [1, 2, 3, 0]
    assert np.allclose(lab[0, :3], (xyz[1] - x0) / h)


def test_network_size_and_weights_file():
    n = sum(k ** 3 * ci * co + co for ci, co, k, _ in cpseed.LAYERS)
    assert 50_000 < n < 100_000
    if not os.path.exists(cpseed.WEIGHTS):
        pytest.skip("no trained weights in the package")
    z = np.load(cpseed.WEIGHTS)
    assert z["bf16"].dtype == np.uint16 and z["bf16"].size == n
    assert np.array_equal(z["layers"], np.array(cpseed.LAYERS, np.int32))
