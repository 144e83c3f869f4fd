"""The oracle's field post-processing against critic2's own POINT records.

Each record (tests/golden/point_records.json, made by make_golden.py from
critic2's test references) prints the Hessian, its eigenvalues, the CP type
and the spin channels of a molecular-wavefunction field at a point; the
values are printed with 10 significant digits, so relations are checked to
1e-8 relative.
"""
import json
import math
import os

import numpy as np
import pytest

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "point_records.json")))["records"]


def test_fixture_present():
    assert len(GOLD) >= 20


@pytest.mark.parametrize("rec", GOLD, ids=lambda r: f"{r['file']}:{r['line']}")
def test_eigenvalues_and_type(oracle_mod, rec):
    H = np.array(rec["hess"])
    ev, r, s = oracle_mod.rsindex(H, 1e-8)
    scale = max(1e-12, np.abs(rec["hfeval"]).max())
    assert np.allclose(ev, rec["hfeval"], rtol=0, atol=2e-9 * scale + 2e-10 * np.abs(H).max())
    assert (r, s) == (rec["r"], rec["s"])
    assert np.all(np.diff(ev) >= 0)  # ascending, like dsyev


@pytest.mark.parametrize("rec", GOLD, ids=lambda r: f"{r['file']}:{r['line']}")
def test_gradient_norm_and_laplacian(rec):
    g = np.array(rec["grad"])
    assert math.isclose(np.linalg.norm(g), rec["gfmod"], rel_tol=2e-9, abs_tol=1e-12)
    H = np.array(rec["hess"])
    assert math.isclose(np.trace(H), rec["lap"], rel_tol=2e-8, abs_tol=2e-9 * np.abs(H).max())
    assert np.allclose(H, H.T)


@pytest.mark.parametrize("rec", [r for r in GOLD if "up" in r], ids=lambda r: f"{r['file']}:{r['line']}")
def test_spin_channels(rec):
    """Spin densities add up to the total (and are halves for closed shells),
    as rho2 assembles them (src/wfn_private@proc.F90:2636-2703)."""
    up, dn = rec["up"], rec["down"]
    if "rohf" in rec["file"]:
        # ROHF: channel 2 sums every MO, channel 3 the first nalpha (the
        # doubly occupied ones), src/wfn_private@proc.F90:2557-2560
        assert math.isclose(up[0], rec["f"], rel_tol=5e-9)
        assert dn[0] < up[0]
        return
    assert math.isclose(up[0] + dn[0], rec["f"], rel_tol=5e-9, abs_tol=1e-12)
    if "up_gkin" in rec and "gkin" in rec:
        assert math.isclose(rec["up_gkin"] + rec["down_gkin"], rec["gkin"], rel_tol=5e-9, abs_tol=1e-12)
    if abs(up[0] - dn[0]) < 1e-12 * abs(rec["f"]) + 1e-15:
        assert math.isclose(up[0], 0.5 * rec["f"], rel_tol=5e-9)
        assert math.isclose(up[1], 0.5 * rec["gfmod"], rel_tol=5e-9, abs_tol=1e-12)
        assert math.isclose(up[2], 0.5 * rec["lap"], rel_tol=5e-8, abs_tol=1e-12)


def test_oracle_eigsym_matches_lapack(oracle_mod):
    rng = np.random.default_rng(0)
    for _ in range(200):
        a = rng.standard_normal((3, 3)) * 10 ** rng.uniform(-4, 3)
        a = a + a.T
        ev = oracle_mod.eigsym3(a)
        ref = np.linalg.eigvalsh(a)
        assert np.allclose(ev, ref, rtol=0, atol=1e-13 * np.abs(ref).max())


def test_oracle_matinvsym(oracle_mod):
    rng = np.random.default_rng(1)
    for _ in range(100):
        a = rng.standard_normal((3, 3))
        a = a + a.T
        inv, ier = oracle_mod.matinvsym3(a)
        assert ier == 0
        assert np.allclose(inv @ a, np.eye(3), atol=1e-10 * np.linalg.cond(a))
    _, ier = oracle_mod.matinvsym3(np.zeros((3, 3)))
    assert ier != 0


def test_nci_constant():
    """const = 2 (3 pi^2)^(1/3) and the 4/3 power (src/nci@proc.f90:90-91)."""
    assert math.isclose(2.0 * (3.0 * math.pi ** 2) ** (1.0 / 3.0), 6.187335452560271, rel_tol=1e-15)
    rec = GOLD[0]
    s = rec["gfmod"] / (6.187335452560271 * rec["f"] ** (4.0 / 3.0))
    assert 0 < s < 100
