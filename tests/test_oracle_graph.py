"""The molecular graph in the oracle: field%gradient with the default
navigation (src/fieldmod@proc.f90:2500-2890) and makegraph
(src/autocp@proc.f90:2116-2268).  The reference's tests hold no molecular
wavefunction with which to replay its graph, so the restatement is pinned by
known answers: spherical densities (radial paths, path length = distance),
the symmetric two-centre bond (terminators, 180 degree angle, end distances),
the eigen-solver against LAPACK, and the structure of a real graph."""
import numpy as np
import pytest

from critic2_gb300 import synth


def atoms_mol(xyz, z, alpha=1.2):
    """s-only molecule: one s primitive per atom, one MO summing them."""
    xyz = np.asarray(xyz, float)
    n = len(xyz)
    return synth.Molecule(xyz, np.array(z, np.int32), np.arange(1, n + 1, dtype=np.int32),
                          np.ones(n, np.int32), np.full(n, alpha), np.array([2.0]),
                          np.ones((n, 1)), wfntyp=0, nalpha=1, name="s-atoms")


def test_eigvec3_against_lapack(oracle_mod):
    rng = np.random.default_rng(0)
    for _ in range(200):
        a = rng.standard_normal((3, 3))
        m = a + a.T
        ev, v = oracle_mod.eigvec3(m)
        ref = np.linalg.eigvalsh(m)
        assert np.allclose(ev, ref, rtol=1e-12, atol=1e-12)
        assert np.allclose(m @ v, v * ev, atol=1e-11)
        assert np.allclose(v.T @ v, np.eye(3), atol=1e-12)
        for j in range(3):  # sign rule: largest component positive
            assert v[np.argmax(np.abs(v[:, j])), j] > 0


def test_radial_path_of_a_spherical_atom(oracle_mod):
    mol = atoms_mol([[0.0, 0.0, 0.0]], [8])
    w = oracle_mod.Wfn(mol)
    cpx, cpt = np.zeros((1, 3)), np.array([-3], np.int32)
    rng = np.random.default_rng(1)
    for _ in range(6):
        d = rng.standard_normal(3)
        r0 = rng.uniform(0.4, 2.0)
        x0 = r0 * d / np.linalg.norm(d)
        xe, ier, nstep, plen = w.gradient(x0, 1, cpx, cpt, x0)
        assert ier == 0 and np.array_equal(xe, np.zeros(3))  # ends on the nucleus
        assert abs(plen - r0) < 1e-4 * r0                       # straight line
        assert nstep >= 2


def test_two_centre_bond(oracle_mod):
    R = 2.4
    mol = atoms_mol([[-R / 2, 0.1, 0.0], [R / 2, 0.1, 0.0]], [6, 6])
    w = oracle_mod.Wfn(mol)
    cp = w.autocritic()
    typ = cp["typ"]
    assert sorted(typ.tolist()) == [-3, -3, -1]
    g = w.makegraph(cp["xyz"], typ)
    b = int(np.nonzero(typ == -1)[0][0])
    assert sorted(g["ipath"][b].tolist()) == [1, 2]
    assert np.all(g["ier"][b] == 0)
    assert np.allclose(g["brdist"][b], R / 2, atol=1e-12)
    assert np.allclose(g["brpathlen"][b], R / 2, rtol=1e-4)
    assert abs(g["brang"][b] - 180.0) < 1e-6
    assert abs(abs(g["brvec"][b][0]) - 1.0) < 1e-10   # along the bond axis
    # nuclei carry no graph data
    n = np.nonzero(typ == -3)[0]
    assert np.all(g["ipath"][n] == 0) and np.all(g["brdist"][n] == 0)


def test_hydrogen_nuclei_are_reached_through_the_cp_list(oracle_mod):
    # critic2 skips hydrogens in the nearest-nucleus shortcut; the CP list
    # still holds them, so a path to an H nucleus ends there
    mol = atoms_mol([[0.0, 0.0, 0.0], [1.8, 0.0, 0.0]], [8, 1])
    w = oracle_mod.Wfn(mol)
    cp = w.autocritic()
    g = w.makegraph(cp["xyz"], cp["typ"])
    b = int(np.nonzero(cp["typ"] == -1)[0][0])
    assert sorted(g["ipath"][b].tolist()) == [1, 2] and np.all(g["ier"][b] == 0)


@pytest.fixture(scope="module")
def graph12(oracle_mod):
    mol = synth.make_molecule("nci12")
    w = oracle_mod.Wfn(mol)
    cp = w.autocritic()
    return mol, cp, w.makegraph(cp["xyz"], cp["typ"])


def test_graph_structure(graph12):
    mol, cp, g = graph12
    typ = cp["typ"]
    nuc = np.nonzero(typ == -3)[0]
    for i in np.nonzero(typ == -1)[0]:
        for j in range(2):
            if g["ier"][i, j] == 0:
                # a bond path that ends normally ends at a nucleus or a
                # non-nuclear attractor, within the beta sphere or at a CP
                t = g["ipath"][i, j]
                assert typ[t - 1] == -3
                assert g["brpathlen"][i, j] >= g["brdist"][i, j] - 1e-9
        if np.all(g["ier"][i] == 0):
            assert g["ipath"][i, 0] != g["ipath"][i, 1]
        assert abs(np.linalg.norm(g["brvec"][i]) - 1.0) < 1e-12
        assert 0.0 <= g["brang"][i] <= 180.0
    for i in np.nonzero(typ == 1)[0]:
        # ring paths go down: to a cage CP, or out of the molecule
        assert all(t == -1 or t == 0 or typ[t - 1] == 3 for t in g["ipath"][i])
    assert len(nuc) >= mol.natom  # nuclei plus any non-nuclear maxima


def test_graph_is_deterministic(oracle_mod, graph12):
    mol, cp, g = graph12
    w = oracle_mod.Wfn(mol)
    g2 = w.makegraph(cp["xyz"], cp["typ"], nthreads=1)
    for k in g:
        assert np.array_equal(g[k], g2[k])


def test_graph_duplicate_cps_keep_first(oracle_mod, graph12):
    """critic2's scan for the nearest beta sphere keeps the first CP of equal
    distance: with the CP list given twice over, every terminator is in the
    first copy and every path is the same (the library's warp-parallel scan
    is held to the same rule by the GPU test of the same name)."""
    mol, cp, g = graph12
    w = oracle_mod.Wfn(mol)
    n = len(cp["typ"])
    two = w.makegraph(np.concatenate([cp["xyz"], cp["xyz"]]), np.concatenate([cp["typ"], cp["typ"]]))
    for k in ("ipath", "brdist", "brpathlen", "ier", "nstep"):
        assert np.array_equal(two[k][:n], g[k]) and np.array_equal(two[k][n:], g[k]), k
    assert np.all(two["ipath"] <= n)


def test_range_test_without_square_root():
    """The device evaluators decide !(sqrt(dd) > dran) without the square
    root except within 1e-12 of dran^2.  In IEEE double arithmetic (numpy)
    that gives the same answer as the square root on squared distances a few
    ulps either side of the cutoff, and far from it, over a range of
    cutoffs."""
    rng = np.random.default_rng(7)
    dran = np.exp(rng.uniform(np.log(0.3), np.log(40.0), 4000))
    r2 = dran * dran
    near = np.concatenate([r2 * (1 + k * 2.0 ** -52) for k in range(-8, 9)])
    far = np.concatenate([r2 * f for f in (0.5, 1 - 2e-12, 1 - 1e-12, 1 + 1e-12, 1 + 2e-12, 2.0)])
    dd = np.concatenate([near, far])
    dr = np.tile(dran, len(dd) // len(dran))
    rr = dr * dr
    fast = np.where(dd < rr * (1 - 1e-12), True, np.where(dd > rr * (1 + 1e-12), False, ~(np.sqrt(dd) > dr)))
    assert np.array_equal(fast, ~(np.sqrt(dd) > dr))
