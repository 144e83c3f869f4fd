"""FP64 plain-form parity: the CUDA evaluator through the C ABI against the
oracle, on seeded synthetic wavefunctions.  Bar: 1e-10 relative."""
import os
import tempfile

import numpy as np
import pytest

from critic2_gb300 import synth

pytestmark = pytest.mark.gpu

REL = 1e-10


@pytest.fixture(scope="module")
def mol12():
    return synth.make_molecule("nci12")


@pytest.fixture(scope="module")
def pair12(gpu_lib, oracle_mod, mol12):
    from critic2_gb300.wfn import Wavefunction
    return Wavefunction(mol12), oracle_mod.Wfn(mol12)


def variant(mol, wfntyp):
    """The same primitives as an open-shell wavefunction."""
    m = synth.Molecule(**{k: getattr(mol, k) for k in
                          ("atom_xyz", "atom_z", "icenter", "itype", "e", "occ", "cmo")},
                       wfntyp=wfntyp, nalpha=mol.nmo // 2 + 1, name=mol.name)
    m.occ = m.occ.copy()
    if wfntyp == 1:
        m.occ[:] = 1.0
    elif wfntyp == 2:
        m.occ[m.nalpha:] = 1.0
    return m


def rel_err(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300))


def close(a, b, rel=REL, scale=None):
    a, b = np.asarray(a, float), np.asarray(b, float)
    s = np.abs(b).max() if scale is None else scale
    return np.all(np.abs(a - b) <= rel * np.maximum(np.abs(b), 1e-6 * s))


def test_rho2_all_outputs(pair12, mol12):
    g, o = pair12
    rng = np.random.default_rng(0)
    lo, hi = mol12.atom_xyz.min(0) - 2, mol12.atom_xyz.max(0) + 2
    pts = rng.uniform(lo, hi, size=(300, 3))
    for nder in (0, 1, 2):
        out = g.rho2(pts, nder=nder, prec="fp64")
        for i in range(0, 300, 7):
            ref = o.rho2(pts[i], nder)
            assert close(out["rho"][i], ref["rho"])
            if nder > 0:
                assert close(out["grad"][i], ref["grad"])
                assert close(out["gkin"][i], ref["gkin"])
            if nder > 1:
                assert close(out["hess"][i], ref["h"])
                assert close(out["stress"][i], ref["stress"], scale=np.abs(ref["h"]).max())
                assert abs(out["vir"][i] - ref["vir"]) <= REL * max(1.0, np.abs(ref["stress"]).max())


@pytest.mark.parametrize("wfntyp", [1, 2])
def test_rho2_open_shell(gpu_lib, oracle_mod, mol12, wfntyp):
    from critic2_gb300.wfn import Wavefunction
    m = variant(mol12, wfntyp)
    g, o = Wavefunction(m), oracle_mod.Wfn(m)
    rng = np.random.default_rng(wfntyp)
    pts = rng.uniform(mol12.atom_xyz.min(0), mol12.atom_xyz.max(0), size=(64, 3))
    out = g.rho2(pts, 2, "fp64")
    for i in range(64):
        ref = o.rho2(pts[i], 2)
        assert close(out["rho"][i], ref["rho"])
        assert close(out["grad"][i], ref["grad"])
        assert close(out["hess"][i], ref["h"])
        assert close(out["gkin"][i], ref["gkin"])
    # the density-only and first-derivative records keep the spin channels
    for nder in (0, 1):
        out = g.rho2(pts, nder, "fp64")
        for i in range(0, 64, 4):
            ref = o.rho2(pts[i], nder)
            assert close(out["rho"][i], ref["rho"])
            if nder:
                assert close(out["grad"][i], ref["grad"])


def test_grd(pair12, mol12):
    g, o = pair12
    rng = np.random.default_rng(3)
    pts = np.concatenate([rng.uniform(mol12.atom_xyz.min(0), mol12.atom_xyz.max(0), size=(50, 3)),
                          mol12.atom_xyz[:3] + 1e-7,          # on nuclei
                          mol12.atom_xyz.max(0) + 40.0 * np.ones((1, 3))])  # wraps in the cell
    out = g.grd(pts, 2, "fp64")
    for i, p in enumerate(pts):
        ref = o.grd(p, 2)
        assert out["isnuc"][i] == ref.isnuc
        assert close(out["f"][i], ref.f)
        assert abs(out["gfmod"][i] - ref.gfmod) <= REL * max(abs(ref.gfmod), 1e-6 * abs(ref.f))
        ev = np.array(ref.hfeval[:])
        assert np.all(np.abs(out["hfeval"][i] - ev) <= REL * np.abs(ev).max())
        assert (out["r"][i], out["s"][i]) == (ref.r, ref.s)


def test_nciplot_small_grid(pair12, mol12):
    g, o = pair12
    x0, xm, ns = synth.nci_grid(mol12, 80, 0.1)
    crho, cgrad, st = g.nciplot(x0, xm, ns, "fp64")
    rr, rg = o.nciplot(x0, xm, ns)
    assert crho.shape == rr.shape == (80, 80, 80)
    assert rel_err(np.abs(crho), np.abs(rr)) < REL
    assert rel_err(cgrad, rg) < REL
    flips = np.sign(crho) != np.sign(rr)
    # a sign may differ only where lambda2 is zero to rounding
    if flips.any():
        pts = synth.grid_points(x0, xm, ns).reshape(-1, 3)[flips.reshape(-1)]
        for p in pts[:20]:
            r = o.grd(p, 2)
            ev = np.array(r.hfeval[:])
            assert abs(ev[1]) < 1e-9 * np.abs(ev).max()
    assert flips.mean() < 1e-4


def test_nciplot_planes_nci60(gpu_lib, oracle_mod):
    from critic2_gb300.wfn import Wavefunction
    mol = synth.make_molecule("nci60")
    g, o = Wavefunction(mol), oracle_mod.Wfn(mol)
    x0, xm, ns = synth.nci_grid(mol, 200, 0.1)
    for i in (0, 113):
        x0i = x0 + i * xm[:, 0]
        nsi = np.array([1, 200, 200], np.int32)
        crho, cgrad, _ = g.nciplot(x0i, xm, nsi, "fp64")
        rr, rg = o.nciplot(x0i, xm, nsi)
        assert rel_err(np.abs(crho), np.abs(rr)) < REL
        assert rel_err(cgrad, rg) < REL


def test_wfx_roundtrip(gpu_lib, pair12, mol12):
    from critic2_gb300.wfn import Wavefunction
    g, _ = pair12
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "m.wfx")
        synth.write_wfx(mol12, path)
        gw = Wavefunction.from_wfx(path)
    assert (gw.natom, gw.npri, gw.nmo) == (g.natom, g.npri, g.nmo)
    pts = np.random.default_rng(4).uniform(2, 10, size=(40, 3))
    a, b = g.rho2(pts, 2), gw.rho2(pts, 2)
    assert close(a["hess"], b["hess"], rel=1e-13)


def noise_floor(o, x):
    """critic2's gfnormeps (1e-12, absolute) can sit below the FP64
    rounding floor of |grad rho| at high-density CPs; there the reference's
    own converged/maxit outcome depends on rounding.  A point is in that band
    when the oracle's |grad| there is below 1e-9."""
    return o.grd(x, 2).gfmod < 1e-9


def test_newton(pair12, mol12):
    g, o = pair12
    seeds = g.pair_seeds()
    ref_seeds = o.pair_seeds()
    assert np.array_equal(seeds, ref_seeds)
    sub = seeds[::11]
    xg, ierg = g.newton(sub, 1e-12, 200, "fp64")
    xo, iero = o.newton_batch(sub, 1e-12, 200)
    same = ierg == iero
    for i in np.nonzero(~same)[0]:
        assert {int(ierg[i]), int(iero[i])} == {0, 2}
        assert noise_floor(o, xo[i]) and noise_floor(o, xg[i])
    assert same.mean() > 0.8
    # a converged point is fixed only to ~|grad|/|lambda_min|: compare that
    # both runs reach the same CP, and that the GPU's point is a CP for the
    # oracle's own evaluation.  In the far tail (rho ~ 1e-13) the absolute
    # threshold |grad| < 1e-12 holds over whole regions, so "converged"
    # positions there are not defined to better than that region; positions
    # are compared where the oracle's density exceeds 1e-8.
    ok = (iero == 0) & (ierg == 0)
    # Two points that both meet |grad| < 1e-12 lie within 2e-12/|lambda|_min
    # of the CP and of each other.
    xs, tol = [], []
    for x in xo[ok]:
        r = o.grd(x, 2)
        xs.append(r.f > 1e-8)
        tol.append(max(1e-6, 1e-11 / max(np.abs(np.array(r.hfeval[:])).min(), 1e-300)))
    dense, tol = np.array(xs, bool), np.array(tol)
    d = np.linalg.norm(xg[ok] - xo[ok], axis=1)
    assert dense.sum() > 0
    bad = dense & (d > tol)
    assert not bad.any(), (d[bad], tol[bad], xg[ok][bad], xo[ok][bad])
    for i in np.nonzero(ierg == 0)[0]:
        assert o.grd(xg[i], 2).gfmod < 1e-9


def test_autocritic(pair12):
    g, o = pair12
    res = g.autocritic(prec="fp64")
    ref = o.autocritic()
    # match CPs by position; unmatched ones must be noise-floor CPs
    matched_g = np.zeros(len(res["xyz"]), bool)
    for j, x in enumerate(ref["xyz"]):
        d = np.linalg.norm(res["xyz"] - x, axis=1)
        i = int(np.argmin(d))
        if d[i] < 1e-6:
            matched_g[i] = True
            assert res["typ"][i] == ref["typ"][j]
            assert abs(res["f"][i] - ref["f"][j]) <= 1e-10 * abs(ref["f"][j])
        else:
            assert noise_floor(o, x)
    for i in np.nonzero(~matched_g)[0]:
        assert noise_floor(o, res["xyz"][i])
    if matched_g.all() and len(res["xyz"]) == len(ref["xyz"]):
        assert list(res["counts"]) == list(ref["counts"]) and res["ph"] == ref["ph"]


def test_autocritic_cp100_vs_oracle(gpu_lib, oracle_mod):
    """cp100 (100 atoms, 22,160 pair seeds), FP64 AUTO on the GPU against
    the oracle's.  critic2 declares Newton converged at an absolute
    |grad rho| < 1e-12 (src/fieldmod@proc.f90:2256), which on these
    densities (rho up to 1e3) lies on the FP64 rounding floor of |grad rho|:
    the two evaluators' summation orders put a CP on either side of it.
    So the CP lists are compared up to that floor: every CP one search lists
    and the other does not is a CP of the other's own field (|grad rho| <=
    1e-10 there, same rank 3 and signature), and the other's Newton with
    gfnormeps 1e-10 converges from it without moving more than 1e-8 bohr.
    CPs found by both have the same type and density (1e-10)."""
    from critic2_gb300.wfn import Wavefunction
    mol = synth.make_molecule("cp100")
    g, o = Wavefunction(mol), oracle_mod.Wfn(mol)
    res = g.autocritic(prec="fp64")
    ref = o.autocritic()
    nat = mol.natom
    gx, ox = res["xyz"][nat:], ref["xyz"][nat:]
    gt, ot = res["typ"][nat:], ref["typ"][nat:]
    d = np.linalg.norm(gx[:, None, :] - ox[None, :, :], axis=2)
    gi = d.argmin(1) if len(ox) else np.zeros(len(gx), int)
    in_ref = d.min(1) < 1e-2 if len(ox) else np.zeros(len(gx), bool)
    in_res = d.min(0) < 1e-2 if len(gx) else np.zeros(len(ox), bool)
    for i in np.nonzero(in_ref)[0]:
        j = gi[i]
        assert gt[i] == ot[j]
        assert abs(res["f"][nat + i] - ref["f"][nat + j]) <= 1e-10 * abs(ref["f"][nat + j])
    # found by the GPU only: CPs of the oracle's field to its rounding floor
    only_g = gx[~in_ref]
    for x, t in zip(only_g, gt[~in_ref]):
        r = o.grd(x, 2)
        assert r.gfmod <= 1e-10 and r.r == 3 and r.s == t
    xo, ier = o.newton_batch(only_g, 1e-10)
    assert np.all(ier == 0) and np.linalg.norm(xo - only_g, axis=1).max() <= 1e-8
    # found by the oracle only: CPs of the GPU's field to its rounding floor
    only_o = ox[~in_res]
    if len(only_o):
        q = g.grd(only_o, 2, "fp64")
        assert np.all(q["gfmod"] <= 1e-10) and np.all(q["r"] == 3) and np.all(q["s"] == ot[~in_res])
        xg, ierg = g.newton(only_o, 1e-10)
        assert np.all(ierg == 0) and np.linalg.norm(xg - only_o, axis=1).max() <= 1e-8
    # nearly every oracle CP is found by the GPU
    assert in_res.mean() >= 0.95
    print(f"\ncp100: GPU {len(gx)} non-nuclear CPs (PH {res['ph']}), oracle {len(ox)} (PH {ref['ph']}), "
          f"{int(in_ref.sum())} common, GPU-only {len(only_g)}, oracle-only {len(only_o)}")


def test_autocritic_distinct_pair_seeds(gpu_lib):
    """The default seeding takes each unordered atom pair once; critic2's own
    list (c2g_pair_seeds: both ordered pairs, every point twice) gives the
    same CP list, types, densities and Poincare-Hopf sum (cp100)."""
    from critic2_gb300.wfn import Wavefunction
    mol = synth.make_molecule("cp100")
    g = Wavefunction(mol)
    full = g.pair_seeds()
    a = g.autocritic(prec="fp64")
    b = g.autocritic(full, prec="fp64")
    assert a["nseed"] * 2 == len(full)
    assert len(a["xyz"]) == len(b["xyz"]) and list(a["counts"]) == list(b["counts"]) and a["ph"] == b["ph"]
    assert np.allclose(a["xyz"], b["xyz"], rtol=0, atol=1e-9)
    assert np.array_equal(a["typ"], b["typ"])
    assert np.allclose(a["f"], b["f"], rtol=1e-12, atol=0)


def test_error_paths(pair12, gpu_lib):
    g, _ = pair12
    with pytest.raises(gpu_lib.C2GError) as e:
        g.rho2(np.zeros((2, 3)), nder=3)
    assert e.value.code == 1
    with pytest.raises(gpu_lib.C2GError):
        g.nciplot(np.zeros(3), np.eye(3), [0, 4, 4])


def test_newton_stall_option(pair12):
    """C2G_PARAM_NEWTON_STALL (off by default): seeds that converge without
    it converge to the same points with it, and a seed it stops sits at the
    FP64 rounding floor of |grad|."""
    g, o = pair12
    seeds = g.pair_seeds()[::5]
    x0, ier0 = g.newton(seeds, 1e-12, 200, "fp64")
    g.set_newton_stall(30)
    try:
        x1, ier1 = g.newton(seeds, 1e-12, 200, "fp64")
    finally:
        g.set_newton_stall(0)
    both = (ier0 == 0) & (ier1 == 0)
    assert np.array_equal(x0[both], x1[both])
    lost = (ier0 == 0) & (ier1 != 0)
    assert lost.sum() <= max(2, 0.02 * (ier0 == 0).sum())
    for i in np.nonzero(lost)[0]:
        assert noise_floor(o, x1[i])


def gh_molecule():
    """nci12 plus one g and one h shell on every heavy atom (li types 21-56)."""
    mol = synth.make_molecule("nci12")
    rng = np.random.default_rng(21)
    ic, it, e = list(mol.icenter), list(mol.itype), list(mol.e)
    for a in np.nonzero(mol.atom_z != 1)[0]:
        for sh in ("g", "h"):
            alpha = float(np.exp(rng.uniform(np.log(0.3), np.log(3.0))))
            for t in synth.SHELL_TYPES[sh]:
                ic.append(a + 1)
                it.append(t)
                e.append(alpha)
    extra = len(e) - mol.npri
    cmo = np.concatenate([mol.cmo, 0.3 * rng.standard_normal((extra, mol.nmo))])
    return synth.Molecule(mol.atom_xyz, mol.atom_z, np.array(ic, np.int32), np.array(it, np.int32),
                          np.array(e), mol.occ, np.ascontiguousarray(cmo), name="nci12gh")


def test_g_and_h_shells(gpu_lib, oracle_mod):
    """g and h primitives (critic2's li rows 21-56): FP64 rho2 against the
    oracle (whose g/h chi are pinned symbolically)."""
    from critic2_gb300.wfn import Wavefunction
    m = gh_molecule()
    g, o = Wavefunction(m), oracle_mod.Wfn(m)
    rng = np.random.default_rng(5)
    pts = rng.uniform(m.atom_xyz.min(0) - 1, m.atom_xyz.max(0) + 1, size=(80, 3))
    out = g.rho2(pts, 2, "fp64")
    for i in range(80):
        ref = o.rho2(pts[i], 2)
        assert close(out["rho"][i], ref["rho"])
        assert close(out["grad"][i], ref["grad"])
        assert close(out["hess"][i], ref["h"])
