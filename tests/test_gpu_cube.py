"""NCI post-pass and cube/dat text on the GPU (c2g_nci_post_dev,
c2g_cube_text, c2g_dat_text, c2g_nciplot_files) against the oracle's
restatement, which reproduces the reference's own NCI text
(tests/test_oracle_cube.py)."""
import ctypes as C
import json
import os
import tempfile

import numpy as np
import pytest

from critic2_gb300 import synth

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
HERE = os.path.dirname(os.path.abspath(__file__))


def _p(t):
    return C.c_void_p(t.data_ptr())


def cube_text(L, lib, ns, vals):
    d = torch.tensor(np.ascontiguousarray(vals, np.float64).reshape(-1), device="cuda")
    n = C.c_long(0)
    ns = np.ascontiguousarray(ns, np.int32)
    lib.check(L.c2g_cube_text(ns, _p(d), None, 0, C.byref(n), None))
    buf = C.create_string_buffer(n.value + 1)
    lib.check(L.c2g_cube_text(ns, _p(d), buf, n.value + 1, C.byref(n), None))
    return buf.raw[: n.value]


def dat_text(L, lib, pairs):
    d = torch.tensor(np.ascontiguousarray(pairs, np.float64).reshape(-1), device="cuda")
    n = C.c_long(0)
    lib.check(L.c2g_dat_text(_p(d), len(pairs), None, 0, C.byref(n), None))
    buf = C.create_string_buffer(n.value + 1)
    lib.check(L.c2g_dat_text(_p(d), len(pairs), buf, n.value + 1, C.byref(n), None))
    return buf.raw[: n.value]


def wide_values(rng, n):
    v = rng.standard_normal(n) * 10.0 ** rng.uniform(-300, 300, n)
    v[:8] = [0.0, -0.0, 100.0, 1.0, 9.999995e-3, 123456.5, 5e-324, -1.7976931348623157e308]
    return v


@pytest.mark.parametrize("ns", [(3, 4, 29), (2, 2, 12), (1, 5, 7)])
def test_cube_text_matches_oracle(gpu_lib, oracle_mod, ns):
    L = gpu_lib.lib()
    rng = np.random.default_rng(sum(ns))
    v = wide_values(rng, int(np.prod(ns)))
    assert cube_text(L, gpu_lib, ns, v) == oracle_mod.cube_body(np.array(ns, np.int32), v)


def test_cube_and_dat_text_reproduce_reference(gpu_lib):
    """The GPU formatter writes the reference's own sampled NCI lines
    exactly from their numbers."""
    L = gpu_lib.lib()
    with open(os.path.join(HERE, "golden", "nci_cube_text.json")) as f:
        gold = json.load(f)
    lines = gold["dens_lines"] + gold["grad_lines"]
    for k in (6, 5):
        sel = [l for l in lines if len(l.split()) == k]
        vals = [[float(t) for t in l.split()] for l in sel]
        txt = cube_text(L, gpu_lib, (len(sel), 1, k), np.array(vals))
        assert txt.decode() == "".join(l + "\n" for l in sel)
    pairs = np.array([[float(t) for t in l.split()] for l in gold["dat_lines"]])
    assert dat_text(L, gpu_lib, pairs).decode() == "".join(l + "\n" for l in gold["dat_lines"])


def test_dat_text_matches_oracle(gpu_lib, oracle_mod):
    L = gpu_lib.lib()
    rng = np.random.default_rng(7)
    pairs = wide_values(rng, 2000).reshape(-1, 2)
    assert dat_text(L, gpu_lib, pairs) == oracle_mod.dat_text(pairs)


def test_nci_post_matches_oracle(gpu_lib, oracle_mod):
    L = gpu_lib.lib()
    rng = np.random.default_rng(3)
    ns = np.array([5, 37, 41], np.int32)
    n = int(ns.prod())
    crho = rng.uniform(-30, 30, n)
    cgrad = rng.uniform(0, 3, n)
    cg_ref, dat_ref = oracle_mod.nci_post(ns, crho, cgrad)
    dr = torch.tensor(crho, device="cuda")
    dg = torch.tensor(cgrad, device="cuda")
    dd = torch.zeros(2 * n, dtype=torch.float64, device="cuda")
    nd = C.c_long(0)
    gpu_lib.check(L.c2g_nci_post_dev(ns, _p(dr), _p(dg), None, _p(dd), n, C.byref(nd), None))
    assert nd.value == len(dat_ref)
    assert np.array_equal(dd[: 2 * nd.value].cpu().numpy().reshape(-1, 2), dat_ref)
    assert np.array_equal(dg.cpu().numpy(), cg_ref)


def test_nciplot_files(gpu_lib, oracle_mod):
    """End to end on the 12-atom molecule (80^3, FP64): the files' bodies are
    the oracle's formatting of the GPU cubes after the oracle's cutoff pass,
    byte for byte, and the headers follow write_cube_header."""
    from critic2_gb300.wfn import Wavefunction
    mol = synth.make_molecule("nci12")
    w = Wavefunction(mol)
    x0, xm, ns = synth.nci_grid(mol, 80, 0.1)
    crho, cgrad, _ = w.nciplot(x0, xm, ns, "fp64")
    cg_ref, dat_ref = oracle_mod.nci_post(ns, crho, cgrad)
    with tempfile.TemporaryDirectory() as d:
        root = os.path.join(d, "nci12")
        st, ms = w.nciplot_files(x0, xm, ns, "fp64", root)
        dens = open(root + "-dens.cube", "rb").read()
        grad = open(root + "-grad.cube", "rb").read()
        dat = open(root + ".dat", "rb").read()
    print(f"\nnci12 80^3 files: eval {ms[0]:.1f} ms, cutoff pass {ms[1]:.1f}, text {ms[2]:.1f}, writes {ms[3]:.1f}")
    x1 = x0 + (ns - 1) * np.diag(xm)
    inside = np.all((mol.atom_xyz > x0 - 0.1) & (mol.atom_xyz < x1 + 0.1), axis=1)
    nat = int(inside.sum()) or mol.natom
    hd = dens.split(b"\n")
    assert hd[0] == b" dens_cube" and hd[1] == b" 3d plot, density"
    assert int(hd[2].split()[0]) == nat
    assert [int(hd[3 + c].split()[0]) for c in range(3)] == [80, 80, 80]
    head_len = sum(len(l) + 1 for l in hd[: 6 + nat])
    assert dens[head_len:] == oracle_mod.cube_body(ns, crho)
    hg = grad.split(b"\n")
    assert hg[0] == b" grad_cube" and hg[1] == b" 3d plot, reduced density gradient"
    assert grad[head_len + (len(hg[0]) - len(hd[0])) + (len(hg[1]) - len(hd[1])):] == \
        oracle_mod.cube_body(ns, cg_ref)
    assert dat == oracle_mod.dat_text(dat_ref)


def precise_text(L, lib, ns, vals):
    d = torch.tensor(np.ascontiguousarray(vals, np.float64).reshape(-1), device="cuda")
    n = C.c_long(0)
    ns = np.ascontiguousarray(ns, np.int32)
    lib.check(L.c2g_cube_precise_text(ns, _p(d), None, 0, C.byref(n), None))
    buf = C.create_string_buffer(n.value + 1)
    lib.check(L.c2g_cube_precise_text(ns, _p(d), buf, n.value + 1, C.byref(n), None))
    return buf.raw[: n.value].decode()


@pytest.mark.parametrize("ns", [(3, 4, 10), (2, 2, 12)])
def test_precise_text_matches_oracle(gpu_lib, oracle_mod, ns):
    L = gpu_lib.lib()
    rng = np.random.default_rng(sum(ns) + 1)
    v = wide_values(rng, int(np.prod(ns)))
    assert precise_text(L, gpu_lib, ns, v) == oracle_mod.precise_body(ns, v)


def test_precise_text_reproduces_reference(gpu_lib):
    L = gpu_lib.lib()
    with open(os.path.join(HERE, "golden", "nci_cube_text.json")) as f:
        gold = json.load(f)
    for c in gold["precise_cubes"].values():
        for k in (6, 4):
            sel = [l for l in c["sample"] if len(l.split()) == k]
            if not sel:
                continue
            vals = np.array([[float(t) for t in l.split()] for l in sel])
            assert precise_text(L, gpu_lib, (len(sel), 1, k), vals) == "".join(l + "\n" for l in sel)


def test_cube_field_file(gpu_lib, oracle_mod):
    """CUBE plots of rho, |grad rho| and the Laplacian on the 12-atom molecule:
    values against the oracle's grd (1e-10), text against the oracle's
    formatting of the same values, header as writegrid_cube."""
    from critic2_gb300.wfn import Wavefunction
    mol = synth.make_molecule("nci12")
    w = Wavefunction(mol)
    o = oracle_mod.Wfn(mol)
    x0, xm, _ = synth.nci_grid(mol, 24, 0.25)
    ns = np.array([24, 20, 17], np.int32)
    pts = synth.grid_points(x0, xm, ns).reshape(-1, 3)
    idx = np.random.default_rng(1).choice(len(pts), 60, replace=False)
    with tempfile.TemporaryDirectory() as d:
        for prop in ("rho", "gmod", "lap", "hxy"):
            path = os.path.join(d, prop + ".cube")
            w.cube_field_file(x0, xm, ns, prop, path, "fp64")
            txt = open(path).read()
            lines = txt.split("\n")
            assert lines[0] == "critic2-cube" and lines[1] == "critic2-cube"
            assert int(lines[2].split()[0]) == mol.natom
            body = "\n".join(lines[6 + mol.natom:])
            vals = np.array([float(t) for t in body.split()])
            assert vals.size == pts.shape[0]
            assert body == oracle_mod.precise_body(ns, vals)
            for i in idx:
                r = o.grd(pts[i], 2)
                h = np.array(r.hf[:]).reshape(3, 3)
                ref = {"rho": r.f, "gmod": r.gfmod, "lap": np.trace(h), "hxy": h[0, 1]}[prop]
                assert abs(vals[i] - ref) <= 1e-10 * max(abs(ref), 1e-6 * abs(r.f)), (prop, vals[i], ref)
