"""makegraph on the GPU (c2g_cp_graph: gradient paths traced together, one
FP64 batch per Runge-Kutta stage) against the oracle's serial restatement,
on the oracle's CP list.  The step control compares error estimates with
1e-4 and |grad| with 1e-7, so where a test sits within rounding of its
threshold a path takes another step sequence; both are solutions of the
same ODE to the integrator's tolerance.  Bars: the graph (every path's
terminator) identical; end distances and angles identical where both paths
end in a beta sphere (the end point is then the CP itself), to 1e-3 for 95%
of all normally ended paths (a path that stops at a new CP stops in a flat
tail, where the stopping point follows the step sequence); path lengths to 1e-5 relative for 95% of the paths
(1e-9 for the median one; paths into flat tails, where |grad| is small and
its direction sensitive, differ by ~1e-6; on cp100 the few paths whose step sequence
differs are within 1.3% of the oracle's length)."""
import numpy as np
import pytest

from critic2_gb300 import synth

pytestmark = pytest.mark.gpu


def compare(g, o, typ, xyz):
    sel = np.abs(typ) == 1
    assert np.array_equal(g["ipath"][sel], o["ipath"][sel])
    assert np.array_equal(g["ipath"][~sel], np.zeros_like(g["ipath"][~sel]))
    assert np.allclose(g["brvec"], o["brvec"], atol=1e-9)
    assert (g["ier"] == o["ier"])[sel].mean() >= 0.95
    both = (g["ier"] == 0) & (o["ier"] == 0) & sel[:, None]
    # paths that end in a beta sphere end on the terminating CP itself
    term = np.clip(o["ipath"] - 1, 0, None)
    to_cp = np.abs(o["brdist"] - np.linalg.norm(xyz[term] - xyz[:, None, :], axis=2)) < 1e-12
    end = both & to_cp
    assert np.allclose(g["brdist"][end], o["brdist"][end], rtol=1e-12, atol=1e-12)
    # a path that stops at a new CP stops where |grad| first drops below
    # 1e-7, in a flat tail: that point moves with the step sequence
    rd = np.abs(g["brdist"][both] - o["brdist"][both]) / o["brdist"][both]
    assert np.quantile(rd, 0.95) <= 1e-3
    rel = np.abs(g["brpathlen"][both] - o["brpathlen"][both]) / o["brpathlen"][both]
    print(f"  {int(end.sum())} of {int(both.sum())} paths end in a beta sphere; path length |rel diff|: "
          f"median {np.median(rel):.1e}, p99 {np.quantile(rel, 0.99):.1e}, max {rel.max():.1e}; "
          f"same step count {np.mean((g['nstep'] == o['nstep'])[sel]):.3f}")
    assert np.median(rel) <= 1e-9
    assert np.mean(rel <= 1e-5) >= 0.95
    assert rel.max() <= 5e-2
    ok = end.all(1)
    assert np.allclose(g["brang"][ok], o["brang"][ok], atol=1e-9)


@pytest.mark.parametrize("name", ["nci12", "cp100"])
def test_graph_vs_oracle(gpu_lib, oracle_mod, name):
    from critic2_gb300.wfn import Wavefunction
    mol = synth.make_molecule(name)
    g, o = Wavefunction(mol), oracle_mod.Wfn(mol)
    cp = o.autocritic()
    typ = cp["typ"]
    og = o.makegraph(cp["xyz"], typ)
    gg = g.cp_graph(cp["xyz"], typ)
    st = gg["stats"]
    print(f"\n{name}: {int((np.abs(typ) == 1).sum())} bond/ring CPs, {st['npath']} paths, "
          f"{st['nbatch']} batches, {st['nevals']} evaluations, {st['ms']:.1f} ms")
    assert st["npath"] == 2 * int((np.abs(typ) == 1).sum())
    compare(gg, og, typ, cp["xyz"])


def test_graph_on_gpu_cp_list(gpu_lib):
    """The graph of the library's own CP search: every bond path that ends
    normally ends at an attractor (nucleus or non-nuclear maximum)."""
    from critic2_gb300.wfn import Wavefunction
    mol = synth.make_molecule("nci12")
    g = Wavefunction(mol)
    cp = g.autocritic(prec="fp64")
    typ = cp["typ"]
    gg = g.cp_graph(cp["xyz"], typ)
    for i in np.nonzero(typ == -1)[0]:
        for j in range(2):
            if gg["ier"][i, j] == 0:
                assert typ[gg["ipath"][i, j] - 1] == -3


def test_graph_rejects_bad_types(gpu_lib):
    from critic2_gb300 import _lib
    from critic2_gb300.wfn import Wavefunction
    g = Wavefunction(synth.make_molecule("nci12"))
    with pytest.raises(_lib.C2GError):
        g.cp_graph(np.zeros((1, 3)), np.array([2], np.int32))
    out = g.cp_graph(np.zeros((0, 3)), np.zeros(0, np.int32))
    assert out["stats"]["npath"] == 0


def test_graph_duplicate_cps_keep_first(gpu_lib, oracle_mod):
    """The beta-sphere candidate is found by a warp (every lane scans every
    32nd CP); equal distances must keep the first CP, as critic2's serial
    scan does.  The CP list given twice over (more than 32 entries, so each
    copy sits on another lane) yields the same terminators, all in the
    first copy, and the same paths."""
    from critic2_gb300.wfn import Wavefunction
    mol = synth.make_molecule("nci12")
    g, o = Wavefunction(mol), oracle_mod.Wfn(mol)
    cp = o.autocritic()
    x, t = cp["xyz"], cp["typ"]
    n = len(t)
    assert n > 32 and n % 32
    one = g.cp_graph(x, t)
    two = g.cp_graph(np.concatenate([x, x]), np.concatenate([t, t]))
    for k in ("ipath", "brdist", "brpathlen", "ier", "nstep"):
        assert np.array_equal(two[k][:n], one[k]), k
        assert np.array_equal(two[k][n:], one[k]), k
    assert np.all(two["ipath"] <= n)
