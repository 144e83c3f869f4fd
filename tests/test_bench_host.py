"""Host-side pieces of bench.py that need no GPU: the roofline record of the
headline line (keys, the issued-work arithmetic, the traffic figure of the
measured launch) and the strided CPU sample grids."""
import dataclasses
import importlib.util
import os

import numpy as np

from critic2_gb300 import synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def bench_module():
    spec = importlib.util.spec_from_file_location("bench_host", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_roofline_record_large500():
    b = bench_module()
    wl = synth.WORKLOADS["large500"]
    mol = synth.make_molecule("large500")
    res = {"npts": wl.grid ** 3, "ms_kernel": 2770.0, "stage_frac": 0.0455}
    r = b.roofline_of(res, mol, mol.npri, "tf32x3", {"bf16_tflops": 1915.4}, "measured", wl)
    assert set(r) >= {"bound", "achieved", "peak", "unit", "frac", "traffic"}
    assert r["bound"] == "tensor" and r["unit"] == "TFLOP/s"
    assert abs(r["peak"] - 1915.4 / 2) < 1e-9 and abs(r["frac"] - r["achieved"] / r["peak"]) < 1e-12
    # issued work: active (tile, K-stage) pairs x MO tiles x 2 x 128 x N x K
    ntiles = wl.grid * (wl.grid // 4) * (wl.grid // 8)
    nstage = -(-mol.npri // 8)
    issued = 0.0455 * ntiles * nstage * 8 * 2.0 * 128 * b.ISSUED_COLUMNS_PER_STAGE * 8
    assert abs(r["achieved"] - issued / 2.770 / 1e12) < 1e-9 * r["achieved"]
    # the one-pass capture of the whole launch: read + written bytes
    assert abs(r["traffic"] - (1.83e9 + 1.76e9)) < 1.0
    # another grid of the same molecule has no measured traffic
    small = dataclasses.replace(wl, grid=48)
    r2 = b.roofline_of({"npts": 48 ** 3, "ms_kernel": 10.0, "stage_frac": 0.2}, mol, mol.npri, "tf32x3",
                       {"bf16_tflops": 1915.4}, "measured", small)
    assert r2["traffic"] is None


def test_sub_grid_covers_the_box():
    """Every stride-th grid point per axis from an offset that moves with the
    step: real points of the grid, spread over the whole box."""
    b = bench_module()
    x0 = np.array([-2.0, 1.0, 0.5])
    xm = np.diag([0.1, 0.2, 0.3])
    ns = np.array([40, 41, 17], np.int32)
    seen = set()
    for k in range(5):
        x0s, xms, nss = b.sub_grid(x0, xm, ns, 5, k)
        assert np.allclose(xms, 5 * xm)
        first = np.linalg.solve(xm, x0s - x0)
        assert np.allclose(first, np.round(first)) and np.all(first >= 0)
        last = first + 5 * (nss - 1)
        assert np.all(last <= ns - 1) and np.all(last + 5 > ns - 1)
        seen.add(tuple(np.round(first).astype(int)))
    assert len(seen) > 1  # the offset moves with the step
