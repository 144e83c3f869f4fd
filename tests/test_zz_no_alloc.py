"""c2g_nciplot_dev_noalloc: the no-allocation NCI entry against the
allocating one (c2g_nciplot_dev), through the C ABI, two calls in a row.

The file is named to be collected last, so that it runs both alone and
after every other GPU test in the same process."""
import numpy as np
import pytest

from critic2_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup(gpu_lib):
    import torch
    from critic2_gb300.wfn import Wavefunction
    mol = synth.make_molecule("nci12")
    w = Wavefunction(mol)
    dev = torch.device("cuda", 0)
    return torch, w, mol, dev


def _bufs(torch, n, dev):
    return (torch.full((n,), np.nan, dtype=torch.float64, device=dev),
            torch.full((n,), np.nan, dtype=torch.float64, device=dev))


@pytest.mark.parametrize("prec", ["tf32x3", "bf16x3", "fp64"])
def test_noalloc_matches_allocating_entry(setup, prec):
    torch, w, mol, dev = setup
    # 48 x 64 x 80 = 245,760 points (below the 2^20 limit), with a nucleus
    # exactly on a grid point so that the device-side nucleus rule is used
    x0, xm, _ = synth.nci_grid(mol, 64, 0.15)
    ns = np.array([48, 64, 80], np.int32)
    x0 = mol.atom_xyz[0] - 0.15 * np.array([20, 30, 40])
    n = int(np.prod(ns))
    stream = torch.cuda.current_stream(dev)
    ref_r, ref_g = _bufs(torch, n, dev)
    w.nciplot_dev(x0, xm, ns, prec, ref_r.data_ptr(), ref_g.data_ptr(), stream.cuda_stream)
    torch.cuda.synchronize()
    inuc = (20 * ns[1] + 30) * ns[2] + 40
    assert ref_g[inuc].item() == 0.0
    outs = [_bufs(torch, n, dev) for _ in range(2)]
    free = []
    for r, g in outs:
        w.nciplot_dev_noalloc(x0, xm, ns, prec, r.data_ptr(), g.data_ptr(), stream.cuda_stream)
        torch.cuda.synchronize()
        free.append(torch.cuda.mem_get_info(dev)[0])
    # the second call takes no device memory (the first one may load the
    # library's GPU code and its static scratch)
    assert free[1] == free[0]
    for r, g in outs:
        # same kernels, same arithmetic: equal to the allocating entry
        # (tolerance 1e-12 relative, FP64 outputs)
        assert torch.isfinite(r).all() and torch.isfinite(g).all()
        assert torch.allclose(r, ref_r, rtol=1e-12, atol=0.0)
        assert torch.allclose(g, ref_g, rtol=1e-12, atol=0.0)
        assert g[inuc].item() == 0.0


def test_noalloc_rejects(setup, gpu_lib):
    torch, w, mol, dev = setup
    x0, xm, _ = synth.nci_grid(mol, 8, 0.1)
    r, g = _bufs(torch, 8, dev)
    big = np.array([1, 1024, 1025], np.int32)  # 1,049,600 > 2^20 points
    with pytest.raises(gpu_lib.C2GError) as e:
        w.nciplot_dev_noalloc(x0, xm, big, "tf32x3", r.data_ptr(), g.data_ptr())
    assert e.value.code == 1 and "at most 1048576" in str(e.value)
    # a fresh handle has no split operands yet: refused, nothing allocated
    from critic2_gb300.wfn import Wavefunction
    w2 = Wavefunction(mol)
    with pytest.raises(gpu_lib.C2GError) as e:
        w2.nciplot_dev_noalloc(x0, xm, np.array([2, 2, 2], np.int32), "bf16x3", r.data_ptr(), g.data_ptr())
    assert e.value.code == 5
