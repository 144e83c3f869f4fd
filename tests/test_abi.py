"""The C-ABI library loads and exports every symbol include/*.h declares."""
import ctypes as C
import glob
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    syms = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        syms.update(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(c2g_\w+)\s*\(", txt, flags=re.M))
    return sorted(syms)


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("c2g_wfn_create", "c2g_rho2", "c2g_grd", "c2g_nciplot", "c2g_newton", "c2g_autocritic"):
        assert s in syms


def test_library_exports_every_declared_symbol(gpu_lib):
    L = gpu_lib.lib()
    missing = [s for s in declared_symbols() if not hasattr(L, s)]
    assert not missing, missing
    assert set(gpu_lib.EXPORTS) <= set(declared_symbols())


def test_abi_version_and_errors(gpu_lib):
    L = gpu_lib.lib()
    assert L.c2g_abi_version() == 1
    # null handle -> argument error with a message, no crash
    rc = L.c2g_rho2(None, 1, None, 0, 0, None, None, None, None, None, None)
    assert rc == 1
    assert "null handle" in gpu_lib.last_error()
    n = C.c_int()
    assert L.c2g_pair_seeds(None, 15.0, 5, None, C.byref(n)) == 1


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the no-device error path")
def test_create_without_gpu_reports_cuda_error(gpu_lib):
    from critic2_gb300 import synth, wfn
    mol = synth.make_molecule("nci12")
    with pytest.raises(gpu_lib.C2GError) as e:
        wfn.Wavefunction(mol)
    assert e.value.code == 2
