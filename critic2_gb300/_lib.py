"""ctypes binding of libcritic2_gb300.so (the C ABI in include/critic2_gb300.h).

Loading fails loudly when the library has not been built: there is no
CPU fallback anywhere in this package.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcritic2_gb300.so")

C2G_OK = 0
PREC = {"fp64": 0, "tf32x3": 1, "bf16x3": 2}
ERRORS = {1: "argument", 2: "cuda", 3: "alloc", 4: "io", 5: "unsupported", 6: "numeric"}

# every symbol include/critic2_gb300.h declares
EXPORTS = ("c2g_abi_version", "c2g_last_error", "c2g_wfn_create", "c2g_wfn_read_wfx", "c2g_wfn_read_wfn", "c2g_wfn_read_fchk", "c2g_wfn_read_molden",
           "c2g_wfn_destroy", "c2g_wfn_set_edf", "c2g_wfn_set_param", "c2g_wfn_info", "c2g_rho2", "c2g_rho2_valence", "c2g_grd", "c2g_nciplot",
           "c2g_nciplot_dev", "c2g_nciplot_dev_noalloc", "c2g_newton", "c2g_pair_seeds",
           "c2g_autocritic", "c2g_nci_post_dev", "c2g_cube_text", "c2g_dat_text", "c2g_nciplot_files",
           "c2g_grid_field_dev", "c2g_cube_precise_text", "c2g_cube_field_file",
           "c2g_nci_chk_write", "c2g_nci_chk_read", "c2g_cp_graph", "c2g_basin_size", "c2g_basin_integrals", "c2g_sphere_integrals",
           "c2g_mesh_size", "c2g_mesh_dev", "c2g_molcalc",
           # learned CP-seed proposer (include/critic2_gb300_cpseed.h)
           "c2g_cs_conv3d", "c2g_cs_conv3d_bwd_data", "c2g_cs_conv3d_bwd_weight", "c2g_cs_loss",
           "c2g_cs_targets", "c2g_cs_features", "c2g_cs_seeds", "c2g_cs_adam")


class C2GError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"critic2_gb300 error {code} ({ERRORS.get(code, '?')}): {msg}")
        self.code = code


class NciStats(C.Structure):
    _fields_ = [("npoints", C.c_long), ("nrecheck", C.c_long), ("ms_kernel", C.c_double),
                ("ms_recheck", C.c_double), ("stage_frac", C.c_double)]


class NciCut(C.Structure):
    _fields_ = [("rhocut", C.c_double), ("dimcut", C.c_double), ("rhoplot", C.c_double),
                ("srho_lo", C.c_double), ("srho_hi", C.c_double), ("onlyneg", C.c_int)]


class GraphStats(C.Structure):
    _fields_ = [("npath", C.c_int), ("nbatch", C.c_int), ("nevals", C.c_long), ("ms_total", C.c_double)]


class BasinStats(C.Structure):
    _fields_ = [("natt", C.c_int), ("nray", C.c_int), ("npath", C.c_long), ("nbatch", C.c_long),
                ("nevals", C.c_long), ("nwarn", C.c_int), ("nrestart", C.c_int), ("ms_total", C.c_double)]


class MeshStats(C.Structure):
    _fields_ = [("npoints", C.c_long), ("ms_mesh", C.c_double), ("ms_total", C.c_double)]


class CpReport(C.Structure):
    _fields_ = [("ncp", C.c_int), ("count", C.c_int * 4), ("poincare_hopf", C.c_int),
                ("nseed", C.c_int), ("nconverged", C.c_int), ("ms_total", C.c_double)]


_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_vp = C.c_void_p

_lib = None


def lib():
    """Loads the shared library (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with critic2_gb300.build.build()")
    L = C.CDLL(LIB_PATH)
    L.c2g_abi_version.restype = C.c_int
    L.c2g_last_error.argtypes = [C.c_char_p, C.c_int]
    L.c2g_wfn_create.argtypes = [C.c_int, _dp, _ip, C.c_int, C.c_int, _ip, _ip, _dp, _dp, _dp,
                                 C.c_int, C.c_int, C.POINTER(_vp)]
    L.c2g_wfn_read_wfx.argtypes = [C.c_char_p, C.POINTER(_vp)]
    L.c2g_wfn_read_wfn.argtypes = [C.c_char_p, C.POINTER(_vp)]
    L.c2g_wfn_read_fchk.argtypes = [C.c_char_p, C.POINTER(_vp)]
    L.c2g_wfn_read_molden.argtypes = [C.c_char_p, C.POINTER(_vp)]
    L.c2g_wfn_destroy.argtypes = [_vp]
    L.c2g_wfn_set_param.argtypes = [_vp, C.c_int, C.c_double]
    L.c2g_wfn_set_edf.argtypes = [_vp, C.c_int, _vp, _vp, _vp, _vp]
    L.c2g_mesh_size.argtypes = [_vp, C.c_int, C.c_int, C.POINTER(C.c_long)]
    L.c2g_mesh_dev.argtypes = [_vp, C.c_int, C.c_int, _vp, _vp, _vp]
    L.c2g_molcalc.argtypes = [_vp, C.c_int, C.c_int, C.c_int, C.c_int, _vp, _vp, C.POINTER(MeshStats)]
    L.c2g_cp_graph.argtypes = [_vp, C.c_int, _vp, _vp] + [_vp] * 7 + [C.POINTER(GraphStats)]
    L.c2g_basin_size.argtypes = [_vp, C.c_int, _vp, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int),
                                 C.POINTER(C.c_int)]
    L.c2g_sphere_integrals.argtypes = [_vp, C.c_int, _vp, _vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                       C.c_double, C.c_double, _vp, _vp, _vp]
    L.c2g_basin_integrals.argtypes = [_vp, C.c_int, _vp, _vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double] + \
        [_vp] * 6 + [C.POINTER(BasinStats)]
    L.c2g_nci_chk_write.argtypes = [C.c_char_p, _dp, _dp, _ip, _dp, _dp]
    L.c2g_nci_chk_read.argtypes = [C.c_char_p, _dp, _dp, _ip, _dp, _dp, C.POINTER(C.c_int)]
    L.c2g_wfn_info.argtypes = [_vp] + [C.POINTER(C.c_int)] * 5
    L.c2g_rho2.argtypes = [_vp, C.c_int, _vp, C.c_int, C.c_int] + [_vp] * 6
    L.c2g_rho2_valence.argtypes = [_vp, C.c_int, _vp, C.c_int] + [_vp] * 3
    L.c2g_grd.argtypes = [_vp, C.c_int, _vp, C.c_int, C.c_int] + [_vp] * 8
    L.c2g_nciplot.argtypes = [_vp, _dp, _dp, _ip, C.c_int, _vp, _vp, C.POINTER(NciStats)]
    L.c2g_nciplot_dev.argtypes = [_vp, _dp, _dp, _ip, C.c_int, _vp, _vp, _vp, C.POINTER(NciStats)]
    L.c2g_nciplot_dev_noalloc.argtypes = [_vp, _dp, _dp, _ip, C.c_int, _vp, _vp, _vp]
    L.c2g_newton.argtypes = [_vp, C.c_int, _vp, C.c_double, C.c_int, C.c_int, _vp]
    L.c2g_pair_seeds.argtypes = [_vp, C.c_double, C.c_int, _vp, C.POINTER(C.c_int)]
    L.c2g_autocritic.argtypes = [_vp, C.c_int, _vp, C.c_int, C.c_int, _vp, _vp, _vp,
                                 C.POINTER(CpReport)]
    L.c2g_nci_post_dev.argtypes = [_ip, _vp, _vp, C.POINTER(NciCut), _vp, C.c_long, C.POINTER(C.c_long), _vp]
    L.c2g_cube_text.argtypes = [_ip, _vp, C.c_char_p, C.c_long, C.POINTER(C.c_long), _vp]
    L.c2g_dat_text.argtypes = [_vp, C.c_long, C.c_char_p, C.c_long, C.POINTER(C.c_long), _vp]
    L.c2g_nciplot_files.argtypes = [_vp, _dp, _dp, _ip, C.c_int, C.c_char_p, C.POINTER(NciCut),
                                    C.POINTER(NciStats), _dp]
    L.c2g_grid_field_dev.argtypes = [_vp, _dp, _dp, _ip, C.c_int, C.c_int, _vp, _vp]
    L.c2g_cube_precise_text.argtypes = [_ip, _vp, C.c_char_p, C.c_long, C.POINTER(C.c_long), _vp]
    L.c2g_cube_field_file.argtypes = [_vp, _dp, _dp, _ip, C.c_int, C.c_int, C.c_char_p, _dp]
    i, f, lg = C.c_int, C.c_float, C.c_long
    L.c2g_cs_conv3d.argtypes = [_vp, i, i, i, i, i, _vp, _vp, i, i, i, _vp, _vp]
    L.c2g_cs_conv3d_bwd_data.argtypes = [_vp, i, i, i, i, i, _vp, i, i, _vp, _vp, _vp]
    L.c2g_cs_conv3d_bwd_weight.argtypes = [_vp, _vp, i, i, i, i, i, i, i, _vp, _vp, _vp]
    L.c2g_cs_loss.argtypes = [_vp, _vp, lg, i, f, f, _vp, _vp, _vp]
    L.c2g_cs_targets.argtypes = [_vp, i, i, _vp, _vp]
    L.c2g_cs_features.argtypes = [_vp, _vp, lg, _vp, _vp]
    L.c2g_cs_seeds.argtypes = [_vp, i, _dp, C.c_double, f, i, i, _vp, _vp, _vp, _vp]
    L.c2g_cs_adam.argtypes = [_vp, _vp, _vp, _vp, i, f, f, f, f, i, _vp]
    _lib = L
    return L


def last_error() -> str:
    buf = C.create_string_buffer(1024)
    lib().c2g_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(rc: int):
    if rc != C2G_OK:
        raise C2GError(rc, last_error())


def ptr(a):
    return None if a is None else a.ctypes.data_as(_vp)
