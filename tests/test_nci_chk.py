"""nciplot's checkpoint file <root>.chk_nci (writechk / readchk,
src/nci@proc.f90:1019-1117) through the library's host entry points
(c2g_nci_chk_write / c2g_nci_chk_read: file I/O only, no GPU needed),
against the oracle's restatement of the records and of gfortran's
unformatted sequential layout."""
import os
import struct

import numpy as np
import pytest

from critic2_gb300 import _lib
from critic2_gb300.wfn import nci_chk_read, nci_chk_write


@pytest.fixture(scope="module")
def lib_built():
    from critic2_gb300 import build
    build.build()
    return _lib.lib()


def grid(seed=0, nstep=(5, 4, 7)):
    rng = np.random.default_rng(seed)
    x0 = rng.uniform(-5, 5, 3)
    xmat = np.diag(rng.uniform(0.05, 0.2, 3)) + 1e-3 * rng.standard_normal((3, 3))
    ns = np.array(nstep, np.int32)
    crho = rng.standard_normal(tuple(ns)) * 10.0 ** rng.uniform(-8, 3, tuple(ns))
    cgrad = rng.uniform(0, 100, tuple(ns))
    return x0, xmat, ns, crho, cgrad


def test_write_matches_the_record_layout(lib_built, oracle_mod, tmp_path):
    x0, xmat, ns, crho, cgrad = grid()
    p = str(tmp_path / "a.chk_nci")
    nci_chk_write(p, x0, xmat, ns, crho, cgrad)
    data = open(p, "rb").read()
    assert data == oracle_mod.fortran_records_bytes(oracle_mod.nci_chk_records(x0, xmat, ns, crho, cgrad))
    recs = oracle_mod.fortran_records_parse(data)
    assert [len(r) for r in recs] == [12, 24, 24, 24, 24, 12, 16 * crho.size]


def test_tiny_file_bytes(lib_built, tmp_path):
    """The bytes of a 1 x 1 x 2 checkpoint, spelled out."""
    p = str(tmp_path / "t.chk_nci")
    x0, xmat, ns = np.array([1.0, 2.0, 3.0]), np.eye(3) * 0.5, np.array([1, 1, 2], np.int32)
    nci_chk_write(p, x0, xmat, ns, np.array([[[-0.25, 4.0]]]), np.array([[[100.0, 0.5]]]))
    rec = lambda b: struct.pack("<i", len(b)) + b + struct.pack("<i", len(b))
    want = (rec(struct.pack("<3i", 0, 0, 0)) + rec(struct.pack("<3d", 1, 2, 3)) +
            rec(struct.pack("<3d", 0.5, 0, 0)) + rec(struct.pack("<3d", 0, 0.5, 0)) +
            rec(struct.pack("<3d", 0, 0, 0.5)) + rec(struct.pack("<3i", 1, 1, 2)) +
            rec(struct.pack("<4d", -0.25, 4.0, 100.0, 0.5)))
    assert open(p, "rb").read() == want


def test_round_trip_and_subrecords(lib_built, oracle_mod, tmp_path):
    x0, xmat, ns, crho, cgrad = grid(1, (6, 5, 9))
    p = str(tmp_path / "b.chk_nci")
    nci_chk_write(p, x0, xmat, ns, crho, cgrad)
    r = nci_chk_read(p, x0, xmat, ns)
    assert r is not None and np.array_equal(r[0], crho) and np.array_equal(r[1], cgrad)
    # a file whose records are split into small subrecords (as gfortran does
    # above 2 GiB), with a promolecular record after the cubes
    q = str(tmp_path / "c.chk_nci")
    recs = oracle_mod.nci_chk_records(x0, xmat, ns, crho, cgrad, rhoat=np.ones(crho.size))
    open(q, "wb").write(oracle_mod.fortran_records_bytes(recs, maxsub=100))
    r = nci_chk_read(q, x0, xmat, ns)
    assert r is not None and np.array_equal(r[0], crho) and np.array_equal(r[1], cgrad)
    o = oracle_mod.nci_chk_read(open(q, "rb").read(), x0, xmat, ns)
    assert np.array_equal(o[0], crho.reshape(-1)) and np.array_equal(o[1], cgrad.reshape(-1))


def test_compatibility_rules(lib_built, oracle_mod, tmp_path):
    x0, xmat, ns, crho, cgrad = grid(2)
    p = str(tmp_path / "d.chk_nci")
    nci_chk_write(p, x0, xmat, ns, crho, cgrad)
    assert nci_chk_read(p, x0 + 5e-14, xmat, ns) is not None      # within 1e-13
    assert nci_chk_read(p, x0 + np.array([0, 2e-13, 0]), xmat, ns) is None
    xm2 = xmat.copy()
    xm2[1, 2] += 2e-13
    assert nci_chk_read(p, x0, xm2, ns) is None
    assert nci_chk_read(p, x0, xmat, ns + np.array([0, 0, 1], np.int32)) is None
    assert nci_chk_read(str(tmp_path / "missing.chk_nci"), x0, xmat, ns) is None
    # fragments in the file: not this caller's checkpoint
    q = str(tmp_path / "e.chk_nci")
    open(q, "wb").write(oracle_mod.fortran_records_bytes(
        oracle_mod.nci_chk_records(x0, xmat, ns, crho, cgrad, nfrag=2)))
    assert nci_chk_read(q, x0, xmat, ns) is None
    assert oracle_mod.nci_chk_read(open(q, "rb").read(), x0, xmat, ns) is None


def test_truncated_file_is_an_error(lib_built, tmp_path):
    x0, xmat, ns, crho, cgrad = grid(3)
    p = str(tmp_path / "f.chk_nci")
    nci_chk_write(p, x0, xmat, ns, crho, cgrad)
    data = open(p, "rb").read()
    open(p, "wb").write(data[:-100])
    with pytest.raises(_lib.C2GError) as e:
        nci_chk_read(p, x0, xmat, ns)
    assert e.value.code == 4
    bad = bytearray(data)
    bad[-1] ^= 0x7F  # trailing marker of the cube record
    open(p, "wb").write(bytes(bad))
    with pytest.raises(_lib.C2GError):
        nci_chk_read(p, x0, xmat, ns)
