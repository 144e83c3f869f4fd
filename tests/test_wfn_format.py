"""The AIMPAC wfn format (read_wfn, src/wfn_private@proc.F90:981-1118): the
test writer against the oracle's restatement of the reader's fixed columns,
and (GPU) the library's reader against the same wavefunction built from
arrays."""
import dataclasses

import numpy as np
import pytest

from critic2_gb300 import synth


def spin(mol, wfntyp):
    occ = np.full(mol.nmo, 2.0)
    nalpha = mol.nmo // 2 + 1
    if wfntyp == 1:
        occ[:] = 1.0
    elif wfntyp == 2:
        occ[nalpha:] = 1.0
    elif wfntyp == 3:
        occ = np.linspace(2.0, 0.1234567, mol.nmo)
    return dataclasses.replace(mol, wfntyp=wfntyp, nalpha=nalpha, occ=occ)


def test_fortran_fields(oracle_mod):
    f = oracle_mod._fortran_field
    assert f(" 0.1722560D+04", 7) == 1722.56
    assert f("  -0.12345678E-01", 8) == -0.012345678
    assert f("    2.0000000", 7) == 2.0
    assert f("      ", 7) == 0.0
    assert f("  12345", 3) == 12.345           # implied decimals
    assert f(" 0.5+003", 7) == 500.0            # exponent without a letter
    assert f(" 1.5d-2", 7) == 0.015


@pytest.mark.parametrize("wfntyp", [0, 1, 2, 3])
def test_writer_against_restated_reader(oracle_mod, tmp_path, wfntyp):
    mol = spin(synth.make_molecule("nci12"), wfntyp)
    p = str(tmp_path / "m.wfn")
    synth.write_wfn(mol, p)
    r = oracle_mod.read_wfn_text(p)
    m = synth.round_for_wfn(mol)
    assert r["natom"] == mol.natom
    assert np.array_equal(r["xyz"], m.atom_xyz)
    assert np.array_equal(r["icenter"], mol.icenter) and np.array_equal(r["itype"], mol.itype)
    assert np.array_equal(r["e"], m.e) and np.array_equal(r["cmo"], m.cmo) and np.array_equal(r["occ"], m.occ)
    assert r["wfntyp"] == wfntyp
    if wfntyp == 1:
        assert r["nalpha"] == mol.nalpha  # from the drop of the orbital energies
    if wfntyp == 2:
        assert r["nalpha"] == mol.nalpha  # the doubly occupied count


def test_ecp_records_are_skipped(oracle_mod, tmp_path):
    mol = synth.make_molecule("nci12")
    p = str(tmp_path / "e.wfn")
    synth.write_wfn(mol, p)
    lines = open(p).read().split("\n")
    i = next(k for k, l in enumerate(lines) if l.startswith("MO"))
    lines[i:i] = ["CORE ELECTRONS ...", "  some ECP data  1 2 3"]
    open(p, "w").write("\n".join(lines))
    r = oracle_mod.read_wfn_text(p)
    assert np.array_equal(r["cmo"], synth.round_for_wfn(mol).cmo)


@pytest.mark.gpu
@pytest.mark.parametrize("wfntyp", [0, 1, 2, 3])
def test_library_reader(gpu_lib, tmp_path, wfntyp):
    from critic2_gb300.wfn import Wavefunction
    mol = spin(synth.make_molecule("nci12"), wfntyp)
    p = str(tmp_path / "m.wfn")
    synth.write_wfn(mol, p)
    m = synth.round_for_wfn(mol)
    if wfntyp == 3:
        m = dataclasses.replace(m, nalpha=0)
    g1, g2 = Wavefunction.from_wfn(p), Wavefunction(m)
    assert (g1.natom, g1.npri, g1.nmo, g1.wfntyp) == (g2.natom, g2.npri, g2.nmo, g2.wfntyp)
    if wfntyp in (1, 2):
        assert g1.nalpha == g2.nalpha
    pts = np.random.default_rng(wfntyp).uniform(mol.atom_xyz.min(0) - 1, mol.atom_xyz.max(0) + 1, (64, 3))
    a, b = g1.rho2(pts, 2, "fp64"), g2.rho2(pts, 2, "fp64")
    for k in ("rho", "grad", "hess", "gkin"):
        assert np.array_equal(a[k], b[k])


@pytest.mark.gpu
def test_library_reader_errors(gpu_lib, tmp_path):
    from critic2_gb300 import _lib
    from critic2_gb300.wfn import Wavefunction
    mol = synth.make_molecule("nci12")
    p = str(tmp_path / "m.wfn")
    synth.write_wfn(mol, p)
    text = open(p).read().split("\n")
    open(p, "w").write("\n".join(text[:40]))  # truncated
    with pytest.raises(_lib.C2GError) as e:
        Wavefunction.from_wfn(p)
    assert e.value.code == 4
    with pytest.raises(_lib.C2GError):
        Wavefunction.from_wfn(str(tmp_path / "missing.wfn"))
