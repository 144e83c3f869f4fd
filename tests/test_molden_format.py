"""molden files with Gaussian-type orbitals (read_molden,
src/wfn_private@proc.F90:1819-2478): the restated reader's functions are
normalised (pure and Cartesian shells); (GPU) the library's reader agrees
with the restatement for RHF/UHF, AU/Angs, standard and ORCA files, and a
one-function-per-MO density integrates to the electron count."""
import numpy as np
import pytest

from critic2_gb300 import synth
from test_fchk_format import overlap


@pytest.mark.parametrize("types", [(0, 1, -2, -3, -4), (0, 1, 2, 3, 4)])
def test_restated_reader_functions_are_normalised(oracle_mod, tmp_path, types):
    b = synth.make_shell_basis(3, natom=1, types=types)
    nb = b.nbas
    b.moa = np.eye(nb)
    b.nalpha = b.nbeta = nb
    b.nelec = 2 * nb
    p = str(tmp_path / "m.molden")
    synth.write_molden(b, p)
    r = oracle_mod.read_molden_text(p)
    LI = synth.LI
    e, t, C = r["e"], r["itype"], r["cmo"]
    assert C.shape[1] == nb
    for m in range(nb):
        nz = np.nonzero(C[:, m])[0]
        s = sum(C[i, m] * C[j, m] * overlap(LI[t[i] - 1], LI[t[j] - 1], e[i], e[j]) for i in nz for j in nz)
        assert abs(s - 1.0) < 1e-9, (m, s)


CASES = [dict(types=(0, 1, -2, -3, -4), spin="rhf", orca=False, angs=False),
         dict(types=(0, 1, 2, 3, 4), spin="uhf", orca=False, angs=True),
         dict(types=(0, 1, -2, -3, -4), spin="rhf", orca=True, angs=False),
         dict(types=(0, 1, -2, -3, -4), spin="uhf", orca=True, angs=True)]


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c['spin']}-{'orca' if c['orca'] else 'std'}")
def test_library_reader_vs_restatement(gpu_lib, oracle_mod, tmp_path, case):
    from critic2_gb300.wfn import Wavefunction
    b = synth.make_shell_basis(6, types=case["types"], spin=case["spin"])
    p = str(tmp_path / "m.molden")
    synth.write_molden(b, p, orca=case["orca"], angs=case["angs"])
    r = oracle_mod.read_molden_text(p)
    mol = synth.Molecule(r["atom_xyz"], r["atom_z"], r["icenter"], r["itype"], r["e"], r["occ"],
                         np.ascontiguousarray(r["cmo"]), wfntyp=r["wfntyp"], nalpha=r["nalpha"], name="molden")
    g1, g2 = Wavefunction.from_molden(p), Wavefunction(mol)
    assert (g1.natom, g1.npri, g1.nmo, g1.wfntyp, g1.nalpha) == (g2.natom, g2.npri, g2.nmo, g2.wfntyp, g2.nalpha)
    pts = np.random.default_rng(7).uniform(b.atom_xyz.min(0) - 1, b.atom_xyz.max(0) + 1, (128, 3))
    a, c = g1.rho2(pts, 2, "fp64"), g2.rho2(pts, 2, "fp64")
    for k in ("rho", "grad", "hess"):
        assert np.allclose(a[k], c[k], rtol=1e-12, atol=1e-14 * np.abs(c[k]).max())


@pytest.mark.gpu
def test_one_function_densities_integrate_to_occupations(gpu_lib, tmp_path):
    from critic2_gb300.wfn import Wavefunction
    b = synth.make_shell_basis(4, natom=1, types=(0, 1, -2, -3, -4))
    nb = b.nbas
    b.moa = np.eye(nb)
    b.nalpha = b.nbeta = nb
    b.nelec = 2 * nb
    b.atom_z[:] = 8
    p = str(tmp_path / "m.molden")
    synth.write_molden(b, p)
    r = Wavefunction.from_molden(p).molcalc(("rho",), "franchini", "vgood", "fp64")
    assert abs(r["rho"] / (2 * nb) - 1) < 1e-5


@pytest.mark.gpu
def test_rejected_files(gpu_lib, tmp_path):
    from critic2_gb300 import _lib
    from critic2_gb300.wfn import Wavefunction
    b = synth.make_shell_basis(4, natom=1, types=(0, 1, -2))
    p = str(tmp_path / "m.molden")
    synth.write_molden(b, p)
    text = open(p).read()
    open(p, "w").write(text.replace(" Occup= 2.000000", " Occup= 1.500000", 1))
    with pytest.raises(_lib.C2GError):
        Wavefunction.from_molden(p)
    open(p, "w").write(text.replace("[GTO]", "[STO]"))
    with pytest.raises(_lib.C2GError):
        Wavefunction.from_molden(p)
