"""Seeded synthetic molecular wavefunctions for the evaluator's workloads.

The generator builds molecules made of Cartesian Gaussian primitives centred
on atoms, with MO coefficients in the wfx convention (coefficients multiply
*unnormalised* primitives, as `read_wfx` stores them;
src/wfn_private@proc.F90:1121-1284 applies no normalisation for wfx files).

Primitive types follow critic2's `li(3,56)` exponent table
(src/wfn_private@proc.F90:3186-3196): type 1 = s; 2-4 = x,y,z; 5-10 =
xx,yy,zz,xy,xz,yz; 11-20 = xxx,yyy,zzz,xxy,xxz,yyz,xyy,xzz,yzz,xyz.

Arrays use critic2's memory layout: `cmo` has shape (npri, nmo) in C order,
which is Fortran's `cmo(nmoocc, npri)` (MO index fastest).  `icenter` and
`itype` are 1-based, exactly as read from a wfx file.

Workloads (all coordinates in bohr):

  nci12     12 atoms (8 H + 4 of C/N/O) as a 2-fragment complex in a
            12-bohr box, ~150 primitives (heavy: 6 s, 3 p, 1 d shells;
            H: 5 s, 1 p), 12 occupied MOs, 80^3 NCI grid at 0.1 bohr.
  nci60     60 atoms, ~1200 primitives (s/p/d), 120 MOs, 200^3 grid.
  prec200   200 atoms, ~4000 primitives (s/p/d/f; f exponents 0.3-5),
            400 MOs, 256^3 grid.
  cp100     100 atoms, ~2000 primitives (s/p/d), 200 MOs; CP search and a
            64^3 coarse density grid.
  large500  500 atoms, ~10000 primitives (s/p/d/f), 1000 MOs, 320^3 grid.

Boxes grow with the atom count at the density of the 12-atom case
(12 atoms per 12^3 bohr^3).  Atoms keep a minimum separation of 1.8 bohr.
The share of hydrogens (which get the reduced 5s1p shell set) is chosen so
that the primitive count meets the stated total.
"""
from __future__ import annotations

import dataclasses
import math
from typing import Dict, List, Optional

import numpy as np

# critic2's li(3,56) table (src/wfn_private@proc.F90:3186-3196): Cartesian
# exponents of types 1-56 (s; p; d; f; g 21-35; h 36-56), 1-based type index.
LI = np.array([
    (0, 0, 0),
    (1, 0, 0), (0, 1, 0), (0, 0, 1),
    (2, 0, 0), (0, 2, 0), (0, 0, 2), (1, 1, 0), (1, 0, 1), (0, 1, 1),
    (3, 0, 0), (0, 3, 0), (0, 0, 3), (2, 1, 0), (2, 0, 1), (0, 2, 1),
    (1, 2, 0), (1, 0, 2), (0, 1, 2), (1, 1, 1),
    (4, 0, 0), (0, 4, 0), (0, 0, 4), (3, 1, 0), (3, 0, 1), (1, 3, 0), (0, 3, 1), (1, 0, 3),
    (0, 1, 3), (2, 2, 0), (2, 0, 2), (0, 2, 2), (2, 1, 1), (1, 2, 1), (1, 1, 2),
    (0, 0, 5), (0, 1, 4), (0, 2, 3), (0, 3, 2), (0, 4, 1), (0, 5, 0), (1, 0, 4), (1, 1, 3),
    (1, 2, 2), (1, 3, 1), (1, 4, 0), (2, 0, 3), (2, 1, 2), (2, 2, 1), (2, 3, 0), (3, 0, 2),
    (3, 1, 1), (3, 2, 0), (4, 0, 1), (4, 1, 0), (5, 0, 0),
], dtype=np.int32)

SHELL_TYPES = {"s": [1], "p": [2, 3, 4], "d": list(range(5, 11)), "f": list(range(11, 21)),
               "g": list(range(21, 36)), "h": list(range(36, 57))}
HEAVY_Z = (6, 7, 8)


@dataclasses.dataclass
class Workload:
    name: str
    natom: int
    target_npri: Optional[int]
    nh: Optional[int]
    with_f: bool
    nmo: int
    grid: int            # grid points per axis (0 = no NCI grid)
    step: float          # grid step (bohr)
    fragments: int
    seed: int
    coarse: int = 0      # coarse density grid for the CP-seed proposer


WORKLOADS: Dict[str, Workload] = {
    "nci12": Workload("nci12", 12, None, 8, False, 12, 80, 0.1, 2, 1),
    "nci60": Workload("nci60", 60, 1200, None, False, 120, 200, 0.1, 1, 2),
    "prec200": Workload("prec200", 200, 4000, None, True, 400, 256, 0.1, 1, 3),
    "cp100": Workload("cp100", 100, 2000, None, False, 200, 0, 0.1, 1, 4, coarse=64),
    "large500": Workload("large500", 500, 10000, None, True, 1000, 320, 0.1, 1, 5),
}


@dataclasses.dataclass
class Molecule:
    """A molecular wavefunction in critic2's molwfn layout (see module doc)."""
    atom_xyz: np.ndarray     # (natom, 3) float64, bohr
    atom_z: np.ndarray       # (natom,) int32
    icenter: np.ndarray      # (npri,) int32, 1-based
    itype: np.ndarray        # (npri,) int32, 1-based li index
    e: np.ndarray            # (npri,) float64
    occ: np.ndarray          # (nmo,) float64
    cmo: np.ndarray          # (npri, nmo) float64, C order == Fortran cmo(nmo,npri)
    wfntyp: int = 0          # 0 rhf, 1 uhf, 2 rohf, 3 frac
    nalpha: int = 0
    name: str = ""
    # EDF core density (wfx <EDF Primitive *> sections), None without one
    edf_icenter: Optional[np.ndarray] = None  # (nedf,) int32, 1-based
    edf_itype: Optional[np.ndarray] = None    # (nedf,) int32, 1-based li index
    edf_e: Optional[np.ndarray] = None        # (nedf,) float64
    edf_c: Optional[np.ndarray] = None        # (nedf,) float64

    @property
    def nedf(self) -> int:
        return 0 if self.edf_e is None else int(self.edf_e.shape[0])

    @property
    def natom(self) -> int:
        return int(self.atom_xyz.shape[0])

    @property
    def npri(self) -> int:
        return int(self.e.shape[0])

    @property
    def nmo(self) -> int:
        return int(self.occ.shape[0])


def _shells(heavy: bool, with_f: bool) -> List[str]:
    if heavy:
        sh = ["s"] * 6 + ["p"] * 3 + ["d"]
        if with_f:
            sh.append("f")
        return sh
    return ["s"] * 5 + ["p"]


def _nprim(shells: List[str]) -> int:
    return sum(len(SHELL_TYPES[s]) for s in shells)


def _place_atoms(rng, natom: int, box: float, fragments: int, dmin: float = 1.8) -> np.ndarray:
    pos = np.zeros((natom, 3))
    n = 0
    gap = 0.75
    tries = 0
    while n < natom:
        tries += 1
        if tries > 2_000_000:
            raise RuntimeError("atom placement failed")
        x = rng.uniform(0.0, box, size=3)
        if fragments == 2:
            # first half of the atoms in the left slab, second half in the right slab
            if n < natom // 2:
                x[0] = rng.uniform(0.0, box / 2 - gap)
            else:
                x[0] = rng.uniform(box / 2 + gap, box)
        if n and np.min(np.sum((pos[:n] - x) ** 2, axis=1)) < dmin * dmin:
            continue
        pos[n] = x
        n += 1
    return pos


def make_molecule(name: str, seed: Optional[int] = None) -> Molecule:
    """Builds the named workload's molecule (deterministic for a given seed)."""
    w = WORKLOADS[name]
    return build_molecule(w, w.seed if seed is None else seed)


def training_molecule(index: int, natom_range=(10, 80)) -> Molecule:
    """Molecule `index` of the CP-seed proposer's training family: the same
    construction as cp100 (s/p/d, ~20 primitives and 2 MOs per atom, one
    fragment, the same atom density) with natom drawn uniformly from
    natom_range.  Indices >= 10**6 are reserved for held-out molecules."""
    rng = np.random.default_rng(7_000_000 + index)
    natom = int(rng.integers(natom_range[0], natom_range[1] + 1))
    w = Workload(f"train{index}", natom, 20 * natom, None, False, 2 * natom, 0, 0.1, 1,
                 8_000_000 + index)
    return build_molecule(w, w.seed)


def build_molecule(w: Workload, seed: int) -> Molecule:
    """The generator behind every workload (see the module doc)."""
    rng = np.random.default_rng(seed)
    per_heavy = _nprim(_shells(True, w.with_f))
    per_h = _nprim(_shells(False, w.with_f))
    if w.nh is not None:
        nh = w.nh
    else:
        nh = int(round(w.natom * (per_heavy - w.target_npri / w.natom) / (per_heavy - per_h)))
        nh = max(0, min(w.natom, nh))
    box = 12.0 * (w.natom / 12.0) ** (1.0 / 3.0)
    pos = _place_atoms(rng, w.natom, box, w.fragments)
    # which atoms are H: spread over both fragments
    isH = np.zeros(w.natom, dtype=bool)
    isH[rng.permutation(w.natom)[:nh]] = True
    if w.fragments == 2:
        half = w.natom // 2
        isH[:] = False
        isH[rng.permutation(half)[: nh // 2]] = True
        isH[half + rng.permutation(w.natom - half)[: nh - nh // 2]] = True
    z = np.where(isH, 1, rng.choice(HEAVY_Z, size=w.natom)).astype(np.int32)

    icenter, itype, e = [], [], []
    for a in range(w.natom):
        for sh in _shells(not isH[a], w.with_f):
            if sh == "f":
                alpha = math.exp(rng.uniform(math.log(0.3), math.log(5.0)))
            else:
                alpha = math.exp(rng.uniform(math.log(0.1), math.log(50.0)))
            for t in SHELL_TYPES[sh]:
                icenter.append(a + 1)
                itype.append(t)
                e.append(alpha)
    npri = len(e)
    cmo = rng.standard_normal((npri, w.nmo))
    occ = np.full(w.nmo, 2.0)
    return Molecule(pos, z, np.array(icenter, np.int32), np.array(itype, np.int32),
                    np.array(e, np.float64), occ, np.ascontiguousarray(cmo),
                    wfntyp=0, nalpha=w.nmo, name=w.name)


def add_edf(mol: Molecule, seed: int, per_atom=(3, 6), lmax: int = 0) -> Molecule:
    """Returns a copy of `mol` with a seeded synthetic EDF core on every
    heavy atom: `per_atom` s-type primitives with exponents 2-2000 and
    positive coefficients (a compact core density, as the EDFs that stand in
    for pseudopotential cores), plus, for lmax >= 1, one primitive of each
    type up to lmax with small signed coefficients (types beyond s exercise
    the full polynomial; they stay within the atom's MO lmax)."""
    rng = np.random.default_rng(seed)
    ic, it, ee, cc = [], [], [], []
    for a in range(mol.natom):
        if int(mol.atom_z[a]) == 1:
            continue
        for _ in range(int(rng.integers(per_atom[0], per_atom[1] + 1))):
            ic.append(a + 1)
            it.append(1)
            ee.append(math.exp(rng.uniform(math.log(2.0), math.log(2000.0))))
            cc.append(math.exp(rng.uniform(math.log(0.5), math.log(200.0))))
        for t in range(2, 57):
            if max(LI[t - 1]) > lmax:
                continue
            ic.append(a + 1)
            it.append(t)
            ee.append(math.exp(rng.uniform(math.log(1.0), math.log(50.0))))
            cc.append(float(rng.uniform(-1.0, 1.0)))
    return dataclasses.replace(mol, edf_icenter=np.array(ic, np.int32), edf_itype=np.array(it, np.int32),
                               edf_e=np.array(ee, np.float64), edf_c=np.array(cc, np.float64),
                               name=mol.name + "+edf")


def nci_grid(mol: Molecule, n: int, step: float):
    """NCI grid geometry in critic2's form (src/nci@proc.f90:430-447).

    For a molecule with explicit limits critic2 uses a diagonal xmat of the
    step and nstep points per axis.  The grid here has n points per axis at
    the given step, centred on the centre of the molecule's bounding box.
    Returns (x0[3], xmat[3,3] with columns = axis steps, nstep[3]).
    """
    lo = mol.atom_xyz.min(axis=0)
    hi = mol.atom_xyz.max(axis=0)
    c = 0.5 * (lo + hi)
    x0 = c - 0.5 * step * (n - 1)
    xmat = np.diag([step, step, step]).astype(np.float64)
    return x0.astype(np.float64), xmat, np.array([n, n, n], np.int32)


def grid_points(x0, xmat, nstep, i_range=None) -> np.ndarray:
    """Cartesian coordinates of grid points in critic2's (k,j,i) order (k fastest).

    x = x0 + i*xmat[:,0] + j*xmat[:,1] + k*xmat[:,2]   (src/nci@proc.f90:548)
    Returns an array of shape (n_i, n2, n3, 3).
    """
    n1, n2, n3 = (int(v) for v in nstep)
    i0, i1 = (0, n1) if i_range is None else i_range
    ii = np.arange(i0, i1, dtype=np.float64)
    jj = np.arange(n2, dtype=np.float64)
    kk = np.arange(n3, dtype=np.float64)
    xm = np.asarray(xmat, np.float64)
    pts = (np.asarray(x0)[None, None, None, :]
           + ii[:, None, None, None] * xm[:, 0]
           + jj[None, :, None, None] * xm[:, 1]
           + kk[None, None, :, None] * xm[:, 2])
    return pts


def write_wfx(mol: Molecule, path: str) -> None:
    """Writes the molecule as a wfx file readable by critic2's read_wfx.

    The MO coefficient block follows the structure read_wfx parses
    (src/wfn_private@proc.F90:1215-1221): one skipped line after the section
    tag, then per MO two skipped lines and the reals, which end at the next
    line that starts with '<'.
    """
    def block(tag, values, fmt):
        lines = [f"<{tag}>"]
        for i in range(0, len(values), 5):
            lines.append(" " + " ".join(fmt(v) for v in values[i:i + 5]))
        lines.append(f"</{tag}>")
        return lines

    out = ["<Title>", f" synthetic {mol.name}", "</Title>",
           "<Keywords>", " GTO", "</Keywords>",
           "<Number of Nuclei>", f" {mol.natom}", "</Number of Nuclei>",
           "<Number of Occupied Molecular Orbitals>", f" {mol.nmo}",
           "</Number of Occupied Molecular Orbitals>",
           "<Number of Perturbations>", " 0", "</Number of Perturbations>",
           "<Net Charge>", " 0", "</Net Charge>",
           "<Electronic Spin Multiplicity>", " 1", "</Electronic Spin Multiplicity>",
           "<Number of Alpha Electrons>", f" {mol.nalpha}", "</Number of Alpha Electrons>",
           "<Number of Beta Electrons>", f" {mol.nalpha}", "</Number of Beta Electrons>",
           "<Nuclear Names>"]
    sym = {1: "H", 6: "C", 7: "N", 8: "O"}
    for a in range(mol.natom):
        out.append(f" {sym.get(int(mol.atom_z[a]), 'X')}{a + 1}")
    out.append("</Nuclear Names>")
    out += block("Atomic Numbers", [int(v) for v in mol.atom_z], lambda v: f"{v:d}")
    out += block("Nuclear Charges", [float(v) for v in mol.atom_z], lambda v: f"{v:.12E}")
    out.append("<Nuclear Cartesian Coordinates>")
    for a in range(mol.natom):
        out.append(" " + " ".join(f"{v: .16E}" for v in mol.atom_xyz[a]))
    out.append("</Nuclear Cartesian Coordinates>")
    out += ["<Number of Primitives>", f" {mol.npri}", "</Number of Primitives>"]
    out += block("Primitive Centers", [int(v) for v in mol.icenter], lambda v: f"{v:d}")
    out += block("Primitive Types", [int(v) for v in mol.itype], lambda v: f"{v:d}")
    out += block("Primitive Exponents", [float(v) for v in mol.e], lambda v: f"{v:.16E}")
    out += block("Molecular Orbital Occupation Numbers", [float(v) for v in mol.occ],
                 lambda v: f"{v:.16E}")
    out.append("<Molecular Orbital Primitive Coefficients>")
    for m in range(mol.nmo):
        out += ["<MO Number>", f" {m + 1}", "</MO Number>"]
        col = mol.cmo[:, m]
        for i in range(0, mol.npri, 4):
            out.append(" " + " ".join(f"{v: .16E}" for v in col[i:i + 4]))
    out.append("</Molecular Orbital Primitive Coefficients>")
    if mol.nedf:
        out += ["<Number of EDF Primitives>", f" {mol.nedf}", "</Number of EDF Primitives>"]
        out += block("EDF Primitive Centers", [int(v) for v in mol.edf_icenter], lambda v: f"{v:d}")
        out += block("EDF Primitive Types", [int(v) for v in mol.edf_itype], lambda v: f"{v:d}")
        out += block("EDF Primitive Exponents", [float(v) for v in mol.edf_e], lambda v: f"{v:.16E}")
        out += block("EDF Primitive Coefficients", [float(v) for v in mol.edf_c], lambda v: f"{v:.16E}")
    with open(path, "w") as fh:
        fh.write("\n".join(out) + "\n")


def _fortran_e(v: float, w: int, d: int, letter: str = "D") -> str:
    """Fortran Ew.d output with a D exponent: [-]0.ddd...D+ee, right-justified."""
    if v == 0.0:
        s = "0." + "0" * d + letter + "+00"
    else:
        t = f"{abs(v):.{d - 1}E}"
        mant, ex = t.split("E")
        digits = mant.replace(".", "")
        s = "0." + digits + letter + f"{int(ex) + 1:+03d}"
        if v < 0:
            s = "-" + s
    return s.rjust(w)


def round_for_wfn(mol: Molecule) -> Molecule:
    """The molecule as a wfn file stores it: exponents with 7 and MO
    coefficients with 8 significant digits, occupations to 1e-7 and
    coordinates to 1e-8."""
    r = lambda a, d: np.array([float(_fortran_e(v, 24, d).replace("D", "E")) for v in np.ravel(a)]).reshape(np.shape(a))
    f = lambda a, d: np.array([float(f"{v:.{d}f}") for v in np.ravel(a)]).reshape(np.shape(a))
    return dataclasses.replace(mol, e=r(mol.e, 7), cmo=np.ascontiguousarray(r(mol.cmo, 8)),
                               occ=f(mol.occ, 7), atom_xyz=f(mol.atom_xyz, 8))


def write_wfn(mol: Molecule, path: str, energies=None) -> None:
    """Writes the molecule as an AIMPAC wfn file in the fixed columns that
    critic2's read_wfn reads (src/wfn_private@proc.F90:1106-1111, formats
    101-106).  Orbital energies: given, or ascending within each spin block
    (the beta block of a UHF wavefunction starts lower, which is how
    read_wfn finds the alpha count)."""
    sym = {1: "H", 6: "C", 7: "N", 8: "O"}
    nmo, npri, nat = mol.nmo, mol.npri, mol.natom
    if energies is None:
        energies = np.array([-1.0 + 0.01 * m if (mol.wfntyp != 1 or m < mol.nalpha)
                             else -1.5 + 0.01 * (m - mol.nalpha) for m in range(nmo)])
    out = [f" synthetic {mol.name}",
           "GAUSSIAN" + " " * 10 + f"{nmo:5d}" + " MOL ORBITALS  " + f"{npri:5d}" + " PRIMITIVES    "
           + f"{nat:5d}" + " NUCLEI"]
    for a in range(nat):
        x = mol.atom_xyz[a]
        out.append("  " + f"{sym.get(int(mol.atom_z[a]), 'X'):<2}" + f"{a + 1:4d}    (CENTRE{a + 1:3d}) "
                   + "".join(f"{v:12.8f}" for v in x) + "  CHARGE =" + f"{float(mol.atom_z[a]):5.1f}")
    for tag, vals in (("CENTRE ASSIGNMENTS  ", mol.icenter), ("TYPE ASSIGNMENTS    ", mol.itype)):
        for i in range(0, npri, 20):
            out.append(tag + "".join(f"{int(v):3d}" for v in vals[i:i + 20]))
    for i in range(0, npri, 5):
        out.append("EXPONENTS " + "".join(_fortran_e(v, 14, 7) for v in mol.e[i:i + 5]))
    for m in range(nmo):
        head = f"MO{m + 1:5d}     MO 0.0        OCC NO =".ljust(35)[:35]
        out.append(head + f"{mol.occ[m]:12.7f}" + "  ORB. ENERGY =" + f"{energies[m]:12.6f}")
        col = mol.cmo[:, m]
        for i in range(0, npri, 5):
            out.append("".join(_fortran_e(v, 16, 8) for v in col[i:i + 5]))
    out.append("END DATA")
    with open(path, "w") as fh:
        fh.write("\n".join(out) + "\n")


@dataclasses.dataclass
class ShellBasis:
    """A contracted-shell basis and MOs as a Gaussian fchk file holds them.
    shells: (type, atom 0-based, exponents, coefficients, sp p-coefficients
    or None); type 0 s, 1 p, -1 sp, +-2 d, +-3 f, +-4 g (negative = pure).
    moa / mob: MO coefficients (nmo, nbas) over the basis functions in
    shell order."""
    atom_xyz: np.ndarray
    atom_z: np.ndarray
    shells: list
    nelec: int
    nalpha: int
    nbeta: int
    moa: np.ndarray
    mob: Optional[np.ndarray] = None

    @property
    def nbas(self) -> int:
        return sum(2 * -t + 1 if t < -1 else (4 if t == -1 else (t + 1) * (t + 2) // 2)
                   for t, *_ in self.shells)


def make_shell_basis(seed: int, natom: int = 5, types=(0, -1, 1, -2, 2, -3, 3, -4, 4),
                     spin: str = "rhf") -> ShellBasis:
    """Seeded molecule with every shell type on each atom (random exponents
    and contractions of 1-3 primitives) and random occupied MOs."""
    rng = np.random.default_rng(seed)
    box = 4.0 + natom
    pos = _place_atoms(rng, natom, box, 1)
    z = rng.choice((1, 6, 7, 8), size=natom).astype(np.int32)
    shells = []
    for a in range(natom):
        for t in types:
            n = int(rng.integers(1, 4))
            e = np.sort(np.exp(rng.uniform(np.log(0.2), np.log(30.0), n)))[::-1].copy()
            c = rng.uniform(0.2, 1.0, n)
            pc = rng.uniform(0.2, 1.0, n) if t == -1 else None
            shells.append((t, a, e, c, pc))
    b = ShellBasis(pos, z, shells, 0, 0, 0, np.zeros((0, 0)))
    nbas = b.nbas
    if spin == "rhf":
        nalpha = nbeta = 6
    elif spin == "uhf":
        nalpha, nbeta = 7, 5
    else:  # rohf
        nalpha, nbeta = 7, 5
    b.nelec, b.nalpha, b.nbeta = nalpha + nbeta, nalpha, nbeta
    nmoa = nbas  # all orbitals, as Gaussian writes them
    b.moa = rng.standard_normal((nmoa, nbas)) * 0.5
    if spin == "uhf":
        b.mob = rng.standard_normal((nmoa, nbas)) * 0.5
    return b


def write_fchk(b: ShellBasis, path: str) -> None:
    """A Gaussian formatted checkpoint file with the sections read_fchk reads
    (integers 6 per line in I12, reals 5 per line in E16.8)."""
    def scalar(name, v):
        return [f"{name:<40}   I     {v:>12d}"]

    def ints(name, vals):
        out = [f"{name:<40}   I   N={len(vals):>12d}"]
        for i in range(0, len(vals), 6):
            out.append("".join(f"{int(v):12d}" for v in vals[i:i + 6]))
        return out

    def reals(name, vals):
        vals = np.ravel(vals)
        out = [f"{name:<40}   R   N={len(vals):>12d}"]
        for i in range(0, len(vals), 5):
            out.append("".join(f"{float(v):16.8E}" for v in vals[i:i + 5]))
        return out

    nat = len(b.atom_z)
    ex, cc, pc = [], [], []
    for t, a, e, c, p in b.shells:
        ex += list(e)
        cc += list(c)
        pc += list(p) if p is not None else [0.0] * len(e)
    lines = [f"synthetic shell basis", "SP        RHF                                                         Gen"]
    lines += scalar("Number of atoms", nat)
    lines += scalar("Charge", 0) + scalar("Multiplicity", 1 + b.nalpha - b.nbeta)
    lines += scalar("Number of electrons", b.nelec)
    lines += scalar("Number of alpha electrons", b.nalpha) + scalar("Number of beta electrons", b.nbeta)
    lines += scalar("Number of basis functions", b.nbas)
    lines += ints("Atomic numbers", b.atom_z)
    lines += reals("Current cartesian coordinates", b.atom_xyz)
    lines += scalar("Number of contracted shells", len(b.shells))
    lines += scalar("Number of primitive shells", len(ex))
    lines += scalar("Highest angular momentum", max(abs(s[0]) for s in b.shells))
    lines += ints("Shell types", [s[0] for s in b.shells])
    lines += ints("Number of primitives per shell", [len(s[2]) for s in b.shells])
    lines += ints("Shell to atom map", [s[1] + 1 for s in b.shells])
    lines += reals("Primitive exponents", ex)
    lines += reals("Contraction coefficients", cc)
    if any(s[0] == -1 for s in b.shells):
        lines += reals("P(S=P) Contraction coefficients", pc)
    lines += reals("Alpha Orbital Energies", np.linspace(-1, 1, b.moa.shape[0]))
    if b.mob is not None:
        lines += reals("Beta Orbital Energies", np.linspace(-1, 1, b.mob.shape[0]))
    lines += reals("Alpha MO coefficients", b.moa)
    if b.mob is not None:
        lines += reals("Beta MO coefficients", b.mob)
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")


def write_molden(b: ShellBasis, path: str, orca: bool = False, angs: bool = False) -> None:
    """A molden file of the basis (no sp shells; pure or Cartesian per l as
    the shells say, flagged with [5D7F] / [9G]); occupied MOs only.  With
    orca=True the title marks an ORCA file."""
    types = {t for t, *_ in b.shells}
    assert -1 not in types
    sym = {1: "H", 6: "C", 7: "N", 8: "O"}
    out = ["[Molden Format]", "[Title]", " created by orca_2mkl" if orca else " synthetic",
           "[Atoms] " + ("Angs" if angs else "AU")]
    f = 0.52917720859 if angs else 1.0
    for a, (x, zz) in enumerate(zip(b.atom_xyz, b.atom_z)):
        out.append(f"{sym.get(int(zz), 'X'):>2} {a + 1:5d} {int(zz):4d} " + " ".join(f"{v * f:20.12f}" for v in x))
    out.append("[GTO]")
    for a in range(len(b.atom_z)):
        out.append(f"  {a + 1} 0")
        for t, at, e, c, _ in b.shells:
            if at != a:
                continue
            out.append(f" {'spdfg'[abs(t)]} {len(e)} 1.00")
            for ei, ci in zip(e, c):
                out.append(f"  {ei:20.12E} {ci:20.12E}")
        out.append("")
    if -2 in types or -3 in types:
        out.append("[5D7F]")
    if -4 in types:
        out.append("[9G]")
    out.append("[MO]")
    spins = [("Alpha", b.moa, b.nalpha)] + ([("Beta", b.mob, b.nbeta)] if b.mob is not None else [])
    for spin, mo, nocc in spins:
        for m in range(mo.shape[0]):
            occ = (2.0 if b.mob is None else 1.0) if m < nocc else 0.0
            out += [" Sym=     1a", f" Ene= {-1.0 + 0.01 * m:.6f}", f" Spin= {spin}", f" Occup= {occ:.6f}"]
            out += [f"{k + 1:6d} {v:20.12E}" for k, v in enumerate(mo[m])]
    with open(path, "w") as fh:
        fh.write("\n".join(out) + "\n")
