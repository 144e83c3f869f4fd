"""ctypes wrapper of the C oracle (oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() to
compare against, and by bench.py's CPU-baseline leg.  The product library
(critic2_gb300) never imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "_build", "liboracle.so")

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def build(force: bool = False) -> str:
    """Compiles oracle.c into oracle/_build/liboracle.so (gcc, OpenMP)."""
    src = os.path.join(_HERE, "oracle.c")
    if force or not os.path.exists(_SO) or os.path.getmtime(_SO) < os.path.getmtime(src):
        os.makedirs(os.path.dirname(_SO), exist_ok=True)
        subprocess.check_call(["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-Wall",
                               src, "-o", _SO, "-lm"])
    return _SO


class ORes(C.Structure):
    _fields_ = [("f", C.c_double), ("fval", C.c_double), ("gf", C.c_double * 3),
                ("gfmod", C.c_double), ("gfmodval", C.c_double), ("hf", C.c_double * 9),
                ("hfeval", C.c_double * 3), ("del2f", C.c_double), ("del2fval", C.c_double),
                ("gkin", C.c_double), ("fspin", C.c_double * 2), ("gkinspin", C.c_double * 2),
                ("lapspin", C.c_double * 2), ("gfmodspin", C.c_double * 2),
                ("stress", C.c_double * 9), ("vir", C.c_double), ("r", C.c_int),
                ("s", C.c_int), ("isnuc", C.c_int), ("valid", C.c_int)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        L = _lib
        L.o_wfn_new.restype = C.c_void_p
        L.o_wfn_new.argtypes = [C.c_int, _dp, _ip, C.c_int, C.c_int, _ip, _ip, _dp, _dp, _dp,
                                C.c_int, C.c_int]
        L.o_wfn_free.argtypes = [C.c_void_p]
        L.o_wfn_set_edf.argtypes = [C.c_void_p, C.c_int, _ip, _ip, _dp, _dp]
        L.o_wfn_npri.argtypes = [C.c_void_p]
        L.o_wfn_cell.argtypes = [C.c_void_p, _dp, _dp, _dp]
        L.o_rho2.argtypes = [C.c_void_p, _dp, C.c_int, _dp, _dp, _dp, _dp, _dp, _dp, _dp,
                             C.POINTER(C.c_double), _dp]
        L.o_grd.argtypes = [C.c_void_p, _dp, C.c_int, C.POINTER(ORes)]
        L.o_eigsym3.argtypes = [_dp, _dp]
        L.o_rsindex.argtypes = [_dp, _dp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_double]
        L.o_matinvsym3.argtypes = [_dp]
        L.o_matinvsym3.restype = C.c_int
        L.o_nci_points.argtypes = [C.c_void_p, C.c_long, _dp, _dp, _dp, C.c_int]
        L.o_nciplot.argtypes = [C.c_void_p, _dp, _dp, _ip, C.c_int, C.c_int, _dp, _dp, C.c_int]
        L.o_rho2_points.argtypes = [C.c_void_p, C.c_long, _dp, C.c_int, _dp, C.c_void_p,
                                    C.c_void_p, C.c_int]
        L.o_newton.argtypes = [C.c_void_p, _dp, C.c_double, C.c_int]
        L.o_newton.restype = C.c_int
        L.o_newton_batch.argtypes = [C.c_void_p, C.c_long, _dp, C.c_double, C.c_int, _ip, C.c_int]
        L.o_pair_seeds.argtypes = [C.c_void_p, C.c_double, C.c_int, _dp, C.c_int]
        L.o_pair_seeds.restype = C.c_int
        L.o_autocritic.argtypes = [C.c_void_p, C.c_int, _dp, C.c_int, C.c_int, _dp, _ip, _dp, _ip]
        L.o_autocritic.restype = C.c_int
        L.o_eigvec3.argtypes = [_dp, _dp, _dp]
        L.o_gradient.argtypes = [C.c_void_p, _dp, C.c_int, C.c_int, _dp, _ip, _dp, C.POINTER(C.c_int),
                                 C.POINTER(C.c_double)]
        L.o_gradient.restype = C.c_int
        L.o_makegraph.argtypes = [C.c_void_p, C.c_int, _dp, _ip, _ip, _dp, _dp, _dp, _dp, _ip, _ip, C.c_int]
        L.o_basin_integrals.argtypes = [C.c_void_p, C.c_int, _dp, _ip, C.c_int, C.c_int, _dp, _dp, C.c_void_p,
                                        C.c_int, C.c_void_p, C.c_int, _dp, _dp, C.c_double, C.c_int, C.c_int,
                                        _ip, _dp, _dp, _dp, _dp, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.o_basin_integrals.restype = C.c_int
        L.o_sphere_integrals.argtypes = [C.c_void_p, C.c_int, _dp, _ip, C.c_int, C.c_int, _dp, _dp, C.c_void_p,
                                         C.c_int, C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_int, _ip, _dp,
                                         _dp]
        L.o_sphere_integrals.restype = C.c_int
        L.o_z2nr.argtypes = [C.c_int, C.c_int]
        L.o_z2nr.restype = C.c_int
        L.o_mesh_size.argtypes = [C.c_void_p, C.c_int, C.c_int]
        L.o_mesh_size.restype = C.c_long
        L.o_mesh.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, _dp, _dp, _dp, C.c_int]
        L.o_fmt_e13_5e3.argtypes = [C.c_double, C.c_char_p]
        L.o_fmt_E15_7.argtypes = [C.c_double, C.c_char_p]
        L.o_fmt_E22_14E3.argtypes = [C.c_double, C.c_char_p]
        L.o_cube_body.argtypes = [_ip, _dp, C.c_char_p]
        L.o_cube_body.restype = C.c_long
        L.o_nci_post.argtypes = [_ip, _dp, _dp, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                                 C.c_int, _dp]
        L.o_nci_post.restype = C.c_long
    return _lib


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


class Wfn:
    """Oracle wavefunction (prune_primitives + complete_struct applied)."""

    def __init__(self, mol):
        L = lib()
        self.mol = mol
        self.h = L.o_wfn_new(mol.natom, _f64(mol.atom_xyz.reshape(-1)), _i32(mol.atom_z),
                             mol.npri, mol.nmo, _i32(mol.icenter), _i32(mol.itype), _f64(mol.e),
                             _f64(mol.occ), _f64(mol.cmo.reshape(-1)), int(mol.wfntyp),
                             int(mol.nalpha))
        if getattr(mol, "edf_e", None) is not None and len(mol.edf_e):
            self.set_edf(mol.edf_icenter, mol.edf_itype, mol.edf_e, mol.edf_c)

    def set_edf(self, icenter, itype, e, c):
        """EDF core density (1-based icenter and li type; empty removes it)."""
        n = len(e)
        lib().o_wfn_set_edf(self.h, n, _i32(icenter), _i32(itype), _f64(e), _f64(c))

    def __del__(self):
        if getattr(self, "h", None):
            lib().o_wfn_free(self.h)
            self.h = None

    @property
    def npri(self):
        return lib().o_wfn_npri(self.h)

    def cell(self):
        lo, aa, mb = np.zeros(3), np.zeros(3), np.zeros(3)
        lib().o_wfn_cell(self.h, lo, aa, mb)
        return lo, aa, mb

    def rho2(self, x, nder=2):
        rho, rv, gv = np.zeros(3), np.zeros(3), np.zeros(9)
        g, h, hv, gk, st = np.zeros(9), np.zeros(27), np.zeros(27), np.zeros(3), np.zeros(9)
        vir = C.c_double()
        lib().o_rho2(self.h, _f64(x), nder, rho, rv, g, gv, h, hv, gk, C.byref(vir), st)
        return dict(rho=rho, rhoval=rv, grad=g.reshape(3, 3), gradval=gv.reshape(3, 3),
                    h=h.reshape(3, 3, 3), hval=hv.reshape(3, 3, 3), gkin=gk, vir=vir.value,
                    stress=st.reshape(3, 3))

    def grd(self, x, nder=2):
        r = ORes()
        lib().o_grd(self.h, _f64(x), nder, C.byref(r))
        return r

    def rho2_points(self, xyz, nder=2, nthreads=0):
        xyz = _f64(xyz).reshape(-1, 3)
        n = xyz.shape[0]
        rho = np.zeros(n)
        grad = np.zeros((n, 3)) if nder > 0 else None
        hess = np.zeros((n, 9)) if nder > 1 else None
        lib().o_rho2_points(self.h, n, xyz.reshape(-1), nder, rho,
                            grad.ctypes.data if grad is not None else None,
                            hess.ctypes.data if hess is not None else None, nthreads)
        return rho, grad, hess

    def nci_points(self, xyz, nthreads=0):
        xyz = _f64(xyz).reshape(-1, 3)
        n = xyz.shape[0]
        crho, cgrad = np.zeros(n), np.zeros(n)
        lib().o_nci_points(self.h, n, xyz.reshape(-1), crho, cgrad, nthreads)
        return crho, cgrad

    def nciplot(self, x0, xmat, nstep, i0=0, i1=None, nthreads=0):
        nstep = _i32(nstep)
        i1 = int(nstep[0]) if i1 is None else i1
        n = (i1 - i0) * int(nstep[1]) * int(nstep[2])
        crho, cgrad = np.zeros(n), np.zeros(n)
        xm = _f64(np.asarray(xmat).T.reshape(-1))  # column-major xmat(:,i)
        lib().o_nciplot(self.h, _f64(x0), xm, nstep, i0, i1, crho, cgrad, nthreads)
        shp = (i1 - i0, int(nstep[1]), int(nstep[2]))
        return crho.reshape(shp), cgrad.reshape(shp)

    def newton_batch(self, xyz, gfnormeps=1e-12, maxit=200, nthreads=0):
        x = _f64(xyz).reshape(-1, 3).copy()
        ier = np.zeros(x.shape[0], np.int32)
        lib().o_newton_batch(self.h, x.shape[0], x.reshape(-1), gfnormeps, maxit, ier, nthreads)
        return x, ier

    def pair_seeds(self, maxdist=15.0, npts=5):
        n = lib().o_pair_seeds(self.h, maxdist, npts, np.zeros(3), 0)
        buf = np.zeros(3 * max(n, 1))
        lib().o_pair_seeds(self.h, maxdist, npts, buf, n)
        return buf[: 3 * n].reshape(n, 3)

    def gradient(self, x, iup, cp_xyz, cp_typ, pathini):
        """field%gradient (molecule, default navigation, up2beta): returns
        (end point, ier, nstep, plen)."""
        xx = _f64(x).copy()
        ns, pl = C.c_int(0), C.c_double(0.0)
        cx, ct = _f64(cp_xyz).reshape(-1), _i32(cp_typ)
        ier = lib().o_gradient(self.h, xx, int(iup), len(ct), cx, ct, _f64(pathini), C.byref(ns), C.byref(pl))
        return xx, ier, ns.value, pl.value

    def makegraph(self, cp_xyz, cp_typ, nthreads=0):
        """makegraph over a CP list: dict of ipath (n,2), brdist (n,2),
        brpathlen (n,2), brang (n,), brvec (n,3), ier (n,2), nstep (n,2)."""
        ct = _i32(cp_typ)
        n = len(ct)
        out = dict(ipath=np.zeros((n, 2), np.int32), brdist=np.zeros((n, 2)), brpathlen=np.zeros((n, 2)),
                   brang=np.zeros(n), brvec=np.zeros((n, 3)), ier=np.zeros((n, 2), np.int32),
                   nstep=np.zeros((n, 2), np.int32))
        lib().o_makegraph(self.h, n, _f64(cp_xyz).reshape(-1), ct, out["ipath"].reshape(-1),
                          out["brdist"].reshape(-1), out["brpathlen"].reshape(-1), out["brang"],
                          out["brvec"].reshape(-1), out["ier"].reshape(-1), out["nstep"].reshape(-1), nthreads)
        return out

    def basin_integrals(self, cp_xyz, cp_typ, u, wang, usph, wsph, ring=None, ringw=None, cpid=0, prec=1e-5,
                        stats=False, nthreads=0):
        """INTEGRALS by bisection (molecule): rays u (nray, 3) with angular
        weights wang (times 4 pi for a Lebedev rule; with ring/ringw the
        gauleg_mquad grouping), beta sphere on usph/wsph.  stats: critic2's
        serial running bracket statistics.  Returns a dict of att_cp,
        props (natt, 2: Pop, Lap), iaserr, rsurf (natt, nray), rbeta_int,
        nwarn, nrestart; raises RuntimeError when a ray has no bracket."""
        ct = _i32(cp_typ)
        n = len(ct)
        nat = self.mol.natom
        cand = [i for i in (range(n) if cpid <= 0 else [cpid - 1]) if i < nat or ct[i] == -3]
        na, nray = len(cand), len(u)
        out = dict(att_cp=np.zeros(max(na, 1), np.int32), props=np.zeros((max(na, 1), 2)),
                   iaserr=np.zeros((max(na, 1), 2)), rsurf=np.zeros((max(na, 1), nray)), rbeta_int=np.zeros(max(na, 1)))
        nw, nr = C.c_int(0), C.c_int(0)
        rg = _i32(ring) if ring is not None else None
        rw = _f64(ringw) if ringw is not None else None
        got = lib().o_basin_integrals(
            self.h, n, _f64(cp_xyz).reshape(-1), ct, int(cpid), nray, _f64(u).reshape(-1), _f64(wang),
            rg.ctypes.data_as(C.c_void_p) if rg is not None else None, len(rw) if rw is not None else 0,
            rw.ctypes.data_as(C.c_void_p) if rw is not None else None, len(usph), _f64(usph).reshape(-1),
            _f64(wsph), float(prec), int(bool(stats)), int(nthreads), out["att_cp"], out["props"].reshape(-1),
            out["iaserr"].reshape(-1), out["rsurf"].reshape(-1), out["rbeta_int"], C.byref(nw), C.byref(nr))
        if got < 0:
            raise RuntimeError("basin bisection: can not find ray limits")
        for k in ("att_cp", "props", "iaserr", "rsurf", "rbeta_int"):
            out[k] = out[k][:got]
        out["nwarn"], out["nrestart"] = nw.value, nr.value
        return out

    def sphere_integrals(self, cp_xyz, cp_typ, u, wang, ring=None, ringw=None, cpid=0, nr=100, r0=1e-3, rend=-1.0,
                         nthreads=0):
        """SPHEREINTEGRALS: dict of att_cp, radii (natt, nr), props (natt, nr, 2: Pop, Lap)."""
        ct = _i32(cp_typ)
        n = len(ct)
        nat = self.mol.natom
        na = len([i for i in (range(n) if cpid <= 0 else [cpid - 1]) if i < nat or ct[i] == -3])
        out = dict(att_cp=np.zeros(max(na, 1), np.int32), radii=np.zeros((max(na, 1), nr)),
                   props=np.zeros((max(na, 1), nr, 2)))
        rg = _i32(ring) if ring is not None else None
        rw = _f64(ringw) if ringw is not None else None
        got = lib().o_sphere_integrals(
            self.h, n, _f64(cp_xyz).reshape(-1), ct, int(cpid), len(u), _f64(u).reshape(-1), _f64(wang),
            rg.ctypes.data_as(C.c_void_p) if rg is not None else None, len(rw) if rw is not None else 0,
            rw.ctypes.data_as(C.c_void_p) if rw is not None else None, int(nr), float(r0), float(rend),
            int(nthreads), out["att_cp"], out["radii"].reshape(-1), out["props"].reshape(-1))
        for k in ("att_cp", "radii", "props"):
            out[k] = out[k][:got]
        return out

    def mesh(self, mesh="franchini", level="good", nthreads=0):
        """genmesh: (xyz (n,3), w (n,)) with the Lebedev rules of
        tests/golden/lebedev_rules.json."""
        t = {"becke": 1, "franchini": 2}[mesh]
        lvl = {"small": 1, "normal": 2, "good": 3, "vgood": 4, "amazing": 5}[level]
        nang = (0, 110, 194, 302, 590, 770)[lvl]
        ang = _f64(lebedev_rule(nang)).reshape(-1)
        n = lib().o_mesh_size(self.h, lvl, nang)
        xyz, wt = np.zeros(3 * n), np.zeros(n)
        lib().o_mesh(self.h, t, lvl, nang, ang, xyz, wt, nthreads)
        return xyz.reshape(n, 3), wt

    def molcalc(self, quantities=("rho",), mesh="franchini", level="good", nthreads=0):
        """molcalc: sum_i w_i f(x_i) for rho, gradrho (|grad rho|), volume."""
        xyz, wt = self.mesh(mesh, level, nthreads)
        # fillmesh evaluates a molecule with periodic = .false. (no wrap),
        # src/molcalc@proc.F90:113
        need = any(q != "volume" for q in quantities)
        rho, grad = self.rho2_points(xyz, 1, nthreads)[:2] if need else (None, None)
        out = {}
        for q in quantities:
            if q == "volume":
                f = np.ones(len(wt))
            elif q == "rho":
                f = rho
            elif q == "gradrho":
                g = grad.reshape(-1, 3).copy()
                # nucleus rule of grd: |grad| := 0 within 1e-5 bohr of a nucleus
                for a in self.mol.atom_xyz:
                    g[np.linalg.norm(xyz - a, axis=1) <= 1e-5] = 0.0
                f = np.linalg.norm(g, axis=1)
            else:
                raise ValueError(q)
            out[q] = float(np.sum(f * wt))
        out["npoints"] = len(wt)
        return out

    def autocritic(self, seeds=None, nthreads=0):
        if seeds is None:
            seeds = self.pair_seeds()
        seeds = _f64(seeds).reshape(-1, 3)
        maxcp = self.mol.natom + seeds.shape[0] + 1
        xyz, typ, f = np.zeros(3 * maxcp), np.zeros(maxcp, np.int32), np.zeros(maxcp)
        cnt = np.zeros(4, np.int32)
        ncp = lib().o_autocritic(self.h, seeds.shape[0], seeds.reshape(-1), nthreads, maxcp,
                                 xyz, typ, f, cnt)
        return dict(xyz=xyz[: 3 * ncp].reshape(ncp, 3), typ=typ[:ncp], f=f[:ncp],
                    counts=cnt, ph=int(cnt[0] - cnt[1] + cnt[2] - cnt[3]))


def eigvec3(m):
    """Ascending eigenvalues and eigenvectors (columns) of a 3x3 matrix."""
    ev, v = np.zeros(3), np.zeros(9)
    lib().o_eigvec3(_f64(np.asarray(m).reshape(-1)), ev, v)
    return ev, v.reshape(3, 3).T


def eigsym3(m):
    ev = np.zeros(3)
    lib().o_eigsym3(_f64(np.asarray(m).T.reshape(-1)), ev)
    return ev


def rsindex(m, eps=1e-8):
    ev = np.zeros(3)
    r, s = C.c_int(), C.c_int()
    lib().o_rsindex(_f64(np.asarray(m).T.reshape(-1)), ev, C.byref(r), C.byref(s), eps)
    return ev, r.value, s.value


def matinvsym3(m):
    a = _f64(np.asarray(m).T.reshape(-1)).copy()
    ier = lib().o_matinvsym3(a)
    return a.reshape(3, 3).T, ier


# ------------------------------------------------------------- NCI output
def fmt_e13(x) -> str:
    """(" ",1p,e13.5e3) of one number (14 characters)."""
    b = C.create_string_buffer(16)
    lib().o_fmt_e13_5e3(float(x), b)
    return b.raw[:14].decode()


def fmt_E15(x) -> str:
    """1p,E15.7 of one number (15 characters)."""
    b = C.create_string_buffer(16)
    lib().o_fmt_E15_7(float(x), b)
    return b.raw[:15].decode()


def cube_body(nstep, values) -> bytes:
    """write_cube_body text of a (k,j,i)-ordered cube."""
    ns = _i32(nstep)
    v = _f64(values).reshape(-1)
    n3 = int(ns[2])
    size = int(ns[0]) * int(ns[1]) * (14 * n3 + (n3 + 5) // 6 + (1 if n3 % 6 else 0))
    b = C.create_string_buffer(size + 16)
    m = lib().o_cube_body(ns, v, b)
    return b.raw[:m]


def dat_text(dat) -> bytes:
    """.dat lines (1p,E15.7,E15.7) of (n,2) pairs."""
    d = _f64(dat).reshape(-1, 2)
    return "".join(fmt_E15(a) + fmt_E15(b) + "\n" for a, b in d).encode()


def nci_post(nstep, crho, cgrad, rhocut=0.2, dimcut=2.0, rhoplot=0.1, srho=(-1e30, 1e30), onlyneg=False):
    """nciplot's cutoff pass: returns (cgrad after the s := 100 rules,
    dat pairs (n, 2))."""
    ns = _i32(nstep)
    cr = _f64(crho).reshape(-1)
    cg = _f64(cgrad).reshape(-1).copy()
    dat = np.zeros(2 * cr.size)
    nd = lib().o_nci_post(ns, cr, cg, rhocut, dimcut, rhoplot, srho[0], srho[1], int(onlyneg), dat)
    return cg, dat[: 2 * nd].reshape(-1, 2)


def fmt_E22(x) -> str:
    """E22.14E3 (no scale factor) of one number (22 characters)."""
    b = C.create_string_buffer(24)
    lib().o_fmt_E22_14E3(float(x), b)
    return b.raw[:22].decode()


def precise_body(nstep, values) -> str:
    """writegrid_cube's (6(" ",E22.14E3)) body of a (k,j,i)-ordered cube."""
    ns = [int(v) for v in nstep]
    v = _f64(values).reshape(-1)
    out = []
    for r in range(ns[0] * ns[1]):
        row = v[r * ns[2]:(r + 1) * ns[2]]
        for c in range(0, ns[2], 6):
            chunk = row[c:c + 6]
            out.append("".join(" " + fmt_E22(x) for x in chunk) + (" " if len(chunk) < 6 else "") + "\n")
    return "".join(out)


# ------------------------------------------------------------ NCI checkpoint
# gfortran's unformatted sequential layout (libgfortran, the runtime of the
# reference's usual compiler; its record format is documented in the GNU
# Fortran manual, "Unformatted sequential file format"): each record is
# one or more subrecords, each framed by 4-byte length markers; the leading
# marker of every subrecord but the last is negative, the trailing marker
# of every subrecord but the first is negative; at most 2^31 - 9 data bytes
# per subrecord.
MAX_SUBRECORD = 2147483639


def fortran_records_bytes(records, maxsub=MAX_SUBRECORD) -> bytes:
    """The bytes of a sequence of records (each a bytes object)."""
    out = []
    for rec in records:
        n = len(rec)
        pos, first = 0, True
        while True:
            m = min(n - pos, maxsub)
            last = pos + m == n
            out.append(np.int32(m if last else -m).tobytes())
            out.append(rec[pos:pos + m])
            out.append(np.int32(m if first else -m).tobytes())
            pos += m
            first = False
            if last:
                break
    return b"".join(out)


def fortran_records_parse(data: bytes):
    """Splits gfortran unformatted sequential bytes into records."""
    recs, pos = [], 0
    while pos < len(data):
        parts, more = [], True
        while more:
            lead = int(np.frombuffer(data[pos:pos + 4], np.int32)[0])
            m = abs(lead)
            parts.append(data[pos + 4:pos + 4 + m])
            trail = int(np.frombuffer(data[pos + 4 + m:pos + 8 + m], np.int32)[0])
            assert abs(trail) == m, "bad record marker"
            pos += 8 + m
            more = lead < 0
        recs.append(b"".join(parts))
    return recs


def nci_chk_records(x0, xmat, nstep, crho, cgrad, rhoat=None, nfrag=0):
    """writechk's records (src/nci@proc.f90:1087-1117); xmat[:, i] is step i;
    logicals as gfortran's default LOGICAL (4 bytes, 1 = .true.)."""
    xm = np.asarray(xmat, np.float64)
    recs = [np.array([int(rhoat is not None), 0, nfrag], np.int32).tobytes(),
            _f64(x0).tobytes()] + [_f64(xm[:, j]).tobytes() for j in range(3)]
    recs.append(_i32(nstep).tobytes())
    recs.append(_f64(crho).reshape(-1).tobytes() + _f64(cgrad).reshape(-1).tobytes())
    if rhoat is not None:
        recs.append(_f64(rhoat).reshape(-1).tobytes())
    return recs


def nci_chk_read(data: bytes, x0, xmat, nstep):
    """readchk (src/nci@proc.f90:1019-1085) for a caller without promolecular
    or fragment densities: (crho, cgrad) flat arrays, or None when the file
    does not match the grid."""
    r = fortran_records_parse(data)
    llat, llfrag, nfrag0 = np.frombuffer(r[0][:12], np.int32)
    if nfrag0 != 0:
        return None
    xm = np.asarray(xmat, np.float64)
    if np.any(np.abs(np.frombuffer(r[1][:24]) - _f64(x0)) > 1e-13):
        return None
    for j in range(3):
        if np.any(np.abs(np.frombuffer(r[2 + j][:24]) - xm[:, j]) > 1e-13):
            return None
    if np.any(np.frombuffer(r[5][:12], np.int32) != _i32(nstep)):
        return None
    n = int(np.prod(nstep))
    v = np.frombuffer(r[6][:16 * n])
    return v[:n].copy(), v[n:].copy()


# -------------------------------------------------------------- wfn format
def _fortran_field(s: str, d: int) -> float:
    t = s.replace(" ", "")
    if not t:
        return 0.0
    t = t.replace("D", "E").replace("d", "E")
    mant, ex = (t.split("E") + ["0"])[:2] if "E" in t else (t, "0")
    if "E" not in t:
        for i in range(1, len(t)):
            if t[i] in "+-":
                mant, ex = t[:i], t[i:]
                break
    e10 = int(ex) - (0 if "." in mant else d)
    return float(f"{mant}E{e10}")  # one correctly rounded conversion


def read_wfn_text(path: str) -> dict:
    """read_wfn (src/wfn_private@proc.F90:981-1118) restated on the fixed
    columns of formats 101-106: returns natom, xyz (natom,3), element labels,
    icenter/itype (1-based), e, occ, cmo (npri, nmo), energies, wfntyp,
    nalpha (before prune_primitives)."""
    lines = open(path).read().split("\n")
    pad = lambda l, n: l + " " * max(0, n - len(l))
    h = pad(lines[1], 80)
    nmo, npri, nat = int(h[18:23]), int(h[38:43]), int(h[58:63])
    pos = 2
    xyz, elem = [], []
    for a in range(nat):
        l = pad(lines[pos + a], 80)
        elem.append(l[2:4])
        xyz.append([_fortran_field(l[24 + 12 * j:36 + 12 * j], 8) for j in range(3)])
    pos += nat

    def fields(n, skip, per, w, d=0, conv=float):
        nonlocal pos
        out = []
        while len(out) < n:
            l = pad(lines[pos], skip + per * w)
            pos += 1
            for k in range(per):
                if len(out) == n:
                    break
                f = l[skip + k * w:skip + (k + 1) * w]
                out.append(conv(f) if conv is int else _fortran_field(f, d))
        return out

    icenter = fields(npri, 20, 20, 3, conv=int)
    itype = fields(npri, 20, 20, 3, conv=int)
    e = fields(npri, 10, 5, 14, 7)
    while not lines[pos].startswith("MO"):
        pos += 1
    occ, ene, cmo = [], [], np.zeros((npri, nmo))
    for m in range(nmo):
        l = pad(lines[pos], 80)
        pos += 1
        occ.append(_fortran_field(l[35:47], 7))
        ene.append(_fortran_field(l[62:74], 6))
        cmo[:, m] = fields(npri, 0, 5, 16, 8)
    frac = any(abs(round(o) - o) > 1e-10 for o in occ)
    n1 = sum(1 for o in occ if abs(round(o) - o) <= 1e-10 and round(o) == 1)
    n2 = sum(1 for o in occ if abs(round(o) - o) <= 1e-10 and round(o) == 2)
    nalpha, found, e0 = -1, False, -1e30
    for m, en in enumerate(ene):
        if en < e0 - 1e-3:
            nalpha, found = m, True
        e0 = en
    if frac:
        typ, na = 3, 0
    elif n1 == 0:
        typ, na = 0, nalpha
    elif n2 == 0:
        typ, na = 1, (nalpha if found else nmo)
    else:
        typ, na = 2, n2
    return dict(natom=nat, xyz=np.array(xyz), elem=elem, icenter=np.array(icenter, np.int32),
                itype=np.array(itype, np.int32), e=np.array(e), occ=np.array(occ), cmo=cmo,
                energies=np.array(ene), wfntyp=typ, nalpha=na)


_LEBEDEV = None


def lebedev_rule(n: int) -> np.ndarray:
    """The n-point Lebedev rule (n, 4): x, y, z, weight (sum 1), from the
    committed fixture tests/golden/lebedev_rules.json."""
    global _LEBEDEV
    if _LEBEDEV is None:
        import json
        here = os.path.dirname(os.path.abspath(__file__))
        with open(os.path.join(here, "..", "tests", "golden", "lebedev_rules.json")) as fh:
            _LEBEDEV = {int(k): np.array(v) for k, v in json.load(fh).items()}
    return _LEBEDEV[n]


# ------------------------------------------------------------- fchk format
_SPHCAR = None
_FCHK_CART = {0: [""], 1: ["x", "y", "z"], 2: ["xx", "yy", "zz", "xy", "xz", "yz"],
              3: ["xxx", "yyy", "zzz", "xyy", "xxy", "xxz", "xzz", "yzz", "yyz", "xyz"],
              4: ["zzzz", "yzzz", "yyzz", "yyyz", "yyyy", "xzzz", "xyzz", "xyyz", "xyyy", "xxzz", "xxyz",
                  "xxyy", "xxxz", "xxxy", "xxxx"]}


def sphcar(l: int) -> np.ndarray:
    """critic2's spherical -> Cartesian matrix for l (tests/golden/sphcar_fchk.json)."""
    global _SPHCAR
    if _SPHCAR is None:
        import json
        here = os.path.dirname(os.path.abspath(__file__))
        with open(os.path.join(here, "..", "tests", "golden", "sphcar_fchk.json")) as fh:
            _SPHCAR = {(int(k) if k.isdigit() else k): np.array(v) for k, v in json.load(fh).items()}
    return _SPHCAR[l]


def _dfac_l(e):
    d = 1
    for v in e:
        for k in range(2 * v - 1, 1, -2):
            d *= k
    return d


def _gnorm(e, a):
    # gnorm (src/wfn_private@proc.F90:3375-3459): 2^((4L+3)/4) a^((2L+3)/4) / pi^(3/4) / sqrt(prod (2l-1)!!)
    L = sum(e)
    return 2.0 ** ((4 * L + 3) / 4) * a ** ((2 * L + 3) / 4) / np.pi ** 0.75 / np.sqrt(_dfac_l(e))


def _aonorm(e, a, c):
    # aonorm (:3461-3540)
    L = sum(e)
    s = sum(c[i] * c[j] / (a[i] + a[j]) ** (L + 1.5) for i in range(len(a)) for j in range(len(a)))
    return 1.0 / np.sqrt(s * _dfac_l(e) * np.pi ** 1.5 / 2 ** L)


def read_fchk_text(path: str) -> dict:
    """read_fchk (src/wfn_private@proc.F90:1287-1812, occupied MOs) restated:
    primitive arrays (icenter 1-based, itype, e, cmo (npri, nmo)), occ,
    wfntyp, nalpha, atoms; before prune_primitives."""
    lines = open(path).read().split("\n")

    def scalar(key):
        for l in lines:
            if l.startswith(key):
                return int(l.split()[-1])
        return 0

    def arr(key, n):
        for i, l in enumerate(lines):
            if l.startswith(key):
                v = []
                j = i + 1
                while len(v) < n:
                    v += [float(t.replace("D", "E")) for t in lines[j].split()]
                    j += 1
                return np.array(v[:n])
        raise KeyError(key)

    nelec, na, nb = scalar("Number of electrons"), scalar("Number of alpha electrons"), scalar("Number of beta electrons")
    nbas, ncs, nps, nat = (scalar("Number of basis functions"), scalar("Number of contracted shells"),
                           scalar("Number of primitive shells"), scalar("Atomic numbers"))
    uhf = any(l.startswith("Beta Orbital Energies") for l in lines)
    if uhf:
        typ, nmo, nalf = 1, nelec, na
    elif na == nb:
        typ, nmo, nalf = 0, nelec // 2, nelec // 2
    else:
        typ, nmo, nalf = 2, na, nb
    namo = nmo if typ == 2 else nalf
    st = arr("Shell types", ncs).astype(int)
    npp = arr("Number of primitives per shell", ncs).astype(int)
    sa = arr("Shell to atom map", ncs).astype(int)
    ex, cc = arr("Primitive exponents", nps), arr("Contraction coefficients", nps)
    pc = arr("P(S=P) Contraction coefficients", nps) if (st == -1).any() else None
    mo = arr("Alpha MO coefficients", namo * nbas).reshape(namo, nbas)
    if nmo > namo:
        mo = np.vstack([mo, arr("Beta MO coefficients", (nmo - namo) * nbas).reshape(nmo - namo, nbas)])
    shells, off = [], 0
    for t, n, a in zip(st, npp, sa):
        e, c = ex[off:off + n], cc[off:off + n]
        if t == -1:
            shells += [(0, a, e, c), (1, a, e, pc[off:off + n])]
        else:
            shells.append((t, a, e, c))
        off += n
    from critic2_gb300.synth import LI
    li = {tuple(v): k + 1 for k, v in enumerate(LI.tolist())}
    icenter, itype, pe, cols = [], [], [], []
    ns = 0
    for t, a, e, c in shells:
        l = abs(t)
        ncar = (l + 1) * (l + 2) // 2
        nsp = 2 * l + 1 if t < 0 else ncar
        blk = mo[:, ns:ns + nsp]
        car = blk @ sphcar(l) if (t < 0 and l >= 2) else blk
        for k, lab in enumerate(_FCHK_CART[l]):
            ev = (lab.count("x"), lab.count("y"), lab.count("z"))
            cn = np.array([ci * _gnorm(ev, ai) for ci, ai in zip(c, e)])
            norm = _aonorm(ev, e, cn)
            for j in range(len(e)):
                icenter.append(a)
                itype.append(li[ev])
                pe.append(e[j])
                cols.append(cn[j] * norm * car[:, k])
        ns += nsp
    occ = np.full(nmo, 1.0 if typ == 1 else 2.0)
    if typ == 2:
        occ[nalf:] = 1.0
    return dict(atom_xyz=arr("Current cartesian coordinates", 3 * nat).reshape(nat, 3),
                atom_z=arr("Atomic numbers", nat).astype(np.int32), icenter=np.array(icenter, np.int32),
                itype=np.array(itype, np.int32), e=np.array(pe), cmo=np.array(cols), occ=occ, wfntyp=typ,
                nalpha=nalf)


_MOLDEN_G = ["xxxx", "yyyy", "zzzz", "xxxy", "xxxz", "xyyy", "yyyz", "xzzz", "yzzz", "xxyy", "xxzz", "yyzz",
             "xxyz", "xyyz", "xyzz"]


def read_molden_text(path: str) -> dict:
    """read_molden (src/wfn_private@proc.F90:1819-2478; GTO, occupied MOs)
    restated: primitive arrays as read_fchk_text returns them."""
    lines = open(path).read().split("\n")
    low = [l.lower() for l in lines]
    key = lambda l: l[l.find("[") + 1:l.find("]")] if "[" in l and "]" in l else ""
    is5d = is7f = is9g = orca = False
    ang, at, gt, mo0 = 1.0, None, None, None
    for i, l in enumerate(low):
        k = key(l)
        if k == "title" and "created by orca_2mkl" in lines[i + 1]:
            orca = True
        elif k == "atoms":
            at = i + 1
            if "angs" in l:
                ang = 1.0 / 0.52917720859
        elif k == "gto":
            gt = i + 1
        elif k == "mo":
            mo0 = i + 1
        elif k in ("5d", "5d7f"):
            is5d = is7f = True
        elif k == "5d10f":
            is5d, is7f = True, False
        elif k == "7f":
            is5d, is7f = False, True
        elif k == "9g":
            is9g = True
    if orca:
        is5d = is7f = is9g = True
    xyz, zs = [], []
    i = at
    while lines[i].strip() and "[" not in lines[i]:
        t = lines[i].split()
        zs.append(int(t[2]))
        xyz.append([float(v.replace("D", "E")) * ang for v in t[3:6]])
        i += 1
    shells, i = [], gt
    for a in range(len(zs)):
        while not lines[i].strip():
            i += 1
        i += 1
        while lines[i].strip() and "[" not in lines[i]:
            lab, n = lines[i].split()[:2]
            n = int(n)
            l = "spdfg".index(lab.lower())
            pure = {2: is5d, 3: is7f, 4: is9g}.get(l, False)
            ps = [list(map(lambda v: float(v.replace("D", "E")), lines[i + 1 + k].split()[:2])) for k in range(n)]
            shells.append((-l if pure else l, a, np.array([p[0] for p in ps]), np.array([p[1] for p in ps])))
            i += n + 1
    nbas = sum(2 * -t + 1 if t < 0 else (t + 1) * (t + 2) // 2 for t, *_ in shells)
    mos, alpha = [], True
    j = mo0
    while j < len(lines):
        l = low[j]
        if "spin=" in l:
            alpha = "alpha" in l
        if "occup=" in l:
            occ = round(float(l.split("occup=")[1].split()[0]))
            c = np.zeros(nbas)
            j += 1
            while j < len(lines):
                t = lines[j].split()
                if len(t) < 2 or not t[0].lstrip("-").isdigit():
                    break
                c[int(t[0]) - 1] = float(t[1].replace("D", "E"))
                j += 1
            if occ > 0:
                mos.append((alpha, occ, c))
            continue
        j += 1
    beta = any(not a for a, _, _ in mos)
    typ = 1 if beta else 0
    mo = np.array([c for a, _, c in mos if a] + [c for a, _, c in mos if not a])
    nalf = sum(1 for a, _, _ in mos if a)
    if orca:
        ns = 0
        for t, *_ in shells:
            if t in (-3, -4):
                mo[:, ns + 5:ns + (7 if t == -3 else 9)] *= -1
            ns += 2 * -t + 1 if t < 0 else (t + 1) * (t + 2) // 2
    from critic2_gb300.synth import LI
    li = {tuple(v): k + 1 for k, v in enumerate(LI.tolist())}
    icenter, itype, pe, cols = [], [], [], []
    ns = 0
    for t, a, e, c in shells:
        l = abs(t)
        cart = _MOLDEN_G if l == 4 else _FCHK_CART[l]
        ncar = len(cart)
        nsp = 2 * l + 1 if t < 0 else ncar
        blk = mo[:, ns:ns + nsp]
        if t < 0 and l >= 2:
            blk = blk @ (sphcar(l) if l < 4 else _sphcar_molden_g())
        for k, lab in enumerate(cart):
            ev = (lab.count("x"), lab.count("y"), lab.count("z"))
            cn = np.array([ci * _gnorm(ev, ai) / (_gnorm((l, 0, 0), ai) if orca else 1.0) for ci, ai in zip(c, e)])
            norm = _aonorm(ev, e, cn)
            for jj in range(len(e)):
                icenter.append(a + 1)
                itype.append(li[ev])
                pe.append(e[jj])
                cols.append(cn[jj] * norm * blk[:, k])
        ns += nsp
    return dict(atom_xyz=np.array(xyz), atom_z=np.array(zs, np.int32), icenter=np.array(icenter, np.int32),
                itype=np.array(itype, np.int32), e=np.array(pe), cmo=np.array(cols),
                occ=np.full(mo.shape[0], 1.0 if typ == 1 else 2.0), wfntyp=typ, nalpha=nalf)


def _sphcar_molden_g():
    sphcar(2)  # loads the fixture
    return _SPHCAR["4molden"]
