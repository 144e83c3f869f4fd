"""Host mirror of critic2's molecular-wavefunction field API over the C ABI.

`Wavefunction` plays the role of critic2's `molwfn` plus the wavefunction
branch of `field` (src/wfn_private.f90:91-141, src/fieldmod.f90:178-269):
`rho2` is molwfn%rho2 for a batch of points, `grd` is field%grd, `newton`
is field%newton for a batch of seeds; `nciplot` and `autocritic` are the
two consumers the reference drives from them (src/nci@proc.f90:540-605,
src/autocp@proc.f90:755-822).  Every call goes to the GPU library; there is
no CPU path.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import _lib as L


def _prec(p) -> int:
    if isinstance(p, str):
        return L.PREC[p]
    return int(p)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


class Wavefunction:
    """A molecular wavefunction resident on the GPU."""

    def __init__(self, mol=None, *, _handle=None):
        self._h = C.c_void_p()
        self.atom_xyz = None if mol is None else np.array(mol.atom_xyz, np.float64).reshape(-1, 3)
        if _handle is not None:
            self._h = _handle
        else:
            lib = L.lib()
            L.check(lib.c2g_wfn_create(
                mol.natom, _f64(mol.atom_xyz.reshape(-1)), _i32(mol.atom_z), mol.npri, mol.nmo,
                _i32(mol.icenter), _i32(mol.itype), _f64(mol.e), _f64(mol.occ),
                _f64(mol.cmo.reshape(-1)), int(mol.wfntyp), int(mol.nalpha), C.byref(self._h)))
        if mol is not None and mol.nedf:
            self.set_edf(mol.edf_icenter, mol.edf_itype, mol.edf_e, mol.edf_c)
        n = [C.c_int() for _ in range(5)]
        L.check(L.lib().c2g_wfn_info(self._h, *[C.byref(v) for v in n]))
        self.natom, self.npri, self.nmo, self.wfntyp, self.nalpha = (v.value for v in n)

    @classmethod
    def from_wfx(cls, path: str) -> "Wavefunction":
        h = C.c_void_p()
        L.check(L.lib().c2g_wfn_read_wfx(path.encode(), C.byref(h)))
        return cls(_handle=h)

    @classmethod
    def from_fchk(cls, path: str) -> "Wavefunction":
        """A Gaussian formatted checkpoint file (c2g_wfn_read_fchk)."""
        h = C.c_void_p()
        L.check(L.lib().c2g_wfn_read_fchk(path.encode(), C.byref(h)))
        return cls(_handle=h)

    @classmethod
    def from_molden(cls, path: str) -> "Wavefunction":
        """A molden file with Gaussian-type orbitals (c2g_wfn_read_molden)."""
        h = C.c_void_p()
        L.check(L.lib().c2g_wfn_read_molden(path.encode(), C.byref(h)))
        return cls(_handle=h)

    @classmethod
    def from_wfn(cls, path: str) -> "Wavefunction":
        """An AIMPAC wfn file (c2g_wfn_read_wfn)."""
        h = C.c_void_p()
        L.check(L.lib().c2g_wfn_read_wfn(path.encode(), C.byref(h)))
        return cls(_handle=h)

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            L.lib().c2g_wfn_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_edf(self, icenter, itype, e, c):
        """EDF core density (c2g_wfn_set_edf): 1-based centres and li types,
        exponents and coefficients; empty arrays remove the core."""
        ic, it, ee, cc = _i32(icenter), _i32(itype), _f64(e), _f64(c)
        n = int(ee.shape[0])
        L.check(L.lib().c2g_wfn_set_edf(self._h, n, L.ptr(ic) if n else None, L.ptr(it) if n else None,
                                        L.ptr(ee) if n else None, L.ptr(cc) if n else None))

    def set_recheck(self, rel: float):
        """Relative |lambda2| below which split-precision NCI points are
        re-evaluated in FP64 (C2G_PARAM_RECHECK_REL); negative restores the
        mode's default (TF32x3 1e-4, BF16x3 1e-3), 0 disables it."""
        L.check(L.lib().c2g_wfn_set_param(self._h, 1, float(rel)))

    def set_newton_stall(self, k: int):
        """Stop a Newton seed after k FP64 steps without a new minimum of
        |grad| (C2G_PARAM_NEWTON_STALL; 0 = off, critic2's semantics)."""
        L.check(L.lib().c2g_wfn_set_param(self._h, 2, float(k)))

    def set_wait_ns(self, ns: float):
        """Limit (ns) of every pipeline wait of the split-precision kernel
        (C2G_PARAM_WAIT_NS, default 4e9); a wait that runs out makes the call
        fail with C2G_ERR_CUDA and leaves the handle usable."""
        L.check(L.lib().c2g_wfn_set_param(self._h, 3, float(ns)))

    # ------------------------------------------------------------ rho2/grd
    def rho2(self, xyz, nder: int = 2, prec="fp64") -> dict:
        """molwfn%rho2 at points xyz (n,3).  Arrays are per point:
        rho (n,3) total/up/down; grad (n,3,3) [spin][xyz]; hess (n,3,3,3)
        [spin][col][row]; gkin (n,3); stress (n,3,3); vir (n,)."""
        x = _f64(xyz).reshape(-1, 3)
        n = x.shape[0]
        out = dict(rho=np.zeros((n, 3)), grad=np.zeros((n, 3, 3)), hess=np.zeros((n, 3, 3, 3)),
                   gkin=np.zeros((n, 3)), stress=np.zeros((n, 3, 3)), vir=np.zeros(n))
        L.check(L.lib().c2g_rho2(self._h, n, L.ptr(x), nder, _prec(prec), L.ptr(out["rho"]),
                                 L.ptr(out["grad"]), L.ptr(out["hess"]), L.ptr(out["gkin"]),
                                 L.ptr(out["stress"]), L.ptr(out["vir"])))
        return out

    def rho2_valence(self, xyz, nder: int = 2) -> dict:
        """The valence outputs of molwfn%rho2 (rhoval, gradval, hval: no
        EDF core), FP64, in rho2's layout: rho (n,3), grad (n,3,3), hess
        (n,3,3,3)."""
        x = _f64(xyz).reshape(-1, 3)
        n = x.shape[0]
        out = dict(rho=np.zeros((n, 3)), grad=np.zeros((n, 3, 3)), hess=np.zeros((n, 3, 3, 3)))
        L.check(L.lib().c2g_rho2_valence(self._h, n, L.ptr(x), nder, L.ptr(out["rho"]),
                                         L.ptr(out["grad"]), L.ptr(out["hess"])))
        return out

    def grd(self, xyz, nder: int = 2, prec="fp64") -> dict:
        """field%grd at points xyz (n,3): f, gf (n,3), gfmod, hf (n,3,3),
        hfeval (n,3) ascending, r, s, isnuc."""
        x = _f64(xyz).reshape(-1, 3)
        n = x.shape[0]
        o = dict(f=np.zeros(n), gf=np.zeros((n, 3)), gfmod=np.zeros(n), hf=np.zeros((n, 3, 3)),
                 hfeval=np.zeros((n, 3)), r=np.zeros(n, np.int32), s=np.zeros(n, np.int32),
                 isnuc=np.zeros(n, np.int32))
        L.check(L.lib().c2g_grd(self._h, n, L.ptr(x), nder, _prec(prec), L.ptr(o["f"]),
                                L.ptr(o["gf"]), L.ptr(o["gfmod"]), L.ptr(o["hf"]),
                                L.ptr(o["hfeval"]), L.ptr(o["r"]), L.ptr(o["s"]),
                                L.ptr(o["isnuc"])))
        return o

    # ---------------------------------------------------------------- NCI
    def nciplot(self, x0, xmat, nstep, prec="fp64"):
        """NCI grid: returns crho, cgrad as (n1, n2, n3) arrays (Fortran
        (k,j,i) order, k fastest) and the stats record.  xmat[:, i] is the
        step of axis i."""
        nstep = _i32(nstep)
        shape = tuple(int(v) for v in nstep)
        crho, cgrad = np.zeros(shape), np.zeros(shape)
        st = L.NciStats()
        xm = _f64(np.asarray(xmat, np.float64).T.reshape(-1))
        L.check(L.lib().c2g_nciplot(self._h, _f64(x0), xm, nstep, _prec(prec), L.ptr(crho),
                                    L.ptr(cgrad), C.byref(st)))
        return crho, cgrad, st

    def nciplot_dev(self, x0, xmat, nstep, prec, d_crho: int, d_cgrad: int, stream: int = 0,
                    stats: bool = False):
        """NCI grid into device buffers (raw pointers), on a CUDA stream."""
        st = L.NciStats()
        xm = _f64(np.asarray(xmat, np.float64).T.reshape(-1))
        L.check(L.lib().c2g_nciplot_dev(self._h, _f64(x0), xm, _i32(nstep), _prec(prec),
                                        C.c_void_p(d_crho), C.c_void_p(d_cgrad),
                                        C.c_void_p(stream), C.byref(st) if stats else None))
        return st

    def nciplot_dev_noalloc(self, x0, xmat, nstep, prec, d_crho: int, d_cgrad: int, stream: int = 0):
        """NCI grid into device buffers without any device allocation by the
        library (c2g_nciplot_dev_noalloc: at most 2^20 points per call, split
        operands of `prec` built by an earlier call, calls on one device
        serialised by the caller)."""
        xm = _f64(np.asarray(xmat, np.float64).T.reshape(-1))
        L.check(L.lib().c2g_nciplot_dev_noalloc(self._h, _f64(x0), xm, _i32(nstep), _prec(prec),
                                                C.c_void_p(d_crho), C.c_void_p(d_cgrad),
                                                C.c_void_p(stream)))

    def nciplot_files(self, x0, xmat, nstep, prec, root: str, cut=None):
        """nciplot end to end into root-dens.cube, root-grad.cube and
        root.dat (c2g_nciplot_files).  cut: None (critic2's defaults) or a
        dict of rhocut, dimcut, rhoplot, srho_lo, srho_hi, onlyneg.  Returns
        (stats, ms) with ms = evaluation, cutoff pass, formatting, writes."""
        st = L.NciStats()
        ms = np.zeros(4)
        c = None
        if cut is not None:
            d = dict(rhocut=0.2, dimcut=2.0, rhoplot=0.1, srho_lo=-1e30, srho_hi=1e30, onlyneg=0)
            d.update(cut)
            c = L.NciCut(**{k: (int(v) if k == "onlyneg" else float(v)) for k, v in d.items()})
        xm = _f64(np.asarray(xmat, np.float64).T.reshape(-1))
        L.check(L.lib().c2g_nciplot_files(self._h, _f64(x0), xm, _i32(nstep), _prec(prec), root.encode(),
                                          C.byref(c) if c is not None else None, C.byref(st), ms))
        return st, ms

    FIELDS = ("rho", "gx", "gy", "gz", "gmod", "hxx", "hxy", "hxz", "hyy", "hyz", "hzz", "lap")

    def cube_field_file(self, x0, xmat, nstep, prop, path: str, prec="fp64"):
        """CUBE plot of one grd quantity (name in FIELDS) into a precise
        critic2 cube file (c2g_cube_field_file); returns the wall times in
        ms of evaluation, text and write."""
        ms = np.zeros(3)
        xm = _f64(np.asarray(xmat, np.float64).T.reshape(-1))
        L.check(L.lib().c2g_cube_field_file(self._h, _f64(x0), xm, _i32(nstep), _prec(prec),
                                            self.FIELDS.index(prop), path.encode(), ms))
        return ms

    # -------------------------------------------------------------- Newton
    def newton(self, xyz, gfnormeps: float = 1e-12, maxit: int = 200, prec="fp64"):
        x = _f64(xyz).reshape(-1, 3).copy()
        ier = np.zeros(x.shape[0], np.int32)
        L.check(L.lib().c2g_newton(self._h, x.shape[0], L.ptr(x), gfnormeps, maxit, _prec(prec),
                                   L.ptr(ier)))
        return x, ier

    def pair_seeds(self, maxdist: float = 15.0, npts: int = 5) -> np.ndarray:
        n = C.c_int(0)
        L.check(L.lib().c2g_pair_seeds(self._h, maxdist, npts, None, C.byref(n)))
        buf = np.zeros((max(n.value, 1), 3))
        L.check(L.lib().c2g_pair_seeds(self._h, maxdist, npts, L.ptr(buf), C.byref(n)))
        return buf[: n.value]

    MESH_TYPES = {"becke": 1, "franchini": 2}
    MESH_LEVELS = {"small": 1, "normal": 2, "good": 3, "vgood": 4, "amazing": 5}
    MOLCALC = {"volume": 0, "rho": 1, "gradrho": 2, "gkin": 3}

    def mesh_size(self, mesh="franchini", level="good") -> int:
        n = C.c_long(0)
        L.check(L.lib().c2g_mesh_size(self._h, self.MESH_TYPES[mesh], self.MESH_LEVELS[level], C.byref(n)))
        return n.value

    def mesh(self, mesh="franchini", level="good"):
        """The integration mesh (c2g_mesh_dev) as host arrays xyz (n,3), w (n,)."""
        import torch
        n = self.mesh_size(mesh, level)
        x = torch.empty((n, 3), dtype=torch.float64, device="cuda")
        w = torch.empty(n, dtype=torch.float64, device="cuda")
        L.check(L.lib().c2g_mesh_dev(self._h, self.MESH_TYPES[mesh], self.MESH_LEVELS[level],
                                     C.c_void_p(x.data_ptr()), C.c_void_p(w.data_ptr()), None))
        return x.cpu().numpy(), w.cpu().numpy()

    def molcalc(self, quantities=("rho",), mesh="franchini", level="good", prec="fp64") -> dict:
        """Mesh integrals (c2g_molcalc): {quantity: integral} plus npoints
        and the wall times."""
        q = _i32([self.MOLCALC[k] for k in quantities])
        out = np.zeros(len(q))
        st = L.MeshStats()
        L.check(L.lib().c2g_molcalc(self._h, self.MESH_TYPES[mesh], self.MESH_LEVELS[level], _prec(prec),
                                    len(q), L.ptr(q), L.ptr(out), C.byref(st)))
        r = {k: float(v) for k, v in zip(quantities, out)}
        r.update(npoints=st.npoints, ms_mesh=st.ms_mesh, ms_total=st.ms_total)
        return r

    def cp_graph(self, cp_xyz, cp_typ) -> dict:
        """makegraph over a CP list (c2g_cp_graph): ipath (n,2) 1-based
        terminator indices (0 none, -1 outside), brdist (n,2), brpathlen
        (n,2), brang (n,), brvec (n,3), ier (n,2), nstep (n,2), stats."""
        x = _f64(cp_xyz).reshape(-1, 3)
        t = _i32(cp_typ)
        n = t.shape[0]
        o = dict(ipath=np.zeros((n, 2), np.int32), brdist=np.zeros((n, 2)), brpathlen=np.zeros((n, 2)),
                 brang=np.zeros(n), brvec=np.zeros((n, 3)), ier=np.zeros((n, 2), np.int32),
                 nstep=np.zeros((n, 2), np.int32))
        st = L.GraphStats()
        L.check(L.lib().c2g_cp_graph(self._h, n, L.ptr(x), L.ptr(t), L.ptr(o["ipath"]), L.ptr(o["brdist"]),
                                     L.ptr(o["brpathlen"]), L.ptr(o["brang"]), L.ptr(o["brvec"]),
                                     L.ptr(o["ier"]), L.ptr(o["nstep"]), C.byref(st)))
        o["stats"] = dict(npath=st.npath, nbatch=st.nbatch, nevals=st.nevals, ms=st.ms_total)
        return o

    def basin_integrals(self, cp_xyz=None, cp_typ=None, meth: str = "lebedev", n: int = 110, nphi: int = 0,
                        cpid: int = 0, iasprec: float = 1e-5) -> dict:
        """Atomic-basin integrals by bisection (c2g_basin_integrals; critic2's
        INTEGRALS LEBEDEV n / GAULEG n nphi [CP cpid]).  The CP list is
        c2g_autocritic's (nuclei first); None for the nuclei alone.  Returns
        att_cp (natt,), props (natt, 2: Pop, Lap), iaserr (natt, 2),
        rays (nray, 3), rsurf (natt, nray), rbeta_int (natt,), stats."""
        if cp_xyz is None:
            x, t, ncp = None, None, 0
        else:
            x, t = _f64(cp_xyz).reshape(-1, 3), _i32(cp_typ)
            ncp = t.shape[0]
        m = {"lebedev": 0, "gauleg": 1}[meth]
        natt, nray = C.c_int(0), C.c_int(0)
        L.check(L.lib().c2g_basin_size(self._h, ncp, L.ptr(t) if t is not None else None, m, int(n), int(nphi),
                                       int(cpid), C.byref(natt), C.byref(nray)))
        na, nr = natt.value, nray.value
        o = dict(att_cp=np.zeros(na, np.int32), props=np.zeros((na, 2)), iaserr=np.zeros((na, 2)),
                 rays=np.zeros((nr, 3)), rsurf=np.zeros((na, nr)), rbeta_int=np.zeros(na))
        st = L.BasinStats()
        L.check(L.lib().c2g_basin_integrals(
            self._h, ncp, L.ptr(x) if x is not None else None, L.ptr(t) if t is not None else None, m, int(n),
            int(nphi), int(cpid), float(iasprec), L.ptr(o["att_cp"]), L.ptr(o["props"]), L.ptr(o["iaserr"]),
            L.ptr(o["rays"]), L.ptr(o["rsurf"]), L.ptr(o["rbeta_int"]), C.byref(st)))
        o["stats"] = dict(natt=st.natt, nray=st.nray, npath=st.npath, nbatch=st.nbatch, nevals=st.nevals,
                          nwarn=st.nwarn, nrestart=st.nrestart, ms=st.ms_total)
        return o

    def sphere_integrals(self, cp_xyz=None, cp_typ=None, meth: str = "gauleg", n: int = 20, nphi: int = 20,
                         cpid: int = 0, nr: int = 100, r0: float = 1e-3, rend: float = -1.0) -> dict:
        """Pop and Lap inside spheres around the attractors
        (c2g_sphere_integrals; critic2's SPHEREINTEGRALS): att_cp (natt,),
        radii (natt, nr), props (natt, nr, 2)."""
        if cp_xyz is None:
            x, t, ncp = None, None, 0
        else:
            x, t = _f64(cp_xyz).reshape(-1, 3), _i32(cp_typ)
            ncp = t.shape[0]
        m = {"lebedev": 0, "gauleg": 1}[meth]
        natt, nray = C.c_int(0), C.c_int(0)
        L.check(L.lib().c2g_basin_size(self._h, ncp, L.ptr(t), m, int(n), int(nphi), int(cpid), C.byref(natt),
                                       C.byref(nray)))
        na = natt.value
        o = dict(att_cp=np.zeros(na, np.int32), radii=np.zeros((na, nr)), props=np.zeros((na, nr, 2)))
        L.check(L.lib().c2g_sphere_integrals(self._h, ncp, L.ptr(x), L.ptr(t), m, int(n), int(nphi), int(cpid),
                                             int(nr), float(r0), float(rend), L.ptr(o["att_cp"]), L.ptr(o["radii"]),
                                             L.ptr(o["props"])))
        return o

    def autocritic(self, seeds: Optional[np.ndarray] = None, prec="fp64") -> dict:
        s = None if seeds is None else _f64(seeds).reshape(-1, 3)
        ns = 0 if s is None else s.shape[0]
        maxcp = self.natom + (ns if s is not None else max(1, len(self.pair_seeds()))) + 1
        xyz, typ, f = np.zeros((maxcp, 3)), np.zeros(maxcp, np.int32), np.zeros(maxcp)
        rep = L.CpReport()
        L.check(L.lib().c2g_autocritic(self._h, ns, L.ptr(s), _prec(prec), maxcp, L.ptr(xyz),
                                       L.ptr(typ), L.ptr(f), C.byref(rep)))
        n = rep.ncp
        return dict(xyz=xyz[:n], typ=typ[:n], f=f[:n], counts=np.array(rep.count[:]),
                    ph=rep.poincare_hopf, nseed=rep.nseed, nconverged=rep.nconverged,
                    ms=rep.ms_total)


def nci_chk_write(path: str, x0, xmat, nstep, crho, cgrad) -> None:
    """critic2's NCI checkpoint <root>.chk_nci (c2g_nci_chk_write): grid and
    the crho, cgrad cubes as (n1, n2, n3) arrays (k fastest in memory)."""
    ns = _i32(nstep)
    n = int(np.prod(ns))
    c, g = _f64(crho).reshape(-1), _f64(cgrad).reshape(-1)
    if c.size != n or g.size != n:
        raise ValueError("crho and cgrad must hold nstep(1)*nstep(2)*nstep(3) values")
    xm = _f64(np.asarray(xmat, np.float64).T.reshape(-1))
    L.check(L.lib().c2g_nci_chk_write(path.encode(), _f64(x0), xm, ns, c, g))


def nci_chk_read(path: str, x0, xmat, nstep):
    """Loads a checkpoint that matches the grid (c2g_nci_chk_read): returns
    (crho, cgrad) as (n1, n2, n3) arrays, or None when the file is missing
    or belongs to another grid (critic2 then recomputes)."""
    ns = _i32(nstep)
    shape = tuple(int(v) for v in ns)
    crho, cgrad = np.zeros(shape), np.zeros(shape)
    found = C.c_int(0)
    xm = _f64(np.asarray(xmat, np.float64).T.reshape(-1))
    L.check(L.lib().c2g_nci_chk_read(path.encode(), _f64(x0), xm, ns, crho.reshape(-1), cgrad.reshape(-1),
                                     C.byref(found)))
    return (crho, cgrad) if found.value else None
