"""Learned critical-point seeds for the AUTO search.

critic2's AUTO seeds Newton from geometric guesses: for molecules, five
points on every pair of atoms closer than 15 bohr (src/autocp@proc.f90:
423-437), which for 100 atoms is tens of thousands of Newton runs.  Here a
small 3D convolutional network reads a coarse grid of the density and
proposes a few seeds per critical point; the seeds go through the unchanged
Newton + addcp stages (`Wavefunction.autocritic(seeds)`), so every CP it
reports is confirmed by exact-field (FP64-finished) Newton convergence and
addcp's gradient check.  The result is accepted if the CP list satisfies
the Poincare-Hopf sum n - b + r - c = 1; otherwise the search is repeated
with a denser seed set and accepted if that satisfies the sum or finds no
new CP outside the nuclear cores; if both fail, critic2's plain pair seeds
are the fallback.

Pieces (all GPU work goes through the library's kernels; torch only holds
device memory and streams):
  coarse_grid / features  the S^3 grid (spacing h, centred on the molecule)
                          evaluated by the NCI kernel (c2g_nciplot_dev),
                          turned into 4 input channels (c2g_cs_features);
  SeedNet                 5 convolutions 4-16-32-32-32-32 (3^3, ReLU) and a
                          1^3 head to 8 channels (4 CP-type heat-map logits,
                          3 sub-voxel offsets); forward, backward and Adam
                          are the library's c2g_cs_* kernels; weights are
                          stored and run as BF16 values;
  cp_labels               training targets from a plain AUTO CP list;
  propose / learned_autocritic  seeds and the confirmed search with the
                          Poincare-Hopf check and fallback;
  train (python -m critic2_gb300.cpseed train)  data generation with plain
                          AUTO on seeded molecules and training on the GPU.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import sys
import time
from dataclasses import dataclass
from typing import List, Optional

import numpy as np

from . import _lib as L
from . import synth

HERE = os.path.dirname(os.path.abspath(__file__))
WEIGHTS = os.path.join(HERE, "cpseed_weights.npz")

# (cin, cout, ksize, relu)
LAYERS = ((4, 16, 3, True), (16, 32, 3, True), (32, 32, 3, True), (32, 32, 3, True), (32, 32, 3, True),
          (32, 8, 1, False))
TYPE_OF_SIGNATURE = {-3: 0, -1: 1, 1: 2, 3: 3}  # non-nuclear maximum, bond, ring, cage
S_DEFAULT, H_DEFAULT = 64, 0.45


def _torch():
    import torch
    return torch


def _vp(t) -> C.c_void_p:
    return C.c_void_p(t.data_ptr())


def bf16_round(a: np.ndarray) -> np.ndarray:
    """Rounds FP32 values to the nearest BF16 value (ties to even)."""
    u = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


# ------------------------------------------------------------------ grid
def coarse_grid(atom_xyz: np.ndarray, S: int = S_DEFAULT, h: float = H_DEFAULT):
    """S^3 grid of spacing h centred on the molecule's bounding box: returns
    x0 (voxel (0,0,0)), xmat (diag h) and nstep."""
    c = 0.5 * (atom_xyz.min(0) + atom_xyz.max(0))
    x0 = c - 0.5 * h * (S - 1)
    return x0.astype(np.float64), np.diag([h, h, h]).astype(np.float64), np.array([S, S, S], np.int32)


def features(wfn, S: int = S_DEFAULT, h: float = H_DEFAULT, prec: str = "tf32x3", out=None, stream=0):
    """Network input for one molecule, on the GPU: the NCI kernel on the
    coarse grid, then the feature kernel.  Returns (x [S^3*4] float32, x0)."""
    torch = _torch()
    x0, xm, ns = coarse_grid(_atoms(wfn), S, h)
    n = S ** 3
    crho = torch.empty(n, dtype=torch.float64, device="cuda")
    cgrad = torch.empty(n, dtype=torch.float64, device="cuda")
    wfn.nciplot_dev(x0, xm, ns, prec, crho.data_ptr(), cgrad.data_ptr(), stream)
    x = out if out is not None else torch.empty(n * 4, dtype=torch.float32, device="cuda")
    L.check(L.lib().c2g_cs_features(_vp(crho), _vp(cgrad), n, _vp(x), C.c_void_p(stream)))
    return x, x0


def _atoms(wfn) -> np.ndarray:
    a = getattr(wfn, "atom_xyz", None)
    if a is None:
        raise ValueError("the wavefunction needs its atom coordinates (Wavefunction(mol) keeps them)")
    return a


def cp_labels(xyz: np.ndarray, typ: np.ndarray, atom_xyz: np.ndarray, x0: np.ndarray, h: float,
              S: int, core: float = 0.5) -> np.ndarray:
    """Training targets from a CP list: rows (fi, fj, fk, type) for every CP
    inside the grid and outside the nuclear cores (within `core` bohr of a
    nucleus: the nuclei themselves, which AUTO adds on its own, and the
    rounding-dependent core CPs), in fractional voxel coordinates."""
    rows = []
    for x, t in zip(np.asarray(xyz).reshape(-1, 3), np.asarray(typ)):
        t = int(t)
        if t not in TYPE_OF_SIGNATURE:
            continue
        if np.min(np.linalg.norm(atom_xyz - x, axis=1)) < core:
            continue
        f = (x - x0) / h
        if np.all(f >= 0) and np.all(f <= S - 1):
            rows.append((f[0], f[1], f[2], TYPE_OF_SIGNATURE[t]))
    return np.array(rows, np.float32).reshape(-1, 4)


# --------------------------------------------------------------- network
class SeedNet:
    """The proposer network on the GPU.  `params` and `grad` are flat FP32
    device buffers; layer l's weights w[tap][cin][cout] and bias[cout]
    are views into them."""

    def __init__(self, seed: int = 0, params: Optional[np.ndarray] = None):
        torch = _torch()
        self.sizes = []
        for cin, cout, k, _ in LAYERS:
            self.sizes += [k ** 3 * cin * cout, cout]
        self.n = int(sum(self.sizes))
        if params is None:
            rng = np.random.default_rng(seed)
            parts = []
            for (cin, cout, k, relu) in LAYERS:
                std = np.sqrt(2.0 / (k ** 3 * cin)) if relu else np.sqrt(1.0 / (k ** 3 * cin))
                parts.append(rng.standard_normal(k ** 3 * cin * cout) * std)
                b = np.zeros(cout)
                if not relu:
                    b[:4] = -4.0  # heat maps start near p = 0.02
                parts.append(b)
            params = np.concatenate(parts)
        assert params.size == self.n
        self.params = torch.tensor(np.asarray(params, np.float32), device="cuda")
        self.grad = torch.zeros_like(self.params)
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.t = 0
        self._acts = None

    def _views(self, buf):
        out, o = [], 0
        for i in range(0, len(self.sizes), 2):
            w = buf[o:o + self.sizes[i]]
            o += self.sizes[i]
            b = buf[o:o + self.sizes[i + 1]]
            o += self.sizes[i + 1]
            out.append((w, b))
        return out

    def forward(self, x, B: int, S: int, keep: bool = False, stream: int = 0):
        """x: [B*S^3*4] float32 on the GPU -> logits [B*S^3*8]."""
        torch = _torch()
        lib = L.lib()
        n = B * S ** 3
        acts = [x]
        cur = x
        for (cin, cout, k, relu), (w, b) in zip(LAYERS, self._views(self.params)):
            y = torch.empty(n * cout, dtype=torch.float32, device="cuda")
            L.check(lib.c2g_cs_conv3d(_vp(cur), B, S, S, S, cin, _vp(w), _vp(b), cout, k, int(relu), _vp(y),
                                      C.c_void_p(stream)))
            acts.append(y)
            cur = y
        self._acts = (acts, B, S) if keep else None
        return cur

    def backward(self, dlogits, stream: int = 0):
        """Accumulates the parameter gradients of the last kept forward."""
        torch = _torch()
        lib = L.lib()
        acts, B, S = self._acts
        n = B * S ** 3
        gviews = self._views(self.grad)
        pviews = self._views(self.params)
        dy = dlogits
        for li in range(len(LAYERS) - 1, -1, -1):
            cin, cout, k, _ = LAYERS[li]
            gw, gb = gviews[li]
            L.check(lib.c2g_cs_conv3d_bwd_weight(_vp(acts[li]), _vp(dy), B, S, S, S, cin, cout, k, _vp(gw),
                                                 _vp(gb), C.c_void_p(stream)))
            if li > 0:
                dx = torch.empty(n * cin, dtype=torch.float32, device="cuda")
                # acts[li] is the ReLU output of layer li-1: its mask
                L.check(lib.c2g_cs_conv3d_bwd_data(_vp(dy), B, S, S, S, cout, _vp(pviews[li][0]), cin, k,
                                                   _vp(acts[li]), _vp(dx), C.c_void_p(stream)))
                dy = dx

    def adam(self, lr: float, b1=0.9, b2=0.999, eps=1e-8, stream: int = 0):
        self.t += 1
        L.check(L.lib().c2g_cs_adam(_vp(self.params), _vp(self.grad), _vp(self.m), _vp(self.v), self.n, lr, b1, b2,
                                    eps, self.t, C.c_void_p(stream)))

    def rounded(self) -> "SeedNet":
        """The network with its weights rounded to BF16 values (as stored)."""
        return SeedNet(params=bf16_round(self.params.cpu().numpy()))

    def save(self, path: str, meta: Optional[dict] = None):
        p = self.params.cpu().numpy().astype(np.float32)
        bits = (bf16_round(p).view(np.uint32) >> 16).astype(np.uint16)
        np.savez_compressed(path, bf16=bits, layers=np.array(LAYERS, np.int32),
                            meta=json.dumps(meta or {}))

    @classmethod
    def load(cls, path: str = WEIGHTS) -> "SeedNet":
        z = np.load(path)
        if not np.array_equal(z["layers"], np.array(LAYERS, np.int32)):
            raise ValueError("weights file does not match the network's layers")
        p = (z["bf16"].astype(np.uint32) << 16).view(np.float32)
        net = cls(params=p)
        net.meta = json.loads(str(z["meta"]))
        return net


def loss_and_grad(net: SeedNet, logits, tgt, nvox: int, npos: int, pos_w: float, off_w: float, stream=0):
    torch = _torch()
    dl = torch.empty_like(logits)
    acc = torch.zeros(1, dtype=torch.float64, device="cuda")
    L.check(L.lib().c2g_cs_loss(_vp(logits), _vp(tgt), nvox, npos, pos_w, off_w, _vp(dl), _vp(acc),
                                C.c_void_p(stream)))
    return dl, acc


def targets(cps: np.ndarray, B: int, S: int, stream=0):
    """Dense targets [B*S^3*8] on the GPU from rows (sample, fi, fj, fk, type)."""
    torch = _torch()
    tgt = torch.zeros(B * S ** 3 * 8, dtype=torch.float32, device="cuda")
    if len(cps):
        d = torch.tensor(np.ascontiguousarray(cps, np.float32).reshape(-1), device="cuda")
        L.check(L.lib().c2g_cs_targets(_vp(d), len(cps), S, _vp(tgt), C.c_void_p(stream)))
    return tgt


# ------------------------------------------------------------- proposing
CORE_RADIUS = 0.5  # bohr


def core_mask(xyz: np.ndarray, atom_xyz: np.ndarray, r: float = CORE_RADIUS) -> np.ndarray:
    """CPs within r of a nucleus.  In these cores the density reaches 10^2-10^3
    and the FP64 rounding of |grad rho| is of the order of AUTO's 1e-12
    convergence threshold, so whether Newton converges there depends on
    rounding (two FP64 codes with different summation orders find different
    core CPs)."""
    xyz = np.asarray(xyz).reshape(-1, 3)
    if len(xyz) == 0:
        return np.zeros(0, bool)
    d = np.linalg.norm(xyz[:, None, :] - atom_xyz[None, :, :], axis=2).min(1)
    return d < r


def proposer_logits(wfn, net: SeedNet, S: int = S_DEFAULT, h: float = H_DEFAULT, prec: str = "tf32x3"):
    x, x0 = features(wfn, S, h, prec)
    return net.forward(x, 1, S), x0


def seeds_from_logits(lg, x0, S: int = S_DEFAULT, h: float = H_DEFAULT, thresh: float = 0.3,
                      mode: int = 2, cap: int = 1 << 17) -> np.ndarray:
    """Seeds (n,3) from the network output, in voxel order (mode: see
    c2g_cs_seeds; 2 = per-type maxima of the heat maps)."""
    torch = _torch()
    seeds = torch.empty(cap * 3, dtype=torch.float64, device="cuda")
    vox = torch.empty(cap, dtype=torch.int32, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    tl = float(np.log(thresh / (1.0 - thresh)))
    L.check(L.lib().c2g_cs_seeds(_vp(lg), S, np.ascontiguousarray(x0, np.float64), h, tl, int(mode), cap,
                                 _vp(seeds), _vp(vox), _vp(cnt), None))
    n = min(int(cnt.item()), cap)
    s = seeds[: 3 * n].cpu().numpy().reshape(n, 3)
    v = vox[:n].cpu().numpy()
    return s[np.argsort(v, kind="stable")]


def cluster_seeds(seeds: np.ndarray, cell: float = 0.2) -> np.ndarray:
    """Keeps the first seed (in the given order) of every cubic cell of edge
    `cell` bohr: voxels around one CP predict nearly the same position, so
    this leaves about one seed per predicted CP."""
    if len(seeds) == 0:
        return seeds
    key = np.floor(seeds / cell).astype(np.int64)
    _, first = np.unique(key, axis=0, return_index=True)
    return seeds[np.sort(first)]


def grid_seeds(wfn, S: int = S_DEFAULT, h: float = H_DEFAULT, prec: str = "tf32x3") -> np.ndarray:
    """Non-learned seeds: coarse-grid voxels where the reduced density
    gradient s (zero at every CP) is a minimum over the 26 neighbours."""
    torch = _torch()
    x0, xm, ns = coarse_grid(_atoms(wfn), S, h)
    crho = torch.empty(S ** 3, dtype=torch.float64, device="cuda")
    cgrad = torch.empty(S ** 3, dtype=torch.float64, device="cuda")
    wfn.nciplot_dev(x0, xm, ns, prec, crho.data_ptr(), cgrad.data_ptr(), 0)
    g = cgrad.cpu().numpy().reshape(S, S, S)
    pad = np.pad(g, 1, constant_values=np.inf)
    m = np.ones_like(g, bool)
    for di in (-1, 0, 1):
        for dj in (-1, 0, 1):
            for dk in (-1, 0, 1):
                if (di, dj, dk) != (0, 0, 0):
                    m &= g <= pad[1 + di:1 + di + S, 1 + dj:1 + dj + S, 1 + dk:1 + dk + S]
    idx = np.argwhere(m)
    return x0 + h * idx.astype(np.float64)


def propose(wfn, net: SeedNet, S: int = S_DEFAULT, h: float = H_DEFAULT, prec: str = "tf32x3",
            thresh: float = 0.3, mode: int = 2) -> np.ndarray:
    lg, x0 = proposer_logits(wfn, net, S, h, prec)
    return seeds_from_logits(lg, x0, S, h, thresh, mode)


def learned_autocritic(wfn, net: SeedNet, prec: str = "fp64", S: int = S_DEFAULT, h: float = H_DEFAULT,
                       thresh=(0.2, 0.05), cell: float = 0.3, feat_prec: str = "tf32x3") -> dict:
    """AUTO with learned seeds, confirmed and checked.

    Seeds: every voxel whose heat map exceeds thresh[0], moved by its
    predicted offset, clustered to one seed per `cell`-bohr cell (on cp100
    with the FP64 search and stall exit 30, (0.2, 0.3 bohr) gives 4,010
    seeds and 97.8% recall of the pair-seed CPs at 3.4x less wall time,
    against 4,625 seeds, 97.5% and 3.1x for (0.3, 0.2 bohr)).  Newton +
    addcp confirm every CP with the exact field.
    Check: accepted if the Poincare-Hopf sum n - b + r - c is 1; otherwise
    the seeds added by lowering the threshold to thresh[1] (those not in an
    already used cell) run a second search, and the CP list is accepted if
    that finds no CP outside the nuclear cores that the first one missed
    (stable under densification); else critic2's plain pair seeds are the
    fallback.  Returns the autocritic dict of the accepted list plus `stage`
    ('learned', 'learned+dense' or 'fallback'), `reason`, `seeds_used`,
    `tries` and `ms` (wall time of the whole search, features and network
    included)."""
    torch = _torch()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    lg, x0 = proposer_logits(wfn, net, S, h, feat_prec)
    sa = cluster_seeds(seeds_from_logits(lg, x0, S, h, thresh[0], 0), cell)
    tries, used = [], len(sa)
    ra = wfn.autocritic(sa, prec) if len(sa) else None
    tries.append({"seeds": len(sa), "ph": None if ra is None else int(ra["ph"])})
    torch.cuda.synchronize()
    proposal = {"xyz": ra["xyz"] if ra is not None else np.zeros((0, 3)),
                "typ": ra["typ"] if ra is not None else np.zeros(0, np.int32),
                "ph": None if ra is None else int(ra["ph"]), "seeds": len(sa),
                "ms": 1e3 * (time.perf_counter() - t0)}
    res = stage = None
    reason = ""
    if ra is not None and ra["ph"] == 1:
        res, stage, reason = ra, "learned", "poincare-hopf"
    elif ra is not None:
        sb = cluster_seeds(seeds_from_logits(lg, x0, S, h, thresh[1], 0), cell)
        used_cells = {tuple(c) for c in np.floor(sa / cell).astype(np.int64)}
        keep = np.array([tuple(c) not in used_cells for c in np.floor(sb / cell).astype(np.int64)], bool)
        sb = sb[keep] if len(sb) else sb
        used += len(sb)
        rb = wfn.autocritic(sb, prec) if len(sb) else None
        tries.append({"seeds": len(sb), "ph": None if rb is None else int(rb["ph"])})
        new = 0
        if rb is not None:
            outer = ~core_mask(rb["xyz"], _atoms(wfn))
            sub = {"xyz": rb["xyz"][outer], "typ": rb["typ"][outer]}
            new = int((~match_cps(sub, ra, tol=1e-2)).sum())
        tries[-1]["new_cps"] = new
        if new == 0:
            res, stage, reason = ra, "learned", "stable under densification"
    if res is None:
        res = wfn.autocritic(None, prec)
        used += int(res["nseed"])
        stage, reason = "fallback", "check failed"
    torch.cuda.synchronize()
    res["ms"] = 1e3 * (time.perf_counter() - t0)
    res["stage"] = stage
    res["reason"] = reason
    res["seeds_used"] = used
    res["tries"] = tries
    res["proposal"] = proposal
    return res


def match_cps(ref: dict, got: dict, tol: float = 1e-3) -> np.ndarray:
    """For each CP of `ref`, whether `got` has a CP of the same type within
    tol bohr."""
    found = np.zeros(len(ref["xyz"]), bool)
    if len(got["xyz"]) == 0:
        return found
    for j, (x, t) in enumerate(zip(ref["xyz"], ref["typ"])):
        d = np.linalg.norm(got["xyz"] - x, axis=1)
        i = int(np.argmin(d))
        found[j] = d[i] <= tol and got["typ"][i] == t
    return found


def compare(ref: dict, got: dict, atom_xyz: np.ndarray) -> dict:
    """Recall of the plain search's CPs, over all of them and over those
    outside the nuclear cores."""
    m = match_cps(ref, got)
    outer = ~core_mask(ref["xyz"], atom_xyz)
    return {"recall": float(m.mean()) if len(m) else 1.0,
            "recall_outside_cores": float(m[outer].mean()) if outer.any() else 1.0,
            "ncp": int(len(m)), "ncp_outside_cores": int(outer.sum())}


# -------------------------------------------------------------- training
@dataclass
class Sample:
    x: object           # features on the GPU, [S^3*4]
    labels: np.ndarray  # (n, 4) fi, fj, fk, type
    natom: int
    ncp: int
    ms_auto: float


def make_sample(mol, S: int, h: float, prec: str, label_prec: str = "fp64") -> Sample:
    """Features and targets of one training molecule.  The targets are the
    CPs of a non-learned AUTO seeded with critic2's pair seeds plus the
    coarse-grid minima of s (grid_seeds): on these random-coefficient
    densities pair seeding alone misses many CPs, and targets that call a
    real CP "none" would teach the network to suppress it."""
    from .wfn import Wavefunction
    w = Wavefunction(mol)
    try:
        x, x0 = features(w, S, h, prec)
        seeds = np.concatenate([w.pair_seeds(), grid_seeds(w, S, h, prec)])
        res = w.autocritic(seeds, label_prec)
        lab = cp_labels(res["xyz"], res["typ"], mol.atom_xyz, x0, h, S)
        return Sample(x, lab, mol.natom, len(res["xyz"]), float(res["ms"]))
    finally:
        w.close()


def train(samples: List[Sample], epochs: int, batch: int, lr: float, S: int, seed: int = 0,
          pos_w: float = 10.0, off_w: float = 4.0, log=print) -> SeedNet:
    torch = _torch()
    net = SeedNet(seed=seed)
    rng = np.random.default_rng(seed)
    nstep = epochs * ((len(samples) + batch - 1) // batch)
    step = 0
    for ep in range(epochs):
        order = rng.permutation(len(samples))
        tot, nb = 0.0, 0
        t0 = time.perf_counter()
        for b0 in range(0, len(order), batch):
            idx = order[b0:b0 + batch]
            B = len(idx)
            x = torch.cat([samples[i].x for i in idx])
            rows = [np.concatenate([np.full((len(samples[i].labels), 1), bi, np.float32), samples[i].labels], 1)
                    for bi, i in enumerate(idx)]
            cps = np.concatenate(rows) if rows else np.zeros((0, 5), np.float32)
            tgt = targets(cps, B, S)
            lg = net.forward(x, B, S, keep=True)
            npos = int(len(cps) * 8)
            dl, acc = loss_and_grad(net, lg, tgt, B * S ** 3, npos, pos_w, off_w)
            net.grad.zero_()
            net.backward(dl)
            frac = step / max(1, nstep - 1)
            net.adam(lr * (0.5 * (1.0 + np.cos(np.pi * frac))) + 1e-5)
            step += 1
            tot += float(acc.item())
            nb += 1
        torch.cuda.synchronize()
        log(f"epoch {ep}: mean loss {tot / max(nb, 1):.5f}  ({time.perf_counter() - t0:.1f} s)")
    return net


def evaluate(mol, net: SeedNet, prec: str = "fp64", stall: int = 0) -> dict:
    """Plain AUTO (critic2's pair seeds) against the learned search on one
    molecule, with the non-learned coarse-grid seeds (minima of s) as the
    method without the network.  Times are wall times of whole searches.
    stall: C2G_PARAM_NEWTON_STALL for every search (0 = critic2's Newton)."""
    from .wfn import Wavefunction
    torch = _torch()
    w = Wavefunction(mol)
    w.set_newton_stall(stall)

    def timed(f, *a):
        torch.cuda.synchronize()
        t = time.perf_counter()
        r = f(*a)
        torch.cuda.synchronize()
        return r, 1e3 * (time.perf_counter() - t)

    try:
        learned_autocritic(w, net, prec)  # warm-up (first-use allocations)
        ref, ms_plain = timed(w.autocritic, None, prec)
        # critic2's own seed list (both ordered pairs: every seed twice)
        ref2, ms_plain2 = timed(w.autocritic, w.pair_seeds(), prec)
        got = learned_autocritic(w, net, prec)
        grid, ms_grid = timed(lambda: w.autocritic(grid_seeds(w), prec))
        prop = got["proposal"]
        out = dict(molecule=mol.name, natom=mol.natom, prec=prec, newton_stall=stall, plain_ph=int(ref["ph"]),
                   plain_seeds=int(ref["nseed"]), ms_plain=round(ms_plain, 1),
                   critic2_seed_list=dict(seeds=int(ref2["nseed"]), ms=round(ms_plain2, 1),
                                          same_cps=bool(len(ref2["xyz"]) == len(ref["xyz"]) and
                                                        np.allclose(ref2["xyz"], ref["xyz"], atol=1e-9))),
                   learned_ph=int(got["ph"]), stage=got["stage"], reason=got["reason"],
                   learned_seeds=int(got["seeds_used"]), ms_learned=round(got["ms"], 1),
                   speedup=round(ms_plain / got["ms"], 2), tries=got["tries"])
        out.update(compare(ref, got, mol.atom_xyz))
        c = compare(ref, prop, mol.atom_xyz)
        out["proposal"] = dict(seeds=prop["seeds"], ms=round(prop["ms"], 1), speedup=round(ms_plain / prop["ms"], 2),
                               speedup_vs_critic2_seed_list=round(ms_plain2 / prop["ms"], 2),
                               ph=prop["ph"], ncp_found=int(len(prop["xyz"])), recall=c["recall"],
                               recall_outside_cores=c["recall_outside_cores"])
        c = compare(ref, grid, mol.atom_xyz)
        out["grid_seeds"] = dict(seeds=int(grid["nseed"]), ms=round(ms_grid, 1), speedup=round(ms_plain / ms_grid, 2),
                                 ph=int(grid["ph"]), ncp_found=int(len(grid["xyz"])), recall=c["recall"],
                                 recall_outside_cores=c["recall_outside_cores"])
        return out
    finally:
        w.close()


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    sub = ap.add_subparsers(dest="cmd", required=True)
    t = sub.add_parser("train", help="generate training data with plain AUTO and train on the GPU")
    t.add_argument("--nmol", type=int, default=2000)
    t.add_argument("--epochs", type=int, default=12)
    t.add_argument("--batch", type=int, default=4)
    t.add_argument("--lr", type=float, default=2e-3)
    t.add_argument("--prec", default="tf32x3", help="precision of the coarse-grid features")
    t.add_argument("--label-prec", default="fp64", help="precision of the plain AUTO that labels")
    t.add_argument("--nval", type=int, default=8)
    t.add_argument("--out", default=WEIGHTS)
    t.add_argument("--log", default=None)
    a = ap.parse_args(argv)
    logf = open(a.log, "a") if a.log else None

    def log(msg):
        print(msg, flush=True)
        if logf:
            logf.write(msg + "\n")
            logf.flush()

    if a.cmd == "train":
        S, h = S_DEFAULT, H_DEFAULT
        t0 = time.perf_counter()
        samples = []
        for i in range(a.nmol):
            samples.append(make_sample(synth.training_molecule(i), S, h, a.prec, a.label_prec))
            if (i + 1) % max(1, a.nmol // 20) == 0:
                log(f"data: {i + 1}/{a.nmol} molecules, {time.perf_counter() - t0:.0f} s, "
                    f"last natom {samples[-1].natom} ncp {samples[-1].ncp} labels {len(samples[-1].labels)}")
        t_data = time.perf_counter() - t0
        t1 = time.perf_counter()
        net = train(samples, a.epochs, a.batch, a.lr, S, log=log)
        t_train = time.perf_counter() - t1
        meta = dict(nmol=a.nmol, epochs=a.epochs, batch=a.batch, lr=a.lr, prec=a.prec, label_prec=a.label_prec,
                    S=S, h=h, s_data=round(t_data, 1), s_train=round(t_train, 1))
        net.save(a.out, meta)
        # held-out check against plain AUTO (FP64 is deterministic; the split
        # mode finishes every Newton run in FP64)
        rn = net.rounded()
        stats = []
        cases = [(synth.training_molecule(10 ** 6 + j), "fp64") for j in range(a.nval)]
        cases += [(synth.make_molecule("cp100"), "fp64"), (synth.make_molecule("cp100"), "tf32x3")]
        for mol, prec in cases:
            st = evaluate(mol, rn, prec)
            st["prec"] = prec
            stats.append(st)
            log("val " + json.dumps(st))
        meta["val"] = stats
        net.save(a.out, meta)
        log("saved " + a.out + " " + json.dumps({k: v for k, v in meta.items() if k != "val"}))
    return 0


if __name__ == "__main__":
    sys.exit(main())
