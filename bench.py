#!/usr/bin/env python
"""Benchmark of the GB300 molecular-wavefunction evaluator on the NCI grid.

Metric: NCI grid points per second (rho, grad rho, Hessian, eigen-sign and
the reduced density gradient s at every point of the grid).  The headline
workload is the largest configuration: large500, 500 atoms, ~10000
primitives (s/p/d/f), 1000 occupied MOs, on a 320^3 grid at 0.1 bohr.  A
step is one full NCI grid pass.  `value` times the kernels with CUDA events
with the outputs in device memory; `e2e` times the public C-ABI call that
writes host arrays (device->host copy of both cubes inside the timed
region).  The split-precision path (TF32x3) is the measured one; its error
against the FP64 plain form (on i-planes spread over the grid) and the FP64
form's own throughput are reported beside it.  `workloads` repeats the
measurement on prec200 (200 atoms, f shells, 400 MOs, 256^3) and nci60 (60
atoms, 120 MOs, 200^3, FP64 comparison on the whole grid).  `cp_search`
holds the metric's second part: the wall time of AUTO's critical-point
search on the 100-atom molecule with critic2's pair seeds and with the
learned seeds.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--prec MODE]
                  [--workload NAME] [--impl ours|reference]

--impl reference times the CPU restatement of critic2's OpenMP loop (the
reference's Fortran cannot be compiled on these machines) on all host
cores: each step evaluates a strided sub-grid of the workload's grid (a
sample spread over the whole box), and ms_per_step is the time that step
took.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from critic2_gb300 import synth  # noqa: E402

PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
HEADLINE = "large500"
EXTRA = ("prec200", "nci60")

# DRAM bytes (read + write) per grid point of the split evaluator's launch,
# from the one-pass ncu capture of the whole 320^3 large500 launch
# (profiles/k_tc_dram_large500_320cubed.md: 1.83 GB read + 1.76 GB written
# over 32,768,000 points).
TRAFFIC_PER_POINT = {("large500", "tf32x3", 320): (1.83e9 + 1.76e9) / 32768000}
BASIN_NLEB = 26  # angular rule of the basin-integral part


def lebedev_dirs(rule):
    """Ray directions rebuilt from (theta, phi) as critic2's lebedev_nodes
    does, and the weights times 4 pi."""
    th, ph = np.arccos(rule[:, 2]), np.arctan2(rule[:, 1], rule[:, 0])
    return np.c_[np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)], rule[:, 3] * 4 * np.pi

# Dense TF32 tensor rate of this GPU model measured with a cuBLAS TF32 GEMM
# (TFLOP/s), a cross-check of the peak used below (half the measured BF16
# dense rate: the tensor core's TF32 rate is half its BF16 rate).
TF32_CUBLAS_TFLOPS = 1006.0

# MMA columns the split kernel issues per active (32-point tile, K-stage)
# pair and 128-MO tile (M = 128, K = 8 TF32 or 16 BF16): the hi*hi products
# of the 10 components (320), the cross products of components 1-9 (2 x 288)
# and the value's two cross products (2 x 32).
ISSUED_COLUMNS_PER_STAGE = 320 + 2 * 288 + 2 * 32


def env_int(k, d):
    try:
        return int(os.environ.get(k, d))
    except ValueError:
        return d


def peaks():
    try:
        with open(PEAKS_FILE) as fh:
            p = json.load(fh)
        return p, "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def config_of(wl, mol):
    """The `config` object, identical in both arms."""
    return {"workload": f"{wl.name}: {mol.natom} atoms, {mol.npri} primitives, {mol.nmo} MOs, "
                        f"{wl.grid}^3 grid at {wl.step} bohr",
            "parallelism": "replicas (one grid per GPU)",
            "l2": "GPU arm: L2 flushed between timed steps (256 MB write); CPU arm: n/a"}


class Clocks:
    """nvidia-smi sampler running during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, dev):
        self.dev = dev
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(5)
            except Exception:
                self.p.kill()

    def summary(self):
        self.f.flush()
        self.f.seek(0)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.f.name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


class _NullCtx:
    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False


def sub_grid(x0, xm, ns, stride, k=0):
    """Strided sub-grid of the grid (every stride-th point per axis, from an
    offset that moves with k): real grid points spread over the whole box."""
    off = np.array([(5 * k + stride // 2) % stride, (3 * k + stride // 3) % stride,
                    (7 * k + stride // 4) % stride])
    off = np.minimum(off, np.asarray(ns) - 1)
    x0s = x0 + xm @ off
    nss = np.array([(int(n) - int(o) + stride - 1) // stride for n, o in zip(ns, off)], np.int32)
    return x0s, xm * stride, nss


def cpu_stride(o, mol, wl, seconds_target, threads):
    """Stride of a sub-grid that the oracle evaluates in about seconds_target
    (calibrated on a coarse sub-grid of about 400 points)."""
    x0, xm, ns = synth.nci_grid(mol, wl.grid, wl.step)
    ntot = int(np.prod(ns))
    s0 = max(1, int(round((ntot / 400.0) ** (1.0 / 3.0))))
    a, b, c = sub_grid(x0, xm, ns, s0)
    t = time.perf_counter()
    o.nciplot(a, b, c, nthreads=threads)
    rate = int(np.prod(c)) / max(time.perf_counter() - t, 1e-6)
    return max(1, int(math.floor((ntot / max(rate * seconds_target, 1.0)) ** (1.0 / 3.0))))


def cpu_run(o, mol, wl, stride, threads, k=0):
    """One oracle pass (C/OpenMP restatement of critic2's nciplot loop) over
    the strided sub-grid; returns (points, seconds, description)."""
    x0, xm, ns = synth.nci_grid(mol, wl.grid, wl.step)
    a, b, c = sub_grid(x0, xm, ns, stride, k)
    npts = int(np.prod(c))
    t = time.perf_counter()
    o.nciplot(a, b, c, nthreads=threads)
    dt = time.perf_counter() - t
    return npts, dt, (f"strided sub-grid of the {wl.name} grid (every {stride}-th point per axis, "
                      f"{c[0]}x{c[1]}x{c[2]} = {npts} points spread over the box)")


def run_reference(args, wl, mol):
    rank = env_int("RANK", 0)
    if rank != 0:
        return 0
    from oracle import oracle
    threads = os.cpu_count()
    o = oracle.Wfn(mol)
    stride = cpu_stride(o, mol, wl, args.ref_seconds, threads)
    ms_steps, pts, secs, sample = [], 0, 0.0, ""
    for s in range(args.warmup + args.steps):
        n, dt, sample = cpu_run(o, mol, wl, stride, threads, k=s)
        if s >= args.warmup:
            ms_steps.append(1e3 * dt)
            pts += n
            secs += dt
    value = pts / secs
    line = {"metric": "NCI grid points/s", "value": value, "unit": "points/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": float(np.mean(ms_steps)),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded generator, wfx convention)", "impl": "reference",
            "config": config_of(wl, mol),
            "cpu_baseline": {"value": value, "unit": "points/s", "cores": threads, "kind": "port",
                             "sample": "per step: " + sample + " (the offset moves with the step); C/OpenMP "
                                       "restatement of critic2's nciplot loop (the reference's Fortran cannot be "
                                       "built here); ms_per_step is the measured time of one such step"},
            "e2e": {"value": value, "unit": "points/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if not args.no_mesh:
        ow = oracle.Wfn(synth.make_molecule("nci60"))
        t0 = time.perf_counter()
        r = ow.molcalc(("rho",), "franchini", "good", nthreads=threads)
        line["molcalc"] = {"workload": "nci60", "mesh": "franchini, good", "quantity": "integral of rho",
                           "unit": "ms", "ms": 1e3 * (time.perf_counter() - t0), "integral": r["rho"],
                           "npoints": r["npoints"], "cores": threads, "kind": "port"}
    if not args.no_basin:
        # basin integrals by bisection on nci60 (the nuclei as attractors),
        # Lebedev 26, all host threads
        bmol = synth.make_molecule("nci60")
        ob = oracle.Wfn(bmol)
        u, wu = lebedev_dirs(oracle.lebedev_rule(BASIN_NLEB))
        us, ws = lebedev_dirs(oracle.lebedev_rule(170))
        t0 = time.perf_counter()
        r = ob.basin_integrals(bmol.atom_xyz, np.full(bmol.natom, -3, np.int32), u, wu, us, ws, nthreads=threads)
        line["basin"] = {"workload": f"nci60: INTEGRALS LEBEDEV {BASIN_NLEB}, nuclei", "unit": "ms",
                         "ms": 1e3 * (time.perf_counter() - t0), "natt": int(len(r["att_cp"])),
                         "nray": int(len(u)), "pop_sum": float(r["props"][:, 0].sum()), "cores": threads,
                         "kind": "port"}
    if not args.no_cp:
        # the metric's second part on the CPU: AUTO with critic2's pair seeds
        # on the 100-atom molecule, all host threads
        cmol = synth.make_molecule("cp100")
        oc = oracle.Wfn(cmol)
        t0 = time.perf_counter()
        r = oc.autocritic(nthreads=threads)
        ms_plain = 1e3 * (time.perf_counter() - t0)
        t0 = time.perf_counter()
        oc.makegraph(r["xyz"], r["typ"], nthreads=threads)
        ms_graph = 1e3 * (time.perf_counter() - t0)
        line["cp_search"] = {"workload": f"cp100: {cmol.natom} atoms, {cmol.npri} primitives, {cmol.nmo} MOs",
                             "unit": "ms", "ms_plain": ms_plain, "ms_graph": ms_graph,
                             "graph_paths": int(2 * (abs(r["typ"]) == 1).sum()),
                             "ncp": int(len(r["xyz"])), "ph": int(r["ph"]), "cores": threads, "kind": "port"}
    print(json.dumps(line), flush=True)
    return 0


def cp_search(args):
    """Second half of the metric: AUTO's CP search on the 100-atom molecule
    (cp100: 1996 primitives, 200 MOs), critic2's pair seeds against the
    learned seeds, wall time of the whole search through the public API."""
    from critic2_gb300 import cpseed
    if not os.path.exists(cpseed.WEIGHTS):
        return None
    mol = synth.make_molecule("cp100")
    net = cpseed.SeedNet.load()
    out = {"workload": f"cp100: {mol.natom} atoms, {mol.npri} primitives, {mol.nmo} MOs; "
                       f"proposer on a {cpseed.S_DEFAULT}^3 grid at {cpseed.H_DEFAULT} bohr",
           "unit": "ms", "higher_is_better": False}
    for mode in args.cp_modes.split(","):
        prec, stall = mode.split(":")
        st = cpseed.evaluate(mol, net, prec, int(stall))
        out[f"{prec}, newton_stall {stall}"] = {k: st[k] for k in (
            "ms_plain", "ms_learned", "speedup", "recall", "recall_outside_cores", "ncp", "ncp_outside_cores",
            "plain_ph", "learned_ph", "stage", "reason", "plain_seeds", "learned_seeds", "critic2_seed_list",
            "proposal", "grid_seeds")
            if k in st}
    # AUTO's graph stage (makegraph: two gradient paths per bond and ring
    # CP) on the FP64 pair-seed CP list, through c2g_cp_graph
    from critic2_gb300.wfn import Wavefunction
    w = Wavefunction(mol)
    cp = w.autocritic(prec="fp64")
    w.cp_graph(cp["xyz"], cp["typ"])  # warm-up
    t0 = time.perf_counter()
    g = w.cp_graph(cp["xyz"], cp["typ"])
    out["graph"] = {"ms": 1e3 * (time.perf_counter() - t0), "cps": int(len(cp["typ"])),
                    "paths": g["stats"]["npath"], "batches": g["stats"]["nbatch"],
                    "evaluations": g["stats"]["nevals"]}
    return out


def fp64_planes(npl, n1):
    """npl i-planes spread evenly over the grid (all of them when npl <= 0 or >= n1)."""
    if npl <= 0 or npl >= n1:
        return list(range(n1))
    return sorted({int(round((k + 0.5) * n1 / npl - 0.5)) for k in range(npl)})


def measure(torch, w, mol, wl, prec, args, dev, stream, flush, steps, warmup, nplanes, binned, world, clocks=None):
    """Times one workload: device-resident steps (CUDA events), the kernel
    split, end to end through c2g_nciplot, and the error against FP64 on
    nplanes i-planes spread over the grid (0: the whole grid)."""
    x0, xm, ns = synth.nci_grid(mol, wl.grid, wl.step)
    npts = int(np.prod(ns))
    crho = torch.empty(npts, dtype=torch.float64, device=dev)
    cgrad = torch.empty(npts, dtype=torch.float64, device=dev)
    sp = stream.cuda_stream

    def step(stats=False):
        return w.nciplot_dev(x0, xm, ns, prec, crho.data_ptr(), cgrad.data_ptr(), sp, stats=stats)

    # W warm-up steps, extended (untimed) to at least ~1.5 s of GPU work so
    # that the clocks have left their idle state before the timed region
    t_w = time.perf_counter()
    nw = 0
    while nw < warmup or (time.perf_counter() - t_w < 1.5 and nw < warmup + 20):
        step()
        torch.cuda.synchronize()
        nw += 1
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    with (clocks if clocks is not None else _NullCtx()):
        for a, b in evs:
            flush.zero_()
            a.record(stream)
            step()
            b.record(stream)
        torch.cuda.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in evs) / steps
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        t = torch.tensor([ms], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    st = step(stats=True)
    torch.cuda.synchronize()
    out = {"npts": npts, "ms": ms, "ms_kernel": float(st.ms_kernel), "ms_recheck": float(st.ms_recheck),
           "nrecheck": int(st.nrecheck), "stage_frac": float(st.stage_frac)}
    # end to end through the public call with host output arrays
    e2e_ms = []
    for _ in range(max(1, min(steps, 3))):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        w.nciplot(x0, xm, ns, prec)
        e2e_ms.append(1e3 * (time.perf_counter() - t0))
    out["e2e_ms"] = float(np.median(e2e_ms))
    if prec != "fp64" and not args.no_fp64:
        n1, plane = int(ns[0]), int(ns[1]) * int(ns[2])
        planes = fp64_planes(nplanes, n1)
        rho64 = torch.empty(len(planes) * plane, dtype=torch.float64, device=dev)
        s64 = torch.empty_like(rho64)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        if len(planes) == n1:
            w.nciplot_dev(x0, xm, ns, "fp64", rho64.data_ptr(), s64.data_ptr(), stream.cuda_stream)
        else:
            nsp = np.array([1, ns[1], ns[2]], np.int32)
            for k, i in enumerate(planes):
                w.nciplot_dev(x0 + i * xm[:, 0], xm, nsp, "fp64", rho64[k * plane:].data_ptr(),
                              s64[k * plane:].data_ptr(), stream.cuda_stream)
        b.record(stream)
        torch.cuda.synchronize()
        t64 = a.elapsed_time(b) * n1 / len(planes)  # per full grid
        sel = torch.cat([torch.arange(i * plane, (i + 1) * plane, device=dev) for i in planes])
        cr, cg = crho[sel], cgrad[sel]
        r64 = rho64.abs() / 100
        r = cr.abs() / 100
        rel = (r - r64).abs() / r64.clamp_min(1e-300)
        ds = (cg - s64).abs()
        flip = torch.sign(cr) != torch.sign(rho64)
        q = rel if rel.numel() <= (1 << 24) else rel[torch.randperm(rel.numel(), device=dev)[:1 << 24]]
        fp = {"value": npts / (t64 / 1e3), "unit": "points/s", "ms_per_step": t64,
              "speedup_split_vs_fp64": t64 / ms, "max_rel_drho": rel.max().item(),
              "p999_rel_drho": torch.quantile(q.float(), 0.999).item(),
              "mean_signed_rel_drho": ((r - r64) / r64.clamp_min(1e-300)).mean().item(),
              "max_abs_ds": ds.max().item(), "sign_flips": int(flip.sum().item()),
              "compared_points": int(len(planes) * plane),
              "sample": "whole grid" if len(planes) == n1 else
              f"{len(planes)} of {n1} i-planes spread over the grid (time scaled to the grid)"}
        if binned:
            lg = torch.floor(torch.log10(r64.clamp_min(1e-300)))
            bins = {}
            for d in range(-8, 4):
                m = lg == d
                n = int(m.sum().item())
                if n:
                    bins[f"1e{d}"] = {"points": n, "max_rel_drho": rel[m].max().item(),
                                      "max_abs_ds": ds[m].max().item(), "sign_flips": int(flip[m].sum().item())}
            fp["by_rho_decade"] = bins
        out["fp64_plain"] = fp
        del rho64, s64, sel
    del crho, cgrad
    return out


def roofline_of(res, mol, npri, prec, pk, pk_kind, wl):
    """Roofline of the evaluation kernel (k_tc): achieved = the MMA work it
    issued (per active (tile, K-stage) pair and MO tile) over its CUDA-event
    time, against the dense TF32 (or BF16) tensor rate."""
    npts = res["npts"]
    t = res["ms_kernel"] / 1e3
    dense = 20.0 * mol.nmo * npri * npts  # algorithmic, no cutoff credit
    kps = 16 if prec == "bf16x3" else 8
    nstage = (npri + kps - 1) // kps
    _, _, ns = synth.nci_grid(mol, wl.grid, wl.step)
    ntiles = int(ns[0]) * ((int(ns[1]) + 3) // 4) * ((int(ns[2]) + 7) // 8)
    nmt = -(-mol.nmo // 128)
    active = res["stage_frac"] * ntiles * nstage  # active (tile, stage) pairs
    issued = active * nmt * 2.0 * 128 * ISSUED_COLUMNS_PER_STAGE * kps
    peak = pk["bf16_tflops"] if prec == "bf16x3" else pk["bf16_tflops"] / 2.0
    ach = issued / t / 1e12
    trf = TRAFFIC_PER_POINT.get((wl.name, prec, wl.grid))
    return {"bound": "tensor", "achieved": ach, "peak": peak, "unit": "TFLOP/s", "frac": ach / peak,
            "traffic": None if trf is None else trf * npts,
            "note": (f"achieved = MMA work issued by the split kernel (M 128 x N {ISSUED_COLUMNS_PER_STAGE} x "
                     f"K {kps} per active (32-point tile, K-stage) pair and 128-MO tile: {active:.4g} pairs x "
                     f"{nmt} MO tiles) over its CUDA-event time; peak = "
                     + ("the measured BF16 dense rate" if prec == "bf16x3" else
                        "half the measured BF16 dense rate (TF32 runs at half the BF16 rate; a cuBLAS TF32 "
                        f"GEMM measured {TF32_CUBLAS_TFLOPS:.0f})") + f" ({pk_kind})"),
            "algorithmic": {"dense_tflops": dense / t / 1e12,
                            "effective_tflops": dense * res["stage_frac"] / t / 1e12,
                            "stage_frac": res["stage_frac"],
                            "note": "20*nmo*npri flops per point (critic2's 10 components x nmo x npri "
                                    "multiply-adds); dense counts the K-stages the cutoffs skip as work, "
                                    "effective scales by the fraction of K-stages the tiles compute"}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=HEADLINE)
    ap.add_argument("--prec", default="auto")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--grid", type=int, default=0, help="grid points per axis (default: the workload's)")
    ap.add_argument("--binned", action="store_true", help="FP64 comparison binned by rho decade")
    ap.add_argument("--no-cp", action="store_true", help="skip the CP-search part")
    ap.add_argument("--no-files", action="store_true", help="skip the cube/dat output part")
    ap.add_argument("--no-mesh", action="store_true", help="skip the molcalc mesh-integral part")
    ap.add_argument("--no-basin", action="store_true", help="skip the basin-integral part")
    ap.add_argument("--no-extra", action="store_true", help="skip the other workloads")
    ap.add_argument("--fp64-planes", type=int, default=-1,
                    help="FP64 comparison on this many i-planes spread over the grid (0: the whole grid; "
                         "default: 8 for grids of 256^3 and more, else the whole grid)")
    ap.add_argument("--ref-seconds", type=float, default=4.0, help="CPU seconds per reference-arm step")
    ap.add_argument("--cp-modes", default="fp64:0,fp64:30,tf32x3:30",
                    help="CP-search precision:stall pairs (stall 0 = critic2's Newton)")
    args = ap.parse_args()
    wl = synth.WORKLOADS[args.workload]
    if args.grid > 0:
        import dataclasses
        wl = dataclasses.replace(wl, grid=args.grid)
    mol = synth.make_molecule(args.workload)
    if args.impl == "reference":
        return run_reference(args, wl, mol)

    import torch
    import torch.distributed as dist
    from critic2_gb300 import _lib
    from critic2_gb300.wfn import Wavefunction

    world = env_int("WORLD_SIZE", 1)
    rank = env_int("RANK", 0)
    local = env_int("LOCAL_RANK", 0)
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)

    prec = args.prec
    if prec == "auto":
        prec = "tf32x3"
        try:
            Wavefunction(synth.make_molecule("nci12")).nciplot(np.zeros(3), np.eye(3) * 0.5, [2, 2, 2], prec)
        except _lib.C2GError:
            prec = "fp64"
    w = Wavefunction(mol)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)

    def planes_for(wl_):
        if args.fp64_planes >= 0:
            return args.fp64_planes
        return 8 if wl_.grid >= 256 else 0

    clk = Clocks(local)
    res = measure(torch, w, mol, wl, prec, args, dev, stream, flush, args.steps, args.warmup, planes_for(wl),
                  args.binned, world, clocks=clk)
    clocks = clk.summary()
    pk, pk_kind = peaks()
    ms, npts = res["ms"], res["npts"]
    line = {"metric": "NCI grid points/s", "value": world * npts / (ms / 1e3), "unit": "points/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": {"fp64": "f64", "tf32x3": "tf32x3 (fp32 accumulate)",
                      "bf16x3": "bf16x3 (fp32 accumulate)"}[prec],
            "data": "synthetic (seeded generator, wfx convention)",
            "config": config_of(wl, mol), "precision": prec, "clocks": clocks,
            "e2e": {"value": world * npts / (res["e2e_ms"] / 1e3), "unit": "points/s",
                    "h2d_bytes_per_step": 3 * 8 + 9 * 8 + 3 * 4, "d2h_bytes_per_step": 2 * 8 * npts},
            # per step: the split evaluator, the FP64 re-check pass (launched
            # even when its device-side list is empty) and the nucleus rule, or
            # the FP64 evaluator alone
            "gpu_launches": args.steps * (1 if prec == "fp64" else 3),
            "fp64_recheck_points": res["nrecheck"], "ms_kernel": res["ms_kernel"], "ms_recheck": res["ms_recheck"]}
    if prec != "fp64":
        line["roofline"] = roofline_of(res, mol, w.npri, prec, pk, pk_kind, wl)
    if "fp64_plain" in res:
        line["fp64_plain"] = res["fp64_plain"]
    if rank == 0 and not args.no_extra and args.workload == HEADLINE:
        extra = {}
        for name in EXTRA:
            wl2 = synth.WORKLOADS[name]
            mol2 = synth.make_molecule(name)
            w2 = Wavefunction(mol2)
            r2 = measure(torch, w2, mol2, wl2, prec, args, dev, stream, flush, 5, 3, planes_for(wl2),
                         args.binned or name == "nci60", 1)
            e = {"config": config_of(wl2, mol2), "value": r2["npts"] / (r2["ms"] / 1e3), "unit": "points/s",
                 "ms_per_step": r2["ms"], "e2e": {"value": r2["npts"] / (r2["e2e_ms"] / 1e3), "unit": "points/s"},
                 "ms_kernel": r2["ms_kernel"], "fp64_recheck_points": r2["nrecheck"]}
            if prec != "fp64":
                e["roofline"] = roofline_of(r2, mol2, w2.npri, prec, pk, pk_kind, wl2)
            if "fp64_plain" in r2:
                e["fp64_plain"] = r2["fp64_plain"]
            extra[name] = e
            del w2
        line["workloads"] = extra
    if rank == 0 and not args.no_files:
        # nciplot end to end into files (nci60): the cutoff pass and the
        # cube/dat text (critic2's output step), timed by parts
        mol3 = synth.make_molecule("nci60")
        wl3 = synth.WORKLOADS["nci60"]
        w3 = Wavefunction(mol3)
        x0, xm, ns = synth.nci_grid(mol3, wl3.grid, wl3.step)
        with tempfile.TemporaryDirectory() as d:
            root = os.path.join(d, "nci")
            _, parts = w3.nciplot_files(x0, xm, ns, prec, root)
            sizes = {k: os.path.getsize(root + k) for k in ("-dens.cube", "-grad.cube", ".dat")}
        line["nci_files"] = {"workload": "nci60", "ms_evaluation": parts[0], "ms_cutoff_pass": parts[1],
                             "ms_text": parts[2], "ms_write": parts[3], "bytes": sizes,
                             "note": "text formatted on the GPU (correctly rounded, near ties on the host)"}
    if rank == 0 and not args.no_mesh:
        # molcalc: the integral of rho over critic2's default molecular mesh
        # (Franchini, good) of nci60, mesh built and field evaluated on the GPU
        w3 = Wavefunction(synth.make_molecule("nci60"))
        mc = {"workload": "nci60", "mesh": "franchini, good", "quantity": "integral of rho", "unit": "ms"}
        for p_ in ("fp64", "tf32x3"):
            w3.molcalc(("rho",), "franchini", "good", p_)  # warm-up
            t0 = time.perf_counter()
            r = w3.molcalc(("rho",), "franchini", "good", p_)
            mc[p_] = {"ms": 1e3 * (time.perf_counter() - t0), "integral": r["rho"], "ms_mesh": r["ms_mesh"]}
            mc["npoints"] = r["npoints"]
        line["molcalc"] = mc
    if rank == 0 and not args.no_basin:
        # basin integrals by bisection (critic2's INTEGRALS LEBEDEV n) on
        # nci60, the nuclei as attractors: surfaces traced on the GPU
        w3 = Wavefunction(synth.make_molecule("nci60"))
        w3.basin_integrals(None, None, "lebedev", 6, cpid=1)  # warm-up
        t0 = time.perf_counter()
        r = w3.basin_integrals(None, None, "lebedev", BASIN_NLEB)
        st = r["stats"]
        line["basin"] = {"workload": f"nci60: INTEGRALS LEBEDEV {BASIN_NLEB}, nuclei", "unit": "ms",
                         "ms": 1e3 * (time.perf_counter() - t0), "natt": st["natt"], "nray": st["nray"],
                         "pop_sum": float(r["props"][:, 0].sum()), "npath": st["npath"], "nbatch": st["nbatch"],
                         "nevals": st["nevals"], "nrestart": st["nrestart"]}
    if rank == 0 and not args.no_cp:
        cps = cp_search(args)
        if cps:
            line["cp_search"] = cps
    if rank == 0 and world == 1 and not args.no_cpu:
        from oracle import oracle
        o = oracle.Wfn(mol)
        cores = os.cpu_count()
        stride = cpu_stride(o, mol, wl, 10.0, cores)
        n, dt, sample = cpu_run(o, mol, wl, stride, cores)
        line["cpu_baseline"] = {"value": n / dt, "unit": "points/s", "cores": cores, "kind": "port",
                                "sample": sample + f", {dt:.1f} s"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
