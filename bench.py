#!/usr/bin/env python
"""Benchmark of the GB300 molecular-wavefunction evaluator on the NCI grid.

Metric: NCI grid points per second (rho, grad rho, Hessian, eigen-sign and
the reduced density gradient s at every point of the grid), for the
60-atom / ~1200-primitive / 120-MO synthetic molecule on a 200^3 grid at
0.1 bohr.  A step is one full NCI grid pass.  `value` times the kernels
with CUDA events with the outputs in device memory; `e2e` times the public
C-ABI call that writes host arrays (device->host copy of both cubes inside
the timed region).  The split-precision path is the measured one; its
error against the FP64 plain form and the FP64 form's own throughput are
reported beside it.  `cp_search` holds the metric's second part: the wall
time of AUTO's critical-point search on the 100-atom molecule with critic2's
pair seeds and with the learned seeds (recall of the plain CP list,
Poincare-Hopf sums, seeds used), in FP64 and in TF32x3 with FP64 final
Newton steps, with critic2's Newton and with the optional stall exit
(C2G_PARAM_NEWTON_STALL = 30).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--prec MODE]
                  [--workload NAME] [--impl ours|reference]

--impl reference times the CPU restatement of critic2's OpenMP loop (the
reference's Fortran cannot be compiled on these machines) on all host
cores, on a bounded sample of the same grid.
"""
from __future__ import annotations

import argparse
import json
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

# DRAM bytes (read + write) per grid point of the split evaluator, from one
# ncu capture of k_tc on the nci60 molecule with a 64^3 grid (1.09 MB per
# 262,144 points; traffic grows with the points, the operands stay in L2).
TRAFFIC_PER_POINT = {("nci60", "tf32x3"): (1.087232e6 + 5.12e3) / 262144}

# Dense TF32 tensor rate of this GPU model, measured with a cuBLAS TF32 GEMM
# on the same GPUs (TFLOP/s); the driver's peaks file holds BF16 only.
TF32_MEASURED_TFLOPS = 1006.0


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


def cpu_sample(mol, wl, seconds_target=15.0, threads=None):
    """Oracle (C/OpenMP restatement of critic2's nciplot loop) on whole
    i-planes of the grid; returns points/s and the sample description."""
    from oracle import oracle
    threads = threads or os.cpu_count()
    o = oracle.Wfn(mol)
    x0, xm, ns = synth.nci_grid(mol, wl.grid, wl.step)
    n1 = int(ns[0])
    # calibrate with one plane, then take as many planes as fit the target
    i = n1 // 2
    t = time.perf_counter()
    o.nciplot(x0, xm, ns, i, i + 1, nthreads=threads)
    dt1 = time.perf_counter() - t
    nplanes = int(max(1, min(n1, seconds_target / max(dt1, 1e-6))))
    i0 = max(0, n1 // 2 - nplanes // 2)
    t = time.perf_counter()
    o.nciplot(x0, xm, ns, i0, i0 + nplanes, nthreads=threads)
    dt = time.perf_counter() - t
    npts = nplanes * int(ns[1]) * int(ns[2])
    return npts / dt, threads, f"{nplanes} of {n1} i-planes ({npts} points) of the {wl.name} grid"


def run_reference(args, wl, mol):
    rank = env_int("RANK", 0)
    if rank != 0:
        return 0
    vals = []
    sample = ""
    threads = os.cpu_count()
    for s in range(args.warmup + args.steps):
        v, threads, sample = cpu_sample(mol, wl, seconds_target=10.0, threads=threads)
        if s >= args.warmup:
            vals.append(v)
    value = float(np.median(vals))
    npts = wl.grid ** 3
    line = {"metric": "NCI grid points/s", "value": value, "unit": "points/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * npts / value,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": f"{wl.name}: {mol.natom} atoms, {mol.npri} primitives, "
                                   f"{mol.nmo} MOs, {wl.grid}^3 grid at {wl.step} bohr",
                       "l2": "n/a (CPU)"},
            "cpu_baseline": {"value": value, "unit": "points/s", "cores": threads, "kind": "port",
                             "sample": sample + " per step; C/OpenMP restatement of critic2's "
                                                "nciplot loop (reference Fortran unbuildable here)"},
            "e2e": {"value": value, "unit": "points/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    if not args.no_mesh:
        from oracle import oracle as _o
        ow = _o.Wfn(mol)
        t0 = time.perf_counter()
        r = ow.molcalc(("rho",), "franchini", "good", nthreads=threads)
        line["molcalc"] = {"mesh": "franchini, good", "quantity": "integral of rho", "unit": "ms",
                           "ms": 1e3 * (time.perf_counter() - t0), "integral": r["rho"], "npoints": r["npoints"],
                           "cores": threads, "kind": "port"}
    if not args.no_cp:
        # the metric's second part on the CPU: AUTO with critic2's pair seeds
        # on the 100-atom molecule, all host threads
        from oracle import oracle
        cmol = synth.make_molecule("cp100")
        o = oracle.Wfn(cmol)
        t0 = time.perf_counter()
        r = o.autocritic(nthreads=threads)
        ms_plain = 1e3 * (time.perf_counter() - t0)
        t0 = time.perf_counter()
        o.makegraph(r["xyz"], r["typ"], nthreads=threads)
        ms_graph = 1e3 * (time.perf_counter() - t0)
        line["cp_search"] = {"workload": f"cp100: {cmol.natom} atoms, {cmol.npri} primitives, {cmol.nmo} MOs",
                             "unit": "ms", "ms_plain": ms_plain, "ms_graph": ms_graph,
                             "graph_paths": int(2 * (abs(r["typ"]) == 1).sum()),
                             "ncp": int(len(r["xyz"])), "ph": int(r["ph"]), "cores": threads,
                             "kind": "port"}
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
        out[f"{prec}, newton_stall {stall}"] = {k: st[k] for k in ("ms_plain", "ms_learned", "speedup", "recall", "recall_outside_cores",
                                        "ncp", "ncp_outside_cores", "plain_ph", "learned_ph", "stage", "reason",
                                        "plain_seeds", "learned_seeds", "proposal", "grid_seeds")}
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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="nci60")
    ap.add_argument("--prec", default="auto")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--grid", type=int, default=0, help="grid points per axis (default: the workload's)")
    ap.add_argument("--binned", action="store_true", help="FP64 comparison binned by rho decade")
    ap.add_argument("--no-cp", action="store_true", help="skip the CP-search part")
    ap.add_argument("--no-files", action="store_true", help="skip the cube/dat output part")
    ap.add_argument("--no-mesh", action="store_true", help="skip the molcalc mesh-integral part")
    ap.add_argument("--fp64-planes", type=int, default=0, help="FP64 comparison on this many i-planes")
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
    x0, xm, ns = synth.nci_grid(mol, wl.grid, wl.step)
    npts = int(np.prod(ns))
    crho = torch.empty(npts, dtype=torch.float64, device=dev)
    cgrad = torch.empty(npts, dtype=torch.float64, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    sp = stream.cuda_stream

    def step(stats=False):
        return w.nciplot_dev(x0, xm, ns, prec, crho.data_ptr(), cgrad.data_ptr(), sp, stats=stats)

    # W warm-up steps, extended (untimed) to at least ~1.5 s of GPU work so
    # that the clocks have left their idle state before the timed region
    t_w = time.perf_counter()
    nw = 0
    while nw < args.warmup or (time.perf_counter() - t_w < 1.5 and nw < args.warmup + 20):
        step()
        torch.cuda.synchronize()
        nw += 1
    # device-resident timed region
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with Clocks(local) as clk:
        for a, b in evs:
            flush.zero_()
            a.record(stream)
            step()
            b.record(stream)
        torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    ms = sum(a.elapsed_time(b) for a, b in evs) / args.steps
    t = torch.tensor([ms], dtype=torch.float64, device=dev)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms = float(t.item())
    clocks = clk.summary()
    # kernel split (evaluation vs FP64 re-check) from the library's events
    st = step(stats=True)
    torch.cuda.synchronize()
    ms_kernel = st.ms_kernel
    nrecheck = int(st.nrecheck)
    stage_frac = float(st.stage_frac)  # K-stages a 32-point tile computes, of all
    # end-to-end through the public call with host output arrays
    e2e_ms = []
    for _ in range(max(1, min(args.steps, 3))):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        hc, hg, _ = w.nciplot(x0, xm, ns, prec)
        e2e_ms.append(1e3 * (time.perf_counter() - t0))
    e2e_ms = float(np.median(e2e_ms))
    # FP64 plain form beside it, and the split-precision error against it
    fp64 = None
    if prec != "fp64" and not args.no_fp64:
        # FP64 on the whole grid, or on --fp64-planes i-planes from the middle
        n1, plane = int(ns[0]), int(ns[1]) * int(ns[2])
        npl = n1 if args.fp64_planes <= 0 else min(n1, args.fp64_planes)
        i0 = (n1 - npl) // 2
        x0p = x0 + i0 * xm[:, 0]
        nsp = np.array([npl, ns[1], ns[2]], np.int32)
        crho = crho[i0 * plane:(i0 + npl) * plane]
        cgrad = cgrad[i0 * plane:(i0 + npl) * plane]
        rf = torch.empty_like(crho)
        gf = torch.empty_like(cgrad)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        w.nciplot_dev(x0p, xm, nsp, "fp64", rf.data_ptr(), gf.data_ptr(), sp)
        b.record(stream)
        torch.cuda.synchronize()
        t64 = a.elapsed_time(b) * n1 / npl  # per full grid
        rho64 = rf.abs() / 100
        rho = crho.abs() / 100
        drel = ((rho - rho64).abs() / rho64.clamp_min(1e-300)).max().item()
        ds = (cgrad - gf).abs().max().item()
        flips = int((torch.sign(crho) != torch.sign(rf)).sum().item())
        fp64 = {"value": npts / (t64 / 1e3), "unit": "points/s", "ms_per_step": t64,
                "speedup_split_vs_fp64": t64 / ms, "max_rel_drho": drel, "max_abs_ds": ds,
                "sign_flips": flips, "compared_points": int(npl * plane),
                "sample": "whole grid" if npl == n1 else f"{npl} of {n1} i-planes (time scaled to the grid)"}
        if args.binned:
            # errors against FP64 binned by rho decade
            lg = torch.floor(torch.log10(rho64.clamp_min(1e-300)))
            bins = {}
            for d in range(-8, 4):
                m = lg == d
                n = int(m.sum().item())
                if n == 0:
                    continue
                bins[f"1e{d}"] = {
                    "points": n,
                    "max_rel_drho": ((rho - rho64).abs() / rho64)[m].max().item(),
                    "max_abs_ds": (cgrad - gf).abs()[m].max().item(),
                    "sign_flips": int((torch.sign(crho) != torch.sign(rf))[m].sum().item())}
            fp64["by_rho_decade"] = bins
    pk, pk_kind = peaks()
    flops = 20.0 * mol.nmo * w.npri * npts  # algorithmic, dense, per step
    achieved = flops / (ms_kernel / 1e3) / 1e12
    peak = pk["bf16_tflops"]
    line = {"metric": "NCI grid points/s", "value": world * npts / (ms / 1e3), "unit": "points/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": {"fp64": "f64", "tf32x3": "tf32x3 (fp32 accumulate)",
                      "bf16x3": "bf16x3 (fp32 accumulate)"}[prec],
            "data": "synthetic (seeded generator, wfx convention)",
            "config": {"workload": f"{wl.name}: {mol.natom} atoms, {w.npri} primitives, {mol.nmo} MOs, "
                                   f"{wl.grid}^3 grid at {wl.step} bohr",
                       "precision": prec, "parallelism": f"replicas x{world}",
                       "l2": "flushed between timed steps (256 MB write)"},
            "clocks": clocks,
            "e2e": {"value": world * npts / (e2e_ms / 1e3), "unit": "points/s",
                    "h2d_bytes_per_step": 3 * 8 + 9 * 8 + 3 * 4,
                    "d2h_bytes_per_step": 2 * 8 * npts},
            # per step: the split evaluator and the FP64 re-check pass (launched even
            # when its device-side list is empty), or the FP64 evaluator alone; the
            # nucleus pass adds one only when a nucleus sits on a grid point (none
            # does on the synthetic grids)
            "gpu_launches": args.steps * (1 if prec == "fp64" else 2),
            "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak,
                         "traffic": (TRAFFIC_PER_POINT[(args.workload, prec)] * npts
                                     if (args.workload, prec) in TRAFFIC_PER_POINT else None),
                         "note": f"algorithmic 20*nmo*npri flops per point over the evaluation "
                                 f"kernel time; peak = bf16 dense burst ({pk_kind})",
                         # the split products issue three MMAs per multiply (hi*hi, hi*lo, lo*hi)
                         "issued": None if prec == "fp64" else {
                             "achieved": 3 * achieved,
                             "peak": peak if prec == "bf16x3" else TF32_MEASURED_TFLOPS,
                             "frac": 3 * achieved / (peak if prec == "bf16x3" else TF32_MEASURED_TFLOPS),
                             "stage_frac": stage_frac,
                             "effective_achieved": 3 * achieved * stage_frac,
                             "effective_frac": 3 * achieved * stage_frac /
                                               (peak if prec == "bf16x3" else TF32_MEASURED_TFLOPS),
                             "note": "3x the algorithmic rate (three products per split multiply); "
                                     "dense count, so K-stages skipped by the cutoffs count as work and "
                                     "frac can exceed 1; effective_* scales it by the fraction of "
                                     "K-stages the tiles compute (MO and stage padding not counted); "
                                     "peak = " + ("bf16 dense burst" if prec == "bf16x3"
                                                                     else "tf32 dense, cuBLAS-measured")}},
            "fp64_recheck_points": nrecheck}
    if fp64:
        line["fp64_plain"] = fp64
    if rank == 0 and not args.no_files:
        # nciplot end to end into files: the cutoff pass and the cube/dat
        # text (critic2's output step), timed by parts
        with tempfile.TemporaryDirectory() as d:
            root = os.path.join(d, "nci")
            _, parts = w.nciplot_files(x0, xm, ns, prec, root)
            sizes = {k: os.path.getsize(root + k) for k in ("-dens.cube", "-grad.cube", ".dat")}
        line["nci_files"] = {"ms_evaluation": parts[0], "ms_cutoff_pass": parts[1], "ms_text": parts[2],
                             "ms_write": parts[3], "bytes": sizes,
                             "note": "text formatted on the GPU (correctly rounded, near ties on the host)"}
    if rank == 0 and not args.no_mesh:
        # molcalc: the integral of rho over critic2's default molecular mesh
        # (Franchini, good), mesh built and field evaluated on the GPU
        mc = {"mesh": "franchini, good", "quantity": "integral of rho", "unit": "ms"}
        for p_ in ("fp64", "tf32x3"):
            w.molcalc(("rho",), "franchini", "good", p_)  # warm-up
            t0 = time.perf_counter()
            r = w.molcalc(("rho",), "franchini", "good", p_)
            mc[p_] = {"ms": 1e3 * (time.perf_counter() - t0), "integral": r["rho"], "ms_mesh": r["ms_mesh"]}
            mc["npoints"] = r["npoints"]
        line["molcalc"] = mc
    if rank == 0 and not args.no_cp:
        cps = cp_search(args)
        if cps:
            line["cp_search"] = cps
    if rank == 0 and world == 1 and not args.no_cpu:
        v, cores, sample = cpu_sample(mol, wl)
        line["cpu_baseline"] = {"value": v, "unit": "points/s", "cores": cores, "kind": "port",
                                "sample": sample}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
