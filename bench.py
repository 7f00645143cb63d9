#!/usr/bin/env python3
"""Chemistry cells/s per CFD step on one GB300.

Workload (default): ``counterflow_53s`` -- the 53-species / 325-reaction
synthetic mechanism with 20 PLOG reactions, 65,536 cells on a 256 x 256
counterflow-like field, one CFD step dt = 1e-6 s integrated by OptRodas34
(absTol 1e-8, relTol 1e-4, exact Jacobian, initial sub-step 1e-7).  A step is
one call of the batched solve over all cells from the same initial state;
the plain method runs it as one CUDA graph (classify, binned work queue,
persistent integrator).

* gated : the same cells through the surrogate-gated method (an MLP ensemble
          trained before timing on ``--train-samples`` other cells of the same
          kind, integrated by the plain method), with its fallback rate and
          audit errors
* accuracy : both methods against the same integrator at absTol 1e-14 /
          relTol 1e-10 on a sample of cells

* value : cells / device time of the step with inputs resident in HBM
          (CUDA events on the library's launching stream; the reset of the
          state from a pristine device copy is inside the timed region)
* e2e   : the same through the C ABI with pinned host buffers: host->device
          copies of the inputs and device->host copies of T, Y, sub-step, RR
          and the cell status are inside the timed region
* roofline : the integrator kernel against the measured dense FP64 FMA rate of
          this GPU (the kernel is FP64-pipe bound, not HBM bound)
* cpu_baseline : the oracle restatement of the reference's CPU integrator on
          a bounded sample of the same cells, all host cores

``--impl reference`` times the reference's CPU path (the oracle restatement:
the reference's own AVX2 core does not build on the aarch64 GPU hosts) on the
host cores with the same metric.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "fastchemistrysolver-openfoam-10_gb300"))
sys.path.insert(0, os.path.join(HERE, "oracle"))

METRIC = "chem cells/s per CFD step, plain GPU Rodas vs surrogate-gated, at <=1e-3 rel T err"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="mine", choices=["mine", "reference"])
    ap.add_argument("--workload", default="counterflow_53s")
    ap.add_argument("--solver", default="OptRodas34")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--mapping", type=int, default=0)
    ap.add_argument("--cells", type=int, default=0, help="0: the workload's full cell count")
    ap.add_argument("--dt", type=float, default=0.0,
                    help="CFD step in s (0: the workload's); a shorter step makes a short launch for profiling")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--method", default="both", choices=["plain", "gated", "both", "mlp"],
                    help="plain GPU method, the surrogate-gated method, or both on the same cells; "
                         "mlp: only the ensemble forward on the tensor cores (untrained weights)")
    ap.add_argument("--train-samples", type=int, default=65536,
                    help="cells integrated by the plain method to train the surrogate (before timing)")
    ap.add_argument("--no-graph", action="store_true",
                    help="launch the plain method's step without a CUDA graph (for profilers)")
    ap.add_argument("--accuracy-cells", type=int, default=256,
                    help="cells checked against a tight-tolerance run (0: skip)")
    return ap.parse_args()


def max_over_ranks(value: float, device=None) -> float:
    """The largest of every rank's value (the whole-job step time is the
    slowest replica's); the value itself when not distributed."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return value
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def workload(args):
    """The named workload, with the CFD step replaced when --dt is given."""
    import dataclasses
    import fcs
    w = fcs.WORKLOADS[args.workload]
    return dataclasses.replace(w, dt=args.dt) if args.dt > 0 else w


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def flops_per_attempt(ns, nr, ntb, nplog, solver, precision):
    """Algorithmic FP64 / FP32 flops of one attempted step (FMA = 2 flops):
    F_rhs = 40 Ns + 12 R + 2 Ns nTB + 10 nP, F_jac = F_rhs + 40 R + 4 Ns nTB +
    10 N^2 (dC/dY as diagonal scaling + rank-1), F_LU = 2/3 N^3, 2 N^2 per
    triangular-solve pair; Rodas34 6 solves / 5 RHS, Rosenbrock34 4 / 2."""
    n = ns + 1
    f_rhs = 40 * ns + 12 * nr + 2 * ns * ntb + 10 * nplog
    f_jac = f_rhs + 40 * nr + 4 * ns * ntb + 10 * n * n
    f_lu = 2.0 / 3.0 * n ** 3
    if solver == "OptRosenbrock34":
        n_solve, n_rhs, c = 4, 2, 30
    else:
        n_solve, n_rhs, c = 6, 5, 40
    if precision == "fp64":
        fp64 = f_jac + f_lu + n_solve * 2 * n * n + n_rhs * f_rhs + c * n
        fp32 = 0.0
    else:
        # LU and the two triangular-solve pairs of each refined solve in FP32;
        # the residual (2 N^2 per solve) in FP64
        fp64 = f_jac + n_solve * 2 * n * n + n_rhs * f_rhs + c * n
        fp32 = f_lu + n_solve * 2 * 2 * n * n
    return fp64, fp32, n_rhs * (ns + nr + 2) + (ns + nr + 2)


def launch_traffic(records, workload, solver, precision, mapping, attempts, cells):
    """DRAM bytes of one integrator launch from an ncu capture of the same
    kernel and mapping on a smaller case (`records`: profiles/integrate_traffic.json),
    scaled by attempts (the lane mapping's workspace traffic) or by cells (the
    cell groups' state I/O and stack write-back); None without a record."""
    name = "lane" if mapping == 1 else f"g{mapping}"
    rec = records.get(f"{workload}/{solver}/{precision}/{name}")
    if not rec:
        return None
    if "bytes_per_attempt" in rec:
        return rec["bytes_per_attempt"] * attempts
    return rec["bytes_per_cell"] * cells


class ClockSampler:
    """nvidia-smi samples during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


PORT_NOTE = ("oracle port (scalar C restatement): the reference core's sources are not present on this host; "
             "per core the port is slower than the reference's vectorised core")
REF_NOTE = ("the reference's own numerical core (Reaction/, LUsolver/, ODE/Opt*) compiled unmodified: with AVX2/FMA "
            "and libmvec on x86-64; on other hosts with the portable SIMD shim (oracle/simd_shim: the AVX "
            "intrinsics on GCC vector extensions, libmvec's exp/log/pow as scalar libm)")


def cpu_integrator(flat, w):
    """The reference's own core (compiled from its sources) where it is built
    on this host, else the oracle port.  Returns (integrate(cells, threads), kind)."""
    import oracle
    if os.path.exists(oracle.REF_SO):
        ref = oracle.Reference(flat, solver=w.solver, abs_tol=w.abs_tol, rel_tol=w.rel_tol)
        return (lambda sub, threads: ref.integrate(sub, w.dt, treact=w.treact, threads=threads)), "reference"
    port = oracle.Port(flat)
    return (lambda sub, threads: port.integrate(sub, w.dt, solver=w.solver, abs_tol=w.abs_tol, rel_tol=w.rel_tol,
                                                treact=w.treact, threads=threads)), "port"


class CellSampler:
    """Disjoint randomly chosen cells of the field, in one seeded order that
    continues across calls (wrapping around after the whole field), so that
    successive CPU steps integrate fresh cells."""

    def __init__(self, n, seed=7):
        self.order = np.random.default_rng(seed).permutation(n)
        self.pos = 0

    def take(self, k):
        n = self.order.size
        idx = self.order[np.arange(self.pos, self.pos + k) % n]
        self.pos += k
        return idx


def cpu_baseline(flat, w, cells, seconds, threads, sampler, stats=None):
    """The reference CPU integrator (its own core, else the oracle port) on a
    bounded sample of the workload's cells (all host threads): batches of
    fresh cells from `sampler` until about `seconds` of wall time.  Returns
    (cells/s, cells done, seconds, kind); `stats` (a dict) also gets the
    attempts per cell (Jacobians per cell: one per Rosenbrock attempt)."""
    run, kind = cpu_integrator(flat, w)
    n = max(threads * 2, 32)
    t_used = 0.0
    done = 0
    jac = 0
    while True:
        sub = cells.subset(sampler.take(n))
        t0 = time.perf_counter()
        out = run(sub, threads)
        dt = time.perf_counter() - t0
        jac += int(out["counters"]["jacobians"])
        t_used += dt
        done += sub.n
        if t_used >= seconds:
            break
        rate = done / t_used
        n = int(max(threads, rate * (seconds - t_used)))
    if stats is not None:
        stats["jacobians_per_cell"] = jac / max(1, done)
    return done / t_used, done, t_used, kind


def cpu_single_core(flat, w, cells, seconds, sampler):
    """One host thread on a few fresh cells: cells/s."""
    run, _ = cpu_integrator(flat, w)
    done, t_used, n = 0, 0.0, 2
    while t_used < seconds:
        sub = cells.subset(sampler.take(n))
        t0 = time.perf_counter()
        run(sub, 1)
        t_used += time.perf_counter() - t0
        done += sub.n
        n = max(1, int(done / t_used * max(0.5, seconds - t_used)) + 1)
    return done / t_used


def workload_config(w, mech, n, solver, precision):
    """The `config` object both arms print: the workload and how it is solved."""
    return {"workload": w.name, "cells": n, "species": mech.n_species, "reactions": mech.n_reactions,
            "solver": solver, "precision": precision, "jacobian": w.jacobian, "dt": w.dt,
            "abs_tol": w.abs_tol, "rel_tol": w.rel_tol, "initial_sub_dt": w.sub_dt0, "treact": w.treact}


def reference_arm(args):
    ws, rank, _ = dist_info()
    if rank != 0:
        return
    import fcs
    w = workload(args)
    mech = w.mechanism()
    flat = fcs.flatten(mech)
    import oracle
    oracle.build(ref=True)  # the reference core where it builds (AVX2 on x86-64, the SIMD shim elsewhere)
    cells = fcs.cells_for(w, mech, n=args.cells or None)
    threads = os.cpu_count() or 1
    per_step = max(2.0, args.cpu_seconds / max(1, args.steps))
    sampler = CellSampler(cells.n)
    for _ in range(max(0, min(args.warmup, 1))):
        cpu_baseline(flat, w, cells, 0.1, threads, CellSampler(cells.n, seed=8))
    rates, secs, total, kind, extra = [], [], 0, "port", {}
    for _ in range(args.steps):
        r, n, t, kind = cpu_baseline(flat, w, cells, per_step, threads, sampler, extra)
        rates.append(r)
        secs.append(t)
        total += n
    value = total / sum(secs)
    sample = (f"{total} distinct cells of the {cells.n}-cell field (seeded random order) over {args.steps} steps "
              f"of ~{per_step:.0f} s each, {total / max(1, args.steps):.0f} cells per step; ms_per_step is the "
              f"measured wall time of a step's sample")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "cells/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(secs),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded generator, no dataset)",
            "config": workload_config(w, mech, cells.n, w.solver, "fp64"),
            "cpu_baseline": {"value": value, "unit": "cells/s", "cores": threads, "kind": kind,
                             "sample": sample, "jacobians_per_cell": extra.get("jacobians_per_cell"),
                             "step_rates": rates,
                             "single_core": cpu_single_core(flat, w, cells, min(5.0, per_step / 2), sampler)},
            "e2e": {"value": value, "unit": "cells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    line["cpu_baseline"]["note"] = PORT_NOTE if kind == "port" else REF_NOTE
    print(json.dumps(line), flush=True)


def device_state(cells, dev):
    import torch
    return {k: torch.from_numpy(np.ascontiguousarray(getattr(cells, k))).to(dev)
            for k in ("p", "rho0", "T", "Y", "subDt")}


def accuracy(ctx, w, cells, idx, results, dev):
    """Max relative T and absolute Y error of each result on cells `idx`
    against the same GPU FP64 integrator at absTol 1e-14 / relTol 1e-10 (the
    FP64 oracle tolerances; the integrator is parity-tested against the
    reference)."""
    import torch
    o = ctx.options
    sub = cells.subset(idx)
    d = device_state(sub, dev)
    ctx.set_options(solver=args_solver(o), jacobian="exact", precision="fp64", mapping=o.mapping,
                    abs_tol=1e-14, rel_tol=1e-10, max_steps=10 ** 7, treact=o.T_react)
    st = torch.zeros(sub.n, dtype=torch.int32, device=dev)
    ctx.integrate_raw(sub.n, w.dt, d["p"], d["rho0"], d["T"], d["Y"], d["subDt"], None, st, device=True)
    ctx.options = o
    ctx._check(ctx.L.fcs_set_options(ctx.h, ctypes.byref(o)))
    Tt, Yt = d["T"].cpu().numpy(), d["Y"].cpu().numpy()
    act = sub.T > o.T_react
    out = {}
    for name, (T, Y) in results.items():
        eT = np.abs(T[idx] - Tt) / Tt
        eY = np.abs(Y[:, idx] - Yt).max(axis=0)
        out[name] = {"max_rel_T": float(eT[act].max()) if act.any() else 0.0,
                     "p99_rel_T": float(np.percentile(eT[act], 99)) if act.any() else 0.0,
                     "max_abs_Y": float(eY[act].max()) if act.any() else 0.0}
    return out


def accuracy_cpu(flat, w, cells, idx, results):
    """Max / p99 relative T and max absolute Y error of each result on cells
    `idx` against the reference's CPU Rodas34 (its own core where it is built,
    else the oracle port) at absTol 1e-14 / relTol 1e-10."""
    import oracle
    sub = cells.subset(idx)
    threads = os.cpu_count() or 1
    if os.path.exists(oracle.REF_SO):
        ref = oracle.Reference(flat, solver="OptRodas34", abs_tol=1e-14, rel_tol=1e-10, max_steps=10 ** 7)
        out = ref.integrate(sub, w.dt, treact=w.treact, threads=threads)
        name = "the reference's own CPU core"
    else:
        out = oracle.Port(flat).integrate(sub, w.dt, solver="OptRodas34", abs_tol=1e-14, rel_tol=1e-10,
                                          max_steps=10 ** 7, treact=w.treact, threads=threads)
        name = "the oracle port of the reference's CPU integrator"
    Tt, Yt = out["T"], out["Y"]
    act = sub.T > w.treact
    res = {"reference": f"{name}, OptRodas34 at absTol 1e-14, relTol 1e-10, maxSteps 1e7 on the sampled cells",
           "cells": int(idx.size)}
    for name_r, (T, Y) in results.items():
        eT = np.abs(T[idx] - Tt) / Tt
        eY = np.abs(Y[:, idx] - Yt).max(axis=0)
        res[name_r] = {"max_rel_T": float(eT[act].max()) if act.any() else 0.0,
                       "p99_rel_T": float(np.percentile(eT[act], 99)) if act.any() else 0.0,
                       "max_abs_Y": float(eY[act].max()) if act.any() else 0.0}
    return res


def args_solver(o):
    from fcs import _lib
    return {v: k for k, v in _lib.SOLVERS.items()}[o.solver]


def mlp_bench(args):
    """The surrogate ensemble's forward over the field on the tensor cores
    (tcgen05 GEMMs): the profiling case of the MLP kernels."""
    import torch
    import fcs
    from fcs import _lib, surrogate
    w = fcs.WORKLOADS[args.workload]
    mech = w.mechanism()
    cells = fcs.cells_for(w, mech, n=args.cells or None)
    ns, n = mech.n_species, cells.n
    mlp = _lib.Mlp(ns + 3, ns + 2, width=256, depth=4, members=4, seed=1)
    x = torch.from_numpy(surrogate.features(cells.T, cells.p, w.dt, cells.Y)).cuda()
    mlp.set_normalization(x.mean(0).cpu().numpy(), x.std(0).cpu().numpy().clip(1e-6), np.zeros(ns + 2),
                          np.ones(ns + 2))
    for _ in range(args.warmup):
        for m in range(mlp.members):
            mlp.forward(m, x, device=True)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        for m in range(mlp.members):
            mlp.forward(m, x, device=True)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    dims = [ns + 3] + [256] * 4 + [ns + 2]
    flop = 2.0 * n * 4 * sum(dims[i] * dims[i + 1] for i in range(len(dims) - 1))
    print(json.dumps({"mlp_forward": {"workload": w.name, "cells": n, "members": 4, "ms_per_ensemble": ms,
                                      "tflops": flop / (ms * 1e-3) / 1e12, "steps": args.steps,
                                      "warmup": args.warmup}}), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        return reference_arm(args)
    if args.method == "mlp":
        return mlp_bench(args)
    ws, rank, local = dist_info()
    import torch
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    import fcs
    from fcs import _lib, surrogate
    w = workload(args)
    mech = w.mechanism()
    flat = fcs.flatten(mech)
    cells = fcs.cells_for(w, mech, n=args.cells or None)
    n, ns = cells.n, mech.n_species
    ctx = _lib.Context(local)
    ctx.load_mechanism(flat)
    ctx.set_options(solver=args.solver, jacobian=w.jacobian, precision=args.precision, mapping=args.mapping,
                    abs_tol=w.abs_tol, rel_tol=w.rel_tol, treact=w.treact)
    dev = torch.device("cuda", local)
    # pristine inputs resident in HBM, and working buffers
    P = device_state(cells, dev)
    T = P["T"].clone(); Y = P["Y"].clone(); S = P["subDt"].clone()
    RR = torch.zeros_like(Y)
    st = torch.zeros(n, dtype=torch.int32, device=dev)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MB > 129 MB L2
    gated = args.method in ("gated", "both")
    plain = args.method in ("plain", "both")

    def reset():
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        T.copy_(P["T"]); Y.copy_(P["Y"]); S.copy_(P["subDt"])
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    def step_plain(graph=True):
        ms = reset()
        code, stats, dmin = ctx.integrate_raw(n, w.dt, P["p"], P["rho0"], T, Y, S, RR, st, device=True,
                                              flags=_lib.CUDA_GRAPH if graph else 0)
        return ms + stats["call_ms"], stats

    def step_gated():
        ms = reset()
        code, stats, gst, dmin = _lib.integrate_gated_raw(ctx, n, w.dt, P["p"], P["rho0"], T, Y, S, RR, st,
                                                          device=True)
        return ms + stats["call_ms"], stats, gst

    def timed(fn):
        times, out = [], []
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            r = fn()
            times.append(r[0])
            out.append(r)
        torch.cuda.synchronize()
        return max_over_ranks(statistics.mean(times), dev), out

    # the first call autotunes the cell-to-thread mapping (outside the graph)
    step_plain(graph=False)
    for _ in range(args.warmup):
        step_plain(graph=not args.no_graph)
    peak64 = _lib.fp64_peak_tflops(local)
    with ClockSampler(local) as clk:
        t_step, outs = timed(lambda: step_plain(graph=not args.no_graph))
    T_plain, Y_plain = T.cpu().numpy(), Y.cpu().numpy()
    value = ws * n / (t_step * 1e-3)
    s0 = outs[-1][1]
    kms = [o[1]["kernel_ms"] for o in outs]
    # e2e through the C ABI with pinned host buffers
    hp = {k: torch.from_numpy(np.ascontiguousarray(getattr(cells, k))).pin_memory() for k in ("p", "rho0", "T", "Y", "subDt")}
    hT, hY, hS = hp["T"].clone().pin_memory(), hp["Y"].clone().pin_memory(), hp["subDt"].clone().pin_memory()
    hRR = torch.zeros_like(hY).pin_memory()
    hst = torch.zeros(n, dtype=torch.int32).pin_memory()
    e2e_ms = []
    for i in range(1 + args.steps):
        hT.copy_(hp["T"]); hY.copy_(hp["Y"]); hS.copy_(hp["subDt"])
        flush.zero_()
        torch.cuda.synchronize()
        code, stats, dmin = ctx.integrate_raw(n, w.dt, hp["p"].numpy(), hp["rho0"].numpy(), hT.numpy(), hY.numpy(),
                                              hS.numpy(), hRR.numpy(), hst.numpy())
        if i >= 1:
            e2e_ms.append(stats["call_ms"])
    t_e2e = max_over_ranks(statistics.mean(e2e_ms), dev)
    h2d = 8 * n * (4 + ns)
    d2h = 8 * n * (2 + 2 * ns) + 4 * n
    # the surrogate-gated method on the same cells
    gated_line = None
    results = {"plain": (T_plain, Y_plain)}
    if gated:
        mlp, info = surrogate.train_for_workload(ctx, w, mech, args.train_samples, seed=1000 + rank)
        surrogate.attach(ctx, mlp, mech)
        for _ in range(args.warmup):
            step_gated()
        t_g, gouts = timed(step_gated)
        results["gated"] = (T.cpu().numpy(), Y.cpu().numpy())
        sg, gg = gouts[-1][1], gouts[-1][2]
        # the tensor-core MLP alone: one ensemble forward over the field
        x = torch.from_numpy(surrogate.features(cells.T, cells.p, w.dt, cells.Y)).to(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        mlp.forward(0, x, device=True)
        torch.cuda.synchronize()
        e0.record()
        for m in range(mlp.members):
            mlp.forward(m, x, device=True)
        e1.record()
        torch.cuda.synchronize()
        mlp_ms = e0.elapsed_time(e1)
        dims = [ns + 3] + [mlp.width] * mlp.depth + [ns + 2]
        mlp_flop = 2.0 * n * mlp.members * sum(dims[i] * dims[i + 1] for i in range(len(dims) - 1))
        peaks = {}
        try:
            with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
                peaks = json.load(f)
        except OSError:
            pass
        bf16_peak = float(peaks.get("bf16_tflops", 1900.0))
        gated_line = {"value": ws * n / (t_g * 1e-3), "unit": "cells/s", "ms_per_step": t_g,
                      "cells_active": gg["cells_active"], "cells_accepted": gg["cells_accepted"],
                      "cells_fallback": gg["cells_fallback"], "cells_audited": gg["cells_audited"],
                      "fallback_rate": gg["cells_fallback"] / max(1, gg["cells_active"]),
                      "audit_max_rel_T": gg["audit_max_rel_T"], "audit_max_abs_Y": gg["audit_max_abs_Y"],
                      "surrogate_ms": gg["surrogate_ms"], "integrate_ms": gg["integrate_ms"],
                      "attempts": sg["attempts"], "training": info,
                      "mlp_roofline": {"bound": "tensor", "achieved": mlp_flop / (mlp_ms * 1e-3) / 1e12,
                                       "peak": bf16_peak, "unit": "TFLOP/s",
                                       "frac": mlp_flop / (mlp_ms * 1e-3) / 1e12 / bf16_peak,
                                       "ms_ensemble_forward": mlp_ms,
                                       "peak_source": "MEASURED_PEAKS.json bf16_tflops (cuBLAS burst)"}}
        _lib.attach_surrogate(ctx, None)
    acc = None
    if args.accuracy_cells > 0:
        rng = np.random.default_rng(5)
        idx = np.sort(rng.choice(n, min(n, args.accuracy_cells), replace=False))
        gpu_tight = accuracy(ctx, w, cells, idx, results, dev)
        gpu_tight["reference"] = "GPU FP64 integrator at absTol 1e-14, relTol 1e-10, maxSteps 1e7 on the sampled cells"
        gpu_tight["cells"] = int(idx.size)
        # the FP64 oracle proper: the reference's CPU integrator at the tight
        # tolerances on the first cells of the same sample
        cidx = idx[:min(idx.size, 32)]
        acc = accuracy_cpu(flat, w, cells, cidx, results)
        acc["gpu_tight"] = gpu_tight
    # roofline of the integrator kernel
    f64, f32, n_exp = flops_per_attempt(ns, mech.n_reactions, mech.count(1), mech.count(2), args.solver,
                                        args.precision)
    attempts = s0["attempts"]
    k_ms = statistics.mean(kms)
    achieved = f64 * attempts / (k_ms * 1e-3) / 1e12
    traffic = None
    tj = os.path.join(HERE, "profiles", "integrate_traffic.json")
    if os.path.exists(tj):
        with open(tj) as f:
            traffic = launch_traffic(json.load(f), args.workload, args.solver, args.precision, s0["mapping"],
                                     s0["attempts"], n)
    if rank != 0:
        return
    line = {"metric": METRIC, "value": value, "unit": "cells/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f64+f32",
            "data": "synthetic (seeded generator, no dataset)",
            "config": workload_config(w, mech, n, args.solver, args.precision),
            "setup": {"method": "plain GPU " + args.solver, "mapping": s0["mapping"],
                      "step": "one CUDA graph per step (classify, binned work queue, persistent integrator)",
                      "l2": "flushed (256 MB write) before every timed step",
                      "parallelism": f"replicas x{ws} (cells independent, no collective)"},
            "e2e": {"value": ws * n / (t_e2e * 1e-3), "unit": "cells/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "gpu_launches": 3 * args.steps,  # classify_bin_kernel, queue_kernel, integrate_kernel
            "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak64, "unit": "TFLOP/s",
                         "frac": achieved / peak64, "traffic": traffic,
                         "peak_source": "measured: dense FP64 FMA chains on this GPU (fcs_bench_fp64_peak)",
                         "flops_per_attempt_fp64": f64, "flops_per_attempt_fp32": f32,
                         "transcendentals_per_attempt": n_exp, "kernel_ms": k_ms},
            "stats": {k: s0[k] for k in ("cells_integrated", "cells_skipped", "cells_failed", "attempts", "accepted",
                                         "jacobians", "rhs_evaluations", "fp64_fallbacks", "mapping")},
            "clocks": clk.summary()}
    if gated_line:
        line["gated"] = gated_line
    if acc:
        line["accuracy"] = acc
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        extra = {}
        sampler = CellSampler(cells.n)
        rate, done, tu, kind = cpu_baseline(flat, w, cells, args.cpu_seconds, threads, sampler, extra)
        line["cpu_baseline"] = {"value": rate, "unit": "cells/s", "cores": threads, "kind": kind,
                                "sample": f"{done} distinct cells of the same field (seeded random order), "
                                          f"{tu:.1f} s of wall time",
                                "jacobians_per_cell": extra["jacobians_per_cell"],
                                "single_core": cpu_single_core(flat, w, cells, min(5.0, args.cpu_seconds / 3), sampler),
                                "note": PORT_NOTE if kind == "port" else REF_NOTE}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
