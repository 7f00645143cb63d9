#!/usr/bin/env python3
"""Chemistry cells/s per CFD step on one GB300.

Workload (default): ``counterflow_53s`` -- the 53-species / 325-reaction
synthetic mechanism with 20 PLOG reactions, 65,536 cells on a 256 x 256
counterflow-like field, one CFD step dt = 1e-6 s integrated by OptRodas34
(absTol 1e-8, relTol 1e-4, exact Jacobian, initial sub-step 1e-7).  A step is
one call of the batched solve over all cells from the same initial state.

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
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


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


def cpu_baseline(flat, w, cells, seconds, threads):
    """The oracle restatement of the reference CPU integrator on a bounded
    sample of the workload's cells (all host threads)."""
    import oracle
    port = oracle.Port(flat)
    rng = np.random.default_rng(7)
    order = rng.permutation(cells.n)
    n = max(threads * 2, 32)
    t_used = 0.0
    done = 0
    while True:
        sub = cells.subset(order[done:done + n])
        t0 = time.perf_counter()
        port.integrate(sub, w.dt, solver=w.solver, abs_tol=w.abs_tol, rel_tol=w.rel_tol,
                       treact=w.treact, threads=threads)
        dt = time.perf_counter() - t0
        t_used += dt
        done += sub.n
        if t_used >= seconds or done >= cells.n:
            break
        rate = done / t_used
        n = int(min(cells.n - done, max(threads, rate * (seconds - t_used))))
        if n <= 0:
            break
    return done / t_used, done, t_used


def reference_arm(args):
    ws, rank, _ = dist_info()
    if rank != 0:
        return
    import fcs
    w = fcs.WORKLOADS[args.workload]
    mech = w.mechanism()
    flat = fcs.flatten(mech)
    import oracle
    oracle.build(ref=False)
    cells = fcs.cells_for(w, mech, n=args.cells or None)
    threads = os.cpu_count() or 1
    per_step = max(2.0, args.cpu_seconds / max(1, args.steps))
    for _ in range(max(0, min(args.warmup, 1))):
        cpu_baseline(flat, w, cells.subset(np.arange(min(cells.n, threads))), 0.1, threads)
    rates, total = [], 0
    for _ in range(args.steps):
        r, n, _t = cpu_baseline(flat, w, cells, per_step, threads)
        rates.append(r)
        total += n
    value = statistics.median(rates)
    sample = f"{total} cells of {cells.n} over {args.steps} steps, each step ~{per_step:.0f} s of CPU work"
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "cells/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": cells.n / value * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded)",
            "config": {"workload": w.name, "cells": cells.n, "solver": w.solver, "precision": "fp64",
                       "dt": w.dt, "abs_tol": w.abs_tol, "rel_tol": w.rel_tol},
            "cpu_baseline": {"value": value, "unit": "cells/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "cells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        return reference_arm(args)
    ws, rank, local = dist_info()
    import torch
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    import fcs
    from fcs import _lib
    w = fcs.WORKLOADS[args.workload]
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
    P = {k: torch.from_numpy(np.ascontiguousarray(getattr(cells, k))).to(dev) for k in ("p", "rho0", "T", "Y", "subDt")}
    T = P["T"].clone(); Y = P["Y"].clone(); S = P["subDt"].clone()
    RR = torch.zeros_like(Y)
    st = torch.zeros(n, dtype=torch.int32, device=dev)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MB > 129 MB L2

    def step():
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        T.copy_(P["T"]); Y.copy_(P["Y"]); S.copy_(P["subDt"])
        e1.record()
        torch.cuda.synchronize()
        code, stats, dmin = ctx.integrate_raw(n, w.dt, P["p"], P["rho0"], T, Y, S, RR, st, device=True)
        return e0.elapsed_time(e1) + stats["call_ms"], stats

    for _ in range(args.warmup):
        step()
    peak64 = _lib.fp64_peak_tflops(local)
    times, kms, all_stats = [], [], []
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            ms, stats = step()
            times.append(ms)
            kms.append(stats["kernel_ms"])
            all_stats.append(stats)
    torch.cuda.synchronize()
    t_step = statistics.mean(times)
    if ws > 1:
        t = torch.tensor([t_step], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        t_step = float(t.item())
        torch.distributed.barrier()
    value = ws * n / (t_step * 1e-3)
    s0 = all_stats[-1]
    # e2e through the C ABI with pinned host buffers
    hp = {k: torch.from_numpy(np.ascontiguousarray(getattr(cells, k))).pin_memory() for k in ("p", "rho0", "T", "Y", "subDt")}
    hT, hY, hS = hp["T"].clone().pin_memory(), hp["Y"].clone().pin_memory(), hp["subDt"].clone().pin_memory()
    hRR = torch.zeros_like(hY).pin_memory()
    hst = torch.zeros(n, dtype=torch.int32).pin_memory()
    e2e_ms = []
    e2e_warm = 1  # the device path above is already warm
    for i in range(e2e_warm + args.steps):
        hT.copy_(hp["T"]); hY.copy_(hp["Y"]); hS.copy_(hp["subDt"])
        flush.zero_()
        torch.cuda.synchronize()
        code, stats, dmin = ctx.integrate_raw(n, w.dt, hp["p"].numpy(), hp["rho0"].numpy(), hT.numpy(), hY.numpy(),
                                              hS.numpy(), hRR.numpy(), hst.numpy())
        if i >= e2e_warm:
            e2e_ms.append(stats["call_ms"])
    t_e2e = statistics.mean(e2e_ms)
    if ws > 1:
        t = torch.tensor([t_e2e], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        t_e2e = float(t.item())
    h2d = 8 * n * (4 + ns)
    d2h = 8 * n * (2 + 2 * ns) + 4 * n
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
            tr = json.load(f)
        key = f"{args.workload}/{args.solver}/{args.precision}"
        if key in tr:
            traffic = tr[key]["bytes_per_cell"] * n
    if rank != 0:
        return
    line = {"metric": METRIC, "value": value, "unit": "cells/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f64+f32",
            "data": "synthetic (seeded generator, no dataset)",
            "config": {"workload": w.name, "cells": n, "species": ns, "reactions": mech.n_reactions,
                       "solver": args.solver, "precision": args.precision, "jacobian": w.jacobian,
                       "dt": w.dt, "abs_tol": w.abs_tol, "rel_tol": w.rel_tol,
                       "l2": "flushed (256 MB write) before every timed step",
                       "parallelism": f"replicas x{ws} (cells independent, no collective)"},
            "e2e": {"value": ws * n / (t_e2e * 1e-3), "unit": "cells/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "gpu_launches": 2 * args.steps,
            "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak64, "unit": "TFLOP/s",
                         "frac": achieved / peak64, "traffic": traffic,
                         "peak_source": "measured: dense FP64 FMA chains on this GPU (fcs_bench_fp64_peak)",
                         "flops_per_attempt_fp64": f64, "flops_per_attempt_fp32": f32,
                         "transcendentals_per_attempt": n_exp, "kernel_ms": k_ms},
            "stats": {k: s0[k] for k in ("cells_integrated", "cells_failed", "attempts", "accepted",
                                         "jacobians", "rhs_evaluations", "fp64_fallbacks")},
            "clocks": clk.summary()}
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        rate, done, tu = cpu_baseline(flat, w, cells, args.cpu_seconds, threads)
        line["cpu_baseline"] = {"value": rate, "unit": "cells/s", "cores": threads, "kind": "port",
                                "sample": f"{done} randomly chosen cells of the same field, {tu:.1f} s of CPU time"}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
