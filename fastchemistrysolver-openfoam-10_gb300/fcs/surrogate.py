"""Training data and set-up of the surrogate ensemble (include/fcs_mlp.h).

The network, its training (forward, backward, Adam) and the gate all run in
the library's own CUDA kernels.  This module only prepares what the network
learns from: cell states drawn like a workload's cells (its own generator
with another seed), keeping the cells that react (T > Treact), and their
state after one CFD step and next initial sub-step from the library's plain
GPU integrator (``fcs_integrate``).

Input features (n_in = Ns + 3): T, ln p, ln dt, Y_0..Y_{Ns-1}.
Outputs (n_out = Ns + 2): T1 - T, Y1_i - max(Y_i, 0), ln sub_dt1 -- exactly
what the gate kernel adds to the cell state.
"""
from __future__ import annotations

import numpy as np

from . import _lib
from .mechanism import ELEMENT_MASS, Mechanism
from .workloads import Cells, Workload, cells_for

def features(T, p, dt, Y) -> np.ndarray:
    """[n][Ns+3] float32 network inputs; Y is species-major [Ns][n]."""
    n = T.shape[0]
    x = np.empty((n, Y.shape[0] + 3), dtype=np.float32)
    x[:, 0] = T
    x[:, 1] = np.log(p)
    x[:, 2] = np.log(dt)
    x[:, 3:] = Y.T
    return x


def targets(T0, Y0, T1, Y1, sub1) -> np.ndarray:
    n, ns = T0.shape[0], Y0.shape[0]
    t = np.empty((n, ns + 2), dtype=np.float32)
    t[:, 0] = T1 - T0
    t[:, 1:ns + 1] = (Y1 - np.maximum(Y0, 0.0)).T
    t[:, ns + 1] = np.log(sub1)
    return t


def predict(mlp: _lib.Mlp, T, p, dt, Y):
    """Ensemble-mean prediction (T1, Y1, sub1) in raw units, the gate's
    reconstruction restated on the host (for tests and diagnostics)."""
    x = features(T, p, dt, Y)
    # members summed in order in FP64, as the gate kernel does
    r = np.zeros((x.shape[0], mlp.n_out))
    for m in range(mlp.members):
        r += mlp.forward(m, x).astype(np.float64)
    r /= mlp.members
    T1 = T + r[:, 0]
    Y1 = np.maximum(np.maximum(Y, 0.0) + r[:, 1:-1].T, 0.0)
    return T1, Y1, np.exp(r[:, -1])


def reacting_cells(w: Workload, mech: Mechanism, n: int, seed: int, per_draw: int = 1024) -> Cells:
    """n cells drawn like w's cells, T > Treact only: `per_draw` random
    reacting cells from each of as many seeded draws of the workload's field
    (seed offsets seed, seed + 7919, ...) as it takes, so that the samples
    cover many fields rather than one."""
    parts, have, k = [], 0, 0
    while have < n:
        c = cells_for(w, mech, seed_offset=seed + 7919 * k)
        keep = np.nonzero(c.T > w.treact)[0]
        rng = np.random.default_rng(seed + 7919 * k)
        keep = np.sort(rng.choice(keep, min(per_draw, keep.size, n - have), replace=False))
        parts.append(c.subset(keep))
        have += keep.size
        k += 1
    T = np.concatenate([c.T for c in parts])
    p = np.concatenate([c.p for c in parts])
    Y = np.ascontiguousarray(np.concatenate([c.Y for c in parts], axis=1))
    rho0 = np.concatenate([c.rho0 for c in parts])
    sub = np.concatenate([c.subDt for c in parts])
    return Cells(T, p, Y, rho0, sub)


def generate(ctx: _lib.Context, cells: Cells, dt: float, chunk: int = 65536):
    """(x, t, stats) training samples from the plain GPU integrator."""
    import torch
    xs, ts = [], []
    tot = {"attempts": 0, "kernel_ms": 0.0, "cells_integrated": 0, "cells_failed": 0}
    for a in range(0, cells.n, chunk):
        b = min(cells.n, a + chunk)
        sub = cells.subset(np.arange(a, b))
        d = {k: torch.from_numpy(np.ascontiguousarray(getattr(sub, k))).cuda() for k in ("p", "rho0", "T", "Y", "subDt")}
        T1, Y1, S1 = d["T"].clone(), d["Y"].clone(), d["subDt"].clone()
        st = torch.zeros(b - a, dtype=torch.int32, device="cuda")
        code, stats, _ = ctx.integrate_raw(b - a, dt, d["p"], d["rho0"], T1, Y1, S1, None, st, device=True)
        for k in tot:
            tot[k] += stats[k]
        ok = (st.cpu().numpy() == 0)
        x = features(sub.T, sub.p, dt, sub.Y)
        t = targets(sub.T, sub.Y, T1.cpu().numpy(), Y1.cpu().numpy(), S1.cpu().numpy())
        xs.append(x[ok])
        ts.append(t[ok])
    return np.concatenate(xs), np.concatenate(ts), tot


def normalisation(x: np.ndarray, t: np.ndarray):
    im = x.mean(axis=0)
    is_ = np.maximum(x.std(axis=0), 1e-6)
    is_[2] = max(is_[2], 1.0)   # ln dt is often constant
    om = t.mean(axis=0)
    os_ = np.maximum(t.std(axis=0), 1e-12)
    return im, is_, om, os_


def fit(x: np.ndarray, t: np.ndarray, members: int = 4, epochs: int = 20, batch: int = 4096, lr: float = 1e-3,
        lr_final: float = 2e-5, seed: int = 1, width: int = 256, depth: int = 4, device: int = 0,
        min_steps: int = 0):
    """A trained ensemble (every member on all samples, its own init and
    shuffles).  With min_steps, small sample sets get smaller batches and
    more epochs so that every member takes at least that many Adam steps."""
    n = x.shape[0]
    if min_steps:
        while batch > 512 and (n // batch) * epochs < min_steps:
            batch //= 2
        epochs = max(epochs, -(-min_steps // max(1, n // batch)))
    mlp = _lib.Mlp(x.shape[1], t.shape[1], width=width, depth=depth, members=members, seed=seed, device=device)
    mlp.set_normalization(*normalisation(x, t))
    hist = mlp.train(x, t, epochs=epochs, batch=batch, lr=lr, lr_final=lr_final, seed=seed)
    return mlp, hist


def train_for_workload(ctx: _lib.Context, w: Workload, mech: Mechanism, n_samples: int, seed: int = 1000,
                       members: int = 4, epochs: int = 20, min_steps: int = 4000):
    """Draw n_samples reacting cells like w's (another seed), integrate them
    with the plain GPU method, train an ensemble on the results.  Returns the
    ensemble and a record of what it took."""
    import time
    t0 = time.perf_counter()
    cells = reacting_cells(w, mech, n_samples, seed=seed)
    x, t, st = generate(ctx, cells, w.dt)
    t1 = time.perf_counter()
    mlp, hist = fit(x, t, members=members, epochs=epochs, min_steps=min_steps, seed=seed)
    t2 = time.perf_counter()
    info = {"samples": int(x.shape[0]), "generate_s": t1 - t0, "generate_kernel_s": st["kernel_ms"] / 1e3,
            "train_s": t2 - t1, "members": members, "loss_first": [float(v) for v in hist[:, 0]],
            "loss_last": [float(v) for v in hist[:, -1]], "epochs": int(hist.shape[1])}
    return mlp, info


def attach(ctx: _lib.Context, mlp: _lib.Mlp, mech: Mechanism, **gate):
    comp = np.asarray(mech.composition, dtype=np.float64)
    em = np.asarray(ELEMENT_MASS[:comp.shape[1]], dtype=np.float64)
    _lib.attach_surrogate(ctx, mlp, comp, em, **gate)
