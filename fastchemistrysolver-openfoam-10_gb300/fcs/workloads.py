"""The benchmark workloads: seeded synthetic mechanisms plus cell states.

Each workload is a constant-pressure batch of independent cells that is
integrated over one CFD step ``dt``; the cell state arrays use the layout of
OpenFOAM fields: ``Y`` is species-major ``[Ns, nCells]`` (one contiguous
field per species), ``T``/``p``/``rho0``/``subDt`` are ``[nCells]``.

Workloads (all seeds fixed):

* ``ignition_10s`` -- 10 species / 27 reactions (3 third-body), 1,024 cells,
  T ~ U[1000, 1500] K, p = 1e5 Pa, Y ~ Dirichlet(0.5), dt = 1e-5 s,
  OptRodas34 absTol 1e-8 relTol 1e-4, exact Jacobian, initial sub-step 1e-7.
* ``counterflow_53s`` -- 53 species / 325 reactions (20 PLOG with 5 rows on
  1e4-1e8 Pa, 13 third-body), 65,536 cells on a 256 x 256 field: T is a tanh
  profile 300 -> 2200 K across x, Y mixes linearly (in y) between two seeded
  Dirichlet end states, p ~ U[1e5, 5e6] Pa, dt = 1e-6 s.
* ``uneven_111s`` -- 111 species / 784 reactions (31 third-body), 262,144
  cells: 80 % near-frozen (half of them below Treact = 700 K: T ~ U[300, 700),
  the other half T ~ U[700, 800]) and 20 % reacting (T ~ U[1200, 2200]),
  Y ~ Dirichlet(0.3), p ~ U[1e5, 1e6] Pa, dt = 5e-6 s.
* ``falloff_16s`` -- 16 species / 48 reactions (3 third-body, 2 PLOG, 3 each of
  Lindemann, Troe and SRI fall-off), 512 cells, T ~ U[900, 1800] K,
  p log-uniform on [1e4, 1e7] Pa, Y ~ Dirichlet(0.5), dt = 1e-5 s: the parity
  case of the fall-off kinds (no benchmark field uses them).
* ``noneq_14s`` -- 14 species / 40 reactions (6 non-equilibrium reversible,
  3 non-equilibrium third-body, 2 third-body, 1 PLOG, 1 Lindemann, 1 Troe),
  512 cells drawn like ``falloff_16s``: the parity case of the
  non-equilibrium kinds.
* ``long_24s`` -- 24 species / 60 reactions, among them 4 irreversible global
  reactions (up to 3 reactants and 7 products) and 2 reversible ones with 6
  products (dnu = 3), plus one of each other kind; 512 cells drawn like
  ``falloff_16s``: the parity case of the long reactions.
* ``large_200s`` -- 200 species / 1,500 reactions (60 PLOG, 40 third-body),
  1,048,576 cells, T ~ U[600, 2400] K, p ~ U[1e5, 4e6] Pa, Y ~ Dirichlet(0.2),
  dt = 1e-5 s.

No public dataset is involved: every input is generated from the seeds here.
"""
from __future__ import annotations

import dataclasses
from typing import Optional

import numpy as np

from .mechanism import Mechanism, synthetic_mechanism

RU = 8314.470066505449722171761095523834228515625  # J/(kmol K), reference value


@dataclasses.dataclass
class Cells:
    T: np.ndarray        # [n]
    p: np.ndarray        # [n]
    Y: np.ndarray        # [Ns, n] species-major
    rho0: np.ndarray     # [n]
    subDt: np.ndarray    # [n]

    @property
    def n(self) -> int:
        return int(self.T.shape[0])

    def subset(self, idx) -> "Cells":
        idx = np.asarray(idx)
        return Cells(self.T[idx].copy(), self.p[idx].copy(),
                     np.ascontiguousarray(self.Y[:, idx]), self.rho0[idx].copy(),
                     self.subDt[idx].copy())

    def copy(self) -> "Cells":
        return Cells(self.T.copy(), self.p.copy(), self.Y.copy(), self.rho0.copy(),
                     self.subDt.copy())


@dataclasses.dataclass
class Workload:
    name: str
    mech_args: dict
    n_cells: int
    dt: float
    solver: str = "OptRodas34"
    abs_tol: float = 1e-8
    rel_tol: float = 1e-4
    jacobian: str = "exact"
    sub_dt0: float = 1e-7
    treact: float = 0.0
    cell_seed: int = 0

    def mechanism(self) -> Mechanism:
        return synthetic_mechanism(name=self.name, **self.mech_args)


WORKLOADS = {
    "ignition_10s": Workload(
        "ignition_10s",
        dict(n_species=10, n_reactions=27, n_third_body=3, n_plog=0, seed=1010),
        n_cells=1024, dt=1e-5, cell_seed=11),
    "counterflow_53s": Workload(
        "counterflow_53s",
        dict(n_species=53, n_reactions=325, n_third_body=13, n_plog=20, seed=5353),
        n_cells=65536, dt=1e-6, cell_seed=53),
    "uneven_111s": Workload(
        "uneven_111s",
        dict(n_species=111, n_reactions=784, n_third_body=31, n_plog=0, seed=111),
        n_cells=262144, dt=5e-6, treact=700.0, cell_seed=111),
    "falloff_16s": Workload(
        "falloff_16s",
        dict(n_species=16, n_reactions=48, n_third_body=3, n_plog=2, seed=1616, n_falloff=(3, 3, 3)),
        n_cells=512, dt=1e-5, cell_seed=16),
    "noneq_14s": Workload(
        "noneq_14s",
        dict(n_species=14, n_reactions=40, n_third_body=2, n_plog=1, seed=1414, n_falloff=(1, 1, 0),
             n_noneq=(6, 3)),
        n_cells=512, dt=1e-5, cell_seed=14),
    "long_24s": Workload(
        "long_24s",
        dict(n_species=24, n_reactions=60, n_third_body=2, n_plog=1, seed=2426, n_falloff=(1, 0, 1),
             n_noneq=(1, 1), n_long=(4, 2)),
        n_cells=512, dt=1e-5, cell_seed=24),
    "large_200s": Workload(
        "large_200s",
        dict(n_species=200, n_reactions=1500, n_third_body=40, n_plog=60, seed=2000),
        n_cells=1048576, dt=1e-5, cell_seed=200),
}


def _rho(mech: Mechanism, T, p, Y):
    # perfect gas: rho = p / (Ru T sum_i Y_i / W_i)
    return p / (RU * T * (Y / mech.W[:, None]).sum(axis=0))


def cells_for(w: Workload, mech: Mechanism, n: Optional[int] = None,
              seed_offset: int = 0) -> Cells:
    """Cell states of workload ``w``; ``n`` < n_cells takes the first n cells
    of the same seeded draw (the full field is generated and cut)."""
    ns = mech.n_species
    n_full = w.n_cells
    rng = np.random.default_rng(w.cell_seed + seed_offset)
    if w.name == "ignition_10s":
        T = rng.uniform(1000.0, 1500.0, n_full)
        p = np.full(n_full, 1e5)
        Y = rng.dirichlet(np.full(ns, 0.5), size=n_full).T
    elif w.name == "counterflow_53s":
        side = int(round(np.sqrt(n_full)))
        x = (np.arange(side) + 0.5) / side
        Tx = 300.0 + (2200.0 - 300.0) * 0.5 * (1.0 + np.tanh((x - 0.5) / 0.08))
        ya = rng.dirichlet(np.full(ns, 0.5))
        yb = rng.dirichlet(np.full(ns, 0.5))
        xi = x  # mixture fraction along the other axis
        T = np.tile(Tx, side)                           # cell = j*side + i
        Y = (np.outer(ya, 1.0 - np.repeat(xi, side)) + np.outer(yb, np.repeat(xi, side)))
        p = rng.uniform(1e5, 5e6, n_full)
    elif w.name == "uneven_111s":
        u = rng.random(n_full)
        T = np.where(u < 0.4, rng.uniform(300.0, 700.0, n_full),
                     np.where(u < 0.8, rng.uniform(700.0, 800.0, n_full),
                              rng.uniform(1200.0, 2200.0, n_full)))
        p = rng.uniform(1e5, 1e6, n_full)
        Y = rng.dirichlet(np.full(ns, 0.3), size=n_full).T
    elif w.name in ("falloff_16s", "noneq_14s", "long_24s"):
        T = rng.uniform(900.0, 1800.0, n_full)
        p = 10.0 ** rng.uniform(4.0, 7.0, n_full)
        Y = rng.dirichlet(np.full(ns, 0.5), size=n_full).T
    elif w.name == "large_200s":
        T = rng.uniform(600.0, 2400.0, n_full)
        p = rng.uniform(1e5, 4e6, n_full)
        Y = rng.dirichlet(np.full(ns, 0.2), size=n_full).T
    else:
        raise KeyError(w.name)
    if n is not None:
        T, p, Y = T[:n], p[:n], Y[:, :n]
    Y = np.ascontiguousarray(Y, dtype=np.float64)
    T = np.ascontiguousarray(T, dtype=np.float64)
    p = np.ascontiguousarray(p, dtype=np.float64)
    rho0 = _rho(mech, T, p, Y)
    subDt = np.full(T.shape[0], w.sub_dt0)
    return Cells(T, p, Y, rho0, subDt)
