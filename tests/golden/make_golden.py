"""Generates the golden fixtures of tests/golden/ from the REFERENCE itself.

The reference's numerical core (Reaction/, LUsolver/, ODE/Opt*) is compiled
unmodified from its own sources by oracle/Makefile into oracle/_ref/ (x86-64
only; needs the reference tree).  This script runs it on seeded cells of the
synthetic workloads and stores its outputs; the tests then check the oracle
restatement and the GPU path against these numbers on any machine.

    python tests/golden/make_golden.py [substring of the fixture names to regenerate]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "fastchemistrysolver-openfoam-10_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import fcs  # noqa: E402
import oracle  # noqa: E402

CASES = [
    # (workload, cells, solver)
    ("ignition_10s", 64, "OptRodas34"),
    ("ignition_10s", 64, "OptRosenbrock34"),
    ("ignition_10s", 64, "OptSeulex"),
    ("counterflow_53s", 8, "OptRodas34"),
    ("counterflow_53s", 4, "OptRosenbrock34"),
    ("counterflow_53s", 4, "OptSeulex"),
    ("ignition_10s", 64, "OptRodas23"),
    ("ignition_10s", 64, "OptRosenbrock23"),
    ("counterflow_53s", 8, "OptRodas23"),
    ("counterflow_53s", 4, "OptRosenbrock23"),
    ("falloff_16s", 64, "OptRodas34"),
    ("falloff_16s", 32, "OptSeulex"),
    ("noneq_14s", 64, "OptRodas34"),
    ("noneq_14s", 32, "OptSeulex"),
    ("long_24s", 64, "OptRodas34"),
    ("falloff_16s", 32, "OptRosenbrock34"),
    ("falloff_16s", 32, "OptRodas23"),
    ("noneq_14s", 32, "OptRosenbrock23"),
    ("long_24s", 32, "OptSeulex"),
    # the two fields whose slots run from the global-memory workspace on the
    # GPU (111 species: with mixed precision or Seulex; 200 species: always)
    ("uneven_111s", 16, "OptRodas34"),
    ("large_200s", 4, "OptRodas34"),
]


def cell_index(w, n):
    return np.linspace(0, w.n_cells - 1, n).astype(np.int64)


FLAT_FIELDS = ("W", "T_low", "T_high", "T_common", "high_coeffs", "low_coeffs", "type", "reversible",
               "lhs_offset", "lhs_species", "rhs_offset", "rhs_species", "arrhenius", "arrhenius2",
               "efficiencies", "falloff_params", "plog_offset", "plog_table")


def inputs(flat, cells):
    """The exact mechanism arrays and cell states the reference ran on (the
    generator rounds differently across platforms' libm/LAPACK, so the
    fixtures carry their inputs)."""
    d = {"mech_" + k: getattr(flat, k) for k in FLAT_FIELDS}
    d.update(in_T=cells.T, in_p=cells.p, in_Y=cells.Y, in_rho0=cells.rho0, in_subDt=cells.subDt)
    return d


TIGHT = [
    # (workload, cells): the reference Rodas34 at absTol 1e-14 / relTol 1e-10
    ("ignition_10s", 64),
    ("counterflow_53s", 8),
    ("large_200s", 4),
]


TC = [
    # (workload, cells): FastChemistryModel::tc() of the reference on the workload's cells
    ("ignition_10s", 64),
    ("counterflow_53s", 64),
    ("uneven_111s", 64),
    ("falloff_16s", 64),
    ("noneq_14s", 64),
    ("long_24s", 64),
]


def make_tc():
    out = {}
    for wname, n in TC:
        w = fcs.WORKLOADS[wname]
        mech = w.mechanism()
        flat = fcs.flatten(mech)
        idx = cell_index(w, n)
        cells = fcs.cells_for(w, mech).subset(idx)
        tc = oracle.Reference(flat).tc(cells.p, cells.T, cells.rho0, cells.Y)
        for k, v in inputs(flat, cells).items():
            out[f"{wname}__{k}"] = v
        out[f"{wname}__tc"] = tc
    name = os.path.join(HERE, "tc.npz")
    np.savez_compressed(name, **out)
    print(name, os.path.getsize(name), "bytes")


# The reference's own tutorial inputs (read from its tree, FCS_REFERENCE):
#   (fixture name, case directory, fuel, cells, dt)
TUTORIAL_IGNITION = [
    ("tutorial_nc12h26_narayanaswamy", "Ignition0D/NC12H26_Narayanaswamy2014", "N-C12H26", 4, 1e-5),
    ("tutorial_ic8h18_yoo", "Ignition0D/IC8H18_Yoo2013", "IC8H18", 4, 1e-5),
]
COUNTERFLOW_CASE = ("tutorial_ch4_gri30_counterflow", "CounterFlowFlame2D/CH4_GRI30", "1", 16, 2e-4)


def ignition_cells(flat, names, fuel, n, seed):
    """Fuel / O2 / N2 near stoichiometry plus a trace of every species (so
    that every reaction runs), T ~ U[1000, 1600] K, p log-uniform on
    [1e5, 2e6] Pa."""
    from fcs.workloads import Cells, RU
    rng = np.random.default_rng(seed)
    low = [s.lower() for s in names]
    ns = flat.n_species
    base = np.zeros(ns)
    for sp, y in ((fuel, 0.06), ("o2", 0.22), ("n2", 0.72)):
        base[low.index(sp.lower())] = y
    Y = np.empty((ns, n))
    for c in range(n):
        trace = rng.dirichlet(np.full(ns, 0.5)) * 1e-3
        Y[:, c] = (base + trace) / (base + trace).sum()
    T = rng.uniform(1000.0, 1600.0, n)
    p = 10.0 ** rng.uniform(5.0, np.log10(2e6), n)
    rho0 = p / (RU * T * (Y / flat.W[:, None]).sum(axis=0))
    return Cells(T, p, np.ascontiguousarray(Y), rho0, np.full(n, 1e-7))


def read_field(path, n=None):
    """internalField of an OpenFOAM volScalarField file: a nonuniform list of
    n values (n taken from the file when None) or a uniform value."""
    import re
    text = open(path).read()
    m = re.search(r"internalField\s+uniform\s+([^;\s]+)\s*;", text)
    if m:
        return np.full(n, float(m.group(1)))
    m = re.search(r"internalField\s+nonuniform\s+List<scalar>\s*(\d+)\s*\((.*?)\)", text, flags=re.S)
    vals = np.array(m.group(2).split(), dtype=np.float64)
    assert int(m.group(1)) == vals.size and (n is None or vals.size == n), (path, vals.size, n)
    return vals


def counterflow_cells(flat, names, case_dir, time, n):
    """Cells of the reference's 2D CH4/air counterflow flame at a written
    time: n cells spread over the temperature range of the flame (the hot
    ones react), with their own p, T and Y; rho0 from the perfect gas."""
    from fcs.workloads import Cells, RU
    d = os.path.join(case_dir, time)
    T = read_field(os.path.join(d, "T"))
    ncell = T.size
    p = read_field(os.path.join(d, "p"), ncell)
    Y = np.stack([read_field(os.path.join(d, s), ncell) if os.path.exists(os.path.join(d, s)) else np.zeros(ncell)
                  for s in names])
    order = np.argsort(T, kind="stable")
    hot = order[T[order] > 1000.0]
    pick = np.unique(np.concatenate([hot[np.linspace(0, hot.size - 1, n - 4).astype(np.int64)],
                                     order[np.linspace(0, order.size - 1, 4).astype(np.int64)]]))
    T, p, Y = T[pick], p[pick], np.ascontiguousarray(Y[:, pick])
    rho0 = p / (RU * T * (Y / flat.W[:, None]).sum(axis=0))
    return pick, Cells(T, p, Y, rho0, np.full(pick.size, 1e-7))


def make_tutorial(only=None):
    """Golden fixtures on the reference's own mechanisms and cell states:
    the flat mechanism as the library's reader produces it, the cells, and
    the reference core's Rodas34 results (plus RHS and Jacobian)."""
    from fcs import _lib
    tut = oracle.reference_tutorial()
    if not tut:
        raise SystemExit("the reference tree is needed: set FCS_REFERENCE")
    jobs = [(name, case, ("ignition", fuel), n, dt) for name, case, fuel, n, dt in TUTORIAL_IGNITION]
    name, case, time, n, dt = COUNTERFLOW_CASE
    jobs.append((name, case, ("field", time), n, dt))
    for name, case, kind, n, dt in jobs:
        if only and only not in name:
            continue
        const = os.path.join(tut, case, "constant")
        flat, names = _lib.parse_mechanism_foam(os.path.join(const, "reactions"),
                                                os.path.join(const, "speciesThermo"))
        if kind[0] == "ignition":
            idx = np.arange(n)
            cells = ignition_cells(flat, names, kind[1], n, seed=len(names))
        else:
            idx, cells = counterflow_cells(flat, names, os.path.join(tut, case), kind[1], n)
        ref = oracle.Reference(flat, solver="OptRodas34", abs_tol=1e-8, rel_tol=1e-4)
        out = ref.integrate(cells, dt, threads=8)
        assert (out["status"] == 0).all(), out["status"]
        tight = oracle.Reference(flat, solver="OptRodas34", abs_tol=1e-14, rel_tol=1e-10, max_steps=10 ** 7)
        tout = tight.integrate(cells, dt, threads=8)
        f = ref.rhs(cells.p, cells.T, cells.Y)
        J, fj = ref.jacobian(cells.p[:1], cells.T[:1], cells.Y[:, :1])
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(
            path, case=np.array(case), species=np.array(names), cell_index=idx, dt=dt,
            abs_tol=1e-8, rel_tol=1e-4,
            T=out["T"], Y=out["Y"], subDt=out["subDt"], RR=out["RR"], status=out["status"],
            deltaTMin=out["deltaTMin"], jacobians=out["counters"]["jacobians"], rhs_calls=out["counters"]["rhs"],
            tight_T=tout["T"], tight_Y=tout["Y"], rhs=f, jac=J, jac_f=fj, **inputs(flat, cells))
        print(path, os.path.getsize(path), "bytes", out["counters"], "tight", tout["counters"])


def main(only=None):
    """Regenerate every fixture, or only those whose file name contains `only`."""
    oracle.build(ref=True)
    if not only or "tutorial" in only:
        make_tutorial(only)
    if only and "tutorial" in only:
        return
    if not only or only in "tc":
        make_tc()
    for wname, n in TIGHT:
        if only and only not in f"{wname}_tight":
            continue
        w = fcs.WORKLOADS[wname]
        mech = w.mechanism()
        flat = fcs.flatten(mech)
        idx = cell_index(w, n)
        cells = fcs.cells_for(w, mech).subset(idx)
        ref = oracle.Reference(flat, solver="OptRodas34", abs_tol=1e-14, rel_tol=1e-10, max_steps=10 ** 7)
        out = ref.integrate(cells, w.dt, treact=w.treact, threads=8)
        assert (out["status"] == 0).all()
        name = os.path.join(HERE, f"{wname}_tight.npz")
        np.savez_compressed(name, digest=np.array(mech.digest()), cell_index=idx, dt=w.dt,
                            abs_tol=1e-14, rel_tol=1e-10, T=out["T"], Y=out["Y"], **inputs(flat, cells))
        print(name, os.path.getsize(name), "bytes", out["counters"])
    for wname, n, solver in CASES:
        if only and only not in f"{wname}_{solver}":
            continue
        w = fcs.WORKLOADS[wname]
        mech = w.mechanism()
        flat = fcs.flatten(mech)
        idx = cell_index(w, n)
        cells = fcs.cells_for(w, mech).subset(idx)
        ref = oracle.Reference(flat, solver=solver, abs_tol=w.abs_tol, rel_tol=w.rel_tol)
        out = ref.integrate(cells, w.dt, treact=w.treact)
        f = ref.rhs(cells.p, cells.T, cells.Y)
        J, fj = ref.jacobian(cells.p, cells.T, cells.Y)
        name = os.path.join(HERE, f"{wname}_{solver}.npz")
        np.savez_compressed(
            name, digest=np.array(mech.digest()), cell_index=idx, dt=w.dt,
            abs_tol=w.abs_tol, rel_tol=w.rel_tol,
            T=out["T"], Y=out["Y"], subDt=out["subDt"], RR=out["RR"], status=out["status"],
            deltaTMin=out["deltaTMin"], jacobians=out["counters"]["jacobians"],
            rhs_calls=out["counters"]["rhs"],
            rhs=f, jac=J[: 1 if flat.n_species > 100 else min(4, n)], jac_f=fj, **inputs(flat, cells))
        print(name, os.path.getsize(name), "bytes", out["counters"])


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else None)
