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


def main(only=None):
    """Regenerate every fixture, or only those whose file name contains `only`."""
    oracle.build(ref=True)
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
            rhs=f, jac=J[: min(4, n)], jac_f=fj, **inputs(flat, cells))
        print(name, os.path.getsize(name), "bytes", out["counters"])


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else None)
