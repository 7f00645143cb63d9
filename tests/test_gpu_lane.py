"""The lane-per-cell mapping of the integrator (FCS_MAPPING_LANE, one thread
per cell, csrc/fcs_lane.cuh) through the C ABI.

It runs the same arithmetic as the cell-group kernels except for the order of
the mixture sums over species (serial here, butterfly reductions there), so it
is held to the same tolerances against the reference's golden outputs as the
group mappings (test_gpu_parity.py), and against the group mapping itself on
the same cells.
"""
import os

import numpy as np
import pytest

import fcs
from conftest import GOLDEN
from golden import fixture

pytestmark = pytest.mark.gpu

LANE = 1


@pytest.fixture(scope="module")
def built():
    import __graft_entry__
    __graft_entry__.build()
    return True


def _ctx(flat, **opt):
    from fcs import _lib
    c = _lib.Context(0)
    c.load_mechanism(flat)
    c.set_options(**opt)
    return c


def _setup(wname, n=None, idx=None):
    w = fcs.WORKLOADS[wname]
    mech = w.mechanism()
    flat = fcs.flatten(mech)
    full = fcs.cells_for(w, mech)
    if idx is None:
        idx = np.linspace(0, w.n_cells - 1, n).astype(np.int64)
    return w, mech, flat, full.subset(idx)


ROSENBROCK_GOLDEN = ["ignition_10s_OptRodas34", "ignition_10s_OptRosenbrock34", "ignition_10s_OptRodas23",
                     "ignition_10s_OptRosenbrock23", "counterflow_53s_OptRodas34", "counterflow_53s_OptRosenbrock34",
                     "counterflow_53s_OptRodas23", "counterflow_53s_OptRosenbrock23", "falloff_16s_OptRodas34",
                     "falloff_16s_OptRosenbrock34", "falloff_16s_OptRodas23", "noneq_14s_OptRodas34",
                     "noneq_14s_OptRosenbrock23", "long_24s_OptRodas34"]


@pytest.mark.parametrize("case", ROSENBROCK_GOLDEN)
def test_lane_integration_matches_reference_golden(built, case):
    wname, solver = case.rsplit("_", 1)
    g = np.load(os.path.join(GOLDEN, case + ".npz"))
    w = fcs.WORKLOADS[wname]
    flat, c = fixture.load(g)
    ctx = _ctx(flat, solver=solver, abs_tol=w.abs_tol, rel_tol=w.rel_tol, mapping=LANE)
    out = ctx.integrate(c, w.dt)
    assert out["stats"]["mapping"] == LANE
    assert (out["status"] == g["status"]).all()
    rtol, atol = (1e-9, 1e-10) if wname == "ignition_10s" else (1e-7, 1e-8)
    np.testing.assert_allclose(out["T"], g["T"], rtol=rtol, atol=0)
    np.testing.assert_allclose(out["Y"], g["Y"], rtol=0, atol=atol)
    np.testing.assert_allclose(out["RR"], g["RR"], rtol=0, atol=atol * np.abs(g["RR"]).max() / 1e-3 + 1e-12)
    # the suggested next sub-step follows the last controller decision, which
    # rounding can tip (as for the group mappings): most cells agree closely
    assert np.isclose(out["subDt"], g["subDt"], rtol=1e-6).mean() >= 0.75
    njac = int(g["jacobians"])
    assert abs(out["stats"]["jacobians"] - njac) <= max(4, 0.01 * njac)


@pytest.mark.parametrize("wname,n", [("counterflow_53s", 2048), ("falloff_16s", 512)])
def test_lane_matches_group_mapping(built, wname, n):
    """Many cells (lanes refill from the queue), Treact skipping a third of
    them: the lane mapping against the 64-thread group mapping."""
    w, mech, flat, c = _setup(wname, n)
    treact = float(np.percentile(c.T, 33))
    a = _ctx(flat, abs_tol=w.abs_tol, rel_tol=w.rel_tol, mapping=64, treact=treact).integrate(c, w.dt)
    b = _ctx(flat, abs_tol=w.abs_tol, rel_tol=w.rel_tol, mapping=LANE, treact=treact).integrate(c, w.dt)
    np.testing.assert_array_equal(b["status"], a["status"])
    assert (a["status"] == 4).sum() > 0 and (a["status"] == 0).sum() > 0
    for k in ("cells_integrated", "cells_skipped", "cells_failed"):
        assert b["stats"][k] == a["stats"][k], k
    assert abs(b["stats"]["attempts"] - a["stats"]["attempts"]) <= 0.002 * a["stats"]["attempts"] + 4
    # the mixture sums run in a different order: rounding-level differences,
    # grown through ~250 stiff steps.  Most cells take the same steps and
    # agree to the golden-fixture tolerances; a cell whose rounding tips one
    # accept/reject decision takes other steps and lands elsewhere within the
    # integration tolerance (relTol 1e-4).
    eT = np.abs(b["T"] - a["T"]) / a["T"]
    eY = np.abs(b["Y"] - a["Y"]).max(axis=0)
    close = (eT <= 1e-7) & (eY <= 1e-8)
    assert close.mean() >= 0.99, close.mean()
    assert eT.max() <= 1e-4 and eY.max() <= 1e-5, (eT.max(), eY.max())
    eR = np.abs(b["RR"] - a["RR"]).max(axis=0) * w.dt / c.rho0  # RR back in units of Y
    assert eR.max() <= 1e-5
    assert b["deltaTMin"] == pytest.approx(a["deltaTMin"], rel=1e-6)


def test_lane_failure_statuses_and_lts(built):
    """maxSteps and NaN pressure fail only their own cells, as with the group
    mapping; the other cells are still integrated; per-cell delta_t (LTS)."""
    import oracle
    w, mech, flat, c = _setup("ignition_10s", 96)
    c.p[5] = np.nan
    ctx = _ctx(flat, abs_tol=w.abs_tol, rel_tol=w.rel_tol, mapping=LANE, max_steps=3)
    out = ctx.integrate(c, w.dt)
    grp = _ctx(flat, abs_tol=w.abs_tol, rel_tol=w.rel_tol, mapping=64, max_steps=3).integrate(c, w.dt)
    np.testing.assert_array_equal(out["status"], grp["status"])
    assert out["status"][5] == 2 and (out["status"] == 1).sum() > 10
    np.testing.assert_array_equal(out["subDt"], grp["subDt"])   # failed cells keep their sub-step
    ctx.set_options(abs_tol=w.abs_tol, rel_tol=w.rel_tol, mapping=LANE)
    out = ctx.integrate(c, w.dt)
    ref = oracle.Port(flat).integrate(c.subset(np.arange(5)), w.dt, abs_tol=w.abs_tol, rel_tol=w.rel_tol)
    assert out["status"][5] == 2 and (np.delete(out["status"], 5) == 0).all()
    np.testing.assert_allclose(out["T"][:5], ref["T"], rtol=1e-9)
    # LTS: per-cell delta_t
    w, mech, flat, c = _setup("ignition_10s", 64)
    dtc = np.geomspace(1e-7, 2e-5, c.n)
    ref = oracle.Port(flat).integrate(c, 0.0, dt_per_cell=dtc, abs_tol=w.abs_tol, rel_tol=w.rel_tol)
    out = _ctx(flat, abs_tol=w.abs_tol, rel_tol=w.rel_tol, mapping=LANE).integrate(c, None, dt_per_cell=dtc)
    assert (out["status"] == 0).all()
    np.testing.assert_allclose(out["T"], ref["T"], rtol=1e-9)
    np.testing.assert_allclose(out["Y"], ref["Y"], atol=1e-10)


def test_lane_graph_and_async_paths(built):
    """The lane mapping inside the per-step CUDA graph and the asynchronous
    step gives the same cells as the synchronous call."""
    import torch
    w, mech, flat, c = _setup("counterflow_53s", 1024)
    ctx = _ctx(flat, abs_tol=w.abs_tol, rel_tol=w.rel_tol, mapping=LANE)

    def dev():
        d = {k: torch.from_numpy(np.ascontiguousarray(getattr(c, k))).cuda() for k in ("p", "rho0", "T", "Y", "subDt")}
        d["RR"] = torch.zeros_like(d["Y"])
        d["status"] = torch.full((c.n,), -1, dtype=torch.int32, device="cuda")
        return d
    outs = []
    for flags in (2, 4, 4):  # natural order; graph captured; graph replayed
        d = dev()
        code, stats, _ = ctx.integrate_raw(c.n, w.dt, d["p"], d["rho0"], d["T"], d["Y"], d["subDt"], d["RR"],
                                           d["status"], device=True, flags=flags)
        assert code == 0 and stats["mapping"] == LANE
        outs.append(d)
    d = dev()
    ctx.integrate_async(c.n, w.dt, d["p"], d["rho0"], d["T"], d["Y"], d["subDt"], d["RR"], d["status"])
    code, stats, _ = ctx.sync()
    assert code == 0 and stats["mapping"] == LANE
    outs.append(d)
    for d in outs[1:]:
        for k in ("T", "Y", "subDt", "RR", "status"):
            np.testing.assert_array_equal(d[k].cpu().numpy(), outs[0][k].cpu().numpy(), err_msg=k)


def test_lane_refused_where_it_does_not_apply(built):
    from fcs import _lib
    w, mech, flat, c = _setup("ignition_10s", 8)
    ctx = _ctx(flat, solver="OptSeulex", mapping=LANE)
    code, _, _ = ctx.integrate_raw(c.n, w.dt, c.p, c.rho0, c.T.copy(), c.Y.copy(), c.subDt.copy(), check=False)
    assert code == 6  # FCS_ERR_UNSUPPORTED: Seulex runs on cell groups
    ctx.set_options(mapping=LANE)
    f = ctx.rhs(c.p, c.T, c.Y)  # the per-cell evaluations use cell groups
    assert np.isfinite(f).all()


@pytest.mark.parametrize("fixture_name,wname", [("counterflow_53s_tight", "counterflow_53s"),
                                                ("large_200s_tight", "large_200s")])
@pytest.mark.parametrize("solver", ["OptRodas34", "OptRosenbrock34"])
def test_lane_mixed_precision_accuracy(built, fixture_name, wname, solver):
    """The lane mapping in mixed precision (FP32 factors of the equilibrated
    iteration matrix, one FP64-residual refinement per solve, an attempt
    whose correction is not small redone in FP64) against the reference's
    tight run: no cell lost, within 2x of the FP64 method's own error plus a
    floor, <= 1e-3 relative in T."""
    g = np.load(os.path.join(GOLDEN, fixture_name + ".npz"))
    w = fcs.WORKLOADS[wname]
    flat, c = fixture.load(g)
    ctx = _ctx(flat, solver=solver, abs_tol=w.abs_tol, rel_tol=w.rel_tol, precision="fp64", mapping=LANE)
    f64 = ctx.integrate(c, w.dt)
    ctx.set_options(solver=solver, abs_tol=w.abs_tol, rel_tol=w.rel_tol, precision="mixed", mapping=LANE)
    mix = ctx.integrate(c, w.dt)
    assert mix["stats"]["mapping"] == LANE
    assert (mix["status"] == 0).all() and (f64["status"] == 0).all()
    eT64 = np.max(np.abs(f64["T"] - g["T"]) / g["T"])
    eY64 = np.max(np.abs(f64["Y"] - g["Y"]))
    eT = np.max(np.abs(mix["T"] - g["T"]) / g["T"])
    eY = np.max(np.abs(mix["Y"] - g["Y"]))
    assert eT <= 2 * eT64 + 1e-5 and eT <= 1e-3, (eT, eT64)
    assert eY <= 2 * eY64 + 1e-6, (eY, eY64)
    # the FP64 redo is the exception, not the rule
    assert mix["stats"]["fp64_fallbacks"] <= 0.25 * mix["stats"]["attempts"]
