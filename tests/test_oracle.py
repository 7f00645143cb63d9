"""The CPU oracle (plain-C restatement) against the reference's own outputs:
golden fixtures made by tests/golden/make_golden.py from the reference core
compiled unmodified, and -- where the reference tree is present on an x86-64
host -- the compiled reference itself."""
import os

import numpy as np
import pytest

import fcs
from conftest import GOLDEN
from golden import fixture

FCS_CELL_MAX_STEPS = 1


def _golden(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


CASES = ["ignition_10s_OptRodas34", "ignition_10s_OptRosenbrock34", "ignition_10s_OptSeulex",
         "counterflow_53s_OptRodas34", "counterflow_53s_OptRosenbrock34", "counterflow_53s_OptSeulex",
         "ignition_10s_OptRodas23", "ignition_10s_OptRosenbrock23",
         "counterflow_53s_OptRodas23", "counterflow_53s_OptRosenbrock23",
         "falloff_16s_OptRodas34", "falloff_16s_OptSeulex",
         "noneq_14s_OptRodas34", "noneq_14s_OptSeulex", "long_24s_OptRodas34",
         "falloff_16s_OptRosenbrock34", "falloff_16s_OptRodas23", "noneq_14s_OptRosenbrock23", "long_24s_OptSeulex"]


def _setup(case):
    wname, solver = case.rsplit("_", 1)
    w = fcs.WORKLOADS[wname]
    g = _golden(case)
    flat, cells = fixture.load(g)
    return w, flat, solver, g, cells


@pytest.mark.parametrize("case", CASES + ["ignition_10s_tight", "counterflow_53s_tight", "large_200s_tight",
                                  "uneven_111s_OptRodas34", "large_200s_OptRodas34"])
def test_generator_reproduces_fixture_inputs(case):
    fixture.check_generator(_golden(case), case.rsplit("_", 1)[0])


@pytest.mark.parametrize("case", CASES)
def test_port_matches_reference_integration(case, port_built):
    import oracle
    w, flat, solver, g, cells = _setup(case)
    port = oracle.Port(flat)
    out = port.integrate(cells, w.dt, solver=solver, abs_tol=w.abs_tol, rel_tol=w.rel_tol, treact=w.treact)
    assert (out["status"] == g["status"]).all()
    # Same algorithm and step sequence: rounding-level differences (libmvec vs
    # libm exp, summation order) grow through ~240 stiff steps per cell of the
    # 53-species workload but stay >1000x below relTol = 1e-4.
    rtol, atol = (1e-9, 1e-10) if case.startswith("ignition") else (1e-7, 1e-8)
    np.testing.assert_allclose(out["T"], g["T"], rtol=rtol, atol=0)
    np.testing.assert_allclose(out["Y"], g["Y"], rtol=0, atol=atol)
    if solver == "OptSeulex":
        # The last Seulex step lands on xEnd or one ulp short of it depending on
        # rounding; one ulp short adds a ~1e-21 s step that changes only the
        # suggested next sub-step (by up to ~2x), not the state.  On the
        # fixtures 84-100 % of the cells agree.
        close = np.isclose(out["subDt"], g["subDt"], rtol=1e-6)
        assert close.mean() >= 0.8
        assert abs(out["counters"]["jacobians"] - int(g["jacobians"])) <= max(4, 0.01 * int(g["jacobians"]))
    else:
        np.testing.assert_allclose(out["subDt"], g["subDt"], rtol=1e-6 if rtol < 1e-8 else 1e-2)
        assert abs(out["counters"]["jacobians"] - int(g["jacobians"])) <= max(2, 0.002 * int(g["jacobians"]))


@pytest.mark.parametrize("case", ["ignition_10s_OptRodas34", "counterflow_53s_OptRodas34", "falloff_16s_OptRodas34",
                                  "noneq_14s_OptRodas34", "long_24s_OptRodas34"])
def test_port_matches_reference_rhs_and_jacobian(case, port_built):
    import oracle
    w, flat, solver, g, cells = _setup(case)
    port = oracle.Port(flat)
    f = port.rhs(cells.p, cells.T, cells.Y)
    scale = np.abs(g["rhs"]).max(axis=1, keepdims=True) + 1e-300
    assert np.max(np.abs(f - g["rhs"]) / scale) < 1e-13
    k = g["jac"].shape[0]
    J, fj = port.jacobian(cells.p[:k], cells.T[:k], cells.Y[:, :k])
    sJ = np.abs(g["jac"]).max(axis=(1, 2), keepdims=True)
    assert np.max(np.abs(J - g["jac"]) / sJ) < 1e-12
    Jw, _ = port.jacobian(cells.p[:k], cells.T[:k], cells.Y[:, :k], as_written=True)
    assert np.max(np.abs(Jw - g["jac"]) / sJ) < 1e-12


def test_port_lu_pivoting_matches_reference(port_built):
    """Panel-restricted pivoting with the reference quirks (signed running max
    in the second step, exact-zero pivots replaced by 2.2e-16)."""
    import oracle
    if not os.path.exists(oracle.REF_SO):
        pytest.skip("reference core not built on this host")
    rng = np.random.default_rng(3)
    w = fcs.WORKLOADS["ignition_10s"]
    flat = fcs.flatten(w.mechanism())
    port, ref = oracle.Port(flat), oracle.Reference(flat)
    for n in (5, 6, 7, 8, 11, 12, 13, 54):
        for trial in range(4):
            a = rng.normal(size=(n, n))
            if trial == 1:
                a[:, 0] *= 1e-6
            if trial == 2:
                a[1, 1] = 0.0
                a[0, 0] = 0.0
            b = rng.normal(size=(3, n))
            _, x1, _, _ = port.lu_solve(a, b)
            _, x0 = ref.lu_solve(a, b)
            np.testing.assert_allclose(x1, x0, rtol=1e-9, atol=1e-9)


def test_port_against_compiled_reference_directly(port_built):
    import oracle
    if not os.path.exists(oracle.REF_SO):
        pytest.skip("reference core not built on this host")
    w = fcs.WORKLOADS["uneven_111s"]
    mech = w.mechanism()
    flat = fcs.flatten(mech)
    cells = fcs.cells_for(w, mech, n=48).subset(np.arange(0, 48, 6))
    ref = oracle.Reference(flat, abs_tol=w.abs_tol, rel_tol=w.rel_tol)
    port = oracle.Port(flat)
    f0 = ref.rhs(cells.p, cells.T, cells.Y)
    f1 = port.rhs(cells.p, cells.T, cells.Y)
    assert np.max(np.abs(f1 - f0) / (np.abs(f0).max(axis=1, keepdims=True) + 1e-300)) < 1e-13
    r0 = ref.integrate(cells, w.dt, treact=w.treact)
    r1 = port.integrate(cells, w.dt, abs_tol=w.abs_tol, rel_tol=w.rel_tol, treact=w.treact)
    assert (r0["status"] == r1["status"]).all()
    np.testing.assert_allclose(r1["T"], r0["T"], rtol=1e-8)
    np.testing.assert_allclose(r1["Y"], r0["Y"], atol=1e-9)


@pytest.mark.parametrize("wname", ["counterflow_53s", "falloff_16s", "noneq_14s"])
def test_port_fast_jacobian_against_compiled_reference(wname, port_built):
    """`jacobian fast` (FastddYdtdY_Vec, Jacobian.C:4541-4568: the dC/dY
    conversion without the rank-1 term): the oracle's Jacobian and a CFD step
    integrated with it, against the reference core compiled from its sources."""
    import oracle
    if not os.path.exists(oracle.REF_SO):
        pytest.skip("reference core not built on this host")
    w = fcs.WORKLOADS[wname]
    mech = w.mechanism()
    flat = fcs.flatten(mech)
    cells = fcs.cells_for(w, mech, n=64).subset(np.arange(0, 64, 16))
    ref = oracle.Reference(flat, jacobian="fast", abs_tol=w.abs_tol, rel_tol=w.rel_tol)
    port = oracle.Port(flat)
    J0, _ = ref.jacobian(cells.p, cells.T, cells.Y)
    J1, _ = port.jacobian(cells.p, cells.T, cells.Y, jacobian="fast")
    Je, _ = port.jacobian(cells.p, cells.T, cells.Y)
    scale = np.abs(J0).max(axis=(1, 2), keepdims=True)
    assert np.max(np.abs(J1 - J0) / scale) < 1e-12
    assert np.max(np.abs(Je - J0) / scale) > 1e-9  # the exact conversion differs: the mode took effect
    r0 = ref.integrate(cells, w.dt, treact=w.treact)
    r1 = port.integrate(cells, w.dt, jacobian="fast", abs_tol=w.abs_tol, rel_tol=w.rel_tol, treact=w.treact)
    assert (r0["status"] == r1["status"]).all()
    np.testing.assert_allclose(r1["T"], r0["T"], rtol=1e-8)
    np.testing.assert_allclose(r1["Y"], r0["Y"], atol=1e-9)
    assert abs(int(r1["counters"]["jacobians"]) - int(r0["counters"]["jacobians"])) <= 2 * cells.n


@pytest.mark.parametrize("solver", ["OptRodas34", "OptSeulex"])
def test_port_max_steps_status_against_compiled_reference(solver, port_built):
    """maxSteps, the reference's only failure path (FatalError at
    OptRodas34.C:193, OptSeulex.C:252): with a step budget that only some of
    the cells finish in, the oracle fails exactly the cells the reference
    core fails, and the others finish as in the reference."""
    import oracle
    if not os.path.exists(oracle.REF_SO):
        pytest.skip("reference core not built on this host")
    w = fcs.WORKLOADS["counterflow_53s"]
    mech = w.mechanism()
    flat = fcs.flatten(mech)
    cells = fcs.cells_for(w, mech).subset(np.linspace(0, w.n_cells - 1, 12).astype(np.int64))
    # the smallest of these budgets that some but not all of the cells finish in
    for steps in (8, 16, 32, 64, 128, 256):
        ref = oracle.Reference(flat, solver=solver, abs_tol=w.abs_tol, rel_tol=w.rel_tol, max_steps=steps)
        r0 = ref.integrate(cells, w.dt)
        failed = r0["status"] == FCS_CELL_MAX_STEPS
        if failed.any() and not failed.all():
            break
    assert failed.any() and not failed.all(), r0["status"]
    r1 = oracle.Port(flat).integrate(cells, w.dt, solver=solver, abs_tol=w.abs_tol, rel_tol=w.rel_tol,
                                     max_steps=steps)
    np.testing.assert_array_equal(r1["status"], r0["status"])
    ok = ~failed  # the 53-species tolerances of the golden comparisons (libm vs libmvec exp, sum order)
    np.testing.assert_allclose(r1["T"][ok], r0["T"][ok], rtol=1e-7)
    np.testing.assert_allclose(r1["Y"][:, ok], r0["Y"][:, ok], atol=1e-8)


@pytest.mark.parametrize("wname", ["ignition_10s", "counterflow_53s", "uneven_111s", "falloff_16s", "noneq_14s", "long_24s"])
def test_port_tc_matches_reference_golden(wname, port_built):
    """FastChemistryModel::tc() of the reference (tests/golden/tc.npz)."""
    import oracle
    g = _golden("tc")
    flat, cells = fixture.load_prefixed(g, wname + "__")
    tc = oracle.Port(flat).tc(cells.p, cells.T, cells.rho0, cells.Y)
    np.testing.assert_allclose(tc, g[wname + "__tc"], rtol=1e-13)


@pytest.mark.parametrize("case", ["uneven_111s_OptRodas34", "large_200s_OptRodas34", "tutorial_nc12h26_narayanaswamy",
                                  "tutorial_ic8h18_yoo", "tutorial_ch4_gri30_counterflow"])
def test_port_matches_reference_on_large_and_tutorial_inputs(case, port_built):
    """The 111- and 200-species fields and the reference's own tutorial
    mechanisms (255 and 140 species) and counterflow-flame cells: the port
    against the reference core's integration, RHS and Jacobian."""
    import oracle
    g = _golden(case)
    flat, cells = fixture.load(g)
    if case.startswith("tutorial"):
        dt, treact = float(g["dt"]), 0.0
    else:
        w = fcs.WORKLOADS[case.rsplit("_", 1)[0]]
        dt, treact = w.dt, w.treact
    port = oracle.Port(flat)
    out = port.integrate(cells, dt, abs_tol=float(g["abs_tol"]), rel_tol=float(g["rel_tol"]), treact=treact,
                         threads=8)
    assert (out["status"] == g["status"]).all()
    np.testing.assert_allclose(out["T"], g["T"], rtol=1e-7, atol=0)
    np.testing.assert_allclose(out["Y"], g["Y"], rtol=0, atol=1e-8)
    assert abs(out["counters"]["jacobians"] - int(g["jacobians"])) <= max(4, 0.01 * int(g["jacobians"]))
    f = port.rhs(cells.p, cells.T, cells.Y)
    assert np.max(np.abs(f - g["rhs"]) / (np.abs(g["rhs"]).max(axis=1, keepdims=True) + 1e-300)) < 1e-12
    k = g["jac"].shape[0]
    J, _ = port.jacobian(cells.p[:k], cells.T[:k], cells.Y[:, :k])
    assert np.max(np.abs(J - g["jac"]) / np.abs(g["jac"]).max(axis=(1, 2), keepdims=True)) < 1e-12
