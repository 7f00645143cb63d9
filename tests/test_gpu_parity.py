"""GPU parity: the sm_103a path through the C ABI against the CPU oracle and
the reference's golden outputs.

Tolerances (written per test): the FP64 method follows the reference's
arithmetic step for step, so its results differ from the oracle only by
rounding (different exp implementation and summation order) amplified through
the stiff integration -- far below the integration tolerance.  The mixed
method (FP32 Jacobian storage and LU + FP64-residual refinement) is compared
with the reference run at absTol 1e-14 / relTol 1e-10 and must stay as close
to it as the FP64 method at the same tolerances.
"""
import ctypes
import os

import numpy as np
import pytest

import fcs
from conftest import GOLDEN
from golden import fixture

pytestmark = pytest.mark.gpu


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


def test_exp_against_cuda(built):
    from fcs import _lib
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.uniform(-706, 706, 200000), rng.uniform(-5, 5, 100000),
                        np.array([0.0, -0.0, 1e-300, -1e-300, 706.9, -706.9, 710.0, -746.0, 800.0, np.inf,
                                  -np.inf, np.nan])])
    a, b = _lib.check_exp(x)
    fin = np.isfinite(b) & (b > 0)
    ulp = np.abs(a[fin] - b[fin]) / np.spacing(b[fin])
    assert ulp.max() <= 2.0, ulp.max()
    assert np.mean(ulp) < 0.5
    np.testing.assert_array_equal(np.isnan(a), np.isnan(b))
    np.testing.assert_array_equal(a[~fin & ~np.isnan(b)], b[~fin & ~np.isnan(b)])


@pytest.mark.parametrize("wname,n", [("ignition_10s", 64), ("counterflow_53s", 32), ("uneven_111s", 16),
                                     ("large_200s", 4), ("falloff_16s", 64), ("noneq_14s", 64),
                                     ("long_24s", 64)])
def test_rhs_and_jacobian_match_oracle(built, wname, n):
    import oracle
    w, mech, flat, c = _setup(wname, n)
    port = oracle.Port(flat)
    ctx = _ctx(flat)
    f0 = port.rhs(c.p, c.T, c.Y)
    f1 = ctx.rhs(c.p, c.T, c.Y)
    scale = np.abs(f0).max(axis=1, keepdims=True) + 1e-300
    assert np.max(np.abs(f1 - f0) / scale) < 1e-12
    J0, g0 = port.jacobian(c.p, c.T, c.Y)
    J1, g1 = ctx.jacobian(c.p, c.T, c.Y)
    sJ = np.abs(J0).max(axis=(1, 2), keepdims=True)
    assert np.max(np.abs(J1 - J0) / sJ) < 1e-12
    assert np.max(np.abs(g1 - g0) / (np.abs(g0).max(axis=1, keepdims=True) + 1e-300)) < 1e-12


def test_fast_jacobian_matches_oracle(built):
    import oracle
    w, mech, flat, c = _setup("counterflow_53s", 16)
    port = oracle.Port(flat)
    ctx = _ctx(flat, jacobian="fast")
    J0, _ = port.jacobian(c.p, c.T, c.Y, jacobian="fast")
    J1, _ = ctx.jacobian(c.p, c.T, c.Y)
    sJ = np.abs(J0).max(axis=(1, 2), keepdims=True)
    assert np.max(np.abs(J1 - J0) / sJ) < 1e-12


GOLDEN_CASES = ["ignition_10s_OptRodas34", "ignition_10s_OptRosenbrock34", "ignition_10s_OptSeulex",
                "counterflow_53s_OptRodas34", "counterflow_53s_OptRosenbrock34", "counterflow_53s_OptSeulex",
                "ignition_10s_OptRodas23", "ignition_10s_OptRosenbrock23",
                "counterflow_53s_OptRodas23", "counterflow_53s_OptRosenbrock23",
                "falloff_16s_OptRodas34", "falloff_16s_OptSeulex",
                "noneq_14s_OptRodas34", "noneq_14s_OptSeulex", "long_24s_OptRodas34",
                "falloff_16s_OptRosenbrock34", "falloff_16s_OptRodas23", "noneq_14s_OptRosenbrock23", "long_24s_OptSeulex"]


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_fp64_integration_matches_reference_golden(built, case):
    """The reference's own integrator outputs (tests/golden, made by the
    reference core compiled from its sources)."""
    wname, solver = case.rsplit("_", 1)
    g = np.load(os.path.join(GOLDEN, case + ".npz"))
    w = fcs.WORKLOADS[wname]
    flat, c = fixture.load(g)
    ctx = _ctx(flat, solver=solver, abs_tol=w.abs_tol, rel_tol=w.rel_tol)
    out = ctx.integrate(c, w.dt)
    assert (out["status"] == g["status"]).all()
    rtol, atol = (1e-9, 1e-10) if wname == "ignition_10s" else (1e-7, 1e-8)
    np.testing.assert_allclose(out["T"], g["T"], rtol=rtol, atol=0)
    np.testing.assert_allclose(out["Y"], g["Y"], rtol=0, atol=atol)
    np.testing.assert_allclose(out["RR"], g["RR"], rtol=0, atol=atol * np.abs(g["RR"]).max() / 1e-3 + 1e-12)
    njac = int(g["jacobians"])
    assert abs(out["stats"]["jacobians"] - njac) <= max(4, 0.01 * njac)


@pytest.mark.parametrize("mapping", [32, 64, 128, 256])
def test_mappings_agree(built, mapping):
    """Every cell-to-thread mapping integrates the same cells to the same result."""
    import oracle
    w, mech, flat, c = _setup("counterflow_53s", 24)
    ref = oracle.Port(flat).integrate(c, w.dt, abs_tol=w.abs_tol, rel_tol=w.rel_tol, threads=8)
    ctx = _ctx(flat, abs_tol=w.abs_tol, rel_tol=w.rel_tol, mapping=mapping)
    out = ctx.integrate(c, w.dt)
    assert (out["status"] == 0).all()
    np.testing.assert_allclose(out["T"], ref["T"], rtol=1e-7)
    np.testing.assert_allclose(out["Y"], ref["Y"], atol=1e-8)


@pytest.mark.parametrize("solver", ["OptRodas34", "OptRosenbrock34", "OptSeulex", "OptRodas23", "OptRosenbrock23"])
def test_mixed_precision_accuracy(built, solver):
    """Mixed precision against the reference Rodas34 run at absTol 1e-14 /
    relTol 1e-10 (tests/golden/*_tight.npz).  At the workload's own tolerances
    (1e-8 / 1e-4) the FP64 method itself sits ~1e-4 (T) / ~4e-5 (Y) away from
    that solution on these stiff cells, so the mixed method must (a) lose no
    cell, (b) stay within 2x (+ a small floor) of the FP64 method's error, and
    (c) for the Rosenbrock methods stay <= 1e-3 relative in T."""
    g = np.load(os.path.join(GOLDEN, "counterflow_53s_tight.npz"))
    w = fcs.WORKLOADS["counterflow_53s"]
    flat, c = fixture.load(g)
    ctx = _ctx(flat, solver=solver, abs_tol=w.abs_tol, rel_tol=w.rel_tol, precision="fp64")
    f64 = ctx.integrate(c, w.dt)
    ctx.set_options(solver=solver, abs_tol=w.abs_tol, rel_tol=w.rel_tol, precision="mixed")
    mix = ctx.integrate(c, w.dt)
    assert (mix["status"] == 0).all() and (f64["status"] == 0).all()
    eT64 = np.max(np.abs(f64["T"] - g["T"]) / g["T"])
    eY64 = np.max(np.abs(f64["Y"] - g["Y"]))
    eT = np.max(np.abs(mix["T"] - g["T"]) / g["T"])
    eY = np.max(np.abs(mix["Y"] - g["Y"]))
    assert eT <= 2 * eT64 + 1e-5, (eT, eT64)
    assert eY <= 2 * eY64 + 1e-6, (eY, eY64)
    if solver != "OptSeulex":
        assert eT <= 1e-3


def test_fp64_error_against_tight_reference(built):
    """FP64 GPU Rodas34 at the workload tolerances vs the tight reference:
    the same error as the reference integrator itself at those tolerances."""
    g = np.load(os.path.join(GOLDEN, "ignition_10s_tight.npz"))
    w = fcs.WORKLOADS["ignition_10s"]
    flat, c = fixture.load(g)
    ctx = _ctx(flat, abs_tol=w.abs_tol, rel_tol=w.rel_tol)
    out = ctx.integrate(c, w.dt)
    assert np.max(np.abs(out["T"] - g["T"]) / g["T"]) <= 1e-5
    assert np.max(np.abs(out["Y"] - g["Y"])) <= 1e-5


def test_treact_skip_and_deltatmin(built):
    import oracle
    w, mech, flat, c = _setup("uneven_111s", 40)
    ctx = _ctx(flat, abs_tol=w.abs_tol, rel_tol=w.rel_tol, treact=w.treact, dt_chem_max=2e-6)
    out = ctx.integrate(c, w.dt)
    ref = oracle.Port(flat).integrate(c, w.dt, abs_tol=w.abs_tol, rel_tol=w.rel_tol, treact=w.treact,
                                      dt_chem_max=2e-6, threads=8)
    skipped = c.T <= w.treact
    assert skipped.any() and (~skipped).any()
    assert (out["status"][skipped] == 4).all() and (out["status"][~skipped] == 0).all()
    assert (out["RR"][:, skipped] == 0).all()
    np.testing.assert_array_equal(out["T"][skipped], c.T[skipped])
    np.testing.assert_allclose(out["T"], ref["T"], rtol=1e-7)
    assert out["subDt"].max() <= 2e-6
    np.testing.assert_allclose(out["deltaTMin"], ref["deltaTMin"], rtol=1e-2)
    assert out["stats"]["cells_skipped"] == int(skipped.sum())


def test_failure_statuses_keep_other_cells(built):
    """Failures come back as per-cell statuses; the other cells are still right."""
    import oracle
    w, mech, flat, c = _setup("ignition_10s", 8)
    c.p[3] = np.nan          # poisoned pressure: non-finite rates in that cell only
    c.T[5] = np.nan          # NaN fails `T > Treact`: skipped like the reference (transientSolve.H:39)
    ctx = _ctx(flat, abs_tol=w.abs_tol, rel_tol=w.rel_tol)
    out = ctx.integrate(c, w.dt)
    assert out["code"] == 5  # FCS_ERR_CELLS
    assert out["status"][3] == 2 and out["status"][5] == 4
    good = (np.arange(8) != 3) & (np.arange(8) != 5)
    assert (out["status"][good] == 0).all()
    ref = oracle.Port(flat).integrate(c.subset(np.where(good)[0]), w.dt, abs_tol=w.abs_tol, rel_tol=w.rel_tol)
    np.testing.assert_allclose(out["T"][good], ref["T"], rtol=1e-9)
    # maxSteps exceeded (fatal in the reference) is a status, not an abort
    ctx.set_options(abs_tol=w.abs_tol, rel_tol=w.rel_tol, max_steps=2)
    c2 = _setup("ignition_10s", 4)[3]
    out2 = ctx.integrate(c2, w.dt)
    assert (out2["status"] == 1).all() and out2["stats"]["cells_failed"] == 4
    # the context stays usable
    ctx.set_options(abs_tol=w.abs_tol, rel_tol=w.rel_tol)
    out3 = ctx.integrate(c2, w.dt)
    assert (out3["status"] == 0).all()


def test_local_time_step_variant(built):
    import oracle
    w, mech, flat, c = _setup("ignition_10s", 16)
    dts = np.geomspace(1e-6, 2e-5, 16)
    ctx = _ctx(flat, abs_tol=w.abs_tol, rel_tol=w.rel_tol)
    out = ctx.integrate(c, None, dt_per_cell=dts)
    ref = oracle.Port(flat).integrate(c, 0.0, dt_per_cell=dts, abs_tol=w.abs_tol, rel_tol=w.rel_tol)
    np.testing.assert_allclose(out["T"], ref["T"], rtol=1e-9)
    np.testing.assert_allclose(out["RR"], ref["RR"], rtol=1e-6, atol=1e-8 * np.abs(ref["RR"]).max())


def test_device_pointer_mode(built):
    import torch
    w, mech, flat, c = _setup("ignition_10s", 32)
    ctx = _ctx(flat, abs_tol=w.abs_tol, rel_tol=w.rel_tol)
    host = ctx.integrate(c, w.dt)
    d = {k: torch.from_numpy(np.ascontiguousarray(getattr(c, k))).cuda() for k in ("p", "rho0", "T", "Y", "subDt")}
    RR = torch.zeros_like(d["Y"])
    st = torch.zeros(c.n, dtype=torch.int32, device="cuda")
    code, stats, dmin = ctx.integrate_raw(c.n, w.dt, d["p"], d["rho0"], d["T"], d["Y"], d["subDt"], RR, st,
                                          device=True)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(d["T"].cpu().numpy(), host["T"])
    np.testing.assert_array_equal(d["Y"].cpu().numpy(), host["Y"])
    np.testing.assert_array_equal(RR.cpu().numpy(), host["RR"])


def test_rates_and_qdot_match_oracle(built):
    import oracle
    w, mech, flat, c = _setup("counterflow_53s", 32)
    ctx = _ctx(flat)
    RR1, Q1 = ctx.rates(c.p, c.T, c.rho0, c.Y)
    RR0, Q0 = oracle.Port(flat).rates(c.p, c.T, c.rho0, c.Y)
    assert np.max(np.abs(RR1 - RR0) / (np.abs(RR0).max(axis=1, keepdims=True) + 1e-300)) < 1e-12
    np.testing.assert_allclose(Q1, Q0, rtol=1e-10, atol=1e-12 * np.abs(Q0).max())


def test_strided_host_inputs(built):
    """Views with strides (a column slice of a species-major field) give the
    same rates, Jacobian and tc as contiguous copies."""
    w, mech, flat, c = _setup("noneq_14s", 32)
    ctx = _ctx(flat)
    p, T, rho, Y = c.p[::2], c.T[::2], c.rho0[::2], c.Y[:, ::2]
    pc, Tc, rc, Yc = (np.ascontiguousarray(a) for a in (p, T, rho, Y))
    np.testing.assert_array_equal(ctx.rhs(p, T, Y), ctx.rhs(pc, Tc, Yc))
    J0, f0 = ctx.jacobian(pc, Tc, Yc)
    J1, f1 = ctx.jacobian(p, T, Y)
    np.testing.assert_array_equal(J1, J0)
    np.testing.assert_array_equal(ctx.tc(p, T, rho, Y), ctx.tc(pc, Tc, rc, Yc))
    np.testing.assert_array_equal(ctx.rates(p, T, rho, Y)[0], ctx.rates(pc, Tc, rc, Yc)[0])


@pytest.mark.parametrize("wname", ["counterflow_53s", "falloff_16s", "noneq_14s", "long_24s"])
def test_mechanism_from_openfoam_files(built, tmp_path, wname):
    """Loading the OpenFOAM reactions / speciesThermo dictionaries gives the
    same chemistry as the flat description: PLOG ArrheniusData, third-body
    coefficient lists, fall-off k0 / kInf / F / thirdBodyEfficiencies and
    non-equilibrium forward / reverse entries."""
    from fcs import foam_io
    w, mech, flat, c = _setup(wname, 8)
    paths = foam_io.write_case(mech, str(tmp_path))
    a = _ctx(flat)
    b = _ctx(flat)
    ns, nr = b.load_mechanism_foam(paths["reactions"], paths["thermo"])
    assert (ns, nr) == (mech.n_species, mech.n_reactions)
    np.testing.assert_allclose(b.rhs(c.p, c.T, c.Y), a.rhs(c.p, c.T, c.Y), rtol=1e-13, atol=0)
    Ja, _ = a.jacobian(c.p, c.T, c.Y)
    Jb, _ = b.jacobian(c.p, c.T, c.Y)
    np.testing.assert_allclose(Jb, Ja, rtol=1e-13, atol=0)


def test_queue_order_and_graph_replay_do_not_change_results(built):
    """The binned work queue (default), the natural order and the CUDA-graph
    step give bit-identical cells: each cell's integration is independent of
    where it sits in the queue."""
    import torch
    w, mech, flat, c = _setup("counterflow_53s", 512)
    c.subDt[::3] = 1e-9  # spread the predicted step counts over several bins
    ctx = _ctx(flat, abs_tol=w.abs_tol, rel_tol=w.rel_tol, mapping=64, treact=float(np.percentile(c.T, 30)))
    from fcs._lib import StepStats
    outs = []
    init = {k: torch.from_numpy(np.ascontiguousarray(getattr(c, k))).cuda() for k in ("p", "rho0", "T", "Y", "subDt")}
    d = {k: v.clone() for k, v in init.items()}
    RR = torch.zeros_like(d["Y"])
    st = torch.zeros(c.n, dtype=torch.int32, device="cuda")
    for flags in (0, 2, 4, 4, 6):
        # the same arrays every call, so that the graph is replayed (calls 3-4)
        for k in d:
            d[k].copy_(init[k])
        RR.zero_()
        st.fill_(-1)
        torch.cuda.synchronize()
        stats, dmin = StepStats(), ctypes.c_double()
        code = ctx.L.fcs_integrate(ctx.h, c.n, w.dt, d["p"].data_ptr(), d["rho0"].data_ptr(), d["T"].data_ptr(),
                                   d["Y"].data_ptr(), d["subDt"].data_ptr(), RR.data_ptr(), st.data_ptr(),
                                   ctypes.byref(stats), ctypes.byref(dmin), 1 | flags)
        assert code == 0, ctx.L.fcs_last_error_string(ctx.h)
        outs.append(({k: v.clone() for k, v in d.items()}, RR.clone(), st.clone(), stats.as_dict(), dmin.value))
    d0, RR0, st0, s0, m0 = outs[0]
    assert s0["cells_skipped"] > 0 and s0["cells_integrated"] == c.n - s0["cells_skipped"]
    for d, RR, st, s, m in outs[1:]:
        for k in ("T", "Y", "subDt"):
            assert torch.equal(d[k], d0[k]), k
        assert torch.equal(RR, RR0) and torch.equal(st, st0)
        assert m == m0
        for k in ("cells_integrated", "cells_skipped", "attempts", "accepted", "jacobians"):
            assert s[k] == s0[k], k


@pytest.mark.parametrize("wname", ["ignition_10s", "counterflow_53s", "uneven_111s", "falloff_16s", "noneq_14s", "long_24s"])
def test_tc_matches_reference_golden(built, wname):
    """fcs_tc against FastChemistryModel::tc() of the reference
    (tests/golden/tc.npz); differences are summation order and exp rounding."""
    g = np.load(os.path.join(GOLDEN, "tc.npz"))
    flat, c = fixture.load_prefixed(g, wname + "__")
    ctx = _ctx(flat)
    tc = ctx.tc(c.p, c.T, c.rho0, c.Y)
    np.testing.assert_allclose(tc, g[wname + "__tc"], rtol=1e-12)


def test_graph_step_recaptures_when_buffers_or_mechanism_change(built):
    """A replayed step graph never uses a buffer that a larger call has
    replaced, nor a mechanism that has been reloaded."""
    import torch
    from fcs._lib import CUDA_GRAPH
    w, mech, flat, c = _setup("ignition_10s", 64)
    ctx = _ctx(flat, abs_tol=w.abs_tol, rel_tol=w.rel_tol, mapping=64)
    d = {k: torch.from_numpy(np.ascontiguousarray(getattr(c, k))).cuda() for k in ("p", "rho0", "T", "Y", "subDt")}
    init = {k: v.clone() for k, v in d.items()}

    def step():
        for k in d:
            d[k].copy_(init[k])
        code, stats, _ = ctx.integrate_raw(c.n, w.dt, d["p"], d["rho0"], d["T"], d["Y"], d["subDt"], device=True,
                                           flags=CUDA_GRAPH)
        assert code == 0
        return d["T"].clone(), stats["attempts"]

    T1, a1 = step()
    # a larger ordinary call grows (and so moves) the context's internal buffers
    big = fcs.cells_for(w, mech, n=1024)
    ctx.integrate(big, w.dt)
    T2, a2 = step()
    assert torch.equal(T1, T2) and a1 == a2
    # reloading the mechanism invalidates the captured step
    ctx.load_mechanism(flat)
    ctx.set_options(abs_tol=w.abs_tol, rel_tol=w.rel_tol, mapping=64)
    T3, a3 = step()
    assert torch.equal(T1, T3) and a1 == a3


def test_async_step_on_a_caller_stream_matches_integrate(built):
    """fcs_integrate_async on a torch stream + fcs_sync equals fcs_integrate."""
    import torch
    w, mech, flat, c = _setup("counterflow_53s", 128)
    ctx = _ctx(flat, abs_tol=w.abs_tol, rel_tol=w.rel_tol, mapping=64)
    ref = ctx.integrate(c, w.dt)
    d = {k: torch.from_numpy(np.ascontiguousarray(getattr(c, k))).cuda() for k in ("p", "rho0", "T", "Y", "subDt")}
    RR = torch.zeros_like(d["Y"])
    st = torch.zeros(c.n, dtype=torch.int32, device="cuda")
    s = torch.cuda.Stream()
    torch.cuda.synchronize()
    ctx.integrate_async(c.n, w.dt, d["p"], d["rho0"], d["T"], d["Y"], d["subDt"], RR, st, stream=s)
    with pytest.raises(Exception):
        ctx.integrate_async(c.n, w.dt, d["p"], d["rho0"], d["T"], d["Y"], d["subDt"], RR, st, stream=s)
    code, stats, dmin = ctx.sync()
    assert code == 0 and stats["cells_integrated"] == c.n
    np.testing.assert_array_equal(d["T"].cpu().numpy(), ref["T"])
    np.testing.assert_array_equal(d["Y"].cpu().numpy(), ref["Y"])
    np.testing.assert_array_equal(RR.cpu().numpy(), ref["RR"])
    assert dmin == ref["deltaTMin"] and stats["attempts"] == ref["stats"]["attempts"]
    # host arrays are refused, not handed to the kernels
    with pytest.raises(Exception):
        ctx.integrate_async(c.n, w.dt, c.p, c.rho0, c.T.copy(), c.Y.copy(), c.subDt.copy())
