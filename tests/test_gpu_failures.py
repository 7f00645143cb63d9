"""Failure paths of the C ABI, made on the host (no GPU fault, trap or hang):

* an allocation that fails (injected with fcs_test_fail_allocations) returns
  FCS_ERR_NOMEM, leaves the mechanism and options in place, and the next call
  integrates normally;
* fcs_sync_timeout gives up on a step that is still running, returns
  FCS_ERR_TIMEOUT and leaves the step in flight, and fcs_sync then collects
  it with the same results as the synchronous entry point;
* while a step of fcs_integrate_async is in flight, the entry points that use
  the context's buffers refuse with FCS_ERR_STATE instead of racing the
  running kernels.

The reference's only failure path is the fatal maxSteps
(src/ODE/OptRodas34/OptRodas34.C:193); it is covered in test_gpu_parity.py.
"""
import numpy as np
import pytest

import fcs

pytestmark = pytest.mark.gpu

OK, NOMEM, STATE, TIMEOUT = 0, 3, 4, 8
NO_QUEUE_SORT = 2


@pytest.fixture(scope="module")
def built():
    import __graft_entry__
    __graft_entry__.build()
    return True


def _cells(wname, n):
    w = fcs.WORKLOADS[wname]
    mech = w.mechanism()
    flat = fcs.flatten(mech)
    idx = np.linspace(0, w.n_cells - 1, n).astype(np.int64)
    return w, flat, fcs.cells_for(w, mech).subset(idx)


def _device(c):
    import torch
    d = {k: torch.from_numpy(np.ascontiguousarray(getattr(c, k))).cuda() for k in ("p", "rho0", "T", "Y", "subDt")}
    d["RR"] = torch.zeros_like(d["Y"])
    d["status"] = torch.full((c.n,), -1, dtype=torch.int32, device="cuda")
    return d


def test_injected_allocation_failure_returns_nomem_and_recovers(built):
    from fcs import _lib
    w, flat, c = _cells("ignition_10s", 256)
    ctx = _lib.Context(0)
    ctx.load_mechanism(flat)
    ctx.set_options(abs_tol=w.abs_tol, rel_tol=w.rel_tol, mapping=64)
    small = c.subset(np.arange(32))
    first = ctx.integrate(small, w.dt)            # buffers sized for 32 cells
    assert first["code"] == OK
    try:
        _lib.fail_allocations(1)                  # the next buffer growth fails
        T, Y, sub = c.T.copy(), c.Y.copy(), c.subDt.copy()
        code, _, _ = ctx.integrate_raw(c.n, w.dt, c.p, c.rho0, T, Y, sub, check=False)
        assert code == NOMEM, (code, ctx.last_error())
        assert "allocation" in ctx.last_error().lower() or "memory" in ctx.last_error().lower()
        np.testing.assert_array_equal(T, c.T)     # nothing was written back
    finally:
        _lib.fail_allocations(0)
    # the mechanism and options survived: the full batch integrates, and the
    # cells of the first call give the same results as before
    again = ctx.integrate(c, w.dt)
    assert again["code"] == OK and (again["status"] == 0).all()
    np.testing.assert_allclose(again["T"][:32], first["T"], rtol=1e-13)
    np.testing.assert_allclose(again["Y"][:, :32], first["Y"], rtol=1e-13, atol=1e-300)
    ctx.close()


def test_sync_timeout_leaves_the_step_in_flight(built):
    import torch
    from fcs import _lib
    w, flat, c = _cells("counterflow_53s", 4096)
    ctx = _lib.Context(0)
    ctx.load_mechanism(flat)
    ctx.set_options(abs_tol=w.abs_tol, rel_tol=w.rel_tol, mapping=64)
    ref = _device(c)
    code, stats_ref, dmin_ref = ctx.integrate_raw(c.n, w.dt, ref["p"], ref["rho0"], ref["T"], ref["Y"],
                                                  ref["subDt"], ref["RR"], ref["status"], device=True,
                                                  flags=NO_QUEUE_SORT)
    assert code == OK
    d = _device(c)
    torch.cuda.synchronize()
    ctx.integrate_async(c.n, w.dt, d["p"], d["rho0"], d["T"], d["Y"], d["subDt"], d["RR"], d["status"],
                        flags=NO_QUEUE_SORT)
    # the step runs for about a second: a 1 ms wait gives up
    code, _, _ = ctx.sync(timeout_ms=1.0)
    assert code == TIMEOUT, (code, ctx.last_error())
    # entry points that use the context's buffers refuse while it runs
    e = _device(c)
    code, _, _ = ctx.integrate_raw(c.n, w.dt, e["p"], e["rho0"], e["T"], e["Y"], e["subDt"], e["RR"],
                                   e["status"], device=True, check=False)
    assert code == STATE, (code, ctx.last_error())
    code, _, _ = ctx.integrate_noalloc(c.n, w.dt, e["p"], e["rho0"], e["T"], e["Y"], e["subDt"], e["RR"],
                                       e["status"], check=False)
    assert code == STATE, (code, ctx.last_error())
    with pytest.raises(_lib.FcsError) as err:
        ctx.rhs(c.p[:4], c.T[:4], c.Y[:, :4])
    assert err.value.code == STATE
    with pytest.raises(_lib.FcsError) as err:
        ctx.load_mechanism(flat)
    assert err.value.code == STATE
    # a second asynchronous step is refused as before
    with pytest.raises(_lib.FcsError) as err:
        ctx.integrate_async(c.n, w.dt, e["p"], e["rho0"], e["T"], e["Y"], e["subDt"], e["RR"], e["status"])
    assert err.value.code == STATE
    # the unbounded wait collects the step: same cells as the synchronous call
    code, stats, dmin = ctx.sync()
    assert code == OK
    for k in ("cells_integrated", "attempts", "accepted", "jacobians"):
        assert stats[k] == stats_ref[k], k
    assert dmin == dmin_ref
    for k in ("T", "Y", "subDt", "RR"):
        np.testing.assert_array_equal(d[k].cpu().numpy(), ref[k].cpu().numpy(), err_msg=k)
    # and the context works again after fcs_sync
    code, _, _ = ctx.integrate_raw(c.n, w.dt, e["p"], e["rho0"], e["T"], e["Y"], e["subDt"], e["RR"],
                                   e["status"], device=True)
    assert code == OK
    ctx.close()


def test_device_pointer_mode_rejects_host_arrays(built):
    from fcs import _lib
    w, flat, c = _cells("ignition_10s", 16)
    ctx = _lib.Context(0)
    ctx.load_mechanism(flat)
    T, Y, sub = c.T.copy(), c.Y.copy(), c.subDt.copy()
    code, _, _ = ctx.integrate_raw(c.n, w.dt, c.p, c.rho0, T, Y, sub, device=True, check=False)
    assert code == 1 and "device memory" in ctx.last_error(), ctx.last_error()
    ctx.close()
