"""fcs_integrate_noalloc (the entry point that allocates no device memory)
against fcs_integrate on the same device arrays, through the C ABI.

Both entry points run the same classify kernel (natural cell order:
fcs_integrate is given FCS_NO_QUEUE_SORT) and the same integrate kernel with
the same cell-to-thread mapping on the same cells, so the results agree to
rounding of identical arithmetic: the test allows 1e-13 relative.  On each
call the no-allocation entry point runs first, so in a fresh process the
first launch of the integrate kernel is its own.  The file is named to be
collected last, and passes alone in a fresh process as well.
"""
import numpy as np
import pytest

import fcs

pytestmark = pytest.mark.gpu

FCS_ERR_INVALID = 1
FCS_NO_QUEUE_SORT = 2
NOALLOC_MAX_CELLS = 1048576
RTOL = 1e-13


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


def _device_state(c):
    import torch
    d = {k: torch.from_numpy(np.ascontiguousarray(getattr(c, k))).cuda() for k in ("p", "rho0", "T", "Y", "subDt")}
    d["RR"] = torch.zeros_like(d["Y"])
    d["status"] = torch.full((c.n,), -1, dtype=torch.int32, device="cuda")
    return d


def test_noalloc_matches_integrate_on_two_calls_in_a_row(built):
    import torch
    from fcs import _lib
    w, flat, c = _cells("counterflow_53s", 2048)
    treact = float(np.median(c.T))  # about half of the cells are skipped
    ctx = _lib.Context(0)
    ctx.load_mechanism(flat)
    ctx.set_options(abs_tol=w.abs_tol, rel_tol=w.rel_tol, mapping=64, treact=treact)
    a, b = _device_state(c), _device_state(c)
    for call in range(2):
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        code_b, stats_b, dmin_b = ctx.integrate_noalloc(c.n, w.dt, b["p"], b["rho0"], b["T"], b["Y"], b["subDt"],
                                                        b["RR"], b["status"])
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info()[0]
        code_a, stats_a, dmin_a = ctx.integrate_raw(c.n, w.dt, a["p"], a["rho0"], a["T"], a["Y"], a["subDt"],
                                                    a["RR"], a["status"], device=True, flags=FCS_NO_QUEUE_SORT)
        torch.cuda.synchronize()
        assert code_a == 0 and code_b == 0, (code_a, code_b, ctx.last_error())
        if call == 1:  # the first call may load the scratch's device module and grow the stack reservation
            assert free_after == free_before
        for k in ("cells_integrated", "cells_skipped", "cells_failed", "attempts", "accepted", "jacobians",
                  "lu_decompositions", "rhs_evaluations", "linear_solves"):
            assert stats_a[k] == stats_b[k], (call, k, stats_a[k], stats_b[k])
        assert 0 < stats_b["cells_skipped"] < c.n and stats_b["mapping"] == 64
        np.testing.assert_allclose(dmin_b, dmin_a, rtol=RTOL)
        np.testing.assert_array_equal(b["status"].cpu().numpy(), a["status"].cpu().numpy())
        for k in ("T", "Y", "subDt", "RR"):
            np.testing.assert_allclose(b[k].cpu().numpy(), a[k].cpu().numpy(), rtol=RTOL, atol=1e-300,
                                       err_msg=f"call {call}: {k}")
    ctx.close()


def test_noalloc_rejects_what_it_cannot_take(built):
    import torch
    from fcs import _lib
    w, flat, c = _cells("ignition_10s", 16)
    ctx = _lib.Context(0)
    ctx.load_mechanism(flat)
    d = _device_state(c)
    args = (d["p"], d["rho0"], d["T"], d["Y"], d["subDt"], d["RR"], d["status"])
    # beyond the fixed queue: refused before any device work
    code, _, _ = ctx.integrate_noalloc(NOALLOC_MAX_CELLS + 1, w.dt, *args, check=False)
    assert code == FCS_ERR_INVALID and str(NOALLOC_MAX_CELLS) in ctx.last_error()
    # host arrays: refused (the kernels would read them as device addresses)
    host = [np.ascontiguousarray(getattr(c, k)) for k in ("p", "rho0", "T", "Y", "subDt")]
    code, _, _ = ctx.integrate_noalloc(c.n, w.dt, *host, check=False)
    assert code == FCS_ERR_INVALID and "device memory" in ctx.last_error()
    # an empty batch is a no-op
    code, stats, _ = ctx.integrate_noalloc(0, w.dt, *args, check=False)
    assert code == 0 and stats["cells_integrated"] == 0
    # and the context still integrates afterwards
    T0 = d["T"].clone()
    code, stats, _ = ctx.integrate_noalloc(c.n, w.dt, *args)
    torch.cuda.synchronize()
    assert code == 0 and stats["cells_integrated"] == c.n
    assert torch.isfinite(d["T"]).all() and not torch.equal(d["T"], T0)
    ctx.close()
