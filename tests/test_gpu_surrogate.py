"""The surrogate-gated method (include/fcs_mlp.h) through the C ABI: an
ensemble trained by the library's own kernels on states the plain GPU
integrator produced, in front of the plain method on unseen cells of the
53-species field.

What is checked:
  * the trained ensemble predicts the state after the step better than an
    untrained one and than "no change" (median errors at most half of
    theirs: on these far-from-equilibrium cells T moves by ~50 % in one
    step, and the ensemble gets within ~10 %);
  * at the default gate (1e-3 relative T, 1e-6 absolute Y: the method's
    accuracy target) no prediction on these stiff cells is good enough:
    every cell falls back, and the method still gains from the network
    through the predicted initial sub-step (fewer attempts than the plain
    method);
  * at a relaxed gate, accepted cells carry exactly the ensemble-mean
    prediction restated on the host, audited cells keep the plain result, and
    the counts add up.
"""
import numpy as np
import pytest

import fcs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup():
    import __graft_entry__
    __graft_entry__.build()
    import torch
    from fcs import _lib, surrogate
    w = fcs.WORKLOADS["counterflow_53s"]
    mech = w.mechanism()
    flat = fcs.flatten(mech)
    ctx = _lib.Context(0)
    ctx.load_mechanism(flat)
    ctx.set_options(abs_tol=w.abs_tol, rel_tol=w.rel_tol, mapping=64)
    mlp, info = surrogate.train_for_workload(ctx, w, mech, 32768, seed=1000, min_steps=3000)
    # unseen cells from the same distribution (other seeds of the field generator)
    ev = surrogate.reacting_cells(w, mech, 4096, seed=777, per_draw=512)

    def run(gated, mlp_=None, **gate):
        d = {k: torch.from_numpy(np.ascontiguousarray(getattr(ev, k))).cuda() for k in ("p", "rho0", "T", "Y", "subDt")}
        RR = torch.zeros_like(d["Y"])
        st = torch.zeros(ev.n, dtype=torch.int32, device="cuda")
        if gated:
            surrogate.attach(ctx, mlp_ or mlp, mech, **gate)
            code, stats, gst, _ = _lib.integrate_gated_raw(ctx, ev.n, w.dt, d["p"], d["rho0"], d["T"], d["Y"],
                                                           d["subDt"], RR, st, device=True)
        else:
            code, stats, _ = ctx.integrate_raw(ev.n, w.dt, d["p"], d["rho0"], d["T"], d["Y"], d["subDt"], RR, st,
                                               device=True)
            gst = None
        assert code == 0
        return dict(T=d["T"].cpu().numpy(), Y=d["Y"].cpu().numpy(), st=st.cpu().numpy(), stats=stats, gate=gst)

    plain = run(False)
    return dict(w=w, mech=mech, ctx=ctx, mlp=mlp, info=info, ev=ev, run=run, plain=plain)


def _err(T, Y, ref):
    return np.abs(T - ref["T"]) / ref["T"], np.abs(Y - ref["Y"]).max(axis=0)


def test_trained_ensemble_beats_untrained_and_no_change(setup):
    from fcs import _lib, surrogate
    s = setup
    ev, w, plain = s["ev"], s["w"], s["plain"]
    assert s["info"]["loss_last"][0] < 0.25 * s["info"]["loss_first"][0]
    T1, Y1, _ = surrogate.predict(s["mlp"], ev.T, ev.p, w.dt, ev.Y)
    eT, eY = _err(T1, Y1, plain)
    nT, nY = _err(ev.T, np.maximum(ev.Y, 0), plain)
    u = _lib.Mlp(s["mlp"].n_in, s["mlp"].n_out, members=4, seed=99)
    u.set_normalization(*s["mlp"].get_normalization())
    T0, Y0, _ = surrogate.predict(u, ev.T, ev.p, w.dt, ev.Y)
    uT, uY = _err(T0, Y0, plain)
    assert np.median(eT) < 0.5 * np.median(nT) and np.median(eY) < 0.5 * np.median(nY)
    # the untrained network still carries the training set's mean change (its
    # output normalisation), a fair baseline for Y
    assert np.median(eT) < 0.5 * np.median(uT) and np.median(eY) < 0.75 * np.median(uY)


def test_default_gate_falls_back_and_gains_through_the_substep(setup):
    s = setup
    plain = s["plain"]
    g = s["run"](True)
    gs = g["gate"]
    assert gs["cells_active"] == s["ev"].n
    assert gs["cells_accepted"] + gs["cells_audited"] + gs["cells_fallback"] == gs["cells_active"]
    assert (g["st"] == 0).all()
    # every integrated cell is the plain method's answer (started from the
    # predicted sub-step, so equal to integration accuracy, not bitwise)
    eT, eY = _err(g["T"], g["Y"], plain)
    assert eT.max() < 1e-3 and eY.max() < 1e-3
    # the network's predicted sub-step saves attempts
    assert g["stats"]["attempts"] < plain["stats"]["attempts"], (g["stats"]["attempts"], plain["stats"]["attempts"])


def test_relaxed_gate_accepts_exactly_the_prediction(setup):
    from fcs import surrogate
    s = setup
    ev, w, plain = s["ev"], s["w"], s["plain"]
    g = s["run"](True, T_rel=0.05, Y_abs=0.05, element_abs=0.05, audit_fraction=0.1)
    gs = g["gate"]
    assert gs["cells_accepted"] > 0, gs
    assert gs["cells_accepted"] + gs["cells_audited"] + gs["cells_fallback"] == gs["cells_active"]
    audited = gs["cells_audited"] / max(1, gs["cells_audited"] + gs["cells_accepted"])
    assert 0.02 < audited < 0.25, gs
    assert gs["audit_max_rel_T"] > 0 or gs["cells_audited"] == 0
    T1, Y1, _ = surrogate.predict(s["mlp"], ev.T, ev.p, w.dt, ev.Y)
    took = np.isclose(g["T"], T1, rtol=1e-13, atol=0) & np.all(np.isclose(g["Y"], Y1, rtol=1e-12, atol=1e-300), axis=0)
    assert took.sum() == gs["cells_accepted"], (took.sum(), gs)
    # cells the plain method integrated: all ok
    assert (g["st"] == 0).all()
    assert g["stats"]["attempts"] < plain["stats"]["attempts"]
