"""Large mechanisms on the GPU against the reference's own outputs.

* the 200-species / 1,500-reaction field (large_200s) and the 111-species /
  784-reaction field (uneven_111s), golden fixtures of the reference core;
* the reference's own tutorial inputs: the 255-species NC12H26
  (Narayanaswamy 2014) and 140-species IC8H18 (Yoo 2013) mechanisms on
  ignition cells, and 15 cells of the 2D CH4/air counterflow flame
  (GRI-Mech 3.0, tutorial/CounterFlowFlame2D/CH4_GRI30/1) over its CFD step
  of 2e-4 s.

Above ~140 species the per-cell slot no longer fits in shared memory and
the cell groups run from the global-memory workspace (fcs_kernels.cuh:
`if (gws) base = ...`); the 111-species slot does so in mixed precision.  Every
mapping is run: the default (auto), explicit group sizes and the lane
mapping.  FP64 is held to the tolerances of test_gpu_parity.py; mixed
precision against the reference's tight run (absTol 1e-14 / relTol 1e-10)
to 2x the FP64 method's own error plus a small floor, and <= 1e-3 relative
in T.
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


def _golden(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def _check_golden(out, g, rtol, atol):
    assert (out["status"] == g["status"]).all(), (out["status"], g["status"])
    np.testing.assert_allclose(out["T"], g["T"], rtol=rtol, atol=0)
    np.testing.assert_allclose(out["Y"], g["Y"], rtol=0, atol=atol)
    np.testing.assert_allclose(out["RR"], g["RR"], rtol=0, atol=atol * np.abs(g["RR"]).max() / 1e-3 + 1e-12)
    njac = int(g["jacobians"])
    assert abs(out["stats"]["jacobians"] - njac) <= max(4, 0.01 * njac), (out["stats"]["jacobians"], njac)


@pytest.mark.parametrize("case,mapping", [("large_200s", 0), ("large_200s", 64), ("large_200s", LANE),
                                          ("uneven_111s", 0), ("uneven_111s", 256), ("uneven_111s", LANE)])
def test_large_fields_match_reference_golden(built, case, mapping):
    g = _golden(case + "_OptRodas34")
    w = fcs.WORKLOADS[case]
    flat, c = fixture.load(g)
    ctx = _ctx(flat, abs_tol=w.abs_tol, rel_tol=w.rel_tol, treact=w.treact, mapping=mapping)
    out = ctx.integrate(c, w.dt)
    _check_golden(out, g, 1e-7, 1e-8)
    if mapping:
        assert out["stats"]["mapping"] == mapping


@pytest.mark.parametrize("case", ["large_200s", "uneven_111s"])
def test_large_fields_rhs_and_jacobian_match_reference(built, case):
    g = _golden(case + "_OptRodas34")
    flat, c = fixture.load(g)
    ctx = _ctx(flat)
    f = ctx.rhs(c.p, c.T, c.Y)
    assert np.max(np.abs(f - g["rhs"]) / (np.abs(g["rhs"]).max(axis=1, keepdims=True) + 1e-300)) < 1e-12
    k = g["jac"].shape[0]
    J, _ = ctx.jacobian(c.p[:k], c.T[:k], c.Y[:, :k])
    assert np.max(np.abs(J - g["jac"]) / np.abs(g["jac"]).max(axis=(1, 2), keepdims=True)) < 1e-12


def test_large_mixed_precision_against_tight_reference(built):
    """The 200-species field in mixed precision (FP32 LU, FP64-residual
    refinement, from the global workspace) against the reference's tight run."""
    g = _golden("large_200s_tight")
    w = fcs.WORKLOADS["large_200s"]
    flat, c = fixture.load(g)
    ctx = _ctx(flat, abs_tol=w.abs_tol, rel_tol=w.rel_tol, precision="fp64")
    f64 = ctx.integrate(c, w.dt)
    ctx.set_options(abs_tol=w.abs_tol, rel_tol=w.rel_tol, precision="mixed")
    mix = ctx.integrate(c, w.dt)
    assert (mix["status"] == 0).all() and (f64["status"] == 0).all()
    eT64 = np.max(np.abs(f64["T"] - g["T"]) / g["T"])
    eY64 = np.max(np.abs(f64["Y"] - g["Y"]))
    eT = np.max(np.abs(mix["T"] - g["T"]) / g["T"])
    eY = np.max(np.abs(mix["Y"] - g["Y"]))
    assert eT <= 2 * eT64 + 1e-5 and eT <= 1e-3, (eT, eT64)
    assert eY <= 2 * eY64 + 1e-6, (eY, eY64)


TUTORIAL = ["tutorial_nc12h26_narayanaswamy", "tutorial_ic8h18_yoo", "tutorial_ch4_gri30_counterflow"]


@pytest.mark.parametrize("name", TUTORIAL)
@pytest.mark.parametrize("mapping", [0, LANE])
def test_tutorial_inputs_match_reference(built, name, mapping):
    """The reference's own mechanisms and flame cells: FP64 Rodas34 against
    the reference core on the same inputs; RHS and Jacobian to 1e-12."""
    g = _golden(name)
    flat, c = fixture.load(g)
    dt = float(g["dt"])
    ctx = _ctx(flat, abs_tol=float(g["abs_tol"]), rel_tol=float(g["rel_tol"]), mapping=mapping)
    out = ctx.integrate(c, dt)
    _check_golden(out, g, 1e-7, 1e-8)
    if mapping == 0:
        f = ctx.rhs(c.p, c.T, c.Y)
        assert np.max(np.abs(f - g["rhs"]) / (np.abs(g["rhs"]).max(axis=1, keepdims=True) + 1e-300)) < 1e-12
        J, _ = ctx.jacobian(c.p[:1], c.T[:1], c.Y[:, :1])
        assert np.max(np.abs(J - g["jac"]) / np.abs(g["jac"]).max(axis=(1, 2), keepdims=True)) < 1e-12


@pytest.mark.parametrize("name", TUTORIAL)
def test_tutorial_inputs_mixed_precision(built, name):
    g = _golden(name)
    flat, c = fixture.load(g)
    dt = float(g["dt"])
    ctx = _ctx(flat, abs_tol=float(g["abs_tol"]), rel_tol=float(g["rel_tol"]), precision="fp64")
    f64 = ctx.integrate(c, dt)
    ctx.set_options(abs_tol=float(g["abs_tol"]), rel_tol=float(g["rel_tol"]), precision="mixed")
    mix = ctx.integrate(c, dt)
    assert (mix["status"] == 0).all()
    Tt, Yt = g["tight_T"], g["tight_Y"]
    eT64 = np.max(np.abs(f64["T"] - Tt) / Tt)
    eY64 = np.max(np.abs(f64["Y"] - Yt))
    eT = np.max(np.abs(mix["T"] - Tt) / Tt)
    eY = np.max(np.abs(mix["Y"] - Yt))
    assert eT <= 2 * eT64 + 1e-5 and eT <= 1e-3, (eT, eT64)
    assert eY <= 2 * eY64 + 1e-6, (eY, eY64)
