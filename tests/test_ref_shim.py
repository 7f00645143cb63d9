"""The reference's numerical core built with the portable SIMD shim
(oracle/simd_shim: <immintrin.h> written on GCC vector extensions, libmvec's
exp/log/pow as scalar libm loops) -- the build the aarch64 GPU hosts use for
the bench's reference arm -- against the golden fixtures made by the
reference's own AVX2/FMA build.

With multiply-adds contracted as in the AVX2 build the shim's LU is
bit-identical to it; what remains is libmvec's vector exp/log against the
scalar libm ones, so the tolerances are those of the oracle restatement
(test_oracle.py).  Runs where the reference tree is known (FCS_REFERENCE or
the checker build's record) on an x86-64 host.
"""
import os

import numpy as np
import pytest

import fcs
from conftest import GOLDEN
from golden import fixture

CASES = ["ignition_10s_OptRodas34", "ignition_10s_OptRosenbrock34", "ignition_10s_OptSeulex",
         "counterflow_53s_OptRodas34", "counterflow_53s_OptRosenbrock34", "counterflow_53s_OptSeulex",
         "ignition_10s_OptRodas23", "counterflow_53s_OptRosenbrock23", "falloff_16s_OptRodas34",
         "noneq_14s_OptRodas34", "long_24s_OptRodas34", "long_24s_OptSeulex"]


@pytest.fixture(scope="module")
def shim_so(port_built):
    import oracle
    so = oracle.build_shim()
    if not so:
        pytest.skip("reference sources not present on this host (set FCS_REFERENCE)")
    return so


@pytest.mark.parametrize("case", CASES)
def test_shim_reference_matches_golden(shim_so, case):
    import oracle
    wname, solver = case.rsplit("_", 1)
    w = fcs.WORKLOADS[wname]
    g = np.load(os.path.join(GOLDEN, case + ".npz"))
    flat, cells = fixture.load(g)
    ref = oracle.Reference(flat, solver=solver, abs_tol=w.abs_tol, rel_tol=w.rel_tol, so=shim_so)
    out = ref.integrate(cells, w.dt, treact=w.treact)
    assert (out["status"] == g["status"]).all()
    rtol, atol = (1e-9, 1e-10) if wname == "ignition_10s" else (1e-7, 1e-8)
    np.testing.assert_allclose(out["T"], g["T"], rtol=rtol, atol=0)
    np.testing.assert_allclose(out["Y"], g["Y"], rtol=0, atol=atol)
    njac = int(g["jacobians"])
    assert abs(out["counters"]["jacobians"] - njac) <= max(4, 0.01 * njac)
    # RHS and Jacobian at the fixture's cells: rounding of exp/log only
    f = ref.rhs(cells.p, cells.T, cells.Y)
    assert np.max(np.abs(f - g["rhs"]) / (np.abs(g["rhs"]).max(axis=1, keepdims=True) + 1e-300)) < 1e-12
    k = g["jac"].shape[0]
    J, _ = ref.jacobian(cells.p[:k], cells.T[:k], cells.Y[:, :k])
    assert np.max(np.abs(J - g["jac"]) / np.abs(g["jac"]).max(axis=(1, 2), keepdims=True)) < 1e-12
