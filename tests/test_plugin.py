"""The OpenFOAM-side plugin libFastChemistryModel.so (plugin/), compiled
against the OpenFOAM-10 stub (plugin/foam_stub) and driven by a stand-in
solver (tests/plugin/driver.C) that loads it as controlDict `libs (...)`
does and selects the model with basicChemistryModel::New.

CPU: the plugin builds, registers the reference's solver names
(src/odeChemistrySolvers.C:63-74) with the method FastChemistryModel, is
selected from a case's chemistryProperties, and ends the run with FatalError
when the GPU library cannot start (no GPU here) -- as OpenFOAM would.

GPU: solve(deltaT), solve(scalarField), tc(), Qdot() and calculate() on a
few cells against the oracle (RR = (Y(t+dt) - Y(t)) rho / dt per cell).
"""
import os
import subprocess

import numpy as np
import pytest

import fcs

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SOLVERS = ("OptRosenbrock34", "OptRosenbrock23", "OptRodas34", "OptRodas23", "OptSeulex")


@pytest.fixture(scope="module")
def plugin(tmp_path_factory):
    from fcs.build import STUB_LIB, PLUGIN, build_plugin
    lib = build_plugin()
    d = tmp_path_factory.mktemp("plugin")
    drv = str(d / "driver")
    stub_dir = os.path.dirname(STUB_LIB)
    subprocess.run(["g++", "-O2", "-std=c++17", os.path.join(ROOT, "tests", "plugin", "driver.C"),
                    "-I" + os.path.join(PLUGIN, "foam_stub"), "-L" + stub_dir, "-lfoamStub", "-ldl",
                    "-Wl,-rpath," + stub_dir, "-o", drv], check=True)
    return lib, drv


def _case(tmp_path, wname, n, solver="OptRodas34", **props):
    from fcs import foam_io
    w = fcs.WORKLOADS[wname]
    mech = w.mechanism()
    case = tmp_path / "case"
    const = case / "constant"
    foam_io.write_case(mech, str(const), solver=solver, abs_tol=w.abs_tol, rel_tol=w.rel_tol, **props)
    # the thermo's species list, in the reverse of the mechanism's order (the
    # plugin maps them by name)
    species = list(reversed(mech.species))
    (const / "species").write_text("\n".join(species) + "\n")
    idx = np.linspace(0, w.n_cells - 1, n).astype(np.int64)
    c = fcs.cells_for(w, mech).subset(idx)
    order = [mech.species.index(s) for s in species]
    with open(tmp_path / "cells.bin", "wb") as f:
        np.array([c.n, mech.n_species], dtype=np.int32).tofile(f)
        np.array([w.dt], dtype=np.float64).tofile(f)
        for a in (c.p, c.T, c.rho0):
            np.ascontiguousarray(a, dtype=np.float64).tofile(f)
        np.ascontiguousarray(c.Y[order], dtype=np.float64).tofile(f)
    return w, mech, c, order, str(case), str(tmp_path / "cells.bin"), str(tmp_path / "out.bin")


def test_plugin_registers_the_reference_solver_names(plugin):
    lib, drv = plugin
    r = subprocess.run([drv, "--list", lib], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    names = set(r.stdout.split())
    thermo = "sutherlandTransportsensibleEnthalpyjanafThermoperfectGasspecie"
    assert names == {f"{s}<FastChemistryModel<{thermo}>>" for s in SOLVERS}


def test_plugin_selected_from_chemistry_properties(plugin, tmp_path):
    """The case's chemistryType selects the model.  Without a GPU the
    model's constructor fails in fcs_create and the run ends with FatalError;
    with one, the step runs (checked in detail by the GPU test)."""
    lib, drv = plugin
    w, mech, c, order, case, cells, out = _case(tmp_path, "ignition_10s", 8)
    r = subprocess.run([drv, lib, case, cells, out], capture_output=True, text=True)
    try:
        import torch
        gpu = torch.cuda.is_available()
    except Exception:
        gpu = False
    if gpu:
        assert r.returncode == 0, r.stderr
    else:
        assert r.returncode == 1 and "FatalError" in r.stderr and "fcs_create" in r.stderr, r.stderr
    # an unknown solver name is refused by the selection, listing the valid ones
    w, mech, c, order, case, cells, out = _case(tmp_path / "x", "ignition_10s", 8, solver="ode")
    r = subprocess.run([drv, lib, case, cells, out], capture_output=True, text=True)
    assert r.returncode == 1 and "Unknown chemistry solver" in r.stderr and "OptRodas34<" in r.stderr


def _read_out(path, ns, n):
    a = np.fromfile(path, dtype=np.float64)
    dmin = a[0]
    o = 1
    RR = a[o:o + ns * n].reshape(ns, n); o += ns * n
    tc = a[o:o + n]; o += n
    Q = a[o:o + n]; o += n
    RRc = a[o:o + ns * n].reshape(ns, n)
    return dmin, RR, tc, Q, RRc


@pytest.mark.gpu
@pytest.mark.parametrize("solver,lts", [("OptRodas34", False), ("OptRosenbrock34", False), ("OptSeulex", False),
                                        ("OptRodas34", True)])
def test_plugin_solve_matches_oracle(plugin, tmp_path, solver, lts):
    import oracle
    lib, drv = plugin
    w, mech, c, order, case, cells, out = _case(tmp_path, "ignition_10s", 32, solver=solver)
    r = subprocess.run([drv, lib, case, cells, out] + (["lts"] if lts else []), capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    ns, n = mech.n_species, c.n
    dmin, RR, tc, Q, RRc = _read_out(out, ns, n)
    flat = fcs.flatten(mech)
    port = oracle.Port(flat)
    dts = w.dt * (1.0 + np.arange(n) / n) if lts else None
    ref = port.integrate(c, 0.0 if lts else w.dt, dt_per_cell=dts, solver=solver, abs_tol=w.abs_tol,
                         rel_tol=w.rel_tol)
    assert (ref["status"] == 0).all()
    RRref = ref["RR"][order]
    scale = np.abs(RRref).max()
    np.testing.assert_allclose(RR, RRref, rtol=0, atol=1e-6 * scale)
    if not lts:
        assert dmin == pytest.approx(ref["deltaTMin"], rel=1e-2)
    # tc and calculate() at the (unchanged) initial state, Qdot from the solve's RR
    np.testing.assert_allclose(tc, port.tc(c.p, c.T, c.rho0, c.Y), rtol=1e-12)
    RRr, _ = port.rates(c.p, c.T, c.rho0, c.Y)
    np.testing.assert_allclose(RRc, RRr[order], rtol=0, atol=1e-12 * np.abs(RRr).max())
    from fcs import _lib
    ctx = _lib.Context(0)
    ctx.load_mechanism(flat)
    hf = np.zeros(ns)
    ctx._check(ctx.L.fcs_formation_enthalpy(ctx.h, hf.ctypes.data_as(_lib.C.POINTER(_lib.C.c_double))))
    ctx.close()
    np.testing.assert_allclose(Q, -(hf[order, None] * RR).sum(axis=0), rtol=1e-12, atol=1e-300)
