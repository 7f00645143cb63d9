"""The reference's own tutorial mechanisms, read by the library's dictionary
reader (fcs_parse_mechanism_foam, host only) and run through the oracle and
the reference core compiled from its sources: rates, Jacobian, tc and one
CFD step of ignition-like cells with Rodas34.

Together the mechanisms cover every reaction kind the tutorials use:
(ir)reversible Arrhenius, third-body, Lindemann / Troe / SRI fall-off, PLOG
and non-equilibrium (third-body) reactions, reactions with more than three
products (the reference's generic RFG/JFG path), species names with parentheses
(CH2(S)) and thermo databases with uniform lists.  The tests run where the
reference tree and its compiled core are present (the x86-64 build host) and
skip elsewhere; no mechanism data is stored in this repository.
"""
import os
import re

import numpy as np
import pytest

MECHS = [
    # (case directory under the tutorials, fuel)
    ("Ignition0D/H2_Burke2011", "H2"),
    ("Ignition0D/H2_Connaire2004", "h2"),          # non-equilibrium (third-body)
    ("Ignition0D/CH4_GRI30", "CH4"),               # Lindemann, Troe, CH2(S)
    ("CounterFlowFlame2D/NH3_Zhang", "NH3"),       # PLOG
    ("Ignition0D/C2H4_Zettervall2024", "C2H4"),    # irreversible fall-off
    ("Ignition0D/DME_LLNL", "CH3OCH3"),            # non-equilibrium, 79 species
    ("Ignition0D/NH3CH4_Konnov", "NH3"),           # SRI, 129 species / 1231 reactions
    ("Ignition0D/C3H8_Qin2000", "C3H8"),           # a reversible reaction with 4 products
    ("Ignition0D/Kerosene_Zettervall2020", "C12H22"),  # global reactions with up to 7 products
    ("Ignition0D/NC12H26_Gao2014", "NC12H26"),     # 15 reactions with 4 products
]


def _files(case):
    import oracle
    d = os.path.join(oracle.reference_tutorial(), case, "constant")
    return os.path.join(d, "reactions"), os.path.join(d, "speciesThermo")


@pytest.fixture(scope="module")
def ref_available(port_built, lib_path):
    import oracle
    if not oracle.reference_tutorial():
        pytest.skip("reference tutorials not present on this host (set FCS_REFERENCE)")
    oracle.build(ref=True)
    if not os.path.exists(oracle.REF_SO):
        pytest.skip("reference core not built on this host")
    return True


def _cells(flat, names, fuel, n, seed):
    """Fuel / O2 / N2 near stoichiometry plus a trace of every species (so
    that every reaction runs), T ~ U[1000, 1600] K, p log-uniform on
    [1e5, 2e6] Pa."""
    from fcs.workloads import Cells, RU
    rng = np.random.default_rng(seed)
    low = [s.lower() for s in names]
    ns = flat.n_species
    base = np.zeros(ns)
    for sp, y in ((fuel, 0.06), ("o2", 0.22), ("n2", 0.72)):
        base[low.index(sp.lower())] = y
    Y = np.empty((ns, n))
    for c in range(n):
        trace = rng.dirichlet(np.full(ns, 0.5)) * 1e-3
        Y[:, c] = (base + trace) / (base + trace).sum()
    T = rng.uniform(1000.0, 1600.0, n)
    p = 10.0 ** rng.uniform(5.0, np.log10(2e6), n)
    rho0 = p / (RU * T * (Y / flat.W[:, None]).sum(axis=0))
    return Cells(T, p, np.ascontiguousarray(Y), rho0, np.full(n, 1e-7))


def _file_kind_counts(reactions_path):
    names = {"Arrhenius": 0, "ThirdBodyArrhenius": 1, "ArrheniusPLOG": 2, "ArrheniusLindemannFallOff": 3,
             "ArrheniusTroeFallOff": 4, "ArrheniusSRIFallOff": 5,
             "nonEquilibriumReversibleArrhenius": 6, "nonEquilibriumReversibleThirdBodyArrhenius": 7}
    counts = np.zeros(8, dtype=np.int64)
    text = re.sub(r"/\*.*?\*/", "", open(reactions_path).read(), flags=re.S)   # block comments
    text = re.sub(r"//[^\n]*", "", text)
    for t in re.findall(r"^\s*type\s+(\w+);", text, flags=re.M):
        base = t if t.startswith("nonEquilibrium") else re.sub(r"^(ir)?reversible", "", t)
        counts[names[base]] += 1
    return counts


@pytest.mark.parametrize("case,fuel", MECHS, ids=[m[0].split("/")[1] for m in MECHS])
def test_tutorial_mechanism_oracle_matches_reference(ref_available, case, fuel):
    import oracle
    from fcs import _lib
    rpath, tpath = _files(case)
    flat, names = _lib.parse_mechanism_foam(rpath, tpath)
    # every reaction of the file read, with its kind
    np.testing.assert_array_equal(np.bincount(flat.type, minlength=8), _file_kind_counts(rpath))
    c = _cells(flat, names, fuel, 8, seed=len(names))
    port, ref = oracle.Port(flat), oracle.Reference(flat)
    f0 = ref.rhs(c.p, c.T, c.Y)
    f1 = port.rhs(c.p, c.T, c.Y)
    assert np.max(np.abs(f1 - f0) / (np.abs(f0).max(axis=1, keepdims=True) + 1e-300)) < 1e-12
    J0, _ = ref.jacobian(c.p[:4], c.T[:4], c.Y[:, :4])
    J1, _ = port.jacobian(c.p[:4], c.T[:4], c.Y[:, :4])
    assert np.max(np.abs(J1 - J0) / np.abs(J0).max(axis=(1, 2), keepdims=True)) < 1e-12
    np.testing.assert_allclose(port.tc(c.p, c.T, c.rho0, c.Y), ref.tc(c.p, c.T, c.rho0, c.Y), rtol=1e-12)
    # one CFD step of 1e-5 s (ignition of the hotter cells)
    ci = c.subset(np.arange(4))
    r0 = oracle.Reference(flat, abs_tol=1e-8, rel_tol=1e-4).integrate(ci, 1e-5)
    r1 = port.integrate(ci, 1e-5, abs_tol=1e-8, rel_tol=1e-4)
    assert (r0["status"] == 0).all() and (r1["status"] == 0).all()
    np.testing.assert_allclose(r1["T"], r0["T"], rtol=1e-8)
    np.testing.assert_allclose(r1["Y"], r0["Y"], atol=1e-9)
    assert abs(r1["counters"]["jacobians"] - r0["counters"]["jacobians"]) <= 2


SOLVER_MECHS = [("Ignition0D/CH4_GRI30", "CH4"), ("CounterFlowFlame2D/NH3_Zhang", "NH3"),
                ("Ignition0D/H2_Connaire2004", "h2")]


@pytest.mark.parametrize("solver", ["OptRosenbrock34", "OptRodas23", "OptRosenbrock23", "OptSeulex"])
@pytest.mark.parametrize("case,fuel", SOLVER_MECHS, ids=[m[0].split("/")[1] for m in SOLVER_MECHS])
def test_tutorial_mechanism_other_solvers(ref_available, case, fuel, solver):
    """The other registered solvers on real mechanisms (fall-off and CH2(S)
    in GRI-3.0, PLOG in NH3_Zhang, non-equilibrium third-body reactions in
    H2_Connaire2004): one 1e-5 s CFD step of ignition-like cells, the oracle
    against the reference core compiled from its sources."""
    import oracle
    from fcs import _lib
    rpath, tpath = _files(case)
    flat, names = _lib.parse_mechanism_foam(rpath, tpath)
    c = _cells(flat, names, fuel, 3, seed=len(names) + 1)
    r0 = oracle.Reference(flat, solver=solver, abs_tol=1e-8, rel_tol=1e-4).integrate(c, 1e-5)
    r1 = oracle.Port(flat).integrate(c, 1e-5, solver=solver, abs_tol=1e-8, rel_tol=1e-4)
    assert (r0["status"] == 0).all() and (r1["status"] == 0).all()
    np.testing.assert_allclose(r1["T"], r0["T"], rtol=1e-8)
    np.testing.assert_allclose(r1["Y"], r0["Y"], atol=1e-9)
    # Seulex may take one ulp-level extra step at the end of the interval
    assert abs(r1["counters"]["jacobians"] - r0["counters"]["jacobians"]) <= (3 if solver == "OptSeulex" else 2)
