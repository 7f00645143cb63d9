"""Host-side pieces of bench.py that its JSON line depends on: the
algorithmic flop count behind roofline.achieved, the DRAM-traffic scaling
behind roofline.traffic, the disjoint CPU samples, and the clock summary."""
import sys

import numpy as np

from conftest import ROOT

sys.path.insert(0, ROOT)
import bench  # noqa: E402


def test_flops_per_attempt_of_the_headline_mechanism():
    import fcs
    mech = fcs.WORKLOADS["counterflow_53s"].mechanism()
    ns, nr = mech.n_species, mech.n_reactions
    ntb, nplog = mech.count(1), mech.count(2)
    f64, f32, n_exp = bench.flops_per_attempt(ns, nr, ntb, nplog, "OptRodas34", "fp64")
    assert (f64, f32) == (232632.0, 0.0)
    assert n_exp == 6 * (ns + nr + 2)
    # mixed: the LU and the FP32 halves of the refined solves move to FP32,
    # the residual (2 N^2 per solve) stays FP64
    m64, m32, _ = bench.flops_per_attempt(ns, nr, ntb, nplog, "OptRodas34", "mixed")
    n = ns + 1
    assert (m64, m32) == (127656.0, 174960.0)
    assert m64 + 2.0 / 3.0 * n ** 3 == f64
    # Rosenbrock34: 4 solves, 2 right-hand sides
    r64, _, _ = bench.flops_per_attempt(ns, nr, ntb, nplog, "OptRosenbrock34", "fp64")
    assert r64 < f64


def test_flops_formula_terms():
    # F_rhs = 40 Ns + 12 R + 2 Ns nTB + 10 nP; F_jac = F_rhs + 40 R + 4 Ns nTB + 10 N^2;
    # F_LU = 2/3 N^3; Rodas34: 6 solves of 2 N^2, 5 RHS, 40 N
    ns, nr, ntb, nplog = 10, 27, 3, 0
    n = ns + 1
    f_rhs = 40 * ns + 12 * nr + 2 * ns * ntb + 10 * nplog
    f_jac = f_rhs + 40 * nr + 4 * ns * ntb + 10 * n * n
    want = f_jac + 2.0 / 3.0 * n ** 3 + 6 * 2 * n * n + 5 * f_rhs + 40 * n
    assert bench.flops_per_attempt(ns, nr, ntb, nplog, "OptRodas34", "fp64")[0] == want


def test_launch_traffic_scales_by_the_records_unit():
    rec = {"w/OptRodas34/fp64/lane": {"bytes_per_attempt": 1000.0},
           "w/OptRodas34/fp64/g64": {"bytes_per_cell": 50.0}}
    assert bench.launch_traffic(rec, "w", "OptRodas34", "fp64", 1, attempts=7, cells=3) == 7000.0
    assert bench.launch_traffic(rec, "w", "OptRodas34", "fp64", 64, attempts=7, cells=3) == 150.0
    # no capture of this mapping, precision or workload: no traffic figure
    assert bench.launch_traffic(rec, "w", "OptRodas34", "fp64", 128, 7, 3) is None
    assert bench.launch_traffic(rec, "w", "OptRodas34", "mixed", 1, 7, 3) is None
    assert bench.launch_traffic(rec, "v", "OptRodas34", "fp64", 1, 7, 3) is None


def test_committed_traffic_records_are_well_formed():
    import json
    import os
    with open(os.path.join(ROOT, "profiles", "integrate_traffic.json")) as f:
        rec = json.load(f)
    for key, r in rec.items():
        if key.startswith("_"):
            continue
        workload, solver, precision, mapping = key.split("/")
        assert precision in ("fp64", "mixed") and (mapping == "lane" or mapping[0] == "g"), key
        assert ("bytes_per_attempt" in r) != ("bytes_per_cell" in r), key


def test_cell_sampler_takes_disjoint_cells_until_the_field_wraps():
    s = bench.CellSampler(100, seed=3)
    a, b = s.take(40), s.take(40)
    assert len(set(a) | set(b)) == 80
    c = s.take(40)  # 20 fresh cells, then the order starts again
    assert len(set(c[:20]) & (set(a) | set(b))) == 0
    assert list(c[20:]) == list(a[:20])
    # the same seed gives the same order
    assert list(bench.CellSampler(100, seed=3).take(10)) == list(a[:10])
    assert sorted(np.concatenate([a, b, c[:20]])) == list(range(100))


def test_clock_summary_reads_median_max_and_throttle_reasons():
    c = bench.ClockSampler(0)
    c.lines = [
        "0, 2070, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active",
        "0, 1980, 2070, 1400.0, 0x4, Not Active, Not Active, Not Active, Active",
        "0, 2070, 2070, 1100.0, 0x0, Not Active, Not Active, Not Active, Not Active",
        "garbage line",
    ]
    s = c.summary()
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0 and s["samples"] == 3
    assert s["reasons"] == ["sw_power_cap"]
    c.lines = ["0, 1200, 2070, 500, 0x0, Active, Not Active, Active, Not Active"]
    assert c.summary()["reasons"] == ["hw_slowdown", "sw_thermal_slowdown"]
