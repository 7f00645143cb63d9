"""Synthetic mechanism generator and workloads (host logic)."""
import numpy as np
import pytest

import fcs
from fcs.mechanism import PLOG, THIRD_BODY


@pytest.mark.parametrize("name", list(fcs.WORKLOADS))
def test_generator_sizes_and_balance(name):
    w = fcs.WORKLOADS[name]
    m = w.mechanism()
    a = w.mech_args
    assert m.n_species == a["n_species"] and m.n_reactions == a["n_reactions"]
    assert m.count(THIRD_BODY) == a["n_third_body"] and m.count(PLOG) == a["n_plog"]
    for r in m.reactions:
        long = a.get("n_long", (0, 0))
        assert 1 <= len(r.lhs) <= (4 if sum(long) else 3) and 1 <= len(r.rhs) <= (8 if sum(long) else 3)
        # atom conservation by construction
        assert np.array_equal(m.composition[r.lhs].sum(0), m.composition[r.rhs].sum(0))
        if r.kinf is not None:
            # fall-off: kInf in the generic ranges, k0 (per unit of M) 10-1000x above it at 1000 K
            A, beta, Ta = r.kinf
            lg = np.log10(r.A * 1000.0 ** r.beta) - np.log10(A * 1000.0 ** beta)
            assert 1.0 - 1e-9 <= lg <= 3.0 + 1e-9
            assert beta - 1.5 <= r.beta <= beta and 0 <= r.Ta <= 0.5 * Ta
        else:
            A, beta, Ta = r.A, r.beta, r.Ta
        assert 6.0 <= np.log10(A * 1000.0 ** beta) <= 14.0 + 1e-9
        assert -2 <= beta <= 3 and 0 <= Ta <= 30000
    # cp(T) of every fit stays in [25, 60] J/mol/K over 300..3000 K (small fit error allowed)
    T = np.linspace(300, 3000, 28)
    for i in range(m.n_species):
        for lo, hi, c in ((300, 1000, m.low[i]), (1000, 3000, m.high[i])):
            t = T[(T >= lo) & (T <= hi)]
            cp = 8.314462618 * (c[0] + c[1] * t + c[2] * t ** 2 + c[3] * t ** 3 + c[4] * t ** 4)
            assert cp.min() > 24.0 and cp.max() < 61.0


def test_generator_is_deterministic():
    w = fcs.WORKLOADS["counterflow_53s"]
    assert w.mechanism().digest() == w.mechanism().digest()


def test_flatten_layout():
    w = fcs.WORKLOADS["counterflow_53s"]
    m = w.mechanism()
    f = fcs.flatten(m)
    assert f.lhs_offset[-1] == len(f.lhs_species) and f.rhs_offset[-1] == len(f.rhs_species)
    assert f.efficiencies.shape == (m.n_reactions * m.n_species,)
    assert f.plog_offset[-1] * 4 == f.plog_table.size
    assert f.arrhenius.shape == (3 * m.n_reactions,)


def test_cells_layout_and_density():
    w = fcs.WORKLOADS["counterflow_53s"]
    m = w.mechanism()
    c = fcs.cells_for(w, m, n=300)
    assert c.Y.shape == (53, 300) and c.Y.flags["C_CONTIGUOUS"]
    np.testing.assert_allclose(c.Y.sum(0), 1.0, rtol=1e-12)
    assert (c.T >= 300).all() and (c.T <= 2200).all()
    rho = c.p / (fcs.workloads.RU * c.T * (c.Y / m.W[:, None]).sum(0))
    np.testing.assert_allclose(c.rho0, rho)
    full = fcs.WORKLOADS["uneven_111s"]
    cu = fcs.cells_for(full, full.mechanism(), n=20000)
    frac_frozen = np.mean(cu.T < 900)
    assert 0.75 < frac_frozen < 0.85
