"""Loads a golden fixture's exact inputs (mechanism arrays and cell states)."""
import numpy as np

import fcs
from fcs.mechanism import FlatMechanism
from fcs.workloads import Cells

FIELDS = ("W", "T_low", "T_high", "T_common", "high_coeffs", "low_coeffs", "type", "reversible",
          "lhs_offset", "lhs_species", "rhs_offset", "rhs_species", "arrhenius", "arrhenius2",
          "efficiencies", "falloff_params", "plog_offset", "plog_table")


def load(g):
    """(FlatMechanism, Cells) stored in the fixture npz ``g``."""
    arrays = {k: np.ascontiguousarray(g["mech_" + k]) for k in FIELDS}
    flat = FlatMechanism(int(arrays["W"].shape[0]), int(arrays["type"].shape[0]), **arrays)
    cells = Cells(g["in_T"].copy(), g["in_p"].copy(), np.ascontiguousarray(g["in_Y"]), g["in_rho0"].copy(),
                  g["in_subDt"].copy())
    return flat, cells


def check_generator(g, wname):
    """The seeded generator still produces this fixture's mechanism and cells
    (to rounding: platforms' libm and LAPACK differ in the last bits)."""
    w = fcs.WORKLOADS[wname]
    mech = w.mechanism()
    flat = fcs.flatten(mech)
    for k in FIELDS:
        a, b = getattr(flat, k), g["mech_" + k]
        assert a.shape == b.shape, k
        np.testing.assert_allclose(a, b, rtol=1e-9, atol=1e-12, err_msg=k)
    cells = fcs.cells_for(w, mech).subset(g["cell_index"])
    np.testing.assert_allclose(cells.T, g["in_T"], rtol=1e-12)
    np.testing.assert_allclose(cells.Y, g["in_Y"], rtol=1e-9, atol=1e-15)


class _Prefixed:
    def __init__(self, g, prefix):
        self.g, self.prefix = g, prefix

    def __getitem__(self, k):
        return self.g[self.prefix + k]


def load_prefixed(g, prefix):
    """load() for a fixture that stores several cases under '<prefix>' keys."""
    return load(_Prefixed(g, prefix))
