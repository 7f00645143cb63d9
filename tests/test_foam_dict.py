"""OpenFOAM dictionary reading at the boundary: chemistryProperties (host only)."""
import pytest

from fcs import _lib, foam_io


def test_chemistry_properties_keys(tmp_path, lib_path):
    path = str(tmp_path / "chemistryProperties")
    foam_io.write_chemistry_properties(path, solver="OptSeulex", jacobian="fast", abs_tol=1e-12,
                                       rel_tol=1e-6, treact=700.0, initial_dt=1e-7, precision="mixed",
                                       mapping="block128")
    o, sub = _lib.read_chemistry_properties(path)
    assert o.solver == 2 and o.jacobian == 1 and o.precision == 1 and o.mapping == 128
    assert o.abs_tol == 1e-12 and o.rel_tol == 1e-6 and o.T_react == 700.0 and sub == 1e-7
    assert o.max_steps == 10000


def test_chemistry_properties_defaults_and_dlb_keys_ignored(tmp_path, lib_path):
    path = str(tmp_path / "chemistryProperties")
    foam_io.write_chemistry_properties(path, extra=["maxChemicalTimeStep 1e-4;", "// comment", "/* block */"])
    o, sub = _lib.read_chemistry_properties(path)
    assert o.solver == 0 and o.jacobian == 0 and o.precision == 0 and o.delta_t_chem_max == 1e-4


def test_chemistry_properties_errors(tmp_path, lib_path):
    p = tmp_path / "cp"
    p.write_text("chemistryType { solver ode; }\nOptRodas34Coeffs { absTol 1e-8; relTol 1e-4; }\n")
    with pytest.raises(_lib.FcsError):
        _lib.read_chemistry_properties(str(p))
    p.write_text("chemistryType { solver OptRodas34; }\n")
    with pytest.raises(_lib.FcsError):  # absTol/relTol are required
        _lib.read_chemistry_properties(str(p))
    with pytest.raises(_lib.FcsError):
        _lib.read_chemistry_properties(str(tmp_path / "missing"))


@pytest.mark.parametrize("solver,code", [("OptRodas23", 3), ("OptRosenbrock23", 4), ("OptRosenbrock34", 1)])
def test_every_registered_solver_name(tmp_path, lib_path, solver, code):
    """All five solvers the plugin registers (odeChemistrySolvers.C:63-74)."""
    path = str(tmp_path / "chemistryProperties")
    foam_io.write_chemistry_properties(path, solver=solver)
    o, _ = _lib.read_chemistry_properties(path)
    assert o.solver == code
