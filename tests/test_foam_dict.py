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


@pytest.mark.parametrize("wname", ["ignition_10s", "counterflow_53s", "falloff_16s", "noneq_14s", "long_24s"])
def test_reactions_file_round_trip(tmp_path, lib_path, wname):
    """The writer's reactions / speciesThermo files read back by the library's
    reader (fcs_parse_mechanism_foam, no GPU) give the generator's mechanism:
    kinds, reversibility, stoichiometry (as multisets: the file groups repeated
    species as "2H"), Arrhenius / kInf / reverse rates, efficiencies of the
    third-body kinds, fall-off parameters, PLOG tables and thermo."""
    import numpy as np
    import fcs
    from fcs.mechanism import FALLOFF_KINDS, NONEQ_THIRD_BODY, THIRD_BODY
    mech = fcs.WORKLOADS[wname].mechanism()
    a = fcs.flatten(mech)
    paths = foam_io.write_case(mech, str(tmp_path))
    b, names = _lib.parse_mechanism_foam(paths["reactions"], paths["thermo"])
    assert names == list(mech.species)
    assert (b.n_species, b.n_reactions) == (a.n_species, a.n_reactions)
    for k in ("W", "T_low", "T_high", "T_common", "high_coeffs", "low_coeffs", "type", "reversible",
              "lhs_offset", "rhs_offset", "arrhenius", "arrhenius2", "falloff_params", "plog_offset"):
        np.testing.assert_array_equal(getattr(b, k), getattr(a, k), err_msg=k)
    np.testing.assert_array_equal(b.plog_table[:a.plog_table.size], a.plog_table)
    ns = a.n_species
    for r in range(a.n_reactions):
        for off, sp in (("lhs_offset", "lhs_species"), ("rhs_offset", "rhs_species")):
            o = getattr(a, off)
            assert sorted(getattr(b, sp)[o[r]:o[r + 1]]) == sorted(getattr(a, sp)[o[r]:o[r + 1]])
        if a.type[r] in (THIRD_BODY, NONEQ_THIRD_BODY) or a.type[r] in FALLOFF_KINDS:
            np.testing.assert_array_equal(b.efficiencies[r * ns:(r + 1) * ns], a.efficiencies[r * ns:(r + 1) * ns])


def test_reader_openfoam_word_and_list_forms(tmp_path, lib_path):
    """Species names with parentheses (CH2(S)), a thermo database holding
    species the mechanism does not use, uniform lists `7 { 0 }`, comments
    and an entry commented out with /* */ are read as OpenFOAM reads them."""
    import numpy as np
    coeffs = "( 3.5 0.001 0 0 0 -1000 3 )"
    thermo = ["species 3 ( CH2(S) CH2 H2 );"]
    for sp, w in (("CH2(S)", 14.027), ("UNUSED", 10.0), ("CH2", 14.027), ("H2", 2.016)):
        body = "highCpCoeffs 7 { 0 }; lowCpCoeffs 7 { 0 };" if sp == "UNUSED" else \
            f"highCpCoeffs {coeffs}; lowCpCoeffs {coeffs};"
        thermo.append(f"{sp} {{ specie {{ molWeight {w}; }} thermodynamics {{ Tlow 200; Thigh 3500; "
                      f"Tcommon 1000; {body} }} }}")
    (tmp_path / "thermo").write_text("\n".join(thermo) + "\n")
    (tmp_path / "reactions").write_text("""// the singlet methylene quench
reactions
{
    un-named-reaction-0
    {
        type            reversibleArrhenius;
        reaction        "CH2(S) + H2 = CH2 + H2";   // collision partner on both sides
        A               7e+09;
        beta            0;
        Ta              0;
    }
    /*un-named-reaction-1
    {
        type            irreversibleArrhenius;
        reaction        "CH2 = CH2(S)";
        A 1; beta 0; Ta 0;
    }*/
    un-named-reaction-1
    {
        type            irreversibleArrhenius;
        reaction        "2CH2(S) = CH2 + CH2";
        A               1e+10;
        beta            0.5;
        Ta              100;
    }
}
""")
    b, names = _lib.parse_mechanism_foam(str(tmp_path / "reactions"), str(tmp_path / "thermo"))
    assert names == ["CH2(S)", "CH2", "H2"]
    assert b.n_reactions == 2
    np.testing.assert_array_equal(b.reversible, [1, 0])
    np.testing.assert_array_equal(b.lhs_species, [0, 2, 0, 0])
    np.testing.assert_array_equal(b.rhs_species, [1, 2, 1, 1])
    np.testing.assert_array_equal(b.arrhenius, [7e9, 0, 0, 1e10, 0.5, 100])
    np.testing.assert_allclose(b.W, [14.027, 14.027, 2.016])


# ---------------------------------------------------------------------------
# Files the reader must refuse (FCS_ERR_PARSE, or FCS_ERR_UNSUPPORTED for a
# reaction type it does not implement) without crashing or hanging: the flow
# solver hands the library whatever its case directory holds.

FCS_ERR_UNSUPPORTED = 6
FCS_ERR_PARSE = 7

_NASA = "( 3.5 0.001 0 0 0 -1000 3 )"
_THERMO = "species 3 ( A B C );\n" + "".join(
    f"{s} {{ specie {{ molWeight {w}; }} thermodynamics {{ Tlow 200; Thigh 3500; Tcommon 1000; "
    f"highCpCoeffs {_NASA}; lowCpCoeffs {_NASA}; }} }}\n" for s, w in (("A", 10), ("B", 20), ("C", 30)))
_ARR = "A 1e10; beta 0; Ta 100;"
_TBE = "thirdBodyEfficiencies { coeffs 3 ( (A 1) (B 2) (C 3) ); }"
_K = "k0 { A 1; beta 0; Ta 0; } kInf { A 2; beta 0; Ta 0; }"


def _reactions(body):
    return "reactions\n{\n    r0\n    {\n        " + body + "\n    }\n}\n"


def _parse(tmp_path, reactions, thermo=_THERMO):
    r, t = tmp_path / "reactions", tmp_path / "thermo"
    r.write_text(reactions)
    t.write_text(thermo)
    return _lib.parse_mechanism_foam(str(r), str(t))


_REFUSED = {
    "empty reactions file": ("", _THERMO),
    "no reactions dictionary": ("foo { }\n", _THERMO),
    "reactions as a list": ("reactions ( );\n", _THERMO),
    "unknown species": (_reactions(f'type reversibleArrhenius; reaction "X + B = C"; {_ARR}'), _THERMO),
    "empty term": (_reactions(f'type reversibleArrhenius; reaction "A + = C"; {_ARR}'), _THERMO),
    "no reactants": (_reactions(f'type reversibleArrhenius; reaction "= C"; {_ARR}'), _THERMO),
    "no products": (_reactions(f'type reversibleArrhenius; reaction "A ="; {_ARR}'), _THERMO),
    "leading +": (_reactions(f'type reversibleArrhenius; reaction "+ A = C"; {_ARR}'), _THERMO),
    "double +": (_reactions(f'type reversibleArrhenius; reaction "A + + B = C"; {_ARR}'), _THERMO),
    "no =": (_reactions(f'type reversibleArrhenius; reaction "A B C"; {_ARR}'), _THERMO),
    "two =": (_reactions(f'type reversibleArrhenius; reaction "A = B = C"; {_ARR}'), _THERMO),
    "negative coefficient": (_reactions(f'type reversibleArrhenius; reaction "-1A = C"; {_ARR}'), _THERMO),
    "fractional coefficient": (_reactions(f'type reversibleArrhenius; reaction "0.5A = C"; {_ARR}'), _THERMO),
    "coefficient without digits": (_reactions(f'type reversibleArrhenius; reaction ".A = C"; {_ARR}'), _THERMO),
    "coefficient out of range": (_reactions(f'type reversibleArrhenius; reaction "99999999999999999999A = C"; {_ARR}'),
                                 _THERMO),
    "reaction order syntax": (_reactions(f'type reversibleArrhenius; reaction "A^2 = C"; {_ARR}'), _THERMO),
    "missing A": (_reactions('type reversibleArrhenius; reaction "A + B = C"; beta 0; Ta 0;'), _THERMO),
    "A not a number": (_reactions('type reversibleArrhenius; reaction "A + B = C"; A abc; beta 0; Ta 0;'), _THERMO),
    "third body without coeffs": (_reactions(f'type reversibleThirdBodyArrhenius; reaction "A + B = C"; {_ARR}'),
                                  _THERMO),
    "sized list of the wrong size": (_reactions(f'type reversibleThirdBodyArrhenius; reaction "A + B = C"; {_ARR} '
                                                'coeffs 3 ( (A 1) (B 1) );'), _THERMO),
    "fall-off without efficiencies": (_reactions(f'type reversibleArrheniusLindemannFallOff; reaction "A + B = C"; {_K}'),
                                      _THERMO),
    "Troe without F": (_reactions(f'type reversibleArrheniusTroeFallOff; reaction "A + B = C"; {_K} {_TBE}'), _THERMO),
    "SRI without e": (_reactions(f'type reversibleArrheniusSRIFallOff; reaction "A + B = C"; {_K} '
                                 f'F {{ a 1; b 2; c 3; d 1; }} {_TBE}'), _THERMO),
    "PLOG without rows": (_reactions('type reversibleArrheniusPLOG; reaction "A + B = C"; ArrheniusData ( );'),
                          _THERMO),
    "PLOG row of three": (_reactions('type reversibleArrheniusPLOG; reaction "A + B = C"; ArrheniusData ( (1e5 1 0) );'),
                          _THERMO),
    "truncated file": (_reactions(f'type reversibleArrhenius; reaction "A + B = C"; {_ARR}')[:-10], _THERMO),
    "unterminated string": (_reactions(f'type reversibleArrhenius; reaction "A + B = C; {_ARR}'), _THERMO),
    "unterminated comment": (_reactions(f'type reversibleArrhenius; reaction "A + B = C"; {_ARR}') + "/* open",
                             _THERMO),
    "unbalanced }": ("reactions\n{\n}\n}\n", _THERMO),
    "NUL bytes": ("reactions { r0 { type \0\0\0; } }\n", _THERMO),
    "nested too deeply": ("reactions\n" + "{ a\n" * 5000 + "}\n" * 5000, _THERMO),
    "thermo missing a listed species": (_reactions(f'type reversibleArrhenius; reaction "A + B = C"; {_ARR}'),
                                        _THERMO.replace("species 3 ( A B C );", "species 4 ( A B C D );")),
    "species list of the wrong size": (_reactions(f'type reversibleArrhenius; reaction "A + B = C"; {_ARR}'),
                                       _THERMO.replace("species 3 ( A B C );", "species 5 ( A B C );")),
    "six NASA coefficients": (_reactions(f'type reversibleArrhenius; reaction "A + B = C"; {_ARR}'),
                              _THERMO.replace(_NASA, "( 3.5 0.001 0 0 0 -1000 )", 1)),
    "empty thermo": (_reactions(f'type reversibleArrhenius; reaction "A + B = C"; {_ARR}'), ""),
}


@pytest.mark.parametrize("case", list(_REFUSED), ids=list(_REFUSED))
def test_reader_refuses_malformed_files(tmp_path, lib_path, case):
    reactions, thermo = _REFUSED[case]
    with pytest.raises(_lib.FcsError) as e:
        _parse(tmp_path, reactions, thermo)
    assert e.value.code == FCS_ERR_PARSE


def test_reader_refuses_unknown_reaction_types(tmp_path, lib_path):
    for t in ("fooArrhenius", "reversibleArrheniusTroeChemicallyActivated", "irreversibleLandauTellerReaction"):
        with pytest.raises(_lib.FcsError) as e:
            _parse(tmp_path, _reactions(f'type {t}; reaction "A + B = C"; {_ARR}'))
        assert e.value.code == FCS_ERR_UNSUPPORTED, t


def test_reader_takes_the_well_formed_neighbours(tmp_path, lib_path):
    """The same files, well formed: the fall-off parameters, a third-body list
    that leaves species out (they keep efficiency 1), integer coefficients,
    and more species than the GPU takes (the loader, not the reader, refuses
    those)."""
    import numpy as np
    troe = _reactions(f'type reversibleArrheniusTroeFallOff; reaction "A + B = C"; {_K} '
                      f'F {{ alpha 0.5; Tsss 100; Ts 1000; Tss 5000; }} {_TBE}')
    b, _ = _parse(tmp_path, troe)
    np.testing.assert_array_equal(b.falloff_params, [0.5, 1000, 5000, 100, 0])
    np.testing.assert_array_equal(b.efficiencies, [1, 2, 3])
    tb = _reactions(f'type reversibleThirdBodyArrhenius; reaction "2A + B = 3C"; {_ARR} coeffs 2 ( (B 2.5) (C 4) );')
    b, _ = _parse(tmp_path, tb)
    np.testing.assert_array_equal(b.efficiencies, [1, 2.5, 4])
    np.testing.assert_array_equal(b.lhs_species, [0, 0, 1])
    np.testing.assert_array_equal(b.rhs_species, [2, 2, 2])
    many = "species 300 (" + " ".join(f"S{i}" for i in range(300)) + ");\n" + "".join(
        f"S{i} {{ specie {{ molWeight 10; }} thermodynamics {{ Tlow 200; Thigh 3500; Tcommon 1000; "
        f"highCpCoeffs {_NASA}; lowCpCoeffs {_NASA}; }} }}\n" for i in range(300))
    b, names = _parse(tmp_path, _reactions(f'type reversibleArrhenius; reaction "S0 + S1 = S299"; {_ARR}'), many)
    assert b.n_species == 300 and names[-1] == "S299"


def test_chemistry_properties_refuses_bad_counts(tmp_path, lib_path):
    for bad in ("maxSteps -5;", "maxSteps 1e12;", "maxSteps 2.5;", "maxSteps abc;"):
        p = tmp_path / "cp"
        p.write_text(f"chemistryType {{ solver OptRodas34; }}\nOptRodas34Coeffs {{ absTol 1e-8; relTol 1e-4; {bad} }}\n")
        with pytest.raises(_lib.FcsError) as e:
            _lib.read_chemistry_properties(str(p))
        assert e.value.code == FCS_ERR_PARSE, bad
    p.write_text("chemistryType { solver OptRodas34; }\nOptRodas34Coeffs { absTol 1e-8; relTol 1e-4; maxSteps 1e6; }\n")
    o, _ = _lib.read_chemistry_properties(str(p))
    assert o.max_steps == 1000000
