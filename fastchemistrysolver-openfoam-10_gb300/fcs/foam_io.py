"""Writers for the OpenFOAM dictionaries the plugin reads: ``reactions`` (with
``species`` list, ``ArrheniusData`` for PLOG reactions, k0 / kInf / F for
fall-off and forward / reverse for non-equilibrium reactions), the species
thermo entries (``specie{molWeight}``, ``thermodynamics{...}``) and a
``chemistryProperties`` file.  The layout follows the reference tutorials
(e.g. tutorial/Ignition0D/*/constant/{reactions,speciesThermo}).
"""
from __future__ import annotations

import os

from typing import List

from .mechanism import (FALLOFF_KINDS, NONEQ_KINDS, NONEQ_THIRD_BODY, PLOG, SRI_FALLOFF, THIRD_BODY, TROE_FALLOFF,
                        TYPE_NAMES, Mechanism)


def _num(x: float) -> str:
    return repr(float(x))


def _coeffs(m: Mechanism, eff, indent: str) -> List[str]:
    return ([f"{indent}coeffs          {m.n_species}", "("] +
            [f"({m.species[i]} {_num(e)})" for i, e in enumerate(eff)] + [")", ";"])


def _arrhenius_block(name: str, abt, indent: str, extra: List[str] = ()) -> List[str]:
    A, beta, Ta = abt
    return ([f"{indent}{name}", f"{indent}{{",
             f"{indent}    A               {_num(A)};",
             f"{indent}    beta            {_num(beta)};",
             f"{indent}    Ta              {_num(Ta)};"] + list(extra) + [f"{indent}}}"])


def write_reactions(m: Mechanism, path: str) -> None:
    """Every kind in the layout of the reference's tutorial mechanisms:
    k0 / kInf / F / thirdBodyEfficiencies for fall-off, forward / reverse
    sub-dictionaries (with the coefficient list in both) for the
    non-equilibrium kinds."""
    lines = [f"species {m.n_species} ( {' '.join(m.species)} );", "", "reactions", "{"]
    for k, r in enumerate(m.reactions):
        if r.kind in NONEQ_KINDS:
            tname = TYPE_NAMES[r.kind]
        else:
            tname = ("reversible" if r.reversible else "irreversible") + TYPE_NAMES[r.kind]
        lines += [f"    un-named-reaction-{k}", "    {",
                  f"        type            {tname};",
                  f'        reaction        "{m.reaction_string(r)}";']
        if r.kind in FALLOFF_KINDS:
            lines += _arrhenius_block("k0", (r.A, r.beta, r.Ta), "        ")
            lines += _arrhenius_block("kInf", r.kinf, "        ")
            names = {TROE_FALLOFF: ("alpha", "Ts", "Tss", "Tsss"), SRI_FALLOFF: ("a", "b", "c", "d", "e")}
            lines += ["        F", "        {"]
            for nm, v in zip(names.get(r.kind, ()), r.falloff or ()):
                lines.append(f"            {nm:<16}{_num(v)};")
            lines += ["        }", "        thirdBodyEfficiencies", "        {"]
            lines += _coeffs(m, r.efficiencies, "            ")
            lines.append("        }")
        elif r.kind in NONEQ_KINDS:
            tb = _coeffs(m, r.efficiencies, "            ") if r.kind == NONEQ_THIRD_BODY else []
            lines += _arrhenius_block("forward", (r.A, r.beta, r.Ta), "        ", tb)
            lines += _arrhenius_block("reverse", r.reverse, "        ", tb)
        else:
            lines += [f"        A               {_num(r.A)};",
                      f"        beta            {_num(r.beta)};",
                      f"        Ta              {_num(r.Ta)};"]
        if r.kind == THIRD_BODY:
            lines += _coeffs(m, r.efficiencies, "        ")
        if r.kind == PLOG:
            lines.append("        ArrheniusData")
            lines.append("        (")
            lines += [f"            ({_num(p)} {_num(a)} {_num(b)} {_num(t)})" for p, a, b, t in r.plog]
            lines.append("        );")
        lines.append("    }")
    lines.append("}")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def write_thermo(m: Mechanism, path: str) -> None:
    lines = []
    for i, s in enumerate(m.species):
        lines += [s, "{", "    specie", "    {", f"        molWeight       {_num(m.W[i])};", "    }",
                  "    thermodynamics", "    {",
                  f"        Tlow            {_num(m.Tlow[i])};",
                  f"        Thigh           {_num(m.Thigh[i])};",
                  f"        Tcommon         {_num(m.Tcommon[i])};",
                  "        highCpCoeffs    ( " + " ".join(_num(x) for x in m.high[i]) + " );",
                  "        lowCpCoeffs     ( " + " ".join(_num(x) for x in m.low[i]) + " );",
                  "    }", "}", ""]
    with open(path, "w") as f:
        f.write("\n".join(lines))


def write_chemistry_properties(path: str, solver="OptRodas34", jacobian="exact", abs_tol=1e-8,
                               rel_tol=1e-4, treact=0.0, initial_dt=1e-7, precision=None,
                               mapping=None, extra=()) -> None:
    lines = ["FoamFile", "{", "    format      ascii;", "    class       dictionary;",
             "    object      chemistryProperties;", "}", "",
             "chemistryType", "{", f"    solver          {solver};", "    method          FastChemistryModel;", "}",
             "", "chemistry       on;", f"initialChemicalTimeStep {_num(initial_dt)};",
             f"jacobian {jacobian};", f"Treact {_num(treact)};",
             "balance off;", "Iter 1;", "DLBthreshold 1.1;", ""]
    for s in ("OptRodas34", "OptRosenbrock34", "OptSeulex", "OptRodas23", "OptRosenbrock23"):
        lines += [f"{s}Coeffs", "{", f"    absTol          {_num(abs_tol)};",
                  f"    relTol          {_num(rel_tol)};", "}"]
    if precision or mapping:
        lines += ["FastChemistryGPU", "{"]
        if precision:
            lines.append(f"    precision {precision};")
        if mapping:
            lines.append(f"    mapping {mapping};")
        lines.append("}")
    lines += list(extra)
    lines += ['', '#include "reactions"', ""]
    with open(path, "w") as f:
        f.write("\n".join(lines))


def write_case(m: Mechanism, directory: str, **props) -> dict:
    os.makedirs(directory, exist_ok=True)
    paths = dict(reactions=os.path.join(directory, "reactions"),
                 thermo=os.path.join(directory, "speciesThermo"),
                 chemistryProperties=os.path.join(directory, "chemistryProperties"))
    write_reactions(m, paths["reactions"])
    write_thermo(m, paths["thermo"])
    write_chemistry_properties(paths["chemistryProperties"], **props)
    return paths
