"""Writers for the OpenFOAM dictionaries the plugin reads: ``reactions`` (with
``species`` list, and ``ArrheniusData`` for PLOG reactions), the species
thermo entries (``specie{molWeight}``, ``thermodynamics{...}``) and a
``chemistryProperties`` file.  The layout follows the reference tutorials
(e.g. tutorial/Ignition0D/*/constant/{reactions,speciesThermo}).
"""
from __future__ import annotations

import os

from .mechanism import ARRHENIUS, PLOG, THIRD_BODY, Mechanism


def _num(x: float) -> str:
    return repr(float(x))


def write_reactions(m: Mechanism, path: str) -> None:
    lines = [f"species {m.n_species} ( {' '.join(m.species)} );", "", "reactions", "{"]
    for k, r in enumerate(m.reactions):
        prefix = "reversible" if r.reversible else "irreversible"
        kind = {ARRHENIUS: "Arrhenius", THIRD_BODY: "ThirdBodyArrhenius", PLOG: "ArrheniusPLOG"}[r.kind]
        lines += [f"    un-named-reaction-{k}", "    {",
                  f"        type            {prefix}{kind};",
                  f'        reaction        "{m.reaction_string(r)}";',
                  f"        A               {_num(r.A)};",
                  f"        beta            {_num(r.beta)};",
                  f"        Ta              {_num(r.Ta)};"]
        if r.kind == THIRD_BODY:
            lines.append(f"        coeffs          {m.n_species}")
            lines.append("(")
            lines += [f"({m.species[i]} {_num(e)})" for i, e in enumerate(r.efficiencies)]
            lines.append(")")
            lines.append(";")
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
