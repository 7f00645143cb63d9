"""Seeded synthetic reaction mechanisms in the OpenFOAM ``reactions`` /
``speciesThermo`` data model.

A :class:`Mechanism` holds one mechanism in *file order* (the order the
reactions would appear in an OpenFOAM ``reactions`` dictionary).  Reordering
into the type blocks the solver uses happens inside the native library, the
same way the reference's loader does it (``src/Reaction/OptReaction.C:348-1339``).

The generator follows the synthetic-mechanism recipe of the benchmark
workloads:

* species are built from a few elements with random small integer atom
  counts; the atoms themselves are always present so that atom-exchange
  templates close;
* NASA-7 low/high coefficient sets are least-squares fits of a smooth,
  monotone cp(T) curve drawn in [25, 60] J/mol/K over 300-3000 K
  (Tcommon = 1000 K), with enthalpy / entropy constants set from a drawn
  formation enthalpy and standard entropy and made continuous at Tcommon;
* reactions are balanced by construction from atom-exchange templates with at
  most three reactants and three products; Arrhenius ``A`` is log-uniform,
  ``beta`` and ``Ta`` uniform in the given ranges;
* third-body reactions are recombination / dissociation templates with one
  efficiency per species (the reference requires every species to be listed,
  ``OptReaction.C:724-731``);
* PLOG reactions carry a table of (p, A, beta, Ta) rows on a log-spaced
  pressure grid (``reversibleArrheniusPLOG`` / ``ArrheniusData``).
"""
from __future__ import annotations

import dataclasses
import hashlib
import math
from typing import List, Optional, Sequence

import numpy as np

# Reaction kinds.  The integer values are the ``fcs_reaction_type`` enum of
# include/fcs.h.
ARRHENIUS = 0
THIRD_BODY = 1
PLOG = 2
LINDEMANN_FALLOFF = 3
TROE_FALLOFF = 4
SRI_FALLOFF = 5
NONEQ = 6
NONEQ_THIRD_BODY = 7

FALLOFF_KINDS = (LINDEMANN_FALLOFF, TROE_FALLOFF, SRI_FALLOFF)
NONEQ_KINDS = (NONEQ, NONEQ_THIRD_BODY)

# OpenFOAM type names; the (ir)reversible prefix is added by the writer except
# for the non-equilibrium kinds, whose names carry it
TYPE_NAMES = {
    ARRHENIUS: "Arrhenius",
    THIRD_BODY: "ThirdBodyArrhenius",
    PLOG: "ArrheniusPLOG",
    LINDEMANN_FALLOFF: "ArrheniusLindemannFallOff",
    TROE_FALLOFF: "ArrheniusTroeFallOff",
    SRI_FALLOFF: "ArrheniusSRIFallOff",
    NONEQ: "nonEquilibriumReversibleArrhenius",
    NONEQ_THIRD_BODY: "nonEquilibriumReversibleThirdBodyArrhenius",
}

ELEMENTS = ("H", "C", "O", "N")
ELEMENT_MASS = (1.00794, 12.0107, 15.9994, 14.0067)
R_MOLAR = 8.314462618  # J/(mol K), only used to build cp/R fits


@dataclasses.dataclass
class Reaction:
    kind: int
    reversible: bool
    lhs: List[int]          # species indices, repeated by stoichiometric coefficient
    rhs: List[int]
    A: float
    beta: float
    Ta: float
    efficiencies: Optional[np.ndarray] = None      # [Ns] for third-body / falloff
    plog: Optional[np.ndarray] = None              # [rows, 4] (p, A, beta, Ta)
    kinf: Optional[Sequence[float]] = None         # (A, beta, Ta) for falloff
    falloff: Optional[Sequence[float]] = None      # Troe (alpha, Ts, Tss, Tsss) / SRI (a,b,c,d,e)
    reverse: Optional[Sequence[float]] = None      # (A, beta, Ta) reverse rate of non-equilibrium kinds


@dataclasses.dataclass
class Mechanism:
    name: str
    species: List[str]
    W: np.ndarray           # [Ns] kg/kmol
    Tlow: np.ndarray        # [Ns]
    Thigh: np.ndarray       # [Ns]
    Tcommon: np.ndarray     # [Ns]
    high: np.ndarray        # [Ns, 7]
    low: np.ndarray         # [Ns, 7]
    composition: np.ndarray  # [Ns, nElements] atom counts
    reactions: List[Reaction]

    @property
    def n_species(self) -> int:
        return len(self.species)

    @property
    def n_reactions(self) -> int:
        return len(self.reactions)

    def count(self, kind: int) -> int:
        return sum(1 for r in self.reactions if r.kind == kind)

    def reaction_string(self, r: Reaction) -> str:
        def side(ix):
            out = []
            seen = []
            for s in ix:
                if s in seen:
                    continue
                seen.append(s)
                n = ix.count(s)
                out.append((f"{n}" if n > 1 else "") + self.species[s])
            return " + ".join(out)
        return f"{side(r.lhs)} = {side(r.rhs)}"

    def digest(self) -> str:
        """Stable hash of every number that defines the mechanism."""
        h = hashlib.sha256()
        for a in (self.W, self.Tlow, self.Thigh, self.Tcommon, self.high, self.low):
            h.update(np.ascontiguousarray(a, dtype=np.float64).tobytes())
        for r in self.reactions:
            h.update(np.array([r.kind, int(r.reversible), len(r.lhs), len(r.rhs)] + r.lhs + r.rhs,
                              dtype=np.int64).tobytes())
            h.update(np.array([r.A, r.beta, r.Ta], dtype=np.float64).tobytes())
            if r.efficiencies is not None:
                h.update(np.asarray(r.efficiencies, dtype=np.float64).tobytes())
            if r.plog is not None:
                h.update(np.asarray(r.plog, dtype=np.float64).tobytes())
            for extra in (r.kinf, r.falloff, r.reverse):
                if extra is not None:
                    h.update(np.asarray(extra, dtype=np.float64).tobytes())
        return h.hexdigest()[:16]


# --------------------------------------------------------------------------
# thermo fits


def _fit_range(Tlo, Thi, cp_over_R, rng_T):
    """Least-squares quartic fit of cp/R on [Tlo, Thi]."""
    T = np.linspace(Tlo, Thi, 64)
    y = cp_over_R(T)
    s = T / 1000.0
    V = np.vander(s, 5, increasing=True)
    c, *_ = np.linalg.lstsq(V, y, rcond=None)
    # back to coefficients in T (not T/1000)
    return np.array([c[0], c[1] / 1e3, c[2] / 1e6, c[3] / 1e9, c[4] / 1e12])


def _minus_G_over_RT(a, T):
    """B = -G/(RT) from one NASA-7 set (the exponent of exp(-G/RT))."""
    return (a[0] * (math.log(T) - 1) + a[1] * T / 2 + a[2] * T**2 / 6 + a[3] * T**3 / 12
            + a[4] * T**4 / 20 - a[5] / T + a[6])


def _H_over_R(a, T):
    return (a[0] * T + a[1] * T**2 / 2 + a[2] * T**3 / 3 + a[3] * T**4 / 4
            + a[4] * T**5 / 5)


def _S_over_R(a, T):
    return (a[0] * math.log(T) + a[1] * T + a[2] * T**2 / 2 + a[3] * T**3 / 3
            + a[4] * T**4 / 4)


def _thermo(rng, hf_kJ, s298):
    cp_lo = rng.uniform(25.0, 40.0)
    cp_hi = rng.uniform(max(cp_lo, 35.0), 60.0)
    tau = rng.uniform(400.0, 1500.0)

    def cp_over_R(T):
        return (cp_lo + (cp_hi - cp_lo) * (1.0 - np.exp(-(T - 300.0) / tau))) / R_MOLAR

    lo = _fit_range(300.0, 1000.0, cp_over_R, None)
    hi = _fit_range(1000.0, 3000.0, cp_over_R, None)
    T0 = 298.15
    a5_lo = hf_kJ * 1e3 / R_MOLAR - _H_over_R(lo, T0)
    a6_lo = s298 / R_MOLAR - _S_over_R(lo, T0)
    Tc = 1000.0
    a5_hi = _H_over_R(lo, Tc) + a5_lo - _H_over_R(hi, Tc)
    a6_hi = _S_over_R(lo, Tc) + a6_lo - _S_over_R(hi, Tc)
    return (np.concatenate([hi, [a5_hi, a6_hi]]),
            np.concatenate([lo, [a5_lo, a6_lo]]))


# --------------------------------------------------------------------------
# species and reactions


def _species(rng, n_species, n_elements, max_count):
    comps = []
    seen = set()
    # the atoms first: they close most atom-exchange templates
    for e in range(n_elements):
        c = [0] * n_elements
        c[e] = 1
        comps.append(tuple(c))
        seen.add(tuple(c))
    tries = 0
    while len(comps) < n_species:
        tries += 1
        c = tuple(int(x) for x in rng.integers(0, max_count + 1, size=n_elements))
        if sum(c) == 0 or sum(c) > 2 * max_count:
            continue
        if c in seen and tries < 50 * n_species:
            continue
        seen.add(c)
        comps.append(c)
    comps = np.array(comps, dtype=np.int64)
    names = []
    counts = {}
    for c in comps:
        base = "".join(f"{ELEMENTS[e]}{'' if c[e] == 1 else c[e]}"
                       for e in range(n_elements) if c[e] > 0)
        k = counts.get(base, 0)
        counts[base] = k + 1
        names.append(base if k == 0 else f"{base}X{k}")
    return names, comps


class _ReactionBuilder:
    def __init__(self, rng, comps):
        self.rng = rng
        self.comps = comps
        self.ns = len(comps)
        self.by_comp = {}
        for i, c in enumerate(comps):
            self.by_comp.setdefault(tuple(c), []).append(i)
        self.keys = set()

    def _key(self, lhs, rhs):
        a, b = tuple(sorted(lhs)), tuple(sorted(rhs))
        return (a, b) if a <= b else (b, a)

    def _accept(self, lhs, rhs):
        if sorted(lhs) == sorted(rhs):
            return False
        k = self._key(lhs, rhs)
        if k in self.keys:
            return False
        self.keys.add(k)
        return True

    def exchange(self):
        """A + B = C + D, or A + B = C + D + E (atom exchange)."""
        rng = self.rng
        for _ in range(400):
            a, b = (int(x) for x in rng.integers(0, self.ns, size=2))
            tot = self.comps[a] + self.comps[b]
            cands = [c for c in range(self.ns)
                     if np.all(self.comps[c] <= tot) and c not in (a, b)]
            rng.shuffle(cands)
            for c in cands:
                rest = tuple(tot - self.comps[c])
                if sum(rest) == 0:
                    continue
                ds = self.by_comp.get(rest)
                if ds:
                    d = ds[int(rng.integers(0, len(ds)))]
                    if self._accept([a, b], [c, d]):
                        return [a, b], [c, d]
                # three products: split the rest once more
                if rng.random() < 0.15:
                    rem = np.array(rest)
                    sub = [e for e in range(self.ns) if np.all(self.comps[e] <= rem)]
                    rng.shuffle(sub)
                    for e in sub:
                        r2 = tuple(rem - self.comps[e])
                        fs = self.by_comp.get(r2)
                        if sum(r2) > 0 and fs:
                            f = fs[int(rng.integers(0, len(fs)))]
                            if self._accept([a, b], [c, e, f]):
                                return [a, b], [c, e, f]
        return None

    def recombination(self):
        """A + B = C (written as dissociation C = A + B half of the time)."""
        rng = self.rng
        for _ in range(400):
            a, b = (int(x) for x in rng.integers(0, self.ns, size=2))
            tot = tuple(self.comps[a] + self.comps[b])
            cs = self.by_comp.get(tot)
            if not cs:
                continue
            c = cs[int(rng.integers(0, len(cs)))]
            if rng.random() < 0.5:
                lhs, rhs = [a, b], [c]
            else:
                lhs, rhs = [c], [a, b]
            if self._accept(lhs, rhs):
                return lhs, rhs
        return None


T_REF_ARRHENIUS = 1000.0


def _arrhenius(rng):
    """A log-uniform in [1e6, 1e14] is the rate-constant prefactor quoted at
    T_ref = 1000 K, k = A (T/T_ref)^beta exp(-Ta/T); the OpenFOAM form
    k = A' T^beta exp(-Ta/T) stores A' = A T_ref^-beta."""
    A = 10.0 ** rng.uniform(6.0, 14.0)
    beta = rng.uniform(-2.0, 3.0)
    Ta = rng.uniform(0.0, 30000.0)
    return A * T_REF_ARRHENIUS ** (-beta), beta, Ta


def synthetic_mechanism(n_species: int, n_reactions: int, n_third_body: int,
                        n_plog: int, seed: int, n_elements: int = 3,
                        max_count: int = 3, plog_points: int = 5,
                        plog_p_range=(1e4, 1e8), hf_range_kJ=(-100.0, 100.0),
                        name: Optional[str] = None, n_falloff=(0, 0, 0), n_noneq=(0, 0),
                        n_long=(0, 0)) -> Mechanism:
    """Build one seeded synthetic mechanism (all reactions reversible).

    The reactions are emitted in a shuffled *file* order so that the type
    reordering of the native loader is exercised.
    """
    rng = np.random.default_rng(seed)
    names, comps = _species(rng, n_species, n_elements, max_count)
    W = comps @ np.array(ELEMENT_MASS[:n_elements])
    high = np.zeros((n_species, 7))
    low = np.zeros((n_species, 7))
    for i in range(n_species):
        hf = rng.uniform(*hf_range_kJ)
        s298 = rng.uniform(150.0, 300.0)
        high[i], low[i] = _thermo(rng, hf, s298)

    # -G/RT of every species at 1000 K: used to write each reaction in its
    # exothermic (Kp >= 1) direction, as real mechanisms quote rate constants;
    # otherwise Kr = Kf/Kc of a reaction written "uphill" exceeds any collision
    # limit by many orders of magnitude.
    Bref = np.array([_minus_G_over_RT(high[i], 1000.0) for i in range(n_species)])

    def orient(lr):
        lhs, rhs = lr
        if Bref[rhs].sum() - Bref[lhs].sum() < 0:
            return rhs, lhs
        return lhs, rhs

    builder = _ReactionBuilder(rng, comps)
    reactions: List[Reaction] = []
    for _ in range(n_third_body):
        lr = builder.recombination() or builder.exchange()
        if lr is None:
            raise RuntimeError("could not close a third-body template; change the seed")
        lr = orient(lr)
        A, beta, Ta = _arrhenius(rng)
        eff = rng.uniform(0.5, 5.0, size=n_species)
        reactions.append(Reaction(THIRD_BODY, True, lr[0], lr[1], A, beta, Ta,
                                  efficiencies=eff))
    for _ in range(n_plog):
        lr = builder.exchange() if rng.random() < 0.6 else builder.recombination()
        if lr is None:
            lr = builder.exchange()
        if lr is None:
            raise RuntimeError("could not close a PLOG template; change the seed")
        lr = orient(lr)
        A, beta, Ta = _arrhenius(rng)
        p = np.logspace(math.log10(plog_p_range[0]), math.log10(plog_p_range[1]), plog_points)
        slope = rng.uniform(-0.6, 0.9)            # d ln A / d ln p
        bslope = rng.uniform(-0.05, 0.05)
        tslope = rng.uniform(-100.0, 100.0)
        x = np.log(p / 1e6)
        rows = np.stack([p,
                         A * np.exp(slope * x),
                         beta + bslope * x,
                         np.clip(Ta + tslope * x, 0.0, None)], axis=1)
        reactions.append(Reaction(PLOG, True, lr[0], lr[1], A, beta, Ta, plog=rows))
    # fall-off (Lindemann, Troe, SRI): recombinations with k0 (per unit of M)
    # above kInf so that Pr = k0 M / kInf crosses 1 over the fields' pressures
    for kind, count in zip((LINDEMANN_FALLOFF, TROE_FALLOFF, SRI_FALLOFF), n_falloff):
        for _ in range(count):
            lr = builder.recombination() or builder.exchange()
            if lr is None:
                raise RuntimeError("could not close a fall-off template; change the seed")
            lr = orient(lr)
            A, beta, Ta = _arrhenius(rng)
            A0 = A * 10.0 ** rng.uniform(1.0, 3.0)
            beta0 = beta - rng.uniform(0.0, 1.5)
            Ta0 = Ta * rng.uniform(0.0, 0.5)
            eff = rng.uniform(0.5, 5.0, size=n_species)
            if kind == TROE_FALLOFF:
                fo = (rng.uniform(0.2, 0.9), rng.uniform(500.0, 5000.0), rng.uniform(2000.0, 10000.0),
                      rng.uniform(50.0, 500.0))          # alpha, T*, T**, T***
            elif kind == SRI_FALLOFF:
                fo = (rng.uniform(0.5, 2.0), rng.uniform(100.0, 1000.0), rng.uniform(200.0, 2000.0),
                      rng.uniform(0.8, 1.2), rng.uniform(-0.5, 0.5))  # a, b, c, d, e
            else:
                fo = None
            reactions.append(Reaction(kind, True, lr[0], lr[1], A0 * T_REF_ARRHENIUS ** (beta - beta0), beta0, Ta0,
                                      efficiencies=eff, kinf=(A, beta, Ta), falloff=fo))
    # non-equilibrium reversible (plain and third-body): the reverse rate is
    # its own Arrhenius, fitted to Kf/Kc at 1000 K and 2000 K with the forward
    # beta and then moved off equilibrium by a factor 10^U(-0.5, 0.5)
    for kind, count in zip(NONEQ_KINDS, n_noneq):
        for _ in range(count):
            lr = builder.exchange() if kind == NONEQ else (builder.recombination() or builder.exchange())
            if lr is None:
                lr = builder.exchange()
            if lr is None:
                raise RuntimeError("could not close a non-equilibrium template; change the seed")
            lr = orient(lr)
            A, beta, Ta = _arrhenius(rng)
            g = []
            for T in (1000.0, 2000.0):
                B = np.array([_minus_G_over_RT(high[i], T) for i in range(n_species)])
                dnu = len(lr[1]) - len(lr[0])
                lnKc = B[lr[1]].sum() - B[lr[0]].sum() + dnu * math.log(1e5 / (8314.47 * T))
                g.append(math.log(A) - Ta / T - lnKc)   # ln(Kf / Kc) - beta ln T
            Ta_r = (g[1] - g[0]) / (1.0 / 1000.0 - 1.0 / 2000.0)
            if Ta_r < 0:
                Ta_r = 0.0
            lnA_r = g[0] + Ta_r / 1000.0 + rng.uniform(-0.5, 0.5) * math.log(10.0)
            eff = rng.uniform(0.5, 5.0, size=n_species) if kind == NONEQ_THIRD_BODY else None
            reactions.append(Reaction(kind, True, lr[0], lr[1], A, beta, Ta, efficiencies=eff,
                                      reverse=(math.exp(lnA_r), beta, Ta_r)))
    # long reactions (the reference's generic RFG/JFG path, more than three
    # species on a side): three balanced templates written as one reaction.
    # Irreversible ones mix exchanges and dissociations (global steps of
    # reduced mechanisms, up to 3 reactants and 7 products); reversible ones
    # join three dissociations (3 reactants, 6 products, dnu = 3).
    for reversible, count in ((False, n_long[0]), (True, n_long[1])):
        for _ in range(count):
            for _attempt in range(200):
                lhs, rhs = [], []
                for _k in range(3):
                    if reversible or rng.random() < 0.6:
                        lr = builder.recombination()
                        if lr is not None and len(lr[0]) == 2:
                            lr = (lr[1], lr[0])          # written as the dissociation
                    else:
                        lr = builder.exchange()
                        lr = orient(lr) if lr is not None else None
                    if lr is None:
                        break
                    lhs += list(lr[0])
                    rhs += list(lr[1])
                if lr is not None and len(lhs) <= 4 and 3 < len(rhs) <= 8:
                    break
            else:
                raise RuntimeError("could not close a long template; change the seed")
            A, beta, Ta = _arrhenius(rng)
            reactions.append(Reaction(ARRHENIUS, reversible, sorted(lhs), sorted(rhs), A, beta, Ta))
    while len(reactions) < n_reactions:
        r = rng.random()
        lr = builder.exchange() if r < 0.8 else builder.recombination()
        if lr is None:
            lr = builder.exchange()
        if lr is None:
            raise RuntimeError("could not close an exchange template; change the seed")
        lr = orient(lr)
        A, beta, Ta = _arrhenius(rng)
        reactions.append(Reaction(ARRHENIUS, True, lr[0], lr[1], A, beta, Ta))
    order = rng.permutation(len(reactions))
    reactions = [reactions[i] for i in order]
    return Mechanism(
        name=name or f"synthetic_{n_species}s_{n_reactions}r_seed{seed}",
        species=names, W=W.astype(np.float64),
        Tlow=np.full(n_species, 300.0), Thigh=np.full(n_species, 3000.0),
        Tcommon=np.full(n_species, 1000.0), high=high, low=low,
        composition=comps, reactions=reactions)


# --------------------------------------------------------------------------
# flat description (the layout of ``fcs_mechanism_desc``)


@dataclasses.dataclass
class FlatMechanism:
    """Numpy arrays laid out exactly as ``fcs_mechanism_desc`` expects."""
    n_species: int
    n_reactions: int
    W: np.ndarray
    T_low: np.ndarray
    T_high: np.ndarray
    T_common: np.ndarray
    high_coeffs: np.ndarray     # [Ns*7]
    low_coeffs: np.ndarray      # [Ns*7]
    type: np.ndarray            # int32 [R]
    reversible: np.ndarray      # int32 [R]
    lhs_offset: np.ndarray      # int32 [R+1]
    lhs_species: np.ndarray     # int32
    rhs_offset: np.ndarray
    rhs_species: np.ndarray
    arrhenius: np.ndarray       # [R*3]
    arrhenius2: np.ndarray      # [R*3]
    efficiencies: np.ndarray    # [R*Ns]
    falloff_params: np.ndarray  # [R*5]
    plog_offset: np.ndarray     # int32 [R+1]
    plog_table: np.ndarray      # [rows*4]


def flatten(m: Mechanism) -> FlatMechanism:
    ns, nr = m.n_species, m.n_reactions
    typ = np.array([r.kind for r in m.reactions], dtype=np.int32)
    rev = np.array([1 if r.reversible else 0 for r in m.reactions], dtype=np.int32)
    lo = np.zeros(nr + 1, dtype=np.int32)
    ro = np.zeros(nr + 1, dtype=np.int32)
    ls, rs = [], []
    for i, r in enumerate(m.reactions):
        ls += r.lhs
        rs += r.rhs
        lo[i + 1] = len(ls)
        ro[i + 1] = len(rs)
    arr = np.array([[r.A, r.beta, r.Ta] for r in m.reactions], dtype=np.float64).reshape(-1)
    arr2 = np.zeros(nr * 3)
    eff = np.zeros(nr * ns)
    fp = np.zeros(nr * 5)
    po = np.zeros(nr + 1, dtype=np.int32)
    pt = []
    for i, r in enumerate(m.reactions):
        if r.kinf is not None:
            arr2[3 * i:3 * i + 3] = r.kinf
        if r.reverse is not None:
            arr2[3 * i:3 * i + 3] = r.reverse
        if r.efficiencies is not None:
            eff[i * ns:(i + 1) * ns] = r.efficiencies
        if r.falloff is not None:
            fp[5 * i:5 * i + len(r.falloff)] = r.falloff
        if r.plog is not None:
            pt.append(np.asarray(r.plog, dtype=np.float64))
        po[i + 1] = po[i] + (0 if r.plog is None else len(r.plog))
    plog_table = (np.concatenate(pt).reshape(-1) if pt else np.zeros(4))
    return FlatMechanism(
        ns, nr, np.ascontiguousarray(m.W, dtype=np.float64),
        np.ascontiguousarray(m.Tlow, dtype=np.float64),
        np.ascontiguousarray(m.Thigh, dtype=np.float64),
        np.ascontiguousarray(m.Tcommon, dtype=np.float64),
        np.ascontiguousarray(m.high, dtype=np.float64).reshape(-1),
        np.ascontiguousarray(m.low, dtype=np.float64).reshape(-1),
        typ, rev, lo, np.array(ls, dtype=np.int32), ro, np.array(rs, dtype=np.int32),
        arr, arr2, eff, fp, po, plog_table)
