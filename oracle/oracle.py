"""ctypes bindings of the two CPU checkers.  TEST INFRASTRUCTURE ONLY.

* :class:`Port` -- the plain-C restatement (``oracle/_build/libfcs_oracle.so``),
  portable, used by tests, ``smoke()`` and the cpu_baseline / reference leg of
  ``bench.py`` as the checker and as the timed CPU baseline.
* :class:`Reference` -- the reference's own numerical core compiled from its
  unmodified sources (``oracle/_ref/libfcs_ref.so``: with AVX2 on x86-64, with
  the portable SIMD shim of ``oracle/simd_shim`` elsewhere), used to validate
  the restatement, to generate the golden fixtures, and as the timed CPU
  baseline of the bench where it is built.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "libfcs_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libfcs_ref.so")
REF_SHIM_SO = os.path.join(HERE, "_ref", "libfcs_ref_shim.so")
STAGED_SRC = os.path.join(HERE, "_ref", "src")   # unmodified reference sources for hosts without the tree
# Where the reference project lives is never assumed: it comes from the
# FCS_REFERENCE environment variable (the project root, holding src/ and
# tutorial/), or from the record the last reference build left in _ref/.
REF_ROOT_RECORD = os.path.join(HERE, "_ref", "REFERENCE_ROOT")


def reference_root():
    """The reference project's root directory, or None when it is unknown
    or absent on this host."""
    root = os.environ.get("FCS_REFERENCE")
    if not root and os.path.exists(REF_ROOT_RECORD):
        root = open(REF_ROOT_RECORD).read().strip()
    return root if root and os.path.isdir(os.path.join(root, "src")) else None


def reference_tutorial():
    """The reference's tutorial tree (mechanisms and cases), or None."""
    root = reference_root()
    d = os.path.join(root, "tutorial") if root else None
    return d if d and os.path.isdir(d) else None

SOLVERS = {"OptRodas34": 0, "OptRosenbrock34": 1, "OptSeulex": 2, "OptRodas23": 3, "OptRosenbrock23": 4}

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_lp = C.POINTER(C.c_int64)


class MechDesc(C.Structure):
    _fields_ = [("n_species", C.c_int32), ("n_reactions", C.c_int32),
                ("W", _dp), ("T_low", _dp), ("T_high", _dp), ("T_common", _dp),
                ("high_coeffs", _dp), ("low_coeffs", _dp),
                ("type", _ip), ("reversible", _ip),
                ("lhs_offset", _ip), ("lhs_species", _ip),
                ("rhs_offset", _ip), ("rhs_species", _ip),
                ("arrhenius", _dp), ("arrhenius2", _dp), ("efficiencies", _dp),
                ("falloff_params", _dp), ("plog_offset", _ip), ("plog_table", _dp)]


def make_desc(flat):
    """fcs_mechanism_desc over the arrays of a FlatMechanism (kept alive on
    the returned object)."""
    d = MechDesc()
    keep = []

    def p(a, t):
        a = np.ascontiguousarray(a)
        keep.append(a)
        return a.ctypes.data_as(C.POINTER(t))
    d.n_species = flat.n_species
    d.n_reactions = flat.n_reactions
    d.W = p(flat.W, C.c_double); d.T_low = p(flat.T_low, C.c_double)
    d.T_high = p(flat.T_high, C.c_double); d.T_common = p(flat.T_common, C.c_double)
    d.high_coeffs = p(flat.high_coeffs, C.c_double); d.low_coeffs = p(flat.low_coeffs, C.c_double)
    d.type = p(flat.type, C.c_int32); d.reversible = p(flat.reversible, C.c_int32)
    d.lhs_offset = p(flat.lhs_offset, C.c_int32); d.lhs_species = p(flat.lhs_species, C.c_int32)
    d.rhs_offset = p(flat.rhs_offset, C.c_int32); d.rhs_species = p(flat.rhs_species, C.c_int32)
    d.arrhenius = p(flat.arrhenius, C.c_double); d.arrhenius2 = p(flat.arrhenius2, C.c_double)
    d.efficiencies = p(flat.efficiencies, C.c_double)
    d.falloff_params = p(flat.falloff_params, C.c_double)
    d.plog_offset = p(flat.plog_offset, C.c_int32); d.plog_table = p(flat.plog_table, C.c_double)
    d._keep = keep
    return d


def _ptr(a, t=C.c_double):
    return None if a is None else a.ctypes.data_as(C.POINTER(t))


def build(ref: bool = True, root: str | None = None):
    """Compile the port (always) and the reference core where it can be built:

    * x86-64 with the reference tree (``root``, else :func:`reference_root`):
      from its sources with AVX2/FMA and libmvec, as the reference builds
      itself; the sources it needs are also staged, unmodified, into
      ``_ref/src`` (git-ignored) for hosts without the tree;
    * other hosts (aarch64): from the staged copy, with ``simd_shim/`` for
      ``<immintrin.h>`` and libmvec.

    The root used is recorded in ``_ref/REFERENCE_ROOT``."""
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    if not ref:
        return
    if root and not os.path.isdir(os.path.join(root, "src")):
        root = None
    root = root or reference_root()
    if root:
        src = os.path.join(root, "src")
        subprocess.run(["make", "-s", "-C", HERE, "ref-stage", "REF=" + src], check=True)
        with open(REF_ROOT_RECORD, "w") as f:
            f.write(root + "\n")
    if os.uname().machine == "x86_64":
        if root:
            subprocess.run(["make", "-s", "-C", HERE, "ref", "REF=" + os.path.join(root, "src")], check=True)
    elif os.path.exists(os.path.join(STAGED_SRC, "Reaction", "OptReaction.H")):
        if os.path.exists(REF_SO) and not _native_elf(REF_SO):
            os.remove(REF_SO)  # built on another architecture
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)


def _native_elf(path) -> bool:
    """Whether the shared object at `path` is for this host's architecture
    (ELF e_machine: 62 x86-64, 183 aarch64)."""
    want = {"x86_64": 62, "aarch64": 183}.get(os.uname().machine)
    with open(path, "rb") as f:
        head = f.read(20)
    return len(head) == 20 and head[:4] == b"\x7fELF" and (want is None or int.from_bytes(head[18:20], "little") == want)


def build_shim() -> str | None:
    """The reference core built with the portable SIMD shim on this host (the
    build the aarch64 hosts use), for checking the shim against the fixtures
    made by the AVX2 build; None when the reference sources are absent."""
    if os.uname().machine != "x86_64":
        return REF_SO if os.path.exists(REF_SO) else None
    root = reference_root()
    if not root:
        return None
    subprocess.run(["make", "-s", "-C", HERE, "ref-shim", "REF=" + os.path.join(root, "src")], check=True)
    return REF_SHIM_SO


class OrcOptions(C.Structure):
    _fields_ = [("solver", C.c_int32), ("jacobian", C.c_int32),
                ("conversion_as_written", C.c_int32), ("max_steps", C.c_int32),
                ("abs_tol", C.c_double), ("rel_tol", C.c_double),
                ("T_react", C.c_double), ("delta_t_chem_max", C.c_double),
                ("n_threads", C.c_int32)]


COUNTER_NAMES = ("attempts", "accepted", "jacobians", "lu", "rhs", "solves", "cells", "failed")


class Port:
    def __init__(self, flat):
        if not os.path.exists(PORT_SO):
            build(ref=False)
        self.lib = C.CDLL(PORT_SO)
        L = self.lib
        L.orc_mech_create.restype = C.c_void_p
        L.orc_mech_create.argtypes = [C.POINTER(MechDesc), _ip]
        L.orc_mech_destroy.argtypes = [C.c_void_p]
        L.orc_integrate.argtypes = [C.c_void_p, C.POINTER(OrcOptions), C.c_int64, C.c_double, _dp,
                                    _dp, _dp, _dp, _dp, _dp, _dp, _ip, _dp, _lp]
        L.orc_rhs.argtypes = [C.c_void_p, C.c_int64, _dp, _dp, _dp, _dp]
        L.orc_jacobian.argtypes = [C.c_void_p, C.POINTER(OrcOptions), C.c_int64, _dp, _dp, _dp, _dp, _dp]
        L.orc_lu_solve.argtypes = [C.c_int32, _dp, C.c_int32, _dp, _ip, _dp]
        L.orc_mech_order.argtypes = [C.c_void_p, _ip]
        L.orc_rates.argtypes = [C.c_void_p, C.c_int64, _dp, _dp, _dp, _dp, _dp, _dp]
        L.orc_tc.argtypes = [C.c_void_p, C.c_int64, _dp, _dp, _dp, _dp, _dp]
        self.ns = flat.n_species
        self.nr = flat.n_reactions
        self.desc = make_desc(flat)
        st = C.c_int32(0)
        self.h = L.orc_mech_create(C.byref(self.desc), C.byref(st))
        if not self.h:
            raise RuntimeError(f"oracle mechanism rejected (status {st.value})")

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.orc_mech_destroy(self.h)
            self.h = None

    def order(self):
        out = np.zeros(self.nr, dtype=np.int32)
        self.lib.orc_mech_order(self.h, _ptr(out, C.c_int32))
        return out

    @staticmethod
    def options(solver="OptRodas34", jacobian="exact", abs_tol=1e-8, rel_tol=1e-4,
                max_steps=10000, treact=0.0, dt_chem_max=1e300, threads=1, as_written=False):
        o = OrcOptions()
        o.solver = SOLVERS[solver]
        o.jacobian = 0 if jacobian == "exact" else 1
        o.conversion_as_written = 1 if as_written else 0
        o.max_steps = max_steps
        o.abs_tol = abs_tol
        o.rel_tol = rel_tol
        o.T_react = treact
        o.delta_t_chem_max = dt_chem_max
        o.n_threads = threads
        return o

    def integrate(self, cells, dt, dt_per_cell=None, **opt):
        """Integrate a copy of ``cells``; returns (T, Y, subDt, RR, status,
        deltaTMin, counters)."""
        o = self.options(**opt)
        n = cells.n
        T = cells.T.copy()
        Y = np.ascontiguousarray(cells.Y.copy())
        sub = cells.subDt.copy()
        RR = np.zeros_like(Y)
        status = np.zeros(n, dtype=np.int32)
        dmin = C.c_double(0)
        cnt = np.zeros(8, dtype=np.int64)
        dtc = None if dt_per_cell is None else np.ascontiguousarray(dt_per_cell, dtype=np.float64)
        self.lib.orc_integrate(self.h, C.byref(o), n, dt, _ptr(dtc), _ptr(cells.p), _ptr(cells.rho0),
                               _ptr(T), _ptr(Y), _ptr(sub), _ptr(RR), _ptr(status, C.c_int32),
                               C.byref(dmin), _ptr(cnt, C.c_int64))
        return dict(T=T, Y=Y, subDt=sub, RR=RR, status=status, deltaTMin=dmin.value,
                    counters=dict(zip(COUNTER_NAMES, cnt.tolist())))

    def rhs(self, p, T, Y):
        n = T.shape[0]
        out = np.zeros((self.ns + 1, n))
        self.lib.orc_rhs(self.h, n, _ptr(np.ascontiguousarray(p)), _ptr(np.ascontiguousarray(T)),
                         _ptr(np.ascontiguousarray(Y)), _ptr(out))
        return out

    def jacobian(self, p, T, Y, jacobian="exact", as_written=False):
        n = T.shape[0]
        N = self.ns + 1
        J = np.zeros((n, N, N))
        f = np.zeros((N, n))
        o = self.options(jacobian=jacobian, as_written=as_written)
        self.lib.orc_jacobian(self.h, C.byref(o), n, _ptr(np.ascontiguousarray(p)),
                              _ptr(np.ascontiguousarray(T)), _ptr(np.ascontiguousarray(Y)),
                              _ptr(J), _ptr(f))
        return J, f

    def rates(self, p, T, rho, Y):
        n = T.shape[0]
        RR = np.zeros((self.ns, n))
        Q = np.zeros(n)
        self.lib.orc_rates(self.h, n, _ptr(np.ascontiguousarray(p)), _ptr(np.ascontiguousarray(T)),
                           _ptr(np.ascontiguousarray(rho)), _ptr(np.ascontiguousarray(Y)), _ptr(RR), _ptr(Q))
        return RR, Q

    def tc(self, p, T, rho, Y):
        n = T.shape[0]
        out = np.zeros(n)
        self.lib.orc_tc(self.h, n, _ptr(np.ascontiguousarray(p)), _ptr(np.ascontiguousarray(T)),
                        _ptr(np.ascontiguousarray(rho)), _ptr(np.ascontiguousarray(Y)), _ptr(out))
        return out

    def lu_solve(self, a, b):
        a = np.ascontiguousarray(a, dtype=np.float64).copy()
        b = np.ascontiguousarray(b, dtype=np.float64).copy()
        n = a.shape[0]
        piv = np.zeros(n, dtype=np.int32)
        invD = np.zeros(n)
        self.lib.orc_lu_solve(n, _ptr(a), b.shape[0], _ptr(b), _ptr(piv, C.c_int32), _ptr(invD))
        return a, b, piv, invD


class Reference:
    """The reference core compiled from its own sources (x86-64 only)."""

    def __init__(self, flat, solver="OptRodas34", jacobian="exact", abs_tol=1e-8, rel_tol=1e-4,
                 max_steps=10000, so=None):
        if so is None and not os.path.exists(REF_SO):
            build(ref=True)
        self.lib = C.CDLL(so or REF_SO)
        L = self.lib
        L.ref_create.restype = C.c_void_p
        L.ref_create.argtypes = [C.POINTER(MechDesc), C.c_int, C.c_int, C.c_double, C.c_double, C.c_int]
        L.ref_destroy.argtypes = [C.c_void_p]
        L.ref_integrate.argtypes = [C.c_void_p, C.c_int64, C.c_double, _dp, _dp, _dp, _dp, _dp, _dp,
                                    _ip, C.c_double, C.c_double, _dp, _lp, C.c_int]
        L.ref_rhs.argtypes = [C.c_void_p, C.c_int64, _dp, _dp, _dp, _dp]
        L.ref_jacobian.argtypes = [C.c_void_p, C.c_int64, _dp, _dp, _dp, _dp, _dp]
        L.ref_lu_solve.argtypes = [C.c_int, _dp, C.c_int, _dp]
        L.ref_tc.argtypes = [C.c_void_p, C.c_int64, _dp, _dp, _dp, _dp, _dp]
        self.ns = flat.n_species
        self.desc = make_desc(flat)
        self.h = L.ref_create(C.byref(self.desc), SOLVERS[solver], 0 if jacobian == "exact" else 1,
                              abs_tol, rel_tol, max_steps)
        if not self.h:
            raise RuntimeError("reference driver rejected the mechanism")

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.ref_destroy(self.h)
            self.h = None

    def integrate(self, cells, dt, treact=0.0, dt_chem_max=1e300, threads=1):
        n = cells.n
        T = cells.T.copy()
        Y = np.ascontiguousarray(cells.Y.copy())
        sub = cells.subDt.copy()
        RR = np.zeros_like(Y)
        status = np.zeros(n, dtype=np.int32)
        dmin = C.c_double(0)
        cnt = np.zeros(4, dtype=np.int64)
        self.lib.ref_integrate(self.h, n, dt, _ptr(cells.p), _ptr(cells.rho0), _ptr(T), _ptr(Y),
                               _ptr(sub), _ptr(RR), _ptr(status, C.c_int32), treact, dt_chem_max,
                               C.byref(dmin), _ptr(cnt, C.c_int64), threads)
        return dict(T=T, Y=Y, subDt=sub, RR=RR, status=status, deltaTMin=dmin.value,
                    counters=dict(jacobians=int(cnt[0]), rhs=int(cnt[1]), cells=int(cnt[2]),
                                  failed=int(cnt[3])))

    def rhs(self, p, T, Y):
        n = T.shape[0]
        out = np.zeros((self.ns + 1, n))
        self.lib.ref_rhs(self.h, n, _ptr(np.ascontiguousarray(p)), _ptr(np.ascontiguousarray(T)),
                         _ptr(np.ascontiguousarray(Y)), _ptr(out))
        return out

    def jacobian(self, p, T, Y):
        n = T.shape[0]
        N = self.ns + 1
        J = np.zeros((n, N, N))
        f = np.zeros((N, n))
        self.lib.ref_jacobian(self.h, n, _ptr(np.ascontiguousarray(p)), _ptr(np.ascontiguousarray(T)),
                              _ptr(np.ascontiguousarray(Y)), _ptr(J), _ptr(f))
        return J, f

    def tc(self, p, T, rho, Y):
        n = T.shape[0]
        out = np.zeros(n)
        self.lib.ref_tc(self.h, n, _ptr(np.ascontiguousarray(p)), _ptr(np.ascontiguousarray(T)),
                        _ptr(np.ascontiguousarray(rho)), _ptr(np.ascontiguousarray(Y)), _ptr(out))
        return out

    def lu_solve(self, a, b):
        a = np.ascontiguousarray(a, dtype=np.float64).copy()
        b = np.ascontiguousarray(b, dtype=np.float64).copy()
        self.lib.ref_lu_solve(a.shape[0], _ptr(a), b.shape[0], _ptr(b))
        return a, b
