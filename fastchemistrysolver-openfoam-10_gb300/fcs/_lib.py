"""ctypes binding of libfcs_cuda.so (the C ABI declared in include/fcs.h).

The product path is the CUDA library only: if ``lib/libfcs_cuda.so`` is
missing, :func:`load` raises -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

from .build import LIB

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)

SOLVERS = {"OptRodas34": 0, "OptRosenbrock34": 1, "OptSeulex": 2, "OptRodas23": 3, "OptRosenbrock23": 4}
PRECISIONS = {"fp64": 0, "mixed": 1}
JACOBIANS = {"exact": 0, "fast": 1}
PTR_DEVICE = 1
NO_QUEUE_SORT = 2
CUDA_GRAPH = 4

CELL_STATUS = {0: "ok", 1: "max_steps", 2: "nonfinite", 3: "dt_underflow", 4: "skipped"}
ERRORS = {0: "OK", 1: "INVALID", 2: "CUDA", 3: "NOMEM", 4: "STATE", 5: "CELLS", 6: "UNSUPPORTED",
          7: "PARSE", 8: "TIMEOUT"}

EXPORTS = ("fcs_create", "fcs_destroy", "fcs_last_error_string", "fcs_version", "fcs_load_mechanism",
           "fcs_load_mechanism_foam", "fcs_parse_mechanism_foam", "fcs_read_chemistry_properties",
           "fcs_default_options",
           "fcs_set_options", "fcs_mechanism_size", "fcs_integrate", "fcs_integrate_lts",
           "fcs_integrate_noalloc", "fcs_integrate_async", "fcs_sync", "fcs_sync_timeout",
           "fcs_test_fail_allocations", "fcs_formation_enthalpy", "fcs_rhs", "fcs_tc",
           "fcs_jacobian", "fcs_rates", "fcs_bench_fp64_peak", "fcs_bench_fp32_peak", "fcs_check_exp",
           # include/fcs_mlp.h
           "fcs_mlp_create", "fcs_mlp_destroy", "fcs_mlp_last_error", "fcs_mlp_get_shape", "fcs_mlp_param_count",
           "fcs_mlp_default_train_options", "fcs_mlp_set_params", "fcs_mlp_get_params",
           "fcs_mlp_set_normalization", "fcs_mlp_get_normalization", "fcs_mlp_forward", "fcs_mlp_gradients",
           "fcs_mlp_train", "fcs_mlp_save", "fcs_mlp_load", "fcs_gate_default_options", "fcs_surrogate_attach",
           "fcs_integrate_gated")


class MechDesc(C.Structure):
    _fields_ = [("n_species", C.c_int32), ("n_reactions", C.c_int32),
                ("W", _dp), ("T_low", _dp), ("T_high", _dp), ("T_common", _dp),
                ("high_coeffs", _dp), ("low_coeffs", _dp),
                ("type", _ip), ("reversible", _ip),
                ("lhs_offset", _ip), ("lhs_species", _ip),
                ("rhs_offset", _ip), ("rhs_species", _ip),
                ("arrhenius", _dp), ("arrhenius2", _dp), ("efficiencies", _dp),
                ("falloff_params", _dp), ("plog_offset", _ip), ("plog_table", _dp)]


MechVisitor = C.CFUNCTYPE(C.c_int32, C.POINTER(MechDesc), C.POINTER(C.c_char_p), C.c_void_p)


class Options(C.Structure):
    _fields_ = [("solver", C.c_int32), ("jacobian", C.c_int32), ("precision", C.c_int32),
                ("mapping", C.c_int32), ("abs_tol", C.c_double), ("rel_tol", C.c_double),
                ("max_steps", C.c_int32), ("max_rejects", C.c_int32), ("T_react", C.c_double),
                ("delta_t_chem_max", C.c_double)]


class StepStats(C.Structure):
    _fields_ = [("cells_integrated", C.c_int64), ("cells_skipped", C.c_int64),
                ("cells_failed", C.c_int64), ("attempts", C.c_int64), ("accepted", C.c_int64),
                ("jacobians", C.c_int64), ("lu_decompositions", C.c_int64),
                ("rhs_evaluations", C.c_int64), ("linear_solves", C.c_int64),
                ("fp64_fallbacks", C.c_int64), ("kernel_ms", C.c_double), ("call_ms", C.c_double),
                ("mapping", C.c_int32), ("reserved", C.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class MlpShape(C.Structure):
    _fields_ = [("n_in", C.c_int32), ("n_out", C.c_int32), ("width", C.c_int32), ("depth", C.c_int32),
                ("members", C.c_int32)]


class MlpTrainOptions(C.Structure):
    _fields_ = [("epochs", C.c_int32), ("batch", C.c_int32), ("lr", C.c_double), ("lr_final", C.c_double),
                ("beta1", C.c_double), ("beta2", C.c_double), ("eps", C.c_double), ("seed", C.c_uint64)]


class GateOptions(C.Structure):
    _fields_ = [("T_rel", C.c_double), ("Y_abs", C.c_double), ("element_abs", C.c_double),
                ("audit_fraction", C.c_double), ("seed_substep", C.c_int32), ("reserved", C.c_int32)]


class GateStats(C.Structure):
    _fields_ = [("cells_active", C.c_int64), ("cells_accepted", C.c_int64), ("cells_fallback", C.c_int64),
                ("cells_audited", C.c_int64), ("audit_max_rel_T", C.c_double), ("audit_max_abs_Y", C.c_double),
                ("surrogate_ms", C.c_double), ("integrate_ms", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_LIB: Optional[C.CDLL] = None


def load(path: str = LIB) -> C.CDLL:
    """Load the CUDA library (raises when it has not been built)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with fcs.build.build() -- there is no CPU fallback")
    L = C.CDLL(path)
    vp = C.c_void_p
    L.fcs_create.argtypes = [C.POINTER(vp), C.c_int]
    L.fcs_destroy.argtypes = [vp]
    L.fcs_last_error_string.argtypes = [vp]
    L.fcs_last_error_string.restype = C.c_char_p
    L.fcs_version.restype = C.c_char_p
    L.fcs_load_mechanism.argtypes = [vp, C.POINTER(MechDesc)]
    L.fcs_load_mechanism_foam.argtypes = [vp, C.c_char_p, C.c_char_p]
    L.fcs_parse_mechanism_foam.argtypes = [C.c_char_p, C.c_char_p, MechVisitor, vp]
    L.fcs_read_chemistry_properties.argtypes = [C.c_char_p, C.POINTER(Options), _dp]
    L.fcs_default_options.argtypes = [C.POINTER(Options)]
    L.fcs_set_options.argtypes = [vp, C.POINTER(Options)]
    L.fcs_mechanism_size.argtypes = [vp, _ip, _ip]
    L.fcs_formation_enthalpy.argtypes = [vp, _dp]
    cell_args = [vp, C.c_int64, C.c_double, vp, vp, vp, vp, vp, vp, vp, C.POINTER(StepStats), _dp, C.c_int32]
    L.fcs_integrate.argtypes = cell_args
    L.fcs_integrate_lts.argtypes = [vp, C.c_int64, vp] + cell_args[3:]
    L.fcs_integrate_noalloc.argtypes = cell_args[:-1]
    L.fcs_integrate_async.argtypes = [vp, C.c_int64, C.c_double] + [vp] * 7 + [C.c_int32, vp]
    L.fcs_sync.argtypes = [vp, C.POINTER(StepStats), _dp]
    L.fcs_sync_timeout.argtypes = [vp, C.c_double, C.POINTER(StepStats), _dp]
    L.fcs_test_fail_allocations.argtypes = [C.c_int32]
    L.fcs_rhs.argtypes = [vp, C.c_int64, vp, vp, vp, vp, C.c_int32]
    L.fcs_jacobian.argtypes = [vp, C.c_int64, vp, vp, vp, vp, vp, C.c_int32]
    L.fcs_rates.argtypes = [vp, C.c_int64, vp, vp, vp, vp, vp, vp, C.c_int32]
    L.fcs_tc.argtypes = [vp, C.c_int64, vp, vp, vp, vp, vp, C.c_int32]
    L.fcs_bench_fp64_peak.argtypes = [C.c_int, C.c_double, _dp]
    L.fcs_bench_fp32_peak.argtypes = [C.c_int, C.c_double, _dp]
    L.fcs_check_exp.argtypes = [C.c_int, C.c_longlong, vp, vp, vp]
    _fp = C.POINTER(C.c_float)
    L.fcs_mlp_create.argtypes = [C.POINTER(vp), C.c_int, C.POINTER(MlpShape), C.c_uint64]
    L.fcs_mlp_destroy.argtypes = [vp]
    L.fcs_mlp_last_error.argtypes = [vp]
    L.fcs_mlp_last_error.restype = C.c_char_p
    L.fcs_mlp_get_shape.argtypes = [vp, C.POINTER(MlpShape)]
    L.fcs_mlp_param_count.argtypes = [vp, C.POINTER(C.c_int64)]
    L.fcs_mlp_default_train_options.argtypes = [C.POINTER(MlpTrainOptions)]
    L.fcs_mlp_set_params.argtypes = [vp, C.c_int32, vp]
    L.fcs_mlp_get_params.argtypes = [vp, C.c_int32, vp]
    L.fcs_mlp_set_normalization.argtypes = [vp, vp, vp, vp, vp]
    L.fcs_mlp_get_normalization.argtypes = [vp, vp, vp, vp, vp]
    L.fcs_mlp_forward.argtypes = [vp, C.c_int32, C.c_int64, vp, vp, C.c_int32]
    L.fcs_mlp_gradients.argtypes = [vp, C.c_int32, C.c_int64, vp, vp, _fp, vp]
    L.fcs_mlp_train.argtypes = [vp, C.c_int64, vp, vp, C.POINTER(MlpTrainOptions), vp]
    L.fcs_mlp_save.argtypes = [vp, C.c_char_p]
    L.fcs_mlp_load.argtypes = [C.POINTER(vp), C.c_int, C.c_char_p]
    L.fcs_gate_default_options.argtypes = [C.POINTER(GateOptions)]
    L.fcs_surrogate_attach.argtypes = [vp, vp, C.c_int32, vp, vp, C.POINTER(GateOptions)]
    L.fcs_integrate_gated.argtypes = cell_args + [C.POINTER(GateStats)]
    _LIB = L
    return L


class FcsError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"fcs error {ERRORS.get(code, code)}: {msg}")
        self.code = code


def _host64(a) -> np.ndarray:
    """A C-contiguous float64 host array (the argument itself when it already is one)."""
    return np.ascontiguousarray(a, dtype=np.float64)


def _addr(a):
    """Address of a C-contiguous numpy array or torch tensor (None -> NULL).
    The caller keeps the array alive for the whole C call; a strided view is
    refused rather than read with the wrong layout."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        if not a.flags.c_contiguous:
            raise ValueError("array arguments must be C-contiguous")
        return a.ctypes.data
    if not a.is_contiguous():  # torch tensor
        raise ValueError("tensor arguments must be contiguous")
    return a.data_ptr()


def make_desc(flat) -> MechDesc:
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


def fail_allocations(count: int) -> None:
    """Test hook: the next `count` device-buffer growths of the library fail
    (host side; fcs_test_fail_allocations)."""
    st = load().fcs_test_fail_allocations(int(count))
    if st:
        raise FcsError(st, "fcs_test_fail_allocations")


def fp64_peak_tflops(device: int = 0, ms: float = 50.0) -> float:
    """Measured dense FP64 FMA throughput of the device (TFLOP/s)."""
    L = load()
    v = C.c_double(0)
    st = L.fcs_bench_fp64_peak(device, ms, C.byref(v))
    if st:
        raise FcsError(st, "fp64 peak probe failed")
    return v.value


def fp32_peak_tflops(device: int = 0, ms: float = 50.0) -> float:
    L = load()
    v = C.c_double(0)
    st = L.fcs_bench_fp32_peak(device, ms, C.byref(v))
    if st:
        raise FcsError(st, "fp32 peak probe failed")
    return v.value


def check_exp(x, device: int = 0):
    """(integrator exp, CUDA exp) of the host array x."""
    L = load()
    x = np.ascontiguousarray(x, dtype=np.float64)
    a = np.empty_like(x)
    b = np.empty_like(x)
    st = L.fcs_check_exp(device, x.size, x.ctypes.data, a.ctypes.data, b.ctypes.data)
    if st:
        raise FcsError(st, "exp check failed")
    return a, b


def parse_mechanism_foam(reactions_path: str, thermo_path: str):
    """The mechanism of an OpenFOAM ``reactions`` + thermo file pair as the
    library reads it (fcs_parse_mechanism_foam; host only, no GPU):
    returns (FlatMechanism, species names)."""
    from .mechanism import FlatMechanism
    L = load()
    got = {}

    def visit(dp, names, _user):
        d = dp.contents
        ns, nr = d.n_species, d.n_reactions

        def arr(ptr, n, dtype):
            return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype, copy=True) if n else np.zeros(0, dtype)
        lo = arr(d.lhs_offset, nr + 1, np.int32)
        ro = arr(d.rhs_offset, nr + 1, np.int32)
        po = arr(d.plog_offset, nr + 1, np.int32)
        got["flat"] = FlatMechanism(
            ns, nr, arr(d.W, ns, np.float64), arr(d.T_low, ns, np.float64), arr(d.T_high, ns, np.float64),
            arr(d.T_common, ns, np.float64), arr(d.high_coeffs, 7 * ns, np.float64),
            arr(d.low_coeffs, 7 * ns, np.float64), arr(d.type, nr, np.int32), arr(d.reversible, nr, np.int32),
            lo, arr(d.lhs_species, int(lo[-1]), np.int32), ro, arr(d.rhs_species, int(ro[-1]), np.int32),
            arr(d.arrhenius, 3 * nr, np.float64), arr(d.arrhenius2, 3 * nr, np.float64),
            arr(d.efficiencies, nr * ns, np.float64), arr(d.falloff_params, 5 * nr, np.float64),
            po, arr(d.plog_table, 4 * max(int(po[-1]), 1), np.float64))
        got["names"] = [names[i].decode() for i in range(ns)]
        return 0

    cb = MechVisitor(visit)
    st = L.fcs_parse_mechanism_foam(reactions_path.encode(), thermo_path.encode(), cb, None)
    if st:
        raise FcsError(st, f"cannot read {reactions_path} / {thermo_path}")
    return got["flat"], got["names"]


def read_chemistry_properties(path: str):
    L = load()
    o = Options()
    sub = C.c_double(-1)
    st = L.fcs_read_chemistry_properties(path.encode(), C.byref(o), C.byref(sub))
    if st:
        raise FcsError(st, f"cannot read {path}")
    return o, sub.value


class Context:
    """One device context (the C ABI's fcs_ctx)."""

    def __init__(self, device: int = 0):
        self.L = load()
        self.h = C.c_void_p()
        st = self.L.fcs_create(C.byref(self.h), device)
        if st:
            raise FcsError(st, "fcs_create failed")
        self.ns = None
        self.options = Options()
        self.L.fcs_default_options(C.byref(self.options))

    def close(self):
        if self.h:
            self.L.fcs_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st):
        if st:
            raise FcsError(st, self.L.fcs_last_error_string(self.h).decode())

    def load_mechanism(self, flat):
        self._desc = make_desc(flat)
        self._check(self.L.fcs_load_mechanism(self.h, C.byref(self._desc)))
        self.ns = flat.n_species

    def load_mechanism_foam(self, reactions_path, thermo_path):
        self._check(self.L.fcs_load_mechanism_foam(self.h, reactions_path.encode(), thermo_path.encode()))
        ns, nr = C.c_int32(), C.c_int32()
        self._check(self.L.fcs_mechanism_size(self.h, C.byref(ns), C.byref(nr)))
        self.ns = ns.value
        return ns.value, nr.value

    def set_options(self, solver="OptRodas34", jacobian="exact", precision="fp64", mapping=0,
                    abs_tol=1e-8, rel_tol=1e-4, max_steps=10000, max_rejects=1000, treact=0.0,
                    dt_chem_max=1e300):
        o = Options()
        o.solver = SOLVERS[solver]; o.jacobian = JACOBIANS[jacobian]
        o.precision = PRECISIONS[precision]; o.mapping = int(mapping)
        o.abs_tol = abs_tol; o.rel_tol = rel_tol; o.max_steps = max_steps
        o.max_rejects = max_rejects; o.T_react = treact; o.delta_t_chem_max = dt_chem_max
        self._check(self.L.fcs_set_options(self.h, C.byref(o)))
        self.options = o

    def integrate_raw(self, n, dt, p, rho0, T, Y, sub, RR=None, status=None, device=False,
                      dt_per_cell=None, check=True, flags=0):
        """Arrays are numpy (host) or torch CUDA tensors with device=True;
        extra fcs_integrate flags (FCS_NO_QUEUE_SORT, FCS_CUDA_GRAPH) in `flags`."""
        stats = StepStats()
        dmin = C.c_double(0)
        flags = (PTR_DEVICE if device else 0) | flags
        if dt_per_cell is not None:
            st = self.L.fcs_integrate_lts(self.h, n, _addr(dt_per_cell), _addr(p), _addr(rho0), _addr(T),
                                          _addr(Y), _addr(sub), _addr(RR), _addr(status), C.byref(stats),
                                          C.byref(dmin), flags)
        else:
            st = self.L.fcs_integrate(self.h, n, 0.0 if dt is None else dt, _addr(p), _addr(rho0), _addr(T), _addr(Y), _addr(sub),
                                      _addr(RR), _addr(status), C.byref(stats), C.byref(dmin), flags)
        if check and st not in (0, 5):
            self._check(st)
        return st, stats.as_dict(), dmin.value

    def integrate_noalloc(self, n, dt, p, rho0, T, Y, sub, RR=None, status=None, check=True):
        """fcs_integrate_noalloc on caller-owned device arrays (torch CUDA tensors)."""
        stats = StepStats()
        dmin = C.c_double(0)
        st = self.L.fcs_integrate_noalloc(self.h, n, dt, _addr(p), _addr(rho0), _addr(T), _addr(Y), _addr(sub),
                                          _addr(RR), _addr(status), C.byref(stats), C.byref(dmin))
        if check and st not in (0, 5):
            self._check(st)
        return st, stats.as_dict(), dmin.value

    def integrate_async(self, n, dt, p, rho0, T, Y, sub, RR=None, status=None, stream=None, flags=0):
        """fcs_integrate_async on torch CUDA tensors; `stream` a torch.cuda.Stream (None: the context's)."""
        st = self.L.fcs_integrate_async(self.h, n, dt, _addr(p), _addr(rho0), _addr(T), _addr(Y), _addr(sub),
                                        _addr(RR), _addr(status), flags,
                                        None if stream is None else stream.cuda_stream)
        self._check(st)

    def sync(self, check=True, timeout_ms=None):
        """fcs_sync, or fcs_sync_timeout when timeout_ms is given (which may
        return code 8, TIMEOUT, with the step still in flight)."""
        stats = StepStats()
        dmin = C.c_double(0)
        if timeout_ms is None:
            st = self.L.fcs_sync(self.h, C.byref(stats), C.byref(dmin))
        else:
            st = self.L.fcs_sync_timeout(self.h, float(timeout_ms), C.byref(stats), C.byref(dmin))
        if check and st not in (0, 5, 8):
            self._check(st)
        return st, stats.as_dict(), dmin.value

    def last_error(self):
        return self.L.fcs_last_error_string(self.h).decode()

    def integrate(self, cells, dt, dt_per_cell=None):
        """Integrate a copy of host ``cells``; returns the same dict as the oracle."""
        n = cells.n
        T = cells.T.copy()
        Y = np.ascontiguousarray(cells.Y.copy())
        sub = cells.subDt.copy()
        RR = np.zeros_like(Y)
        status = np.zeros(n, dtype=np.int32)
        dtc = None if dt_per_cell is None else np.ascontiguousarray(dt_per_cell, dtype=np.float64)
        st, stats, dmin = self.integrate_raw(n, dt, cells.p, cells.rho0, T, Y, sub, RR, status,
                                             dt_per_cell=dtc)
        return dict(T=T, Y=Y, subDt=sub, RR=RR, status=status, deltaTMin=dmin, stats=stats, code=st)

    # The contiguous float64 copies are bound to locals for the whole call:
    # an address taken from a temporary copy would dangle once the copy is freed.
    def rhs(self, p, T, Y):
        p, T, Y = _host64(p), _host64(T), _host64(Y)
        n = T.shape[0]
        out = np.zeros((self.ns + 1, n))
        self._check(self.L.fcs_rhs(self.h, n, _addr(p), _addr(T), _addr(Y), _addr(out), 0))
        return out

    def jacobian(self, p, T, Y):
        p, T, Y = _host64(p), _host64(T), _host64(Y)
        n = T.shape[0]
        N = self.ns + 1
        J = np.zeros((n, N, N))
        f = np.zeros((N, n))
        self._check(self.L.fcs_jacobian(self.h, n, _addr(p), _addr(T), _addr(Y), _addr(J), _addr(f), 0))
        return J, f

    def tc(self, p, T, rho, Y):
        p, T, rho, Y = _host64(p), _host64(T), _host64(rho), _host64(Y)
        n = T.shape[0]
        out = np.zeros(n)
        self._check(self.L.fcs_tc(self.h, n, _addr(p), _addr(T), _addr(rho), _addr(Y), _addr(out), 0))
        return out

    def rates(self, p, T, rho, Y):
        p, T, rho, Y = _host64(p), _host64(T), _host64(rho), _host64(Y)
        n = T.shape[0]
        RR = np.zeros((self.ns, n))
        Q = np.zeros(n)
        self._check(self.L.fcs_rates(self.h, n, _addr(p), _addr(T), _addr(rho), _addr(Y), _addr(RR), _addr(Q), 0))
        return RR, Q


class Mlp:
    """The surrogate MLP ensemble (include/fcs_mlp.h)."""

    def __init__(self, n_in=None, n_out=None, width=256, depth=4, members=4, seed=0, device=0, path=None):
        self.L = load()
        self.h = C.c_void_p()
        if path is not None:
            st = self.L.fcs_mlp_load(C.byref(self.h), device, os.fsencode(path))
            if st:
                raise FcsError(st, f"cannot load {path}")
        else:
            sh = MlpShape(n_in, n_out, width, depth, members)
            st = self.L.fcs_mlp_create(C.byref(self.h), device, C.byref(sh), seed)
            if st:
                raise FcsError(st, "fcs_mlp_create failed")
        sh = MlpShape()
        self.L.fcs_mlp_get_shape(self.h, C.byref(sh))
        self.n_in, self.n_out, self.width, self.depth, self.members = (sh.n_in, sh.n_out, sh.width, sh.depth,
                                                                       sh.members)
        n = C.c_int64()
        self.L.fcs_mlp_param_count(self.h, C.byref(n))
        self.n_params = n.value

    def close(self):
        if self.h:
            self.L.fcs_mlp_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st):
        if st:
            raise FcsError(st, self.L.fcs_mlp_last_error(self.h).decode())

    def layer_shapes(self):
        """[(out, in)] per layer, in parameter order."""
        dims = [self.n_in] + [self.width] * self.depth + [self.n_out]
        return [(dims[i + 1], dims[i]) for i in range(len(dims) - 1)]

    def unflatten(self, flat):
        out, o = [], 0
        for (no, ni) in self.layer_shapes():
            W = flat[o:o + no * ni].reshape(no, ni)
            o += no * ni
            b = flat[o:o + no]
            o += no
            out.append((W, b))
        return out

    def get_params(self, member):
        p = np.zeros(self.n_params, dtype=np.float32)
        self._check(self.L.fcs_mlp_get_params(self.h, member, _addr(p)))
        return p

    def set_params(self, member, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.n_params
        self._check(self.L.fcs_mlp_set_params(self.h, member, _addr(p)))

    def set_normalization(self, in_mean, in_std, out_mean, out_std):
        a = [np.ascontiguousarray(v, dtype=np.float32) for v in (in_mean, in_std, out_mean, out_std)]
        self._check(self.L.fcs_mlp_set_normalization(self.h, *[_addr(v) for v in a]))

    def get_normalization(self):
        a = [np.zeros(self.n_in, np.float32), np.zeros(self.n_in, np.float32), np.zeros(self.n_out, np.float32),
             np.zeros(self.n_out, np.float32)]
        self._check(self.L.fcs_mlp_get_normalization(self.h, *[_addr(v) for v in a]))
        return a

    def forward(self, member, x, device=False):
        if device:
            import torch
            y = torch.empty((x.shape[0], self.n_out), dtype=torch.float32, device=x.device)
        else:
            x = np.ascontiguousarray(x, dtype=np.float32)
            y = np.zeros((x.shape[0], self.n_out), dtype=np.float32)
        self._check(self.L.fcs_mlp_forward(self.h, member, x.shape[0], _addr(x), _addr(y),
                                           PTR_DEVICE if device else 0))
        return y

    def gradients(self, member, x, target):
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(target, dtype=np.float32)
        g = np.zeros(self.n_params, dtype=np.float32)
        loss = C.c_float()
        self._check(self.L.fcs_mlp_gradients(self.h, member, x.shape[0], _addr(x), _addr(t), C.byref(loss),
                                             _addr(g)))
        return loss.value, g

    def train(self, x, target, epochs=20, batch=4096, lr=1e-3, lr_final=2e-5, seed=1):
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(target, dtype=np.float32)
        o = MlpTrainOptions()
        self.L.fcs_mlp_default_train_options(C.byref(o))
        o.epochs, o.batch, o.lr, o.lr_final, o.seed = epochs, batch, lr, lr_final, seed
        hist = np.zeros((self.members, epochs), dtype=np.float32)
        self._check(self.L.fcs_mlp_train(self.h, x.shape[0], _addr(x), _addr(t), C.byref(o), _addr(hist)))
        return hist

    def save(self, path):
        self._check(self.L.fcs_mlp_save(self.h, os.fsencode(path)))


def gate_options(**kw) -> GateOptions:
    o = GateOptions()
    load().fcs_gate_default_options(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def attach_surrogate(ctx: "Context", mlp: Optional[Mlp], composition=None, element_mass=None, **gate):
    """Attach the ensemble to a chemistry context (None detaches)."""
    if mlp is None:
        ctx._check(ctx.L.fcs_surrogate_attach(ctx.h, None, 0, None, None, None))
        return
    comp = np.ascontiguousarray(composition, dtype=np.float64)
    em = np.ascontiguousarray(element_mass, dtype=np.float64)
    o = gate_options(**gate)
    ctx._gate_keep = (mlp, comp, em, o)
    ctx._check(ctx.L.fcs_surrogate_attach(ctx.h, mlp.h, comp.shape[1], _addr(comp), _addr(em), C.byref(o)))


def integrate_gated_raw(ctx: "Context", n, dt, p, rho0, T, Y, sub, RR=None, status=None, device=False, check=True):
    stats, gst = StepStats(), GateStats()
    dmin = C.c_double(0)
    st = ctx.L.fcs_integrate_gated(ctx.h, n, dt, _addr(p), _addr(rho0), _addr(T), _addr(Y), _addr(sub), _addr(RR),
                                   _addr(status), C.byref(stats), C.byref(dmin), PTR_DEVICE if device else 0,
                                   C.byref(gst))
    if check and st not in (0, 5):
        ctx._check(st)
    return st, stats.as_dict(), gst.as_dict(), dmin.value
