"""The C-ABI library builds, loads and exports every symbol the headers declare
(no compute calls: no GPU needed)."""
import ctypes
import glob
import os
import re

from conftest import ROOT


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(?:fcs_status|int|const char\*|void)\s+(fcs_\w+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_library_exports_declared_symbols(lib_path):
    lib = ctypes.CDLL(lib_path)
    names = declared_symbols()
    assert len(names) >= 17
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_lists_exports(lib_path):
    from fcs import _lib
    assert set(_lib.EXPORTS) == declared_symbols()


def test_version_and_options_without_gpu(lib_path):
    from fcs import _lib
    L = _lib.load(lib_path)
    assert b"sm_103a" in L.fcs_version()
    o = _lib.Options()
    assert L.fcs_default_options(ctypes.byref(o)) == 0
    assert o.max_steps == 10000 and o.abs_tol == 1e-8 and o.rel_tol == 1e-4


def test_no_cpu_fallback_when_library_missing(tmp_path):
    from fcs import _lib
    import pytest
    saved = _lib._LIB
    _lib._LIB = None
    try:
        with pytest.raises(RuntimeError, match="no CPU fallback"):
            _lib.load(str(tmp_path / "missing.so"))
    finally:
        _lib._LIB = saved


def test_binding_refuses_strided_arrays():
    """A strided view handed to the C ABI would be read with the wrong layout:
    the binding refuses it (the evaluation helpers copy their inputs first)."""
    import numpy as np
    import pytest
    from fcs import _lib
    a = np.zeros((4, 6))
    assert _lib._addr(a) == a.ctypes.data
    with pytest.raises(ValueError):
        _lib._addr(a[:, ::2])
    assert _lib._host64(a[:, ::2]).flags.c_contiguous
