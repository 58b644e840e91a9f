"""The C-ABI library builds for sm_103a, loads without a GPU, and exports every
function include/fv3g.h declares (no compute calls: there is no GPU here)."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "fv3g.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*int\s+(fv3g_\w+)\s*\(", src, flags=re.M)))


def test_library_exports_every_declared_function():
    from fv3atm_gb300 import _lib
    from fv3atm_gb300 import build as B
    path = B.build()
    lib = ctypes.CDLL(path)
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) == set(_lib.EXPORTS), set(names) ^ set(_lib.EXPORTS)


def test_version_and_error_reporting_without_gpu():
    from fv3atm_gb300 import _lib
    L = _lib.load()
    assert L.fv3g_version() == 100
    # argument validation happens before any CUDA call
    rc = L.fv3g_remap_columns_noalloc(5000, 10, ctypes.c_void_p(8), ctypes.c_void_p(8), None, 10,
                                      ctypes.c_void_p(8), ctypes.c_void_p(8), 1, 0, 9, ctypes.c_double(0.0), None)
    assert rc == -1 and "1024 columns" in _lib.last_error()
    rc = L.fv3g_state_create(None, None)
    assert rc == -1
