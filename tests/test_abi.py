"""The C ABI library builds for sm_103a, loads, and exports every function
include/allium_sweep.h declares.  No compute calls (CPU only)."""
import ctypes
import os
import re

from allium_gb300 import _lib, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    names = []
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if h.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", h)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names += re.findall(r"\b(allium_[a-z0-9_]+)\s*\(", txt)
    return sorted(set(names))


def test_library_exports_header():
    lib = _lib.lib()
    names = declared()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) <= set(_lib.EXPORTS), set(names) - set(_lib.EXPORTS)


def test_status_strings_without_gpu():
    lib = _lib.lib()
    assert lib.allium_status_string(0) == b"ok"
    assert lib.allium_status_string(2) == b"upwind graph is not a DAG"


def test_build_is_current():
    build.build()
    assert build.up_to_date()


def test_create_rejects_null_arguments():
    lib = _lib.lib()
    out = ctypes.c_void_p()
    assert lib.allium_sweep_create(None, None, None, 1, None, None, ctypes.byref(out)) == 1
    assert not out.value
