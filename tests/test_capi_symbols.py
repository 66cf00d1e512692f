"""The C-ABI library builds for sm_103a, loads without a GPU, and exports every
entry point include/genie_gb300.h declares (no compute calls here)."""
import ctypes
import os
import re

from conftest import ROOT


def _declared():
    with open(os.path.join(ROOT, "include", "genie_gb300.h")) as f:
        src = f.read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(genie_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    from genie_gb300 import build, _lib
    build.build()
    lib = ctypes.CDLL(_lib.LIB_PATH)
    names = _declared()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # the Python binding declares a prototype for each of them
    assert set(names) <= set(_lib.PROTOTYPES)


def test_library_loads_and_reports_errors_without_gpu():
    import genie_gb300 as g
    assert g.lib().genie_version() >= 10000
    # invalid arguments are rejected on the host before any device work
    rc = g.lib().genie_index_create(None, 0, 0, None)
    assert rc == 1
    assert b"NULL" in g.lib().genie_last_error() or b"data" in g.lib().genie_last_error()
