"""The C-ABI library loads without a GPU and exports every function include/*.h declares."""
import ctypes
import os
import re

import meso_gpu as mg
from conftest import ROOT


def _declared():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            txt = open(os.path.join(inc, f)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"\b(meso_[a-z0-9_]+)\s*\(", txt))
    return names


def test_exports_every_declared_symbol():
    lib = ctypes.CDLL(mg.LIB_PATH)
    declared = _declared()
    assert len(declared) >= 20
    missing = [n for n in declared if not hasattr(lib, n)]
    assert not missing, missing
    # the binding declares signatures for all of them
    assert declared <= set(mg.EXPORTED), declared - set(mg.EXPORTED)


def test_version_and_error_strings():
    assert b"sm_103a" in mg.lib().meso_version()
    rc = mg.lib().meso_case_load(b"/nonexistent/case.txt", ctypes.byref(ctypes.c_void_p()))
    assert rc == mg.ERR_IO
    assert b"file open error" in mg.lib().meso_last_error()


def test_null_arguments_are_rejected():
    L = mg.lib()
    assert L.meso_step(None, 1, None) == mg.ERR_INVALID
    assert L.meso_get_macros(None, None, None, None, None) == mg.ERR_INVALID
    assert L.meso_ctx_create(None, None, None, 0, None, None, None) == mg.ERR_INVALID
