"""CPU checks of the C-ABI library: it loads, exports every declared symbol,
and rejects bad arguments before touching a GPU."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = []
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", f)).read()
            names += re.findall(r"^\s*(?:int|void|double|const char \*)\s*\*?\s*(umt\w+)\s*\(", txt, re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    from umt_gb300 import build
    lib = C.CDLL(build.build())
    names = _declared()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n


def test_python_binding_lists_every_symbol():
    from umt_gb300 import capi
    assert set(_declared()) <= set(capi.EXPORTED)


def test_calls_before_init_fail_cleanly():
    from umt_gb300 import build, capi
    build.build()
    lib = capi.load()
    assert lib.umt103_sweep_resident(0, 0) == -2
    assert b"init" in lib.umt103_error_string()
