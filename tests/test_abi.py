"""The C-ABI library builds, loads and exports every entry point that
include/soundersim_gb300.h declares (no compute: runs without a GPU)."""

import os
import re

from radar_sounder_simulator_gb300 import _lib, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for fn in os.listdir(inc):
        if fn.endswith(".h"):
            src = open(os.path.join(inc, fn)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(ss_[a-z0-9_]+)\s*\(", src))
    return names


def test_library_exports_header_symbols():
    build.build()
    L = _lib.lib()
    decl = declared_symbols()
    assert decl, "no entry points declared"
    for name in decl:
        assert hasattr(L, name), f"{name} declared but not exported"
    assert set(_lib.SIGNATURES) <= decl | {"ss_version", "ss_last_error"}
    assert b"sm_103a" in L.ss_version()
