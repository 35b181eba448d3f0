"""The C-ABI library loads and exports every function include/topomax_gb300.h declares (no GPU calls)."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            src = open(os.path.join(ROOT, "include", f)).read()
            names |= set(re.findall(r"\b(topo_[a-z0-9_]+)\s*\(", src))
    return names


def test_library_exports_declared_symbols():
    from topomax_gb300 import build, _capi
    build.build()
    lib = _capi.load_library()
    declared = _declared()
    assert len(declared) >= 15
    missing = [n for n in declared if not hasattr(lib, n)]
    assert not missing, missing
    assert set(_capi.EXPORTED) <= declared


def test_missing_library_fails_loudly(tmp_path):
    from topomax_gb300 import _capi
    with pytest.raises(ImportError):
        _capi.load_library(str(tmp_path / "nope.so"))
