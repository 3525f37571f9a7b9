"""CPU checks of the drop-in boundary: the C-ABI library builds, loads and exports every entry point
that include/mlegs_gb300.h declares (no compute calls: this container has no GPU)."""
import ctypes
import os
import re

from conftest import ROOT

HDR = os.path.join(ROOT, "include", "mlegs_gb300.h")


def declared():
    txt = open(HDR).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(mlg_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    from mlegs_gb300 import build
    path = build.build()
    lib = ctypes.CDLL(path)
    missing = [s for s in declared() if not hasattr(lib, s)]
    assert not missing, missing
    assert len(declared()) > 50


def test_kit_requires_init():
    from mlegs_gb300.kit import load
    L = load()
    d = (ctypes.c_int * 9)()
    assert L.mlg_kit_dims(d) == 2
    assert b"not initialized" in L.mlg_last_error()


def test_params_default_matches_reference():
    from mlegs_gb300.kit import load
    from mlegs_gb300.params import MlgParams, make_params
    L = load()
    p = MlgParams()
    L.mlg_params_default(ctypes.byref(p))
    q = make_params()
    for f, _ in MlgParams._fields_:
        assert getattr(p, f) == getattr(q, f), f
