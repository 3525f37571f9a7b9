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


def test_fortran_interface_binds_every_export():
    """include/mlegs_gb300_iface.f90 (the ISO_C_BINDING module a Fortran host adds) declares a
    bind(c) interface for every entry point of the header, and its wrapper module makes public
    every procedure it defines (no Fortran compiler here: the check is textual)."""
    f90 = open(os.path.join(ROOT, "include", "mlegs_gb300_iface.f90")).read()
    code = "\n".join(l.split("!")[0] for l in f90.splitlines())
    bound = set(re.findall(r"bind\(\s*c\s*,\s*name\s*=\s*'(mlg_[a-z0-9_]+)'\s*\)", code, flags=re.I))
    missing = sorted(set(declared()) - bound)
    assert not missing, f"header exports without a Fortran binding: {missing}"
    extra = sorted(bound - set(declared()))
    assert not extra, f"Fortran bindings of names the header does not declare: {extra}"
    wrap = code[code.index("module mlegs_scalar_gpu"):]
    defined = set(re.findall(r"^\s*subroutine\s+([a-z0-9_]+)", wrap, flags=re.I | re.M)) - {"check"}
    public = set()
    for line in re.findall(r"^\s*public\s*::\s*(.*)$", wrap, flags=re.I | re.M):
        public |= {n.strip() for n in line.split(",")}
    generic = {"idel2_preln", "idel2_proln"}   # reached through the generic idel2
    hidden = sorted(defined - public - generic)
    assert not hidden, f"wrapper procedures that are not public: {hidden}"
    for name in ("adjoint_run", "axpby", "vortex_step", "vortex_run", "read_input", "set_stream"):
        assert name in public, name
