"""ctypes front end of the CPU oracle (oracle/liboracle.so) — test infrastructure only.

Exposes the same operator names as the GPU kit (mlegs_gb300.Kit) so that a parity test runs one
call sequence on both and compares the fields.  Only tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg use this module.
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
from mlegs_gb300.params import MlgParams, make_params, dims_of  # noqa: E402
from oracle.build import build  # noqa: E402

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build()
        L = ctypes.CDLL(path)
        L.orc_last_error.restype = ctypes.c_char_p
        L.orc_new.restype = ctypes.c_int
        for name in ["orc_svv_filter"]:
            getattr(L, name).argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
        for name in ["orc_idel2_preln", "orc_helm", "orc_ihelm"]:
            getattr(L, name).argtypes = [ctypes.c_int, ctypes.c_double]
        for name in ["orc_helmp", "orc_ihelmp"]:
            getattr(L, name).argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double]
        for name in ["orc_fefe", "orc_febe"]:
            getattr(L, name).argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double]
        L.orc_abab.argtypes = [ctypes.c_int] * 4 + [ctypes.c_double, ctypes.c_int]
        L.orc_abcn.argtypes = [ctypes.c_int] * 4 + [ctypes.c_double]
        L.orc_vortex_step.argtypes = [ctypes.c_int] * 9 + [ctypes.c_double, ctypes.POINTER(ctypes.c_double)]
        L.orc_set.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_double, ctypes.c_char_p, ctypes.c_void_p]
        L.orc_get.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_char_p,
                              ctypes.c_void_p]
        L.orc_axpby.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_double, ctypes.c_int]
        L.orc_kit_get.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_longlong]
        _lib = L
    return _lib


class OracleError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code


def _chk(rc):
    if rc != 0:
        raise OracleError(rc, lib().orc_last_error().decode())
    return rc


class OScalar:
    def __init__(self, kit):
        self.kit = kit
        self.h = lib().orc_new()
        if self.h < 0:
            _chk(2)

    def free(self):
        if self.h >= 0:
            lib().orc_free(self.h)
            self.h = -1

    def set(self, e, ln=0.0, space="PPP", offsets=(0, 0, 0)):
        a = np.asfortranarray(e, dtype=np.complex128)
        assert a.shape == self.kit.dims, (a.shape, self.kit.dims)
        offs = (ctypes.c_int * 3)(*offsets)
        _chk(lib().orc_set(self.h, a.ctypes.data, float(ln), space.encode(), offs))
        return self

    def get(self):
        a = np.zeros(self.kit.dims, dtype=np.complex128, order="F")
        ln = ctypes.c_double()
        sp = ctypes.create_string_buffer(4)
        offs = (ctypes.c_int * 3)()
        _chk(lib().orc_get(self.h, a.ctypes.data, ctypes.byref(ln), sp, offs))
        return a, ln.value, sp.value.decode(), tuple(offs)

    @property
    def e(self):
        return self.get()[0]

    @property
    def ln(self):
        return self.get()[1]

    @property
    def space(self):
        return self.get()[2]

    def copy_from(self, other):
        _chk(lib().orc_copy(self.h, other.h))
        return self

    def chop_offset(self, a, b=0, c=0):
        _chk(lib().orc_chop_offset(self.h, a, b, c))


class Oracle:
    """The CPU restatement behind the same operator names as mlegs_gb300.Kit."""

    def __init__(self, params=None, threads=None, **kw):
        self.params = params if params is not None else make_params(**kw)
        L = lib()
        L.orc_finalize()
        if threads:
            L.orc_set_threads(int(threads))
        _chk(L.orc_init(ctypes.byref(self.params)))
        d = (ctypes.c_int * 9)()
        _chk(L.orc_kit_dims(d))
        self.dims = (d[0], d[1], d[2])
        self.chopzl, self.chopzu, self.nrh, self.ne, self.npchop, self.nr = d[3], d[4], d[5], d[6], d[7], d[8]

    @staticmethod
    def threads():
        return lib().orc_get_threads()

    def close(self):
        lib().orc_finalize()

    def kit_get(self, name):
        sizes = {"x": self.nr, "w": self.nr, "r": self.nr, "ln": self.nr, "ak": self.dims[2],
                 "lognorm": self.ne * self.npchop, "pf": self.nrh * self.ne * self.npchop,
                 "at0": self.params.nrchop, "at1": self.params.nrchop}
        n = sizes[name]
        out = np.zeros(n)
        _chk(lib().orc_kit_get(name.encode(), out.ctypes.data, n))
        if name == "lognorm":
            return out.reshape((self.ne, self.npchop), order="F")
        if name == "pf":
            return out.reshape((self.nrh, self.ne, self.npchop), order="F")
        return out

    def scalar(self, e=None, ln=0.0, space="PPP"):
        s = OScalar(self)
        if e is not None:
            s.set(e, ln, space)
        return s

    # ---- operator API (names of mlegs_scalar.f90) ----
    def trans(self, s, space): _chk(lib().orc_trans(s.h, space.encode()))
    def chop(self, s): _chk(lib().orc_chop(s.h))
    def dealias(self, s): _chk(lib().orc_dealias(s.h))

    def svv_filter(self, s, gain):
        g = ctypes.c_double(gain)
        _chk(lib().orc_svv_filter(s.h, ctypes.byref(g)))
        return g.value

    def calcat0(self, s):
        out = np.zeros(self.dims[2], dtype=np.complex128)
        _chk(lib().orc_calcat0(s.h, ctypes.c_void_p(out.ctypes.data)))
        return out

    def calcat1(self, s):
        out = np.zeros(self.dims[2], dtype=np.complex128)
        _chk(lib().orc_calcat1(s.h, ctypes.c_void_p(out.ctypes.data)))
        return out

    def zeroat1(self, s): _chk(lib().orc_zeroat1(s.h))
    def delsqp(self, s): _chk(lib().orc_delsqp(s.h))
    def idelsqp(self, s): _chk(lib().orc_idelsqp(s.h))
    def xxdx(self, s): _chk(lib().orc_xxdx(s.h))
    def del2h(self, s): _chk(lib().orc_del2h(s.h))
    def del2(self, s): _chk(lib().orc_del2(s.h))

    def idel2(self, s, preln=None):
        if preln is None:
            _chk(lib().orc_idel2_proln(s.h))
        else:
            _chk(lib().orc_idel2_preln(s.h, float(preln)))

    def helm(self, s, alpha): _chk(lib().orc_helm(s.h, float(alpha)))
    def ihelm(self, s, alpha): _chk(lib().orc_ihelm(s.h, float(alpha)))
    def helmp(self, s, power, alpha, beta): _chk(lib().orc_helmp(s.h, int(power), float(alpha), float(beta)))
    def ihelmp(self, s, power, alpha, beta): _chk(lib().orc_ihelmp(s.h, int(power), float(alpha), float(beta)))
    def fftreat(self, s): _chk(lib().orc_fftreat(s.h))
    def fefe(self, s, nl, dt): _chk(lib().orc_fefe(s.h, nl.h, float(dt)))
    def abab(self, s, sp, nl, nlp, dt, is_2nd_svis_p=False):
        _chk(lib().orc_abab(s.h, sp.h, nl.h, nlp.h, float(dt), int(bool(is_2nd_svis_p))))
    def febe(self, s, nl, dt): _chk(lib().orc_febe(s.h, nl.h, float(dt)))
    def abcn(self, s, sp, nl, nlp, dt): _chk(lib().orc_abcn(s.h, sp.h, nl.h, nlp.h, float(dt)))
    def vecprod(self, vr, vp, vz, ur, up, uz): _chk(lib().orc_vecprod(vr.h, vp.h, vz.h, ur.h, up.h, uz.h))
    def vec2tp(self, vr, vp, vz, psi, chi): _chk(lib().orc_vec2tp(vr.h, vp.h, vz.h, psi.h, chi.h))
    def tp2vec(self, psi, chi, vr, vp, vz): _chk(lib().orc_tp2vec(psi.h, chi.h, vr.h, vp.h, vz.h))
    def tp2curlvec(self, psi, chi, wr, wp, wz): _chk(lib().orc_tp2curlvec(psi.h, chi.h, wr.h, wp.h, wz.h))
    def advection_rhs(self, psi, chi, nlpsi, nlchi, uz):
        _chk(lib().orc_advection_rhs(psi.h, chi.h, nlpsi.h, nlchi.h, uz.h))

    def axpby(self, d, a, x, b=0.0, y=None):
        _chk(lib().orc_axpby(d.h, float(a), x.h, float(b), y.h if y is not None else -1))

    def vortex_step(self, psi, chi, nlpsi, nlchi, psip, chip, nlpsip, nlchip, uz, dt, gains):
        g = (ctypes.c_double * 2)(*gains)
        _chk(lib().orc_vortex_step(psi.h, chi.h, nlpsi.h, nlchi.h, psip.h, chip.h, nlpsip.h, nlchip.h,
                                   uz.h, float(dt), g))
        gains[0], gains[1] = g[0], g[1]
