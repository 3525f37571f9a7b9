"""Python front end of the GB300 library (ctypes over the C ABI in include/mlegs_gb300.h).

This mirrors the reference's Fortran operator API (module mlegs_scalar, src/modules/mlegs_scalar.f90):
`Kit` plays the role of the global transform kit `tfm` (one per process), `Scalar` of type(scalar),
and the methods keep the reference's names and argument meanings (trans, chop, dealias, svv_filter,
calcat0/1, zeroat1, delsqp, idelsqp, xxdx, del2h, del2, idel2, helm, ihelm, helmp, ihelmp, fefe,
abab, febe, abcn, vecprod, vec2tp, tp2vec, tp2curlvec).  Errors the reference reports with `stop`
raise MlgError with the same message.
"""
import ctypes
import os

import numpy as np

from .params import MlgParams, make_params

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmlegs_gb300.so")

_lib = None
_P = ctypes.c_void_p
_D = ctypes.c_double
_I = ctypes.c_int


def load(path=None):
    """Loads the CUDA library; fails loudly if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: build it with `python -m mlegs_gb300.build` "
                          "(the GPU path has no fallback)")
    L = ctypes.CDLL(path)
    L.mlg_last_error.restype = ctypes.c_char_p
    L.mlg_mem_bytes.restype = ctypes.c_longlong
    L.mlg_mem_high_water.restype = ctypes.c_longlong
    L.mlg_launch_count.restype = ctypes.c_longlong
    L.mlg_scalar_device_ptr.restype = _P
    L.mlg_scalar_device_ptr.argtypes = [_P]
    sig = {
        "mlg_init": [_P], "mlg_kit_dims": [_P], "mlg_kit_get": [ctypes.c_char_p, _P, ctypes.c_longlong],
        "mlg_set_precision": [_I], "mlg_set_stream": [_P],
        "mlg_scalar_alloc": [_P], "mlg_scalar_free": [_P],
        "mlg_scalar_upload": [_P, _P, _D, ctypes.c_char_p],
        "mlg_scalar_upload_device": [_P, _P, _D, ctypes.c_char_p],
        "mlg_scalar_download": [_P, _P, _P, _P], "mlg_scalar_download_device": [_P, _P, _P, _P],
        "mlg_scalar_copy": [_P, _P], "mlg_scalar_chop_offset": [_P, _I, _I, _I],
        "mlg_scalar_get_meta": [_P, _P, _P, _P], "mlg_scalar_set_ln": [_P, _D],
        "mlg_scalar_set_space": [_P, ctypes.c_char_p],
        "mlg_trans": [_P, ctypes.c_char_p], "mlg_svv_filter": [_P, _P],
        "mlg_calcat0": [_P, _P], "mlg_calcat1": [_P, _P],
        "mlg_idel2_preln": [_P, _D], "mlg_helm": [_P, _D], "mlg_ihelm": [_P, _D],
        "mlg_helmp": [_P, _I, _D, _D], "mlg_ihelmp": [_P, _I, _D, _D],
        "mlg_fefe": [_P, _P, _D], "mlg_febe": [_P, _P, _D],
        "mlg_abab": [_P, _P, _P, _P, _D, _I], "mlg_abcn": [_P, _P, _P, _P, _D],
        "mlg_vecprod": [_P] * 6, "mlg_vec2tp": [_P] * 5, "mlg_tp2vec": [_P] * 5, "mlg_tp2curlvec": [_P] * 5,
        "mlg_advection_rhs": [_P] * 5,
        "mlg_vortex_step": [_P] * 9 + [_D, _P], "mlg_vortex_run": [_P] * 9 + [_D, _I, _P],
        "mlg_scalar_axpby": [_P, _D, _P, _D, _P],
        "mlg_kernel_timing": [_I], "mlg_kernel_timing_read": [_I, _P, _P, _P],
        "mlg_adjoint_run": [_P, _P, _P, _D, _I, _I, _P, _P, _P], "mlg_adj_vortex_step": [_P, _P, _D, _P],
        "mlg_adj_trans": [_P, ctypes.c_char_p], "mlg_adj_band": [_P, _I], "mlg_adj_ihelm": [_P, _D],
        "mlg_adj_idel2_proln": [_P], "mlg_adj_zeroat1": [_P],
        "mlg_adj_tp2vec": [_P] * 5, "mlg_adj_tp2curlvec": [_P] * 5, "mlg_adj_vec2tp": [_P] * 5,
        "mlg_adj_advection": [_P] * 7,
        "mlg_msave": [_P, ctypes.c_char_p, _I, _I], "mlg_mload": [_P, ctypes.c_char_p, _I, _I],
        "mlg_fftreat": [_P], "mlg_vort_mag": [_P, _P, _P], "mlg_ke_spectrum": [_P, _P, _P],
        "mlg_read_input": [ctypes.c_char_p, _P, _P, _I],
        "mlg_selftest_bounded_wait": [ctypes.c_longlong, _I],
    }
    for name in ["mlg_chop", "mlg_dealias", "mlg_zeroat1", "mlg_delsqp", "mlg_idelsqp", "mlg_xxdx", "mlg_del2h",
                 "mlg_del2", "mlg_idel2_proln"]:
        sig[name] = [_P]
    for name, args in sig.items():
        getattr(L, name).argtypes = args
        getattr(L, name).restype = _I
    _lib = L
    return L


class MlgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code


def _chk(rc):
    if rc != 0:
        raise MlgError(rc, load().mlg_last_error().decode())
    return rc


PLAIN_FP64 = 0
MIXED = 1


class Scalar:
    """type(scalar): a device-resident field with ln, chop offsets and space tag."""

    def __init__(self, kit):
        self.kit = kit
        h = ctypes.c_void_p()
        _chk(load().mlg_scalar_alloc(ctypes.byref(h)))
        self.h = h

    def free(self):
        if self.h:
            load().mlg_scalar_free(self.h)
            self.h = None

    def set(self, e, ln=0.0, space="PPP"):
        a = np.asfortranarray(e, dtype=np.complex128)
        assert a.shape == self.kit.dims, (a.shape, self.kit.dims)
        _chk(load().mlg_scalar_upload(self.h, a.ctypes.data, float(ln), space.encode()))
        return self

    def get(self):
        a = np.zeros(self.kit.dims, dtype=np.complex128, order="F")
        ln = ctypes.c_double()
        sp = ctypes.create_string_buffer(4)
        _chk(load().mlg_scalar_download(self.h, a.ctypes.data, ctypes.byref(ln), sp))
        offs = (ctypes.c_int * 3)()
        _chk(load().mlg_scalar_get_meta(self.h, None, None, offs))
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
        _chk(load().mlg_scalar_copy(self.h, other.h))
        return self

    def chop_offset(self, a, b=0, c=0):
        _chk(load().mlg_scalar_chop_offset(self.h, a, b, c))

    def device_ptr(self):
        return load().mlg_scalar_device_ptr(self.h)


class Kit:
    """tfm%init(): the transform kit on the GPU (one per process, as in the reference)."""

    def __init__(self, params=None, precision=PLAIN_FP64, stream=None, **kw):
        L = load()
        self.params = params if params is not None else make_params(**kw)
        L.mlg_finalize()
        if stream is not None:
            _chk(L.mlg_set_stream(ctypes.c_void_p(stream)))
        _chk(L.mlg_init(ctypes.byref(self.params)))
        d = (ctypes.c_int * 9)()
        _chk(L.mlg_kit_dims(d))
        self.dims = (d[0], d[1], d[2])
        self.chopzl, self.chopzu, self.nrh, self.ne, self.npchop, self.nr = d[3], d[4], d[5], d[6], d[7], d[8]
        self.set_precision(precision)

    def close(self):
        load().mlg_finalize()

    def set_precision(self, mode):
        _chk(load().mlg_set_precision(int(mode)))
        self.precision = int(mode)

    def sync(self):
        _chk(load().mlg_sync())

    def mem_bytes(self):
        return load().mlg_mem_bytes()

    def mem_high_water(self):
        return load().mlg_mem_high_water()

    def launch_count(self):
        return load().mlg_launch_count()

    def kit_get(self, name):
        sizes = {"x": self.nr, "w": self.nr, "r": self.nr, "ln": self.nr, "ak": self.dims[2],
                 "lognorm": self.ne * self.npchop, "pf": self.nrh * self.ne * self.npchop,
                 "at0": self.params.nrchop, "at1": self.params.nrchop}
        n = sizes[name]
        out = np.zeros(n)
        _chk(load().mlg_kit_get(name.encode(), out.ctypes.data, n))
        if name == "lognorm":
            return out.reshape((self.ne, self.npchop), order="F")
        if name == "pf":
            return out.reshape((self.nrh, self.ne, self.npchop), order="F")
        return out

    def scalar(self, e=None, ln=0.0, space="PPP"):
        s = Scalar(self)
        if e is not None:
            s.set(e, ln, space)
        return s

    # ---- operator API (names of mlegs_scalar.f90) ----
    def trans(self, s, space): _chk(load().mlg_trans(s.h, space.encode()))
    def chop(self, s): _chk(load().mlg_chop(s.h))
    def dealias(self, s): _chk(load().mlg_dealias(s.h))

    def svv_filter(self, s, gain):
        g = ctypes.c_double(gain)
        _chk(load().mlg_svv_filter(s.h, ctypes.byref(g)))
        return g.value

    def calcat0(self, s):
        out = np.zeros(self.dims[2], dtype=np.complex128)
        _chk(load().mlg_calcat0(s.h, out.ctypes.data))
        return out

    def calcat1(self, s):
        out = np.zeros(self.dims[2], dtype=np.complex128)
        _chk(load().mlg_calcat1(s.h, out.ctypes.data))
        return out

    def zeroat1(self, s): _chk(load().mlg_zeroat1(s.h))
    def delsqp(self, s): _chk(load().mlg_delsqp(s.h))
    def idelsqp(self, s): _chk(load().mlg_idelsqp(s.h))
    def xxdx(self, s): _chk(load().mlg_xxdx(s.h))
    def del2h(self, s): _chk(load().mlg_del2h(s.h))
    def del2(self, s): _chk(load().mlg_del2(s.h))

    def idel2(self, s, preln=None):
        if preln is None:
            _chk(load().mlg_idel2_proln(s.h))
        else:
            _chk(load().mlg_idel2_preln(s.h, float(preln)))

    def helm(self, s, alpha): _chk(load().mlg_helm(s.h, float(alpha)))
    def ihelm(self, s, alpha): _chk(load().mlg_ihelm(s.h, float(alpha)))
    def helmp(self, s, power, alpha, beta): _chk(load().mlg_helmp(s.h, int(power), float(alpha), float(beta)))
    def ihelmp(self, s, power, alpha, beta): _chk(load().mlg_ihelmp(s.h, int(power), float(alpha), float(beta)))
    def fefe(self, s, nl, dt): _chk(load().mlg_fefe(s.h, nl.h, float(dt)))

    def abab(self, s, sp, nl, nlp, dt, is_2nd_svis_p=False):
        _chk(load().mlg_abab(s.h, sp.h, nl.h, nlp.h, float(dt), int(bool(is_2nd_svis_p))))

    def febe(self, s, nl, dt): _chk(load().mlg_febe(s.h, nl.h, float(dt)))
    def abcn(self, s, sp, nl, nlp, dt): _chk(load().mlg_abcn(s.h, sp.h, nl.h, nlp.h, float(dt)))
    def vecprod(self, vr, vp, vz, ur, up, uz): _chk(load().mlg_vecprod(vr.h, vp.h, vz.h, ur.h, up.h, uz.h))
    def vec2tp(self, vr, vp, vz, psi, chi): _chk(load().mlg_vec2tp(vr.h, vp.h, vz.h, psi.h, chi.h))
    def tp2vec(self, psi, chi, vr, vp, vz): _chk(load().mlg_tp2vec(psi.h, chi.h, vr.h, vp.h, vz.h))
    def tp2curlvec(self, psi, chi, wr, wp, wz): _chk(load().mlg_tp2curlvec(psi.h, chi.h, wr.h, wp.h, wz.h))

    # ---- field I/O (mlegs_scalar_io.f90) and diagnostics ----
    def msave(self, s, fn, is_binary=False, is_global=True):
        """msave: the reference's optional arguments default to formatted and global."""
        _chk(load().mlg_msave(s.h, os.fsencode(fn), int(bool(is_binary)), int(bool(is_global))))

    def mload(self, s, fn, is_binary=False, is_global=True):
        _chk(load().mlg_mload(s.h, os.fsencode(fn), int(bool(is_binary)), int(bool(is_global))))

    def fftreat(self, s): _chk(load().mlg_fftreat(s.h))

    def vort_mag(self, psi, chi, out):
        """The field of save_vort_mag: out (PPP) <- |curl v| per physical sample."""
        _chk(load().mlg_vort_mag(psi.h, chi.h, out.h))

    def ke_spectrum(self, psi, chi):
        """Kinetic-energy spectrum E[m, k] (npdim x nzdim) of the velocity of (psi, chi), FP64."""
        E = np.zeros((self.dims[2], self.dims[1]), dtype=np.float64)   # k-major rows: E[m + npdim*k]
        _chk(load().mlg_ke_spectrum(psi.h, chi.h, E.ctypes.data))
        return E.T.copy()

    def advection_rhs(self, psi, chi, nlpsi, nlchi, uz):
        _chk(load().mlg_advection_rhs(psi.h, chi.h, nlpsi.h, nlchi.h, uz.h))

    def vortex_step(self, psi, chi, nlpsi, nlchi, psip, chip, nlpsip, nlchip, uz, dt, gains):
        g = (ctypes.c_double * 2)(*gains)
        _chk(load().mlg_vortex_step(psi.h, chi.h, nlpsi.h, nlchi.h, psip.h, chip.h, nlpsip.h, nlchip.h, uz.h,
                                    float(dt), g))
        gains[0], gains[1] = g[0], g[1]

    def vortex_run(self, psi, chi, nlpsi, nlchi, psip, chip, nlpsip, nlchip, uz, dt, nsteps, gains):
        g = (ctypes.c_double * 2)(*gains)
        _chk(load().mlg_vortex_run(psi.h, chi.h, nlpsi.h, nlchi.h, psip.h, chip.h, nlpsip.h, nlchip.h, uz.h,
                                   float(dt), int(nsteps), g))
        gains[0], gains[1] = g[0], g[1]

    def axpby(self, d, a, x, b=0.0, y=None):
        """d%e = a*x%e + b*y%e (the apps' direct array arithmetic on s%e)."""
        _chk(load().mlg_scalar_axpby(d.h, float(a), x.h, float(b), y.h if y is not None else None))

    # ---- adjoint (no counterpart in the reference) ----
    def adjoint_run(self, psi0, chi0, uz, dt, nsteps, k_ckpt, grad_psi=None, grad_chi=None):
        """J at step nsteps and, with grad scalars given, dJ/d(psi0, chi0) written into them."""
        J = ctypes.c_double()
        _chk(load().mlg_adjoint_run(psi0.h, chi0.h, uz.h, float(dt), int(nsteps), int(k_ckpt),
                                    grad_psi.h if grad_psi is not None else None,
                                    grad_chi.h if grad_chi is not None else None, ctypes.byref(J)))
        return J.value

    def adj_vortex_step(self, state, uz, dt, adj):
        st = (_P * 6)(*[q.h.value for q in state])
        ad = (_P * 6)(*[q.h.value for q in adj])
        _chk(load().mlg_adj_vortex_step(st, uz.h, float(dt), ad))

    def adj_trans(self, s, forward_from): _chk(load().mlg_adj_trans(s.h, forward_from.encode()))
    def adj_band(self, s, op): _chk(load().mlg_adj_band(s.h, int(op)))
    def adj_ihelm(self, s, alpha): _chk(load().mlg_adj_ihelm(s.h, float(alpha)))
    def adj_idel2_proln(self, s): _chk(load().mlg_adj_idel2_proln(s.h))
    def adj_zeroat1(self, s): _chk(load().mlg_adj_zeroat1(s.h))
    def adj_tp2vec(self, vr, vp, vz, psi, chi): _chk(load().mlg_adj_tp2vec(vr.h, vp.h, vz.h, psi.h, chi.h))
    def adj_tp2curlvec(self, wr, wp, wz, psi, chi): _chk(load().mlg_adj_tp2curlvec(wr.h, wp.h, wz.h, psi.h, chi.h))
    def adj_vec2tp(self, psi, chi, vr, vp, vz): _chk(load().mlg_adj_vec2tp(psi.h, chi.h, vr.h, vp.h, vz.h))

    def adj_advection(self, psi, chi, uz, nlpsi_bar, nlchi_bar, psi_bar, chi_bar):
        _chk(load().mlg_adj_advection(psi.h, chi.h, uz.h, nlpsi_bar.h, nlchi_bar.h, psi_bar.h, chi_bar.h))

    # ---- kernel timing ----
    def kernel_timing(self, enable):
        _chk(load().mlg_kernel_timing(int(bool(enable))))

    def kernel_timing_read(self, kind):
        ms, n, w = ctypes.c_double(), ctypes.c_longlong(), ctypes.c_double()
        _chk(load().mlg_kernel_timing_read(int(kind), ctypes.byref(ms), ctypes.byref(n), ctypes.byref(w)))
        return ms.value, n.value, w.value
