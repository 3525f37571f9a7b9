"""Kit parameters: the module globals of the reference's mlegs_base (src/modules/mlegs_base.f90:7-41),
as the POD struct `mlg_params` of include/mlegs_gb300.h."""
import ctypes
import math


class MlgParams(ctypes.Structure):
    _fields_ = [
        ("nr", ctypes.c_int), ("np", ctypes.c_int), ("nz", ctypes.c_int),
        ("nrchop", ctypes.c_int), ("npchop", ctypes.c_int), ("nzchop", ctypes.c_int),
        ("ell", ctypes.c_double), ("zlen", ctypes.c_double), ("visc", ctypes.c_double),
        ("hyperpow", ctypes.c_int), ("hypervisc", ctypes.c_double),
        ("is_svv", ctypes.c_int),
        ("svv_cutoff", ctypes.c_double), ("svv_target", ctypes.c_double),
        ("svv_strength", ctypes.c_double), ("svv_relax", ctypes.c_double),
    ]


DEFAULTS = dict(nr=256, np=128, nz=128, nrchop=256, npchop=65, nzchop=65, ell=4.0,
                zlen=2.0 * math.pi, visc=1.0e-3, hyperpow=0, hypervisc=0.0, is_svv=1,
                svv_cutoff=0.75, svv_target=2.0e-2, svv_strength=0.12, svv_relax=0.25)


def make_params(**kw):
    """Reference defaults (mlegs_base.f90:7-41) overridden by keyword arguments."""
    d = dict(DEFAULTS)
    for k, v in kw.items():
        if k not in d:
            raise KeyError(f"unknown kit parameter {k!r}")
        d[k] = v
    p = MlgParams()
    for k, v in d.items():
        setattr(p, k, int(v) if isinstance(DEFAULTS[k], int) and not isinstance(DEFAULTS[k], bool) else v)
    return p


def dims_of(p):
    """(nrdim, npdim, nzdim) of a field for these parameters (mlegs_spectfm_init.f90:117-136)."""
    return (p.nr + max(3, p.hyperpow), p.np // 2 + 1, p.nz)


class MlgRunParams(ctypes.Structure):
    """The time-stepping and output settings of an input file (mlg_run_params)."""
    _fields_ = [
        ("dt", ctypes.c_double), ("ti", ctypes.c_double), ("totaltime", ctypes.c_double),
        ("ni", ctypes.c_int), ("totaln", ctypes.c_int),
        ("isfldsav", ctypes.c_int), ("fldsavintvl", ctypes.c_int),
        ("islogsav", ctypes.c_int), ("logsavintvl", ctypes.c_int),
        ("flddir", ctypes.c_char * 260), ("logdir", ctypes.c_char * 260),
    ]


def read_input(fn, make_dirs=False):
    """read_input (mlegs_misc_io.f90:307-388): (kit parameters, run settings as a dict) from an input
    file in the reference's layout; raises MlgError with the reference's message when it is invalid."""
    import os
    from .kit import load, _chk
    p, r = MlgParams(), MlgRunParams()
    _chk(load().mlg_read_input(os.fsencode(fn), ctypes.byref(p), ctypes.byref(r), int(bool(make_dirs))))
    run = {f: getattr(r, f) for f, _ in MlgRunParams._fields_}
    run["flddir"] = r.flddir.decode()
    run["logdir"] = r.logdir.decode()
    return p, run
