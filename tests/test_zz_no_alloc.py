"""mlg_ihelm_noalloc: the Helmholtz solve for callers that cannot let the library allocate device
memory (hosts whose own allocator or fixed arena owns the GPU, or that forbid allocation inside the
step loop).  Through the C ABI it must give the same field and ln as mlg_ihelm, on two calls in a
row, for a small grid and for the 192 x 128 x 128 grid (whose 8320 radial systems do not fit the
fixed workspace at once and are solved in batches), and the same field as the oracle's ihelm.  This
file runs last so that a failure here leaves every other test already run."""
import ctypes

import numpy as np
import pytest

from mlegs_gb300 import fields
from helpers import params, rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-12


@pytest.mark.parametrize("cfg", ["c1", "big"])
def test_ihelm_noalloc_matches_ihelm(cfg):
    from mlegs_gb300.kit import Kit, load
    from mlegs_gb300.params import make_params
    if cfg == "big":
        p = make_params(nr=192, np=128, nz=128, nrchop=192, npchop=65, nzchop=65, ell=4.0, visc=1.0e-4)
    else:
        p = params(cfg)
    k = Kit(p)
    L = load()
    L.mlg_ihelm_noalloc.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_double]
    L.mlg_ihelm_noalloc.restype = ctypes.c_int
    e0 = fields.spectral_noise(p, k.dims, 5, amp=1.0, decay=0.05)
    ref = k.scalar(e0, 0.3, "FFF")
    out = k.scalar(e0, 0.3, "FFF")
    ln = ctypes.c_double(0.3)
    alpha = -2.0 / (1.0e-3 * 1.0e-3)
    for call in range(2):
        k.ihelm(ref, alpha)
        rc = L.mlg_ihelm_noalloc(ctypes.c_void_p(out.device_ptr()), ctypes.byref(ln), alpha)
        assert rc == 0, L.mlg_last_error().decode()
        k.sync()
        er, lr, _, _ = ref.get()
        eo, _, _, _ = out.get()
        err = rel_l2(eo, er)
        assert err < TOL, f"call {call + 1}: relative L2 difference {err:.3e}"
        assert abs(ln.value - lr) <= 1e-15 * max(1.0, abs(lr)), (ln.value, lr)
    ref.free()
    out.free()
    k.close()


def test_ihelm_noalloc_matches_oracle():
    """Two calls in a row on the reference's small case, each against the oracle's ihelm
    (mlegs_scalar_ops.f90:791-854, banded LU mlegs_bndmat_ops.f90:369-457)."""
    from mlegs_gb300.kit import Kit, load
    from oracle.oracle import Oracle
    p = params("c1")
    o = Oracle(p)
    k = Kit(p)
    L = load()
    L.mlg_ihelm_noalloc.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_double]
    L.mlg_ihelm_noalloc.restype = ctypes.c_int
    e0 = fields.spectral_noise(p, k.dims, 6, amp=1.0, decay=0.05)
    ref = o.scalar(e0, 0.2, "FFF")
    out = k.scalar(e0, 0.2, "FFF")
    ln = ctypes.c_double(0.2)
    alpha = -1.0 / (1.0e-3 * 1.0e-3)
    for call in range(2):
        o.ihelm(ref, alpha)
        rc = L.mlg_ihelm_noalloc(ctypes.c_void_p(out.device_ptr()), ctypes.byref(ln), alpha)
        assert rc == 0, L.mlg_last_error().decode()
        k.sync()
        err = rel_l2(out.e, ref.e)
        assert err < TOL, f"call {call + 1}: relative L2 difference from the oracle {err:.3e}"
        assert abs(ln.value - ref.ln) <= 1e-15 * max(1.0, abs(ref.ln)), (ln.value, ref.ln)
    out.free()
    k.close()
    o.close()


def test_ihelm_noalloc_rejects_zero_alpha():
    from mlegs_gb300.kit import Kit, load
    k = Kit(params("c1"))
    L = load()
    s = k.scalar(np.zeros(k.dims, complex, order="F"), 0.0, "FFF")
    ln = ctypes.c_double(0.0)
    L.mlg_ihelm_noalloc.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_double]
    rc = L.mlg_ihelm_noalloc(ctypes.c_void_p(s.device_ptr()), ctypes.byref(ln), 0.0)
    assert rc == 5 and b"alpha equals to zero" in L.mlg_last_error()
    s.free()
    k.close()
