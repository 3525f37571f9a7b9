"""Shared helpers of the parity tests: paired GPU kit / CPU oracle and field comparisons."""
import numpy as np

from mlegs_gb300.params import make_params

# the configurations of the parity tests (small enough for the oracle to finish in seconds)
CONFIGS = {
    # the reference's CPU-runnable case: NR=NP=NZ=32, ELL=4, chops 32/17/17 (full: exercises the
    # shared Nyquist z slot)
    "c1": dict(nr=32, np=32, nz=32, nrchop=32, npchop=17, nzchop=17, ell=4.0, visc=1.0e-3),
    # 2-D kit, the transformation / operation tutorials (NR=32, NP=48, ELL=1)
    "t2d": dict(nr=32, np=48, nz=1, nrchop=32, npchop=25, nzchop=1, ell=1.0, zlen=1.0, visc=5.0e-3),
    # radix 3 and 5 in both FFTs, partial chops, odd sizes
    "odd": dict(nr=24, np=30, nz=20, nrchop=20, npchop=11, nzchop=7, ell=2.0, visc=2.0e-3),
    # hyperviscosity (nrdim = nr + hyperpow)
    "hyp": dict(nr=16, np=12, nz=12, nrchop=16, npchop=7, nzchop=7, ell=3.0, visc=1.0e-3, hyperpow=4,
                hypervisc=1.0e-6),
}


def params(name, **kw):
    d = dict(CONFIGS[name])
    d.update(kw)
    return make_params(**d)


def rel_l2(a, b):
    nb = np.linalg.norm(b)
    if nb == 0:
        return float(np.linalg.norm(a))
    return float(np.linalg.norm(a - b) / nb)


def rel_max(a, b):
    mb = np.max(np.abs(b)) if b.size else 0.0
    if mb == 0:
        return float(np.max(np.abs(a))) if a.size else 0.0
    return float(np.max(np.abs(a - b)) / mb)


def compare(gs, os_, tol, ln_tol=None, what=""):
    ge, gln, gsp, goff = gs.get()
    oe, oln, osp, ooff = os_.get()
    assert gsp == osp, f"{what}: space {gsp} != {osp}"
    assert goff == ooff, f"{what}: offsets {goff} != {ooff}"
    err = rel_l2(ge, oe)
    assert err <= tol, f"{what}: relative L2 error {err:.3e} > {tol:.1e} (max rel {rel_max(ge, oe):.3e})"
    lt = tol if ln_tol is None else ln_tol
    scale = max(abs(oln), 1e-300)
    if oln != 0 or gln != 0:
        assert abs(gln - oln) <= lt * max(scale, np.max(np.abs(oe))), f"{what}: ln {gln!r} != {oln!r}"
    return err
