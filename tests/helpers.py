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


def qvortex_closed_form(p, dims, r, q=1.0, xo=0.0, yo=0.0):
    """The q-vortex V = (1 - exp(-r'^2))/r' e_phi' + exp(-r'^2)/q e_z about (xo, yo)
    (docs/tutorial/vector_field.md:88-106) and W = curl V, sampled at the collocation points and
    packed as PPP fields (real part of slot j at phi_{2j}, imaginary part at phi_{2j+1}, every z).
    Returns ([V_r, V_phi, V_z], [W_r, W_phi, W_z])."""
    nph = p.np // 2
    phi = 2 * np.pi / p.np * np.arange(p.np)
    R, PH = np.asarray(r)[:, None], phi[None, :]
    dx, dy = R * np.cos(PH) - xo, R * np.sin(PH) - yo
    rp2 = dx * dx + dy * dy
    g = np.where(rp2 > 0, -np.expm1(-rp2) / np.where(rp2 > 0, rp2, 1.0), 1.0)
    vx, vy, vz = -dy * g, dx * g, np.exp(-rp2) / q
    wx, wy, wz = -2 * dy * vz, 2 * dx * vz, 2 * np.exp(-rp2)
    c, s = np.cos(PH), np.sin(PH)

    def pack(a):
        e = np.zeros(dims, complex, order="F")
        e[: p.nr, :nph, :] = (a[:, 0::2] + 1j * a[:, 1::2])[:, :, None]
        return e
    return ([pack(a) for a in (vx * c + vy * s, -vx * s + vy * c, vz)],
            [pack(a) for a in (wx * c + wy * s, -wx * s + wy * c, wz)])


def qvortex_tp(kit, q=1.0, xo=0.0, yo=0.0):
    """psi and chi of the q-vortex by the reference's recipe (vecfld_reconstruction.f90:155-215): the
    closed-form vorticity and axial flow over (1-x)^2 in PPP, to FFF, idelsqp, zeroat1."""
    from mlegs_gb300 import fields
    a, b = fields.qvort_ppp(kit.params, kit.dims, kit.kit_get("r"), kit.kit_get("x"), q=q, centers=((xo, yo),))
    out = []
    for src in (a, b):
        s = kit.scalar(src, 0.0, "PPP")
        kit.trans(s, "FFF")
        kit.idelsqp(s)
        kit.zeroat1(s)
        out.append(s)
    return out
