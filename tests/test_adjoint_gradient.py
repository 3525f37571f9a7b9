"""The adjoint's gradient against the FP64 oracle's forward (central differences of J computed on the
CPU), the mixed form's gradient against the FP64 one, and the refusal with SVV on.  Each test makes
its own kit (the library holds one kit at a time)."""
import numpy as np
import pytest

from helpers import params
from test_adjoint import base_state, get, ip, perturbed

pytestmark = pytest.mark.gpu


def oracle_J(o, p, psi0, chi0, uz, dt, nsteps):
    """J through the FP64 oracle's own forward (same startup and steps as mlg_adjoint_run)."""
    dims = psi0[0].shape
    z = lambda: o.scalar(np.zeros(dims, complex, order="F"), 0.0, "FFF")
    P, C = o.scalar(psi0[0], psi0[1], "FFF"), o.scalar(chi0[0], chi0[1], "FFF")
    NP, NC = z(), z()
    U = o.scalar(uz, 0.0, "PPP")
    o.advection_rhs(P, C, NP, NC, U)
    NPP, NCP = z(), z()
    NPP.copy_from(NP); NCP.copy_from(NC)
    PP, CP = z(), z()
    for _ in range(nsteps):
        o.vortex_step(P, C, NP, NC, PP, CP, NPP, NCP, U, dt, [0.0, 0.0])
    pe, ce = P.get()[0].copy(), C.get()[0].copy()
    pe[:, 0, 0] = 0
    ce[:, 0, 0] = 0
    PT, CT = o.scalar(pe, 0.0, "FFF"), o.scalar(ce, 0.0, "FFF")
    V = [o.scalar() for _ in range(3)]
    o.tp2vec(PT, CT, *V)
    x, w, r = o.kit_get("x"), o.kit_get("w"), o.kit_get("r")
    W = w * r ** 2 / (1 - x ** 2) * (2 * np.pi / p.np) * (p.zlen / p.nz)
    J = 0.0
    for v in V:
        e = v.get()[0][: p.nr, : p.np // 2, :]
        J += 0.5 * np.sum(W[:, None, None] * (e.real ** 2 + e.imag ** 2))
    return J


def test_gradient_against_oracle_forward():
    from mlegs_gb300.kit import Kit, MIXED
    from oracle.oracle import Oracle
    p = params("c1", is_svv=0)
    k = Kit(p)
    o = Oracle(p)
    st = base_state(k, 81, pert=1e-3)
    dt, nsteps = 1e-2, 4
    psi0, chi0 = get(st.psi), get(st.chi)
    uz = st.uz.get()[0]
    gp, gc = k.scalar(), k.scalar()
    J = k.adjoint_run(st.psi, st.chi, st.uz, dt, nsteps, 3, gp, gc)
    Jo = oracle_J(o, p, psi0, chi0, uz, dt, nsteps)
    assert abs(J - Jo) <= 1e-11 * abs(Jo), (J, Jo)
    g = (get(gp), get(gc))
    h = 1e-6
    for seed in range(2):
        dp = perturbed(p, k.dims, 300 + seed, 1.0)
        dc = perturbed(p, k.dims, 400 + seed, 1.0)
        sc = 1.0 / np.sqrt(np.sum(np.abs(dp) ** 2) + np.sum(np.abs(dc) ** 2))
        dp, dc = dp * sc, dc * sc
        fd = (oracle_J(o, p, (psi0[0] + h * dp, psi0[1]), (chi0[0] + h * dc, chi0[1]), uz, dt, nsteps)
              - oracle_J(o, p, (psi0[0] - h * dp, psi0[1]), (chi0[0] - h * dc, chi0[1]), uz, dt, nsteps)) / (2 * h)
        an = ip(g[0], (dp, 0.0)) + ip(g[1], (dc, 0.0))
        assert abs(fd - an) <= 1e-5 * abs(an) + 1e-9 * abs(J), (seed, fd, an)
    # the mixed form's gradient against the FP64 one
    k.set_precision(MIXED)
    mp, mc = k.scalar(), k.scalar()
    Jm = k.adjoint_run(st.psi, st.chi, st.uz, dt, nsteps, 3, mp, mc)
    k.set_precision(0)
    num = np.sqrt(np.sum(np.abs(get(mp)[0] - g[0][0]) ** 2) + np.sum(np.abs(get(mc)[0] - g[1][0]) ** 2))
    den = np.sqrt(np.sum(np.abs(g[0][0]) ** 2) + np.sum(np.abs(g[1][0]) ** 2))
    assert abs(Jm - J) <= 1e-5 * J
    assert num / den <= 1e-4, num / den
    k.close()
    o.close()


def test_adjoint_rejects_svv_on():
    from mlegs_gb300.kit import Kit, MlgError
    p = params("c1")   # SVV on by default
    k = Kit(p)
    s = k.scalar(np.zeros(k.dims, complex, order="F"), 0.0, "FFF")
    u = k.scalar(np.zeros(k.dims, complex, order="F"), 0.0, "PPP")
    with pytest.raises(MlgError):
        k.adjoint_run(s, s, u, 1e-2, 1, 1)
    k.close()


def test_gradient_over_many_steps_with_svv_off():
    """128 x 64 x 64 Lamb-Oseen vortex, SVV off, 60 steps with checkpoints every 20: the gradient
    with respect to the active coefficients stays finite and matches central differences.  (The
    chopped coefficients the step reads through its vector reconstruction would otherwise enter the
    adjoint with a growth of ~5e6 per step.)"""
    from mlegs_gb300 import fields, vortex
    from mlegs_gb300.kit import Kit
    from mlegs_gb300.params import make_params
    p = make_params(nr=128, np=64, nz=64, nrchop=128, npchop=33, nzchop=33, ell=4.0, visc=2.0e-4, is_svv=0)
    k = Kit(p)
    st = vortex.VortexState(k)
    pert = (fields.spectral_noise(p, k.dims, 2001, amp=1e-5, decay=0.3, m_max=4, k_max=8),
            fields.spectral_noise(p, k.dims, 2002, amp=1e-5, decay=0.3, m_max=4, k_max=8))
    vortex.qvort_init(k, st, q=np.inf, uz_b=0.0, pert=pert)
    psi0, chi0 = get(st.psi), get(st.chi)
    dt, n, kc = 2e-3, 60, 20
    gp, gc = k.scalar(), k.scalar()
    J = k.adjoint_run(st.psi, st.chi, st.uz, dt, n, kc, gp, gc)
    g = (get(gp), get(gc))
    assert np.all(np.isfinite(g[0][0])) and np.all(np.isfinite(g[1][0]))
    # zero off the active set
    act = fields.active_mask(p, k.dims)
    assert np.all(g[0][0][~act] == 0) and np.all(g[1][0][~act] == 0)
    h = 1e-6
    for seed in range(2):
        dp = perturbed(p, k.dims, 500 + seed, 1.0)
        dc = perturbed(p, k.dims, 600 + seed, 1.0)
        sc = 1.0 / np.sqrt(np.sum(np.abs(dp) ** 2) + np.sum(np.abs(dc) ** 2))
        dp, dc = dp * sc, dc * sc
        Js = []
        for sgn in (1.0, -1.0):
            P = k.scalar(psi0[0] + sgn * h * dp, psi0[1], "FFF")
            C = k.scalar(chi0[0] + sgn * h * dc, chi0[1], "FFF")
            Js.append(k.adjoint_run(P, C, st.uz, dt, n, kc))
        fd = (Js[0] - Js[1]) / (2 * h)
        an = ip(g[0], (dp, 0.0)) + ip(g[1], (dc, 0.0))
        assert abs(fd - an) <= 1e-5 * abs(an) + 1e-9 * abs(J), (seed, fd, an)
    k.close()
