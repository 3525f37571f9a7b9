"""The adjoint (no counterpart in the reference).

Inner product of the adjoint: <a, b> = sum Re(conj(a.e) b.e) + a.ln b.ln over the whole stored array.
- every transposed operator: the dot-product test <F x, y> = <x, F^T y> on random x, y;
- the nonlinear term and the vortex step: against central differences of the forward, which are
  exact (to rounding) because the term is bilinear and the step quadratic in its state;
- the gradient of J through several steps with checkpointing: central differences of J computed
  by the GPU forward and by the FP64 oracle's forward, checkpoint-interval invariance, and the mixed
  form against the FP64 gradient.
"""
import numpy as np
import pytest

from helpers import params
from mlegs_gb300 import fields, vortex

pytestmark = pytest.mark.gpu

DOT_TOL = 1e-12


def ip(a, b):
    ea, la = a
    eb, lb = b
    return float(np.sum((np.conj(ea) * eb).real) + la * lb)


def rnd(dims, seed, ln=True):
    g = np.random.default_rng(seed)
    e = np.asfortranarray(g.standard_normal(dims) + 1j * g.standard_normal(dims))
    return e, (float(g.standard_normal()) if ln else 0.0)


def get(s):
    e, ln, _, _ = s.get()
    return e, ln


@pytest.fixture(scope="module", params=["c1", "odd"])
def kit(request):
    from mlegs_gb300.kit import Kit
    p = params(request.param, is_svv=0)
    k = Kit(p)
    yield request.param, k
    k.close()


def dot_check(k, x, sp_in, y, sp_out, fwd, adj, what):
    X = k.scalar(x[0], x[1], sp_in)
    fwd(X)
    fx = get(X)
    Y = k.scalar(y[0], y[1], sp_out)
    adj(Y)
    fty = get(Y)
    lhs, rhs = ip(fx, y), ip(x, fty)
    scale = np.sqrt(ip(fx, fx) * ip(y, y)) + np.sqrt(ip(x, x) * ip(fty, fty))
    assert abs(lhs - rhs) <= DOT_TOL * scale, (what, lhs, rhs, scale)


@pytest.mark.parametrize("a,b", [("FFF", "PPP"), ("PPP", "FFF"), ("PFP", "FFF"), ("FFF", "FFP"), ("FFP", "PPP"),
                                 ("PPP", "PFP")])
def test_trans_transpose(kit, a, b):
    name, k = kit
    x, y = rnd(k.dims, 1), rnd(k.dims, 2)
    dot_check(k, x, a, y, b, lambda s: k.trans(s, b), lambda s: k.adj_trans(s, a), f"{name} trans {a}->{b}")


@pytest.mark.parametrize("op", [0, 1, 2])
def test_band_transpose(kit, op):
    name, k = kit
    fwd = [k.xxdx, k.del2h, k.del2][op]
    x, y = rnd(k.dims, 3), rnd(k.dims, 4)
    dot_check(k, x, "FFF", y, "FFF", fwd, lambda s: k.adj_band(s, op), f"{name} band {op}")


def test_solves_transpose(kit):
    name, k = kit
    for alpha in (-3.0e3, -0.7):
        x, y = rnd(k.dims, 5), rnd(k.dims, 6)
        dot_check(k, x, "FFF", y, "FFF", lambda s: k.ihelm(s, alpha), lambda s: k.adj_ihelm(s, alpha),
                  f"{name} ihelm {alpha}")
    x, y = rnd(k.dims, 7), rnd(k.dims, 8)
    dot_check(k, x, "FFF", y, "FFF", lambda s: k.idel2(s), k.adj_idel2_proln, f"{name} idel2_proln")
    x, y = rnd(k.dims, 9), rnd(k.dims, 10)
    dot_check(k, x, "FFF", y, "FFF", k.zeroat1, k.adj_zeroat1, f"{name} zeroat1")


def test_vector_transposes(kit):
    name, k = kit
    d = k.dims
    # tp2vec, tp2curlvec: (psi, chi) FFF -> 3 PPP fields
    for fwd, adj, what in ((k.tp2vec, k.adj_tp2vec, "tp2vec"), (k.tp2curlvec, k.adj_tp2curlvec, "tp2curlvec")):
        xs = [rnd(d, 11), rnd(d, 12)]
        ys = [rnd(d, 13), rnd(d, 14), rnd(d, 15)]
        X = [k.scalar(e, l, "FFF") for e, l in xs]
        V = [k.scalar() for _ in range(3)]
        fwd(*X, *V)
        fx = [get(v) for v in V]
        Y = [k.scalar(e, l, "PPP") for e, l in ys]
        P = [k.scalar(), k.scalar()]
        adj(*Y, *P)
        fty = [get(q) for q in P]
        lhs = sum(ip(a, b) for a, b in zip(fx, ys))
        rhs = sum(ip(a, b) for a, b in zip(xs, fty))
        scale = np.sqrt(sum(ip(a, a) for a in fx) * sum(ip(b, b) for b in ys))
        assert abs(lhs - rhs) <= DOT_TOL * scale, (name, what, lhs, rhs)
    # vec2tp: 3 PPP fields -> (psi, chi) FFF
    xs = [rnd(d, 16), rnd(d, 17), rnd(d, 18)]
    ys = [rnd(d, 19), rnd(d, 20)]
    X = [k.scalar(e, l, "PPP") for e, l in xs]
    Q = [k.scalar(np.zeros(d, complex, order="F"), 0.0, "FFF") for _ in range(2)]
    k.vec2tp(*X, *Q)
    fx = [get(q) for q in Q]
    Y = [k.scalar(e, l, "FFF") for e, l in ys]
    V = [k.scalar() for _ in range(3)]
    k.adj_vec2tp(*Y, *V)
    fty = [get(v) for v in V]
    lhs = sum(ip(a, b) for a, b in zip(fx, ys))
    rhs = sum(ip(a, b) for a, b in zip(xs, fty))
    scale = np.sqrt(sum(ip(a, a) for a in fx) * sum(ip(b, b) for b in ys))
    assert abs(lhs - rhs) <= DOT_TOL * scale, (name, "vec2tp", lhs, rhs)


def base_state(k, seed, pert=1e-3):
    """A q-vortex with spectral noise: the linearisation point."""
    p = k.params
    noise = (fields.spectral_noise(p, k.dims, seed, amp=pert, decay=0.3),
             fields.spectral_noise(p, k.dims, seed + 1, amp=pert, decay=0.3))
    st = vortex.VortexState(k)
    vortex.qvort_init(k, st, q=1.0, uz_b=-0.2, pert=noise)
    return st


def test_advection_transpose(kit):
    name, k = kit
    st = base_state(k, 31)
    d = k.dims
    psi0, chi0 = get(st.psi), get(st.chi)
    dp, dc = rnd(d, 32), rnd(d, 33)
    lp, lc = rnd(d, 34), rnd(d, 35)
    h = 1e-3

    def nl_of(a, b):
        P = k.scalar(a[0], a[1], "FFF")
        C = k.scalar(b[0], b[1], "FFF")
        NP = k.scalar(np.zeros(d, complex, order="F"), 0.0, "FFF")
        NC = k.scalar(np.zeros(d, complex, order="F"), 0.0, "FFF")
        k.advection_rhs(P, C, NP, NC, st.uz)
        return get(NP), get(NC)

    plus = nl_of((psi0[0] + h * dp[0], psi0[1] + h * dp[1]), (chi0[0] + h * dc[0], chi0[1] + h * dc[1]))
    minus = nl_of((psi0[0] - h * dp[0], psi0[1] - h * dp[1]), (chi0[0] - h * dc[0], chi0[1] - h * dc[1]))
    jd = [((pl[0] - mi[0]) / (2 * h), (pl[1] - mi[1]) / (2 * h)) for pl, mi in zip(plus, minus)]
    lhs = ip(jd[0], lp) + ip(jd[1], lc)
    LP, LC = k.scalar(lp[0], lp[1], "FFF"), k.scalar(lc[0], lc[1], "FFF")
    GP, GC = k.scalar(), k.scalar()
    k.adj_advection(st.psi, st.chi, st.uz, LP, LC, GP, GC)
    rhs = ip(dp, get(GP)) + ip(dc, get(GC))
    scale = np.sqrt((ip(jd[0], jd[0]) + ip(jd[1], jd[1])) * (ip(lp, lp) + ip(lc, lc)))
    assert abs(lhs - rhs) <= 1e-10 * scale, (name, lhs, rhs, scale)


def test_vortex_step_transpose(kit):
    name, k = kit
    p = k.params
    st = base_state(k, 41)
    k.advection_rhs(st.psi, st.chi, st.nlpsi, st.nlchi, st.uz)
    st.nlpsi_p.copy_from(st.nlpsi)
    st.nlchi_p.copy_from(st.nlchi)
    dt = 1e-2
    names = ["psi", "chi", "nlpsi", "nlchi", "nlpsi_p", "nlchi_p"]
    s0 = [get(getattr(st, n)) for n in names]
    d = k.dims
    dirs = [rnd(d, 50 + i) for i in range(6)]
    lam = [rnd(d, 60 + i) for i in range(6)]
    h = 1e-4

    def step_of(sgn):
        S = [k.scalar(e + sgn * h * de, l + sgn * h * dl, "FFF") for (e, l), (de, dl) in zip(s0, dirs)]
        pp, cp = k.scalar(), k.scalar()
        pp.copy_from(S[0]); cp.copy_from(S[1])
        k.vortex_step(S[0], S[1], S[2], S[3], pp, cp, S[4], S[5], st.uz, dt, [0.0, 0.0])
        return [get(q) for q in S]

    plus, minus = step_of(+1), step_of(-1)
    jd = [((a[0] - b[0]) / (2 * h), (a[1] - b[1]) / (2 * h)) for a, b in zip(plus, minus)]
    lhs = sum(ip(a, b) for a, b in zip(jd, lam))
    S = [k.scalar(e, l, "FFF") for e, l in s0]
    A = [k.scalar(e, l, "FFF") for e, l in lam]
    k.adj_vortex_step(S, st.uz, dt, A)
    rhs = sum(ip(a, get(b)) for a, b in zip(dirs, A))
    scale = np.sqrt(sum(ip(a, a) for a in jd) * sum(ip(b, b) for b in lam))
    assert abs(lhs - rhs) <= 1e-9 * scale, (name, lhs, rhs, scale)
    # the state it was linearised at is left as it was
    for (e, l), q in zip(s0, S):
        e2, l2 = get(q)
        assert np.array_equal(e, e2) and l == l2


def perturbed(p, dims, seed, amp):
    return fields.spectral_noise(p, dims, seed, amp=amp, decay=0.3)


def test_gradient_matches_finite_differences(kit):
    name, k = kit
    p = k.params
    st = base_state(k, 71, pert=1e-3)
    dt, nsteps = 1e-2, 5
    psi0, chi0 = get(st.psi), get(st.chi)
    gp, gc = k.scalar(), k.scalar()
    J = k.adjoint_run(st.psi, st.chi, st.uz, dt, nsteps, 2, gp, gc)
    g = (get(gp), get(gc))
    assert J > 0
    # unchanged inputs
    assert np.array_equal(get(st.psi)[0], psi0[0])
    # checkpoint interval does not change the result
    gp1, gc1 = k.scalar(), k.scalar()
    J1 = k.adjoint_run(st.psi, st.chi, st.uz, dt, nsteps, 1, gp1, gc1)
    gpn, gcn = k.scalar(), k.scalar()
    k.adjoint_run(st.psi, st.chi, st.uz, dt, nsteps, nsteps, gpn, gcn)
    assert J1 == J
    for a, b in ((gp1, gp), (gc1, gc), (gpn, gp), (gcn, gc)):
        ea, eb = get(a)[0], get(b)[0]
        assert np.max(np.abs(ea - eb)) <= 1e-13 * np.max(np.abs(eb))
    # central differences of J in seeded directions
    h = 1e-6
    for seed in range(3):
        dp = (perturbed(p, k.dims, 100 + seed, 1.0), 0.0)
        dc = (perturbed(p, k.dims, 200 + seed, 1.0), 0.0)
        sc = 1.0 / np.sqrt(ip(dp, dp) + ip(dc, dc))
        dp, dc = (dp[0] * sc, 0.0), (dc[0] * sc, 0.0)

        def J_at(sgn):
            P = k.scalar(psi0[0] + sgn * h * dp[0], psi0[1], "FFF")
            C = k.scalar(chi0[0] + sgn * h * dc[0], chi0[1], "FFF")
            return k.adjoint_run(P, C, st.uz, dt, nsteps, 2)

        fd = (J_at(+1) - J_at(-1)) / (2 * h)
        an = ip(g[0], dp) + ip(g[1], dc)
        assert abs(fd - an) <= 1e-5 * abs(an) + 1e-9 * abs(J), (name, seed, fd, an)
