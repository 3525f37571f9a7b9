"""GPU parity: every operator of the C ABI against the CPU oracle on the same seeded inputs.

The plain form (all FP64) must agree with the oracle's FP64 restatement of the reference to 1e-12
relative (L2 over the field), the drop-in's bar; the Poisson solves, the steppers over three calls
and five vortex steps, which compound rounding through the solves, are held to 1e-11.  The mixed
form is checked against the same oracle per operator at 1e-6 (transforms, vector fields and the
projection, on three kits including 192 x 128 x 128), and against the FP64 form over 20 vortex steps at
192 x 128 x 128 at 1e-6.  (C1 with its 100 febe and abcn steps is
in tests/test_gpu_configs.py.)
"""
import numpy as np
import pytest

from mlegs_gb300 import fields
from helpers import CONFIGS, params, compare, rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-12
# Poisson solves (idel2) are not diagonally dominant: their condition number (~1e4 at these sizes)
# multiplies the rounding difference between two correct FP64 evaluations.
TOL_POISSON = 1e-11


@pytest.fixture(scope="module", params=["c1", "t2d", "odd", "hyp"])
def pair(request):
    from mlegs_gb300.kit import Kit
    from oracle.oracle import Oracle
    p = params(request.param)
    o = Oracle(p)
    k = Kit(p)
    yield request.param, k, o
    k.close()
    o.close()


def both(k, o, e, ln=0.0, space="FFF"):
    return k.scalar(e, ln, space), o.scalar(e, ln, space)


def fff_input(p, dims, seed, amp=1.0):
    return fields.spectral_noise(p, dims, seed, amp=amp, decay=0.05)


def test_kit_arrays(pair):
    name, k, o = pair
    for a in ["x", "w", "r", "ln", "ak", "lognorm", "at0", "at1"]:
        g, c = k.kit_get(a), o.kit_get(a)
        assert np.array_equal(g, c) or rel_l2(g, c) < 1e-15, (a, rel_l2(g, c))
    g, c = k.kit_get("pf"), o.kit_get("pf")
    # the table: double-double recurrence on the GPU, binary128 in the oracle, both rounded to FP64
    big = np.abs(c) > 1e-250
    rel = np.abs(g[big] - c[big]) / np.abs(c[big])
    assert rel.max() < 1e-14, rel.max()
    assert np.all(np.abs(g[~big]) < 1e-240)


def test_trans_roundtrip(pair):
    name, k, o = pair
    p = k.params
    e = fields.ppp_random(p, k.dims, seed=11)
    gs, os_ = both(k, o, e, 0.0, "PPP")
    for sp in ["PFP", "FFP", "FFF"]:
        k.trans(gs, sp); o.trans(os_, sp)
        compare(gs, os_, TOL, what=f"{name} PPP->{sp}")
    c = fff_input(p, k.dims, 12)
    gs, os_ = both(k, o, c, 0.3, "FFF")
    for sp in ["FFP", "PFP", "PPP"]:
        k.trans(gs, sp); o.trans(os_, sp)
        compare(gs, os_, TOL, what=f"{name} FFF->{sp}")
    k.trans(gs, "FFF"); o.trans(os_, "FFF")
    compare(gs, os_, TOL, what=f"{name} round trip")


@pytest.mark.parametrize("op", ["chop", "dealias", "zeroat1", "delsqp", "idelsqp", "xxdx", "del2h", "del2",
                                "idel2_pro", "idel2_pre", "helm", "ihelm", "svv"])
def test_single_operator(pair, op):
    name, k, o = pair
    p = k.params
    c = fff_input(p, k.dims, 21)
    for ln in (0.0, 0.7):
        gs, os_ = both(k, o, c, ln, "FFF")
        if op == "idel2_pro":
            k.idel2(gs); o.idel2(os_)
        elif op == "idel2_pre":
            k.idel2(gs, 0.25); o.idel2(os_, 0.25)
        elif op in ("helm", "ihelm"):
            getattr(k, op)(gs, -3.5e3); getattr(o, op)(os_, -3.5e3)
        elif op == "svv":
            # a field with a heavy tail, so that the filter engages
            big = fields.spectral_noise(p, k.dims, 22, amp=1.0, decay=0.0)
            gs.set(big, ln, "FFF"); os_.set(big, ln, "FFF")
            g1 = k.svv_filter(gs, 0.5)
            g2 = o.svv_filter(os_, 0.5)
            assert abs(g1 - g2) <= 1e-14 * max(1.0, abs(g2)), (g1, g2)
        else:
            getattr(k, op)(gs); getattr(o, op)(os_)
        compare(gs, os_, TOL_POISSON if op.startswith("idel2") else TOL, what=f"{name} {op} ln={ln}")


def test_chop_offset_and_partial_space(pair):
    name, k, o = pair
    p = k.params
    c = fff_input(p, k.dims, 31)
    gs, os_ = both(k, o, c, 0.0, "FFF")
    gs.chop_offset(3); os_.chop_offset(3)
    k.xxdx(gs); o.xxdx(os_)
    compare(gs, os_, TOL, what=f"{name} xxdx offset 3")
    k.del2h(gs); o.del2h(os_)
    compare(gs, os_, TOL, what=f"{name} del2h offset 3")
    gs.chop_offset(0); os_.chop_offset(0)
    k.chop(gs); o.chop(os_)
    compare(gs, os_, TOL, what=f"{name} chop")


def test_calcat(pair):
    name, k, o = pair
    p = k.params
    c = fff_input(p, k.dims, 41)
    gs, os_ = both(k, o, c, 0.0, "FFF")
    for f in ("calcat0", "calcat1"):
        g, r = getattr(k, f)(gs), getattr(o, f)(os_)
        assert rel_l2(g, r) < TOL, (f, rel_l2(g, r))
    # from a physical field (calcat transforms a copy)
    e = fields.ppp_random(p, k.dims, seed=42)
    gs, os_ = both(k, o, e, 0.0, "PPP")
    g, r = k.calcat0(gs), o.calcat0(os_)
    assert rel_l2(g, r) < TOL
    compare(gs, os_, 0.0, what="calcat leaves its argument unchanged")


@pytest.mark.parametrize("op", ["helmp", "ihelmp"])
def test_powered_helmholtz(pair, op):
    name, k, o = pair
    p = k.params
    c = fff_input(p, k.dims, 51)
    # alpha = -2/(dt*hypervisc) as the steppers use it (dt = 1e-3, hypervisc = 1e-6): the identity
    # term dominates, as in every hyperviscous step of the reference
    for power in (4, 6, 8):
        gs, os_ = both(k, o, c, 0.2, "FFF")
        getattr(k, op)(gs, power, -2.0e9, 0.5); getattr(o, op)(os_, power, -2.0e9, 0.5)
        compare(gs, os_, 1e-11, what=f"{name} {op} p={power}")


@pytest.mark.parametrize("op", ["fefe", "abab", "febe", "abcn"])
def test_steppers(pair, op):
    name, k, o = pair
    p = k.params
    s0, sp0 = fff_input(p, k.dims, 61), fff_input(p, k.dims, 62)
    n0, np0 = fff_input(p, k.dims, 63, 0.1), fff_input(p, k.dims, 64, 0.1)
    g = [k.scalar(a, ln, "FFF") for a, ln in ((s0, 0.1), (sp0, 0.2), (n0, 0.05), (np0, 0.0))]
    r = [o.scalar(a, ln, "FFF") for a, ln in ((s0, 0.1), (sp0, 0.2), (n0, 0.05), (np0, 0.0))]
    dt = 1e-3
    for _ in range(3):
        if op in ("fefe", "febe"):
            getattr(k, op)(g[0], g[2], dt); getattr(o, op)(r[0], r[2], dt)
        else:
            getattr(k, op)(g[0], g[1], g[2], g[3], dt); getattr(o, op)(r[0], r[1], r[2], r[3], dt)
    for i in range(4):
        compare(g[i], r[i], 1e-11, what=f"{name} {op} arg{i}")


def test_vector_fields(pair):
    name, k, o = pair
    p = k.params
    if p.np < 4:
        pytest.skip("needs an azimuthal direction")
    psi, chi = fff_input(p, k.dims, 71), fff_input(p, k.dims, 72)
    gp, op_ = both(k, o, psi, 0.0, "FFF")
    gc, oc = both(k, o, chi, 0.0, "FFF")
    gv = [k.scalar() for _ in range(3)]
    ov = [o.scalar() for _ in range(3)]
    k.tp2vec(gp, gc, *gv); o.tp2vec(op_, oc, *ov)
    for i in range(3):
        compare(gv[i], ov[i], TOL, what=f"{name} tp2vec {i}")
    gw = [k.scalar() for _ in range(3)]
    ow = [o.scalar() for _ in range(3)]
    k.tp2curlvec(gp, gc, *gw); o.tp2curlvec(op_, oc, *ow)
    for i in range(3):
        compare(gw[i], ow[i], TOL, what=f"{name} tp2curlvec {i}")
    k.vecprod(*gv, *gw); o.vecprod(*ov, *ow)
    for i in range(3):
        compare(gv[i], ov[i], TOL, what=f"{name} vecprod {i}")
    gq = [k.scalar(np.zeros(k.dims, complex, order="F"), 0.0, "FFF") for _ in range(2)]
    oq = [o.scalar(np.zeros(k.dims, complex, order="F"), 0.0, "FFF") for _ in range(2)]
    k.vec2tp(*gv, *gq); o.vec2tp(*ov, *oq)
    for i in range(2):
        compare(gq[i], oq[i], 1e-11, what=f"{name} vec2tp {i}")


def test_vortex_steps(pair):
    name, k, o = pair
    p = k.params
    if p.nz < 4 or p.np < 4:
        pytest.skip("3-D case only")
    from mlegs_gb300 import vortex
    # identical initial state on both sides: the oracle builds it, the GPU receives the same bytes
    so = vortex.VortexState(o)
    pert = (fields.spectral_noise(p, o.dims, 81, amp=1e-3, decay=0.3, m_max=4, k_max=8),
            fields.spectral_noise(p, o.dims, 82, amp=1e-3, decay=0.3, m_max=4, k_max=8))
    vortex.qvort_init(o, so, q=4.0, uz_b=-0.5, pert=pert)
    sg = vortex.VortexState(k)
    for n in vortex.VortexState.names:
        e, ln, sp, _ = getattr(so, n).get()
        getattr(sg, n).set(e, ln, sp)
    dt = 1e-3
    vortex.bootstrap(k, sg, dt)
    vortex.bootstrap(o, so, dt)
    for n in ("psi", "chi", "nlpsi", "nlchi"):
        compare(getattr(sg, n), getattr(so, n), 1e-11, what=f"{name} bootstrap {n}")
    for _ in range(5):
        vortex.step(k, sg, dt)
        vortex.step(o, so, dt)
    for n in ("psi", "chi", "nlpsi", "nlchi", "psi_p", "nlpsi_p"):
        compare(getattr(sg, n), getattr(so, n), 1e-11, what=f"{name} 5 steps {n}")
    assert abs(sg.gains[0] - so.gains[0]) < 1e-12 and abs(sg.gains[1] - so.gains[1]) < 1e-12


# ---- the mixed form (exact-slice contractions, FP32 FFTs; FP64 state, solves and reductions) ----
MIXED_TOL = 1e-6


@pytest.fixture(scope="module", params=["c1", "odd", "big"])
def mixed_pair(request):
    from mlegs_gb300.kit import Kit, MIXED
    from oracle.oracle import Oracle
    from mlegs_gb300.params import make_params
    if request.param == "big":
        # the benchmark grid: radial contractions of the full size
        p = make_params(nr=192, np=128, nz=128, nrchop=192, npchop=65, nzchop=65, ell=4.0, visc=1.0e-4)
    else:
        p = params(request.param)
    o = Oracle(p)
    k = Kit(p, precision=MIXED)
    yield request.param, k, o
    k.close()
    o.close()


def test_mixed_transforms(mixed_pair):
    name, k, o = mixed_pair
    p = k.params
    e = fields.ppp_random(p, k.dims, seed=91)
    gs, os_ = both(k, o, e, 0.0, "PPP")
    k.trans(gs, "FFF"); o.trans(os_, "FFF")
    compare(gs, os_, MIXED_TOL, ln_tol=1.0, what=f"{name} mixed forward")
    c = fff_input(p, k.dims, 92)
    gs, os_ = both(k, o, c, 0.0, "FFF")
    k.trans(gs, "PPP"); o.trans(os_, "PPP")
    compare(gs, os_, MIXED_TOL, ln_tol=1.0, what=f"{name} mixed backward")


def test_mixed_vector_fields(mixed_pair):
    # spectra decaying like the physical fields: the projection ends with a Poisson solve whose
    # condition number would amplify FP32-level differences of heavy high modes
    name, k, o = mixed_pair
    p = k.params
    psi = fields.spectral_noise(p, k.dims, 93, amp=1.0, decay=0.3)
    chi = fields.spectral_noise(p, k.dims, 94, amp=1.0, decay=0.3)
    gp, op_ = both(k, o, psi, 0.0, "FFF")
    gc, oc = both(k, o, chi, 0.0, "FFF")
    gv = [k.scalar() for _ in range(3)]
    ov = [o.scalar() for _ in range(3)]
    k.tp2vec(gp, gc, *gv); o.tp2vec(op_, oc, *ov)
    for i in range(3):
        compare(gv[i], ov[i], MIXED_TOL, ln_tol=1.0, what=f"{name} mixed tp2vec {i}")
    # the projection from the same (FP64) vectors on both sides: chi ends with an inverse horizontal
    # Laplacian that turns a 1e-6 difference of u_z into ~1e-3 in chi, so feeding each side its own
    # tp2vec output would measure tp2vec's rounding, not vec2tp's
    gin = [k.scalar(v.e, v.ln, v.space) for v in ov]
    gq = [k.scalar(np.zeros(k.dims, complex, order="F"), 0.0, "FFF") for _ in range(2)]
    oq = [o.scalar(np.zeros(k.dims, complex, order="F"), 0.0, "FFF") for _ in range(2)]
    k.vec2tp(*gin, *gq); o.vec2tp(*ov, *oq)
    for i in range(2):
        compare(gq[i], oq[i], 1e-6, ln_tol=1.0, what=f"{name} mixed vec2tp {i}")


def test_mixed_vortex_steps_within_1e6_of_fp64():
    """The mixed form against the FP64 form over 20 vortex steps at 192x128x128 (q = 4 Batchelor
    vortex, Re = 1e4, dt = 1e-3, SVV on, perturbation 1e-4 on |m| <= 4, |k| <= 8): the state fields
    psi, chi (and their history) and the nonlinear-term fields nlpsi, nlchi, all within 1e-6 relative.
    The FP64 form itself matches the oracle to 1e-11 (test_vortex_steps)."""
    from mlegs_gb300 import vortex
    from mlegs_gb300.kit import Kit, MIXED, PLAIN_FP64
    from mlegs_gb300.params import make_params
    p = make_params(nr=192, np=128, nz=128, nrchop=192, npchop=65, nzchop=65, ell=4.0, visc=1.0e-4)
    k = Kit(p)
    st = vortex.VortexState(k)
    pert = (fields.spectral_noise(p, k.dims, 1001, amp=1e-4, decay=0.3, m_max=4, k_max=8),
            fields.spectral_noise(p, k.dims, 1002, amp=1e-4, decay=0.3, m_max=4, k_max=8))
    vortex.qvort_init(k, st, q=4.0, uz_b=0.0, pert=pert)
    vortex.bootstrap(k, st, 1e-3)
    snap = {n: getattr(st, n).get() for n in st.names}
    out = {}
    for mode in (PLAIN_FP64, MIXED):
        k.set_precision(mode)
        for n, (e, ln, sp, _) in snap.items():
            getattr(st, n).set(e, ln, sp)
        st.gains = [0.0, 0.0]
        k.vortex_run(*st.args(), 1e-3, 20, st.gains)
        out[mode] = {n: getattr(st, n).get() for n in ("psi", "chi", "nlpsi", "nlchi", "psi_p", "chi_p")}
    k.close()
    for n in out[MIXED]:
        a, b = out[MIXED][n], out[PLAIN_FP64][n]
        err = np.linalg.norm(a[0] - b[0]) / np.linalg.norm(b[0])
        tol = 1e-6
        assert err < tol, f"mixed {n} after 20 steps: {err:.3e} relative to FP64"
        assert abs(a[1] - b[1]) <= 1e-6 * max(1.0, abs(b[1])), f"mixed {n} ln: {a[1]} vs {b[1]}"


@pytest.mark.parametrize("nsteps", [4, 5])
def test_vortex_run_equals_single_steps(nsteps):
    """A run of nsteps steps leaves the same bytes in all eight fields as nsteps single-step calls, in
    both forms: a run writes psi_p and chi_p on its last step only, and nlpsi_p and nlchi_p take the
    buffers of nlpsi and nlchi each step, which the step's advection then recomputes.  A run of four or
    more steps replays its interior steps as a captured graph of two steps (4: one pair; 5: one pair
    and one step as launched)."""
    from mlegs_gb300 import vortex
    from mlegs_gb300.kit import Kit, MIXED, PLAIN_FP64
    from mlegs_gb300.params import make_params
    p = make_params(nr=48, np=32, nz=32, nrchop=48, npchop=17, nzchop=17, ell=4.0, visc=1.0e-3)
    k = Kit(p)
    st = vortex.VortexState(k)
    pert = (fields.spectral_noise(p, k.dims, 91, amp=1e-3, decay=0.3, m_max=4, k_max=8),
            fields.spectral_noise(p, k.dims, 92, amp=1e-3, decay=0.3, m_max=4, k_max=8))
    vortex.qvort_init(k, st, q=4.0, uz_b=-0.5, pert=pert)
    vortex.bootstrap(k, st, 1e-3)
    snap = {n: getattr(st, n).get() for n in st.names}
    names = ("psi", "chi", "nlpsi", "nlchi", "psi_p", "chi_p", "nlpsi_p", "nlchi_p")
    for mode in (PLAIN_FP64, MIXED):
        k.set_precision(mode)
        out = []
        for run in (True, False):
            for n, (e, ln, sp, _) in snap.items():
                getattr(st, n).set(e, ln, sp)
            st.gains = [0.0, 0.0]
            if run:
                k.vortex_run(*st.args(), 1e-3, nsteps, st.gains)
            else:
                for _ in range(nsteps):
                    vortex.step(k, st, 1e-3)
            out.append(({n: getattr(st, n).get() for n in names}, list(st.gains)))
        (a, ga), (b, gb) = out
        assert ga == gb, f"form {mode}: gains {ga} vs {gb}"
        for n in names:
            assert np.array_equal(a[n][0], b[n][0]) and a[n][1] == b[n][1] and a[n][2] == b[n][2], \
                f"form {mode}: {n} of a {nsteps}-step run differs from {nsteps} single steps"
    k.close()


@pytest.mark.parametrize("op", ["idel2_pro", "idel2_pre", "ihelm", "abcn"])
def test_mixed_solves_stay_fp64(mixed_pair, op):
    """The mixed form keeps the banded solves in FP64 (only abcn's explicit increment is summed in
    FP32 for m >= 1): held to 1e-10 of the FP64 oracle (1e-9 for the Poisson solves, whose condition
    number is ~1e4), far inside the 1e-6 of the mixed transforms."""
    name, k, o = mixed_pair
    p = k.params
    c = fff_input(p, k.dims, 121)
    for ln in ((0.0,) if op == "abcn" else (0.0, 0.7)):
        if op == "abcn":
            g = [k.scalar(fff_input(p, k.dims, 122 + i, 1.0 if i < 2 else 0.1), 0.1 * i, "FFF") for i in range(4)]
            r = [o.scalar(*x.get()[:3]) for x in g]
            k.abcn(*g, 1e-3); o.abcn(*r, 1e-3)
            for i in range(4):
                compare(g[i], r[i], 1e-10, what=f"{name} mixed abcn arg{i} ln={ln}")
            continue
        gs, os_ = both(k, o, c, ln, "FFF")
        if op == "idel2_pro":
            k.idel2(gs); o.idel2(os_)
        elif op == "idel2_pre":
            k.idel2(gs, 0.25); o.idel2(os_, 0.25)
        else:
            k.ihelm(gs, -3.5e3); o.ihelm(os_, -3.5e3)
        compare(gs, os_, 1e-9 if op.startswith("idel2") else 1e-10, what=f"{name} mixed {op} ln={ln}")
