"""GPU parity on the benchmark's configurations and on the reference's closed-form vortex.

* C1 exactly as the benchmark states it: NR = NP = NZ = 32, ELL = 4, chops 32/17/17, axial period
  2 pi; exp(-r^2) plus seeded spectral noise 1e-3 exp(-0.3 (n + |m| + |k|)); a round trip, then 100
  febe and (separately) 100 abcn diffusion steps with nu = 1e-3, dt = 1e-3 (mlegs_scalar_ops.f90:
  1157-1262), against the oracle: 1e-12 for the transforms, 1e-11 for the steps.
* The 3-D vortex step at the metric's grid, 192 x 128 x 128, in the plain form against the oracle:
  3 steps from the same state, psi, chi and nlpsi at 1e-11 and nlchi at 5e-11.  nlchi ends in
  k X - Y and the inverse Laplacian, which cancel: two FP64 evaluations that only order their sums
  differently (this library's all-DFMA contractions and the oracle) already differ by up to 2.4e-11
  there after one step.
* The q-vortex closed forms (docs/tutorial/vector_field.md:88-106) through the CUDA path: tp2vec,
  tp2curlvec and vec2tp of the off-centre and the centred vortex, and the vanishing nonlinear term of
  the axisymmetric vortex, in both precision forms.
"""
import numpy as np
import pytest

from mlegs_gb300 import fields
from helpers import compare, params, qvortex_closed_form, qvortex_tp, rel_l2

pytestmark = pytest.mark.gpu

NU = DT = 1.0e-3


def c1_input(k):
    """exp(-r^2) in PPP, to FFF, plus the seeded noise on the active coefficients (Hermitian at m = 0)."""
    p = k.params
    r = k.kit_get("r")
    e = np.zeros(k.dims, complex, order="F")
    g = np.exp(-r ** 2)
    e[: p.nr, : p.np // 2, :] = (g + 1j * g)[:, None, None]
    s = k.scalar(e, 0.0, "PPP")
    k.trans(s, "FFF")
    c = s.e + fields.spectral_noise(p, k.dims, 2024, amp=1.0e-3, decay=0.3)
    s.free()
    return c


@pytest.fixture(scope="module")
def c1():
    from mlegs_gb300.kit import Kit
    from oracle.oracle import Oracle
    p = params("c1", visc=NU)
    o = Oracle(p)
    k = Kit(p)
    yield k, o, c1_input(o)
    k.close()
    o.close()


def test_c1_round_trip(c1):
    k, o, c = c1
    gs, os_ = k.scalar(c, 0.0, "FFF"), o.scalar(c, 0.0, "FFF")
    for sp in ("PPP", "FFF"):
        k.trans(gs, sp); o.trans(os_, sp)
        compare(gs, os_, 1e-12, what=f"C1 -> {sp}")


@pytest.mark.parametrize("stepper", ["febe", "abcn"])
def test_c1_100_diffusion_steps(c1, stepper):
    k, o, c = c1
    zero = np.zeros(k.dims, complex, order="F")
    g = [k.scalar(c, 0.0, "FFF"), k.scalar(c, 0.0, "FFF"), k.scalar(zero, 0.0, "FFF"), k.scalar(zero, 0.0, "FFF")]
    h = [o.scalar(c, 0.0, "FFF"), o.scalar(c, 0.0, "FFF"), o.scalar(zero, 0.0, "FFF"), o.scalar(zero, 0.0, "FFF")]
    for _ in range(100):
        if stepper == "febe":
            k.febe(g[0], g[2], DT); o.febe(h[0], h[2], DT)
        else:
            k.abcn(g[0], g[1], g[2], g[3], DT); o.abcn(h[0], h[1], h[2], h[3], DT)
    compare(g[0], h[0], 1e-11, what=f"C1 100 {stepper} steps")
    # the steps did diffuse the field: the noise's high modes decayed
    assert rel_l2(g[0].e, c) > 1e-6
    for s in g + h:
        s.free()


def test_c3_plain_vortex_steps_match_oracle():
    """Three 3-D vortex steps at 192 x 128 x 128 (the benchmark's workload) from the same state."""
    import bench
    from mlegs_gb300 import vortex
    from mlegs_gb300.kit import Kit
    from oracle.oracle import Oracle
    p = bench.workload_params()
    k = Kit(p)
    sg = vortex.VortexState(k)
    vortex.qvort_init(k, sg, q=bench.Q, uz_b=0.0, pert=bench.perturbation(p, k.dims))
    vortex.bootstrap(k, sg, bench.DT)
    o = Oracle(p)
    so = vortex.VortexState(o)
    for n in vortex.VortexState.names:
        e, ln, sp, _ = getattr(sg, n).get()
        getattr(so, n).set(e, ln, sp)
    so.gains = list(sg.gains)
    for _ in range(3):
        vortex.step(k, sg, bench.DT)
        vortex.step(o, so, bench.DT)
    for n, tol in (("psi", 1e-11), ("chi", 1e-11), ("nlpsi", 1e-11), ("nlchi", 5e-11)):
        compare(getattr(sg, n), getattr(so, n), tol, what=f"C3 3 steps {n}")
    k.close()
    o.close()


# ---- the q-vortex closed forms through the CUDA path ------------------------------------------
QV = dict(nr=96, np=64, nz=4, nrchop=96, npchop=33, nzchop=3, ell=3.0, visc=1.0e-4)
CASES = [(1.0, 1.0, 1.0), (4.0, 0.0, 0.0)]
# plain: the oracle's own bars (tests/test_oracle_known_answers.py); mixed: the precision form's
# (largest pointwise deviation relative to the largest value, which the 1/r of the velocity near the
# axis magnifies; the mixed form's FP32 FFTs put it near 1e-6 there)
TOLS = {0: dict(v=1e-12, w=2e-11, psi=1e-10, chi=5e-10, ln=1e-10, nl=1e-14),
        1: dict(v=1e-5, w=1e-5, psi=2e-6, chi=2e-6, ln=1e-8, nl=1e-9)}


@pytest.fixture(scope="module", params=[0, 1], ids=["plain", "mixed"])
def qkit(request):
    from mlegs_gb300.kit import Kit
    from mlegs_gb300.params import make_params
    k = Kit(make_params(**QV), precision=request.param)
    yield request.param, k
    k.close()


def _vmax_err(got, ref):
    scale = max(np.max(np.abs(c)) for c in ref)
    return max(np.max(np.abs(g - c)) for g, c in zip(got, ref)) / scale


@pytest.mark.parametrize("case", [0, 1], ids=["offcentre_q1", "centred_q4"])
def test_qvortex_closed_form_on_gpu(qkit, case):
    mode, k = qkit
    t = TOLS[mode]
    q, xo, yo = CASES[case]
    psi, chi = qvortex_tp(k, q, xo, yo)
    assert abs(psi.ln + 0.5) < t["ln"] and abs(chi.ln + 1 / (4 * q)) < t["ln"], (psi.ln, chi.ln)
    V, W = qvortex_closed_form(k.params, k.dims, k.kit_get("r"), q, xo, yo)
    z = np.zeros(k.dims, complex, order="F")
    v = [k.scalar(z, 0.0, "PPP") for _ in range(3)]
    k.tp2vec(psi, chi, *v)
    assert _vmax_err([s.e for s in v], V) < t["v"]
    w = [k.scalar(z, 0.0, "PPP") for _ in range(3)]
    k.tp2curlvec(psi, chi, *w)
    assert _vmax_err([s.e for s in w], W) < t["w"]
    u = [k.scalar(a, 0.0, "PPP") for a in V]
    pp, cc = k.scalar(z, 0.0, "FFF"), k.scalar(z, 0.0, "FFF")
    k.vec2tp(*u, pp, cc)
    assert rel_l2(pp.e, psi.e) < t["psi"] and rel_l2(cc.e, chi.e) < t["chi"]
    assert abs(pp.ln + 0.5) < t["ln"] and abs(cc.ln + 1 / (4 * q)) < t["ln"], (pp.ln, cc.ln)
    for s in v + w + u + [pp, cc, psi, chi]:
        s.free()


def test_axisymmetric_vortex_nonlinear_term_vanishes_on_gpu(qkit):
    mode, k = qkit
    from mlegs_gb300 import vortex
    st = vortex.VortexState(k)
    vortex.qvort_init(k, st, q=4.0)
    k.advection_rhs(st.psi, st.chi, st.nlpsi, st.nlchi, st.uz)
    scale = np.linalg.norm(st.psi.e)
    assert np.linalg.norm(st.nlpsi.e) < TOLS[mode]["nl"] * scale
    assert np.linalg.norm(st.nlchi.e) < TOLS[mode]["nl"] * scale
    st.free()
