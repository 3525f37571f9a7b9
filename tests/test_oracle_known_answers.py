"""The oracle (CPU restatement) pinned against the reference's analytic known answers and a 50-digit
evaluation of the P_L^m table (tests/golden/known_answers.json, made by tests/golden/make_golden.py).
CPU only."""
import json
import math
import os

import numpy as np
import pytest

from oracle.oracle import Oracle, OracleError

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "known_answers.json")))


@pytest.fixture(scope="module")
def tut():
    g = GOLD["two_mode"]
    o = Oracle(nr=g["nr"], np=g["np"], nz=1, nrchop=32, npchop=25, nzchop=1, ell=float(g["ell"]), zlen=1.0,
               visc=0.1)
    yield o
    o.close()


def two_mode_field(o):
    e = np.zeros(o.dims, complex, order="F")
    e[1, 1, 0] = 1.0   # s_2^{1,0} (backward_trans.f90:69)
    e[1, 2, 0] = 1.0   # s_3^{2,0} (backward_trans.f90:70)
    return e


def test_nodes_match_50_digit_roots(tut):
    x = tut.kit_get("x")
    g = np.array(GOLD["two_mode"]["x"])
    # the reference's FP64 Newton nodes: bit-identical to its restatement, within 2 ulp of the roots
    assert np.array_equal(x, np.array(GOLD["table"]["x_fp64_newton"]))
    assert np.max(np.abs(x - g)) <= 2.3e-16


def test_backward_two_mode_closed_form(tut):
    g = GOLD["two_mode"]
    s = tut.scalar(two_mode_field(tut), 0.0, "FFF")
    tut.trans(s, "PPP")
    e = s.e
    nph = g["np"] // 2
    ref = np.array(g["s_re"]) + 1j * np.array(g["s_im"])
    err = np.max(np.abs(e[: g["nr"], :nph, 0] - ref)) / np.max(np.abs(ref))
    assert err < 1e-14, err


def test_forward_recovers_two_unit_coefficients(tut):
    s = tut.scalar(two_mode_field(tut), 0.0, "FFF")
    tut.trans(s, "PPP")
    tut.trans(s, "FFF")
    e = s.e
    ref = two_mode_field(tut)
    assert np.max(np.abs(e - ref)) < 1e-14


def test_laplacian_closed_form(tut):
    g = GOLD["two_mode"]
    s = tut.scalar(two_mode_field(tut), 0.0, "FFF")
    tut.del2(s)
    tut.trans(s, "PPP")
    e = s.e
    nph = g["np"] // 2
    ref = np.array(g["lap_re"]) + 1j * np.array(g["lap_im"])
    err = np.max(np.abs(e[: g["nr"], :nph, 0] - ref)) / np.max(np.abs(ref))
    assert err < 1e-13, err


def test_table_against_50_digit_recurrence():
    t = GOLD["table"]
    o = Oracle(nr=t["nr"], np=32, nz=32, nrchop=t["nrchop"], npchop=t["npchop"], nzchop=17, ell=t["ell"])
    pf = o.kit_get("pf")
    for smp in t["samples"]:
        v = pf[smp["i"], smp["nn"] - 1, smp["m"]]
        ref = smp["value"]
        # binary128 against 50 digits, both rounded to FP64: at most one rounding apart
        assert abs(v - ref) <= 1.2e-16 * max(abs(ref), 1e-300) + 1e-300, (smp, v)
    o.close()


def lamb_oseen_origin(o, dt, scheme, tfinal=10.0):
    """time_integration_first/second (src/apps): w0 = exp(-r^2/2)/(2 pi) in PPP, nonlinear term 0."""
    p = o.params
    r = o.kit_get("r")
    e = np.zeros(o.dims, complex, order="F")
    v = np.exp(-r ** 2 / 2.0) / (2 * np.pi)
    e[: p.nr, : p.np // 2, 0] = (v + 1j * v)[:, None]
    w = o.scalar(e, 0.0, "PPP")
    nl = o.scalar(np.zeros(o.dims, complex, order="F"), 0.0, "FFF")
    o.trans(w, "FFF")
    n = int(round(tfinal / dt))
    if scheme == "febe":
        for _ in range(n):
            o.febe(w, nl, dt)
    else:
        # Richardson start (time_integration_second.f90:92-121), then abcn
        wp = o.scalar(); wp.copy_from(w)
        nlp = o.scalar(); nlp.copy_from(nl)
        wr = o.scalar(); wr.copy_from(w)
        o.febe(wr, nl, dt)
        for _ in range(2):
            o.febe(w, nl, dt / 2)
        o.axpby(w, 2.0, w, -1.0, wr)
        for _ in range(n - 1):
            o.abcn(w, wp, nl, nlp, dt)
    return o.calcat0(w)[0].real


def test_lamb_oseen_decay_and_order():
    o = Oracle(nr=32, np=48, nz=1, nrchop=32, npchop=25, nzchop=1, ell=1.0, zlen=1.0, visc=0.1)
    exact = GOLD["lamb_oseen"]["omega0"]
    assert abs(exact - 1.0 / (6 * math.pi)) < 1e-15
    e1 = {dt: abs(lamb_oseen_origin(o, dt, "febe") - exact) for dt in (0.2, 0.4)}
    e2 = {dt: abs(lamb_oseen_origin(o, dt, "abcn") - exact) for dt in (0.2, 0.4)}
    # first order in dt for febe, second order for abcn (time_integration.md:268, 487)
    assert 1.7 < e1[0.4] / e1[0.2] < 2.3, e1
    assert 3.2 < e2[0.4] / e2[0.2] < 4.8, e2
    assert e2[0.2] < e1[0.2] and e1[0.2] < 2e-3
    o.close()


def test_invalid_inputs_are_rejected():
    # tools/validate_tutorials.py:438-471: invalid parameters must fail
    from mlegs_gb300.params import make_params
    from oracle.oracle import lib
    import ctypes
    for kw in (dict(nr=31), dict(np=14), dict(nz=22), dict(nrchop=40, nr=32), dict(npchop=70, np=128)):
        p = make_params(**kw)
        lib().orc_finalize()
        assert lib().orc_init(ctypes.byref(p)) == 1
    o = Oracle(nr=16, np=8, nz=8, nrchop=16, npchop=5, nzchop=5)
    s = o.scalar(np.zeros(o.dims, complex, order="F"), 0.0, "FFF")
    with pytest.raises(OracleError):
        o.ihelm(s, 0.0)
    o.close()


# ---- the q-vortex closed forms (docs/tutorial/vector_field.md:88-106) -----------------------------
QV = GOLD["qvortex"]


@pytest.fixture(scope="module")
def qkit():
    o = Oracle(nr=QV["nr"], np=QV["np"], nz=QV["nz"], nrchop=QV["nr"], npchop=QV["np"] // 2 + 1,
               nzchop=QV["nz"] // 2 + 1, ell=QV["ell"], visc=1.0e-4)
    yield o
    o.close()


def _zeros(o, space):
    return o.scalar(np.zeros(o.dims, complex, order="F"), 0.0, space)


def _vmax_err(got, ref):
    """Largest deviation over the three components, relative to the largest component value."""
    scale = max(np.max(np.abs(c)) for c in ref)
    return max(np.max(np.abs(g - c)) for g, c in zip(got, ref)) / scale


@pytest.mark.parametrize("case", [0, 1], ids=["offcentre_q1", "centred_q4"])
def test_qvortex_closed_form_samples(qkit, case):
    """The numpy closed form used below agrees with the 60-digit samples of the golden file."""
    from helpers import qvortex_closed_form
    c = QV["cases"][case]
    V, W = qvortex_closed_form(qkit.params, qkit.dims, qkit.kit_get("r"), c["q"], c["xo"], c["yo"])
    for smp in c["samples"]:
        i, j = smp["i"], smp["j"]
        for ref, fld in ((smp["v"], V), (smp["w"], W)):
            for comp in range(3):
                z = fld[comp][i, j // 2, 0]
                got = z.real if j % 2 == 0 else z.imag
                assert abs(got - ref[comp]) <= 4e-15 * max(1.0, abs(ref[comp])), (i, j, comp, got, ref[comp])


@pytest.mark.parametrize("case", [0, 1], ids=["offcentre_q1", "centred_q4"])
def test_qvortex_tp2vec_and_curl_closed_form(qkit, case):
    """tp2vec and tp2curlvec (mlegs_scalar_ops.f90:1455-1560) of the recipe's psi and chi reproduce the
    closed-form V and curl V, and the recipe's log coefficients are the closed-form -1/2, -1/(4q)."""
    from helpers import qvortex_closed_form, qvortex_tp
    c = QV["cases"][case]
    psi, chi = qvortex_tp(qkit, c["q"], c["xo"], c["yo"])
    assert abs(psi.ln - c["ln_psi"]) < 1e-12 and abs(chi.ln - c["ln_chi"]) < 1e-12, (psi.ln, chi.ln)
    V, W = qvortex_closed_form(qkit.params, qkit.dims, qkit.kit_get("r"), c["q"], c["xo"], c["yo"])
    v = [_zeros(qkit, "PPP") for _ in range(3)]
    qkit.tp2vec(psi, chi, *v)
    assert _vmax_err([s.e for s in v], V) < 1e-12
    w = [_zeros(qkit, "PPP") for _ in range(3)]
    qkit.tp2curlvec(psi, chi, *w)
    assert _vmax_err([s.e for s in w], W) < 2e-11


@pytest.mark.parametrize("case", [0, 1], ids=["offcentre_q1", "centred_q4"])
def test_qvortex_vec2tp_recovers_psi_chi(qkit, case):
    """vec2tp (mlegs_scalar_ops.f90:1308-1453) of the closed-form V returns the recipe's psi and chi
    (what src/apps/tp_project.f90 does with the vectors that vecfld_reconstruction.f90 saves)."""
    from helpers import qvortex_closed_form, qvortex_tp
    c = QV["cases"][case]
    psi, chi = qvortex_tp(qkit, c["q"], c["xo"], c["yo"])
    V, _ = qvortex_closed_form(qkit.params, qkit.dims, qkit.kit_get("r"), c["q"], c["xo"], c["yo"])
    u = [qkit.scalar(a, 0.0, "PPP") for a in V]
    pp, cc = _zeros(qkit, "FFF"), _zeros(qkit, "FFF")
    qkit.vec2tp(*u, pp, cc)
    # the projection ends with an inverse Laplacian on chi: its truncation error at this resolution is
    # about 1e-11 absolute, 1.3e-10 of the q = 4 vortex's smaller chi
    assert np.linalg.norm(pp.e - psi.e) / np.linalg.norm(psi.e) < 1e-10
    assert np.linalg.norm(cc.e - chi.e) / np.linalg.norm(chi.e) < 5e-10
    assert abs(pp.ln - c["ln_psi"]) < 1e-10 and abs(cc.ln - c["ln_chi"]) < 1e-10, (pp.ln, cc.ln)


def test_qvortex_vecprod_closed_form(qkit):
    """vector_product (mlegs_scalar_ops.f90:1264-1306) of the closed-form V and curl V is V x curl V
    sample by sample."""
    from helpers import qvortex_closed_form
    c = QV["cases"][0]
    V, W = qvortex_closed_form(qkit.params, qkit.dims, qkit.kit_get("r"), c["q"], c["xo"], c["yo"])
    v = [qkit.scalar(a, 0.0, "PPP") for a in V]
    w = [qkit.scalar(a, 0.0, "PPP") for a in W]
    qkit.vecprod(*v, *w)

    def cross(a, b):   # on the packed samples: real and imaginary parts are separate samples
        out = []
        for i, j, k in ((1, 2, 0), (2, 0, 1), (0, 1, 2)):
            re = a[i].real * b[j].real - a[j].real * b[i].real
            im = a[i].imag * b[j].imag - a[j].imag * b[i].imag
            out.append(re + 1j * im)
        return out
    ref = cross(V, W)
    assert _vmax_err([s.e for s in v], ref) < 1e-15


def test_axisymmetric_vortex_has_no_nonlinear_term(qkit):
    """For the centred Batchelor vortex u x omega is radial and depends on r only, a pure gradient: its
    curl, and with it the TP projection that advection_rhs (vortical_flow_3d.f90:353-395) returns,
    vanish.  The step's nonlinear term must come out at round-off of the vortex's own size."""
    from mlegs_gb300 import vortex
    c = QV["cases"][1]
    st = vortex.VortexState(qkit)
    vortex.qvort_init(qkit, st, q=c["q"])
    qkit.advection_rhs(st.psi, st.chi, st.nlpsi, st.nlchi, st.uz)
    scale = np.linalg.norm(st.psi.e)
    assert np.linalg.norm(st.nlpsi.e) < 1e-14 * scale and np.linalg.norm(st.nlchi.e) < 1e-14 * scale
    assert st.nlpsi.ln == 0.0 and st.nlchi.ln == 0.0
