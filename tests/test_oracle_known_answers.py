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
