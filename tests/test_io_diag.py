"""Field I/O (msave / mload, mlegs_scalar_io.f90:6-249) and the diagnostics (fftreat, save_vort_mag's
field, the kinetic-energy spectrum) on the GPU.

The binary files are compared byte for byte with the layout of the reference's stream-access writes,
assembled here with struct; the formatted files are checked line by line against the reference's edit
descriptors ('(3(1X,I10))' and '1PE24.15E3'), and a file in the reference's formatted layout with
list-directed tail lines written by hand is read back.  fftreat is held to the oracle; the vorticity
magnitude to numpy on the oracle's curl; the spectrum to numpy FFTs of the FP64 velocity."""
import struct

import numpy as np
import pytest

from mlegs_gb300 import fields
from mlegs_gb300.kit import MlgError
from helpers import params, compare, rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", params=["c1", "hyp"])
def pair(request):
    from mlegs_gb300.kit import Kit
    from oracle.oracle import Oracle
    p = params(request.param)
    o = Oracle(p)
    k = Kit(p)
    yield request.param, k, o
    k.close()
    o.close()


def field(k, seed, ln=0.3, offs=(0, 0, 0), space="FFF"):
    e = fields.spectral_noise(k.params, k.dims, seed, amp=1.0, decay=0.05)
    s = k.scalar(e, ln, space)
    if any(offs):
        s.chop_offset(*offs)
    return s, e


def test_msave_binary_is_the_reference_layout(pair, tmp_path):
    name, k, o = pair
    s, e = field(k, 301, ln=-0.25, offs=(2, 1, 0))
    for is_global in (True, False):
        fn = tmp_path / f"b_{int(is_global)}"
        k.msave(s, str(fn), is_binary=True, is_global=is_global)
        d = k.dims
        hdr = struct.pack("<3i", *d) if is_global else struct.pack("<9i", *d, *d, 0, 0, 0)
        want = hdr + np.asfortranarray(e).tobytes(order="F") + struct.pack("<d3i", -0.25, 2, 1, 0) + b"FFF"
        got = (tmp_path / (fn.name if is_global else fn.name + "_0")).read_bytes()
        assert got == want, f"{name} binary msave (global={is_global})"
        t = k.scalar()
        k.mload(t, str(fn), is_binary=True, is_global=is_global)
        te, tln, tsp, toff = t.get()
        assert np.array_equal(te, e) and tln == -0.25 and tsp == "FFF" and tuple(toff) == (2, 1, 0)


def test_msave_formatted_layout_and_round_trip(pair, tmp_path):
    name, k, o = pair
    s, e = field(k, 302, ln=0.125, offs=(3, 0, 0), space="FFF")
    fn = tmp_path / "f"
    k.msave(s, str(fn))
    lines = fn.read_text().split("\n")
    n1, n2, n3 = k.dims
    assert lines[0] == "".join(f" {v:10d}" for v in (n1, n2, n3))
    body = lines[1:1 + n3 * n1 + (n3 - 1)]
    rows = [ln for ln in body if ln.strip()]
    assert len(rows) == n1 * n3 and all(len(ln) == 48 * n2 for ln in rows)
    assert sum(1 for ln in body if not ln.strip()) == n3 - 1
    # each value: '1PE24.15E3' -- one leading digit, 15 after the point, a signed 3-digit exponent
    for tok in rows[0].split():
        mant, ex = tok.split("E")
        assert len(mant.lstrip("-").split(".")[1]) == 15 and len(ex) == 4 and ex[0] in "+-"
    vals = np.array([float(v) for ln in rows for v in ln.split()])
    ref = np.stack([e.real, e.imag], axis=-1).transpose(2, 0, 1, 3).reshape(-1)   # (k, i, j, re/im)
    assert np.max(np.abs(vals - ref)) <= 1e-15 * np.max(np.abs(ref)) * 10
    t = k.scalar()
    k.mload(t, str(fn))
    te, tln, tsp, toff = t.get()
    assert rel_l2(te, e) < 1e-15 and tln == 0.125 and tsp == "FFF" and tuple(toff) == (3, 0, 0)


def test_mload_reads_the_reference_formatted_tail(pair, tmp_path):
    name, k, o = pair
    n1, n2, n3 = k.dims
    rng = np.random.default_rng(7)
    a = rng.standard_normal((n1, n2, n3)) + 1j * rng.standard_normal((n1, n2, n3))
    out = ["".join(f" {v:10d}" for v in (n1, n2, n3)) + " "]
    for kk in range(n3):
        for i in range(n1):
            out.append("".join(f"{x:24.15E}" for j in range(n2) for x in (a[i, j, kk].real, a[i, j, kk].imag)) + " ")
        if kk + 1 < n3:
            out.append(" ")
    out.append("   0.50000000000000000                1           0           0")   # list-directed
    out.append(" PPP")
    fn = tmp_path / "ref_layout"
    fn.write_text("\n".join(out) + "\n")
    t = k.scalar()
    k.mload(t, str(fn))
    te, tln, tsp, toff = t.get()
    assert rel_l2(te, a) < 1e-15 and tln == 0.5 and tsp == "PPP" and tuple(toff) == (1, 0, 0)


def test_mload_rejects_a_size_mismatch(pair, tmp_path):
    name, k, o = pair
    n1, n2, n3 = k.dims
    fn = tmp_path / "bad"
    fn.write_bytes(struct.pack("<3i", n1 + 1, n2, n3) + bytes(16 * (n1 + 1) * n2 * n3 + 23))
    with pytest.raises(MlgError) as ex:
        k.mload(k.scalar(), str(fn), is_binary=True)
    assert "size inconsistency" in str(ex.value)


def test_fftreat_matches_oracle(pair):
    name, k, o = pair
    e = fields.spectral_noise(k.params, k.dims, 303, amp=1.0, decay=0.05)
    for ln in (0.0, 0.4):
        g, r = k.scalar(e, ln, "FFF"), o.scalar(e, ln, "FFF")
        k.fftreat(g); o.fftreat(r)
        compare(g, r, 1e-11, what=f"{name} fftreat ln={ln}")


def test_vort_mag_matches_the_oracle_curl(pair):
    name, k, o = pair
    p = k.params
    psi = fields.spectral_noise(p, k.dims, 304, amp=1.0, decay=0.3)
    chi = fields.spectral_noise(p, k.dims, 305, amp=1.0, decay=0.3)
    out = k.scalar(np.zeros(k.dims, complex, order="F"), 0.0, "PPP")
    k.vort_mag(k.scalar(psi, 0.0, "FFF"), k.scalar(chi, 0.0, "FFF"), out)
    w = [o.scalar() for _ in range(3)]
    o.tp2curlvec(o.scalar(psi, 0.0, "FFF"), o.scalar(chi, 0.0, "FFF"), *w)
    we = [x.get()[0] for x in w]
    want = np.sqrt(sum(x.real ** 2 for x in we)) + 1j * np.sqrt(sum(x.imag ** 2 for x in we))
    ge, gln, gsp, _ = out.get()
    assert gsp == "PPP" and gln == 0.0
    assert rel_l2(ge, want) < 1e-12, f"{name} vort_mag"


def test_ke_spectrum_matches_numpy(pair):
    name, k, o = pair
    p = k.params
    psi = fields.spectral_noise(p, k.dims, 306, amp=1.0, decay=0.3)
    chi = fields.spectral_noise(p, k.dims, 307, amp=1.0, decay=0.3)
    E = k.ke_spectrum(k.scalar(psi, 0.0, "FFF"), k.scalar(chi, 0.0, "FFF"))
    x, w, r = k.kit_get("x"), k.kit_get("w"), k.kit_get("r")
    nr = len(x)
    v = [k.scalar(np.zeros(k.dims, complex, order="F"), 0.0, "PPP") for _ in range(3)]
    k.tp2vec(k.scalar(psi, 0.0, "FFF"), k.scalar(chi, 0.0, "FFF"), *v)
    W = w * r ** 2 / (1.0 - x ** 2) * 2.0 * np.pi * p.zlen
    want = 0.0
    for s in v:
        e = s.get()[0][:nr, : p.np // 2, :]
        f = np.empty((nr, p.np, k.dims[2]))
        f[:, 0::2, :] = e.real
        f[:, 1::2, :] = e.imag
        F = np.fft.fft(np.fft.rfft(f, axis=1) / p.np, axis=2) / k.dims[2]
        cm = np.full(F.shape[1], 2.0)
        cm[0] = 1.0
        if p.np % 2 == 0:
            cm[-1] = 1.0
        want = want + 0.5 * np.einsum("i,imk->mk", W, np.abs(F) ** 2) * cm[:, None]
    assert E.shape == want.shape
    assert np.max(np.abs(E - want)) <= 1e-12 * np.max(want), f"{name} ke spectrum"
