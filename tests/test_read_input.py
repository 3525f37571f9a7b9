"""read_input (mlegs_misc_io.f90:307-388) through the C ABI: the reference's input-file layout (a comment
line before each group of values, Fortran D exponents, T/F logicals, the optional SVV section) and its
validation messages.  Host-only: runs without a GPU."""
import math
import os

import pytest

from mlegs_gb300.kit import MlgError
from mlegs_gb300.params import read_input

LAYOUT = """!!! COMPUTATIONAL DOMAIN INFO !!!
# ---------- NR ----------- NP ----------- NZ ---
            {nr}            {np}            {nz}
# ------ NRCHOP ------- NPCHOP ------- NZCHOP ---
            {nrchop}             {npchop}             {nzchop}
# --------- ELL --------- ZLEN ------ ZLENxPI ---
           3.D0           {zlen}              {xpi}
#
!!! TIME STEPPING INFO !!!
# ---------- DT ----------- TI --------- TOTT ----------- NI --------- TOTN ---
          2.5D-3           0.D0           4.D1              7           1600
#
!!! FIELD PROPERTY INFO !!!
# -------- VISC ----- HYPERPOW ---- HYPERVISC ---
          {visc}              {hp}          {hv}
#
!!! FIELD SAVE INFO !!!
# --------------------- FLDDIR ---
                  {fld}
# ---- ISFLDSAV -- FLDSAVINTVL ---
              T            250
#
!!! DATA LOGGING INFO !!!
# --------------------- LOGDIR ---
                  {log}
# ---- ISLOGSAV -- LOGSAVINTVL ---
              F              3
"""
SVV = """!!! STABILITY CONTROL INFO (OPTIONAL) !!!
# ------- IS_SVV ------- CUTOFF ------- TARGET ------ STRENGTH ------- RELAX ---
              {svv}          {cut}          3.D-2          0.2          0.5
/* ------------------------------ END OF INPUT ------------------------------ */
"""


def write(tmp_path, svv=True, **kw):
    v = dict(nr=64, np=32, nz=16, nrchop=64, npchop=17, nzchop=9, zlen="2.D0", xpi="T", visc="1.D-4", hp=0,
             hv="0.D0", fld=str(tmp_path / "fld"), log=str(tmp_path / "log" / "a"), svv="F", cut="0.6")
    v.update(kw)
    txt = LAYOUT.format(**v) + (SVV.format(**v) if svv else "")
    fn = tmp_path / "input.params"
    fn.write_text(txt)
    return str(fn)


def test_reads_every_value(tmp_path):
    p, run = read_input(write(tmp_path))
    assert (p.nr, p.np, p.nz, p.nrchop, p.npchop, p.nzchop) == (64, 32, 16, 64, 17, 9)
    assert p.ell == 3.0 and p.zlen == pytest.approx(2.0 * math.pi, rel=1e-15)
    assert p.visc == 1e-4 and p.hyperpow == 0 and p.hypervisc == 0.0
    assert (run["dt"], run["ti"], run["totaltime"], run["ni"], run["totaln"]) == (2.5e-3, 0.0, 40.0, 7, 1600)
    assert run["isfldsav"] == 1 and run["fldsavintvl"] == 250
    assert run["islogsav"] == 0 and run["logsavintvl"] == 3
    assert run["flddir"] == str(tmp_path / "fld") + "/" and run["logdir"] == str(tmp_path / "log" / "a") + "/"
    assert p.is_svv == 0 and p.svv_cutoff == 0.6 and p.svv_target == 3e-2 and p.svv_strength == 0.2
    assert p.svv_relax == 0.5
    assert not os.path.exists(run["flddir"])   # created only when asked


def test_zlen_without_pi_and_older_files_keep_svv_defaults(tmp_path):
    p, _ = read_input(write(tmp_path, svv=False, xpi="F", zlen="6.D0"))
    assert p.zlen == 6.0
    assert (p.is_svv, p.svv_cutoff, p.svv_target, p.svv_strength, p.svv_relax) == (1, 0.75, 2e-2, 0.12, 0.25)


def test_make_dirs(tmp_path):
    _, run = read_input(write(tmp_path), make_dirs=True)
    assert os.path.isdir(run["flddir"]) and os.path.isdir(run["logdir"])


@pytest.mark.parametrize("kw,msg", [
    (dict(nr=63), "nr must be positive and even"),
    (dict(nrchop=65), "invalid chopping sizes"),
    (dict(npchop=18), "invalid chopping sizes"),
    (dict(hp=3, hv="1.D-6"), "hyperpow must be zero, 4, 6, or 8"),
    (dict(hp=4, hv="0.D0"), "hypervisc must be positive when enabled"),
    (dict(visc="-1.D-4"), "viscosities must be non-negative"),
    (dict(cut="1.0"), "invalid SVV controls"),
    (dict(fld="out put"), "invalid field output directory"),
])
def test_rejects_as_the_reference(tmp_path, kw, msg):
    with pytest.raises(MlgError) as e:
        read_input(write(tmp_path, **kw))
    assert msg in str(e.value)


def test_missing_file(tmp_path):
    with pytest.raises(MlgError) as e:
        read_input(str(tmp_path / "none.params"))
    assert "could not open input file" in str(e.value)
