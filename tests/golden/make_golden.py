"""Generates tests/golden/known_answers.json: the reference's own analytic known answers, evaluated
independently of the oracle (mpmath, 40+ digits), plus a 50-digit evaluation of the P_L^m table
recurrence at a sample of entries.

Sources in the reference:
  * two-mode field s_2^{1,0} = s_3^{2,0} = 1 at ELL = 1, NR = 32, NP = 48 (backward_trans.f90:69-70)
    and its closed form (docs/tutorial/transformation.md:209-223);
  * its Laplacian (docs/tutorial/operation.md:144-150);
  * Lamb-Oseen: omega(0, t) = 1/(2 pi (1 + 2 nu t)), nu = 0.1, t = 10 (time_integration.md:37-60, 265);
  * the table recurrence of leg_tbl (mlegs_spectfm_init.f90:254-300) evaluated with 50 digits as FM
    does (fm_parallel.f90:60), with log_fact and lognorm in FP64 as the reference computes them;
  * the q-vortex V = (1 - exp(-r'^2))/r' e_phi' + exp(-r'^2)/q e_z about a centre (xo, yo)
    (docs/tutorial/vector_field.md:88-106): its cylindrical components and those of its curl
    (2 exp(-r'^2) e_z plus the curl of the axial jet) at a sample of the collocation points, and the
    log coefficients of psi and chi that its circulation and axial flux fix, -1/2 and -1/(4q) (the
    recipe builds psi and chi from the closed-form vorticity and axial flow,
    src/apps/vecfld_reconstruction.f90:155-215, and tp_project.f90 projects V back to them).
Run: python tests/golden/make_golden.py
"""
import ctypes
import ctypes.util
import json
import math
import os

import mpmath as mp

mp.mp.dps = 60
HERE = os.path.dirname(os.path.abspath(__file__))


def gauss_legendre_nodes(n):
    """Roots of P_n in increasing order, by Newton iteration in 60 digits."""
    xs = []
    for i in range(1, (n + 1) // 2 + 1):
        z = mp.cos(mp.pi * (i - mp.mpf(1) / 4) / (n + mp.mpf(1) / 2))
        for _ in range(100):
            p1, p2 = mp.mpf(1), mp.mpf(0)
            for j in range(1, n + 1):
                p3 = p2
                p2 = p1
                p1 = ((2 * j - 1) * z * p2 - (j - 1) * p3) / j
            pp = n * (z * p1 - p2) / (z * z - 1)
            dz = p1 / pp
            z = z - dz
            if abs(dz) < mp.mpf(10) ** -55:
                break
        xs.append(z)
    lo = [-z for z in xs]
    hi = list(reversed(xs))
    if n % 2:
        hi = hi[1:]
    return sorted(lo + hi)


def gauss_legendre_fp64(n):
    """The reference's own FP64 Newton iteration (mlegs_spectfm_init.f90:181-214) in Python floats,
    which round every operation like the Fortran (no fused multiply-add)."""
    x = [0.0] * n
    m = math.ceil((n + 1) / 2.0)
    for i in range(1, m + 1):
        z = math.cos(math.pi * (i - .25) / (n + .5))
        z1 = z + 1.0
        while abs(z - z1) > 1.0e-15:
            p1, p2 = 1.0, 0.0
            for j in range(1, n + 1):
                p3 = p2
                p2 = p1
                p1 = ((2 * j - 1) * z * p2 - (j - 1) * p3) / j
            pp = n * (z * p1 - p2) / (z * z - 1)
            z1 = z
            z = z1 - p1 / pp
        x[i - 1] = -z
        x[n - i] = z
    return x


def two_mode(r, ph):
    return 2 * (mp.sqrt(mp.mpf(5) / 12) * (-6 * r * (r ** 2 - 1) / (r ** 2 + 1) ** 2) * mp.cos(ph)
                + mp.sqrt(mp.mpf(7) / 240) * (60 * r ** 2 * (r ** 2 - 1) / (r ** 2 + 1) ** 3) * mp.cos(2 * ph))


def two_mode_lap(r, ph):
    return (48 * mp.sqrt(15) * r * (r ** 2 - 1) * ((r ** 2 + 1) * mp.cos(ph) - 2 * mp.sqrt(7) * r * mp.cos(2 * ph))
            / (r ** 2 + 1) ** 5)


def lognorm_fp64(ndim, m):
    """leg_lognorm (mlegs_spectfm_init.f90:218-250) in FP64, column m."""
    wk = [math.log(.5)]
    for mm in range(1, m + 1):
        wk.append(wk[-1] + math.log(2.0 * mm + 1.0) - math.log(2.0 * mm * (2.0 * mm - 1.0) ** 2))
    l = [wk[m]]
    for nn in range(2, ndim + 1):
        n = m + nn - 1
        l.append(l[-1] + math.log(2.0 * n + 1.0) - math.log(2.0 * n - 1.0) + math.log(1.0 * (n - m)) - math.log(1.0 * (n + m)))
    return [.5 * v for v in l]


# the reference's log_gamma is gfortran's intrinsic, i.e. the C library's lgamma; CPython's
# math.lgamma is a separate implementation whose last bits differ, and exp(log_fact + lognorm)
# carries those bits into the table (about 1e-14 relative at n ~ 20)
_libm = ctypes.CDLL(ctypes.util.find_library("m") or "libm.so.6")
_libm.lgamma.restype = ctypes.c_double
_libm.lgamma.argtypes = [ctypes.c_double]


def log_fact(n):
    """log_fact (mlegs_spectfm_init.f90:351-357) with the C library's lgamma."""
    return _libm.lgamma(2 * n + 1.0) - n * math.log(2.0) - _libm.lgamma(n + 1.0)


def table_entries(x, m, ne, lnrm):
    """leg_tbl recurrence for one x and m with 50 digits (FM's precision)."""
    with mp.workdps(50):
        xq = mp.mpf(x)
        f = [(-1) ** m * mp.sqrt(1 - xq * xq) ** m]
        f.append(xq * f[0])
        for nn in range(3, ne + 1):
            n = m + nn - 1
            f.append(mp.mpf(1) / (n - m) * (f[nn - 2] * xq - f[nn - 3] * (n + m - 1) / (2 * n - 1) / (2 * n - 3)))
        out = []
        for nn in range(1, ne + 1):
            n = m + nn - 1
            out.append(float(f[nn - 1] * mp.exp(mp.mpf(log_fact(n)) + mp.mpf(lnrm[nn - 1]))))
    return out


def qvortex(r, ph, q, xo, yo):
    """(V_r, V_phi, V_z) and (W_r, W_phi, W_z) = curl V of the q-vortex about (xo, yo) at (r, phi)."""
    x, y = r * mp.cos(ph), r * mp.sin(ph)
    dx, dy = x - xo, y - yo
    rp2 = dx * dx + dy * dy
    g = -mp.expm1(-rp2) / rp2 if rp2 != 0 else mp.mpf(1)     # (1 - exp(-r'^2)) / r'^2
    vx, vy, vz = -dy * g, dx * g, mp.exp(-rp2) / q
    wx, wy, wz = -2 * dy * vz, 2 * dx * vz, 2 * mp.exp(-rp2)
    c, s = mp.cos(ph), mp.sin(ph)
    return ((vx * c + vy * s, -vx * s + vy * c, vz), (wx * c + wy * s, -wx * s + wy * c, wz))


def qvortex_samples(nr, np_, ell, q, xo, yo):
    """The closed form at every 5th radial node and every 7th azimuthal sample of an (nr, np_) kit whose
    nodes are the reference's FP64 Newton roots, r_i = ell sqrt((1 + x_i)/(1 - x_i))."""
    xref = gauss_legendre_fp64(nr)
    out = []
    for i in range(0, nr, 5):
        xi = mp.mpf(xref[i])
        r = ell * mp.sqrt((1 + xi) / (1 - xi))
        for j in range(0, np_, 7):
            ph = 2 * mp.pi / np_ * j
            v, w = qvortex(r, ph, q, xo, yo)
            out.append({"i": i, "j": j, "v": [float(a) for a in v], "w": [float(a) for a in w]})
    return out


def main():
    NR, NP, ELL = 32, 48, 1
    xs = gauss_legendre_nodes(NR)
    r = [ELL * mp.sqrt((1 + x) / (1 - x)) for x in xs]
    phi = [2 * mp.pi / NP * j for j in range(NP)]
    s_re = [[float(two_mode(ri, phi[2 * j])) for j in range(NP // 2)] for ri in r]
    s_im = [[float(two_mode(ri, phi[2 * j + 1])) for j in range(NP // 2)] for ri in r]
    l_re = [[float(two_mode_lap(ri, phi[2 * j])) for j in range(NP // 2)] for ri in r]
    l_im = [[float(two_mode_lap(ri, phi[2 * j + 1])) for j in range(NP // 2)] for ri in r]
    # table samples at the reference's FP64 nodes of an NR = 32 kit, npchop = 17, nrchop = 32 (ne = 46)
    x64 = [float(x) for x in xs]
    xref = gauss_legendre_fp64(NR)
    samples = []
    ne = 32 + 14
    for m in (0, 1, 5, 16):
        lnrm = lognorm_fp64(ne, m)
        for xi in (0, 3, 9, 15):
            vals = table_entries(xref[xi], m, ne, lnrm)
            for nn in (1, 2, 7, 20, 33, 46):
                samples.append({"i": xi, "nn": nn, "m": m, "value": vals[nn - 1]})
    data = {
        "two_mode": {"nr": NR, "np": NP, "ell": ELL, "x": x64, "r": [float(v) for v in r],
                     "s_re": s_re, "s_im": s_im, "lap_re": l_re, "lap_im": l_im},
        "lamb_oseen": {"nu": 0.1, "t": 10.0, "omega0": float(1 / (2 * mp.pi * (1 + 2 * mp.mpf("0.1") * 10)))},
        "table": {"nr": 32, "nrchop": 32, "npchop": 17, "ell": 4.0, "x_fp64_newton": xref, "samples": samples},
        # the tutorial's off-centre vortex (centre (1, 1), q = 1) and the centred Batchelor vortex of the 3-D
        # app (q = 4), on a kit that resolves both to round-off
        "qvortex": {"nr": 96, "np": 64, "nz": 4, "ell": 3.0,
                    "cases": [{"q": q, "xo": xo, "yo": yo, "ln_psi": -0.5, "ln_chi": float(-1 / (4 * mp.mpf(q))),
                               "samples": qvortex_samples(96, 64, 3.0, q, xo, yo)}
                              for q, xo, yo in ((1.0, 1.0, 1.0), (4.0, 0.0, 0.0))]},
    }
    with open(os.path.join(HERE, "known_answers.json"), "w") as f:
        json.dump(data, f)
    print("wrote", os.path.join(HERE, "known_answers.json"))


if __name__ == "__main__":
    main()
