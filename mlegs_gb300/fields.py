"""Seeded synthetic fields and initial conditions (host side, numpy).

The same bytes are handed to the GPU library and to the CPU oracle, so a comparison between them
measures the implementations and not the inputs.

* `qvort_ppp` restates the initial-condition recipe of the reference's 3-D vortex app
  (src/apps/vortical_flow_3d.f90:258-326): in PPP space, psi-source = -exp(-rr^2)*2/(1-x)^2 and
  chi-source = -exp(-rr^2)/q/(1-x)^2 summed over the vortex centres, later mapped to (psi, chi) by
  trans -> idelsqp -> zeroat1.  The reference's gfortran `rand()` noise (which reseeds on every call,
  :467-487) is replaced by a seeded spectral perturbation (`spectral_noise`).
* `spectral_noise` draws complex coefficients with a uniform phase and magnitude
  amp*exp(-decay*(n+|m|+|k|)) on the active (chopped) coefficients, made Hermitian in k on the m=0
  and m=np/2 planes so that the physical field is real.
"""
import numpy as np


def _kz(nz):
    k = np.arange(nz)
    return np.where(k <= nz // 2, k, k - nz)   # slot -> signed wavenumber index (mlegs_spectfm_init.f90:133-134)


def active_mask(p, dims, offset=0):
    """Boolean mask of the coefficients kept by chop (mlegs_scalar_ops.f90:6-41)."""
    nrdim, npdim, nzdim = dims
    nrc = p.nrchop + offset
    n = np.arange(nrdim)[:, None, None]
    m = np.arange(npdim)[None, :, None]
    kk = np.arange(1, nzdim + 1)[None, None, :]
    nrcs = np.where(m < p.npchop, np.maximum(np.minimum(nrc, nrc - m), 0), 0)
    chopzl, chopzu = p.nzchop, p.nz - p.nzchop + 2
    kmask = ~((chopzl < chopzu) & (kk >= chopzl + 1) & (kk <= chopzu - 1))
    return (n < nrcs) & (m < p.npchop) & kmask


def hermitian_fix(e, p):
    """Make the m = 0 (and m = np/2) planes Hermitian in k: c(n,0,-k) = conj c(n,0,k)."""
    nz = e.shape[2]
    planes = [0] + ([e.shape[1] - 1] if p.np > 1 and e.shape[1] > 1 else [])
    for mm in planes:
        sl = e[:, mm, :]
        ref = sl.copy()
        for k in range(nz):
            kn = (-k) % nz
            if k == kn:
                sl[:, k] = ref[:, k].real
            elif k < kn:
                sl[:, kn] = np.conj(ref[:, k])
        e[:, mm, :] = sl
    return e


def spectral_noise(p, dims, seed, amp=1.0, decay=0.05, m_max=None, k_max=None):
    rng = np.random.default_rng(seed)
    nrdim, npdim, nzdim = dims
    n = np.arange(nrdim)[:, None, None]
    m = np.arange(npdim)[None, :, None]
    k = np.abs(_kz(nzdim))[None, None, :]
    mag = amp * np.exp(-decay * (n + m + k))
    ph = rng.uniform(0.0, 2 * np.pi, size=dims)
    e = mag * np.exp(1j * ph)
    mask = active_mask(p, dims)
    if m_max is not None:
        mask &= (m <= m_max)
    if k_max is not None:
        mask &= (k <= k_max)
    e = np.where(mask, e, 0.0)
    e = np.asfortranarray(e.astype(np.complex128))
    return hermitian_fix(e, p)


def ppp_random(p, dims, seed, amp=1.0):
    """Random physical field (packed reals in the first nr rows and np/2 slots)."""
    rng = np.random.default_rng(seed)
    e = np.zeros(dims, dtype=np.complex128, order="F")
    nph = max(p.np // 2, 1)
    e[: p.nr, :nph, :] = amp * (rng.standard_normal((p.nr, nph, dims[2])) + 1j * rng.standard_normal((p.nr, nph, dims[2])))
    return e


def qvort_ppp(p, dims, r, x, q=1.0, centers=((0.0, 0.0),)):
    """PPP sources of the q-vortex recipe (vortical_flow_3d.f90:278-316); returns (psi_src, chi_src)."""
    nph = max(p.np // 2, 1)
    phi = 2 * np.pi / p.np * np.arange(p.np + 1)
    R = np.asarray(r)[:, None]
    X = np.asarray(x)[:, None]
    pr = phi[0:2 * nph:2][None, :]       # p(2j-1): real part
    pi_ = phi[1:2 * nph:2][None, :]      # p(2j):   imag part
    ps = np.zeros((p.nr, nph), dtype=np.complex128)
    ch = np.zeros((p.nr, nph), dtype=np.complex128)
    for xo, yo in centers:
        rr = np.sqrt((R * np.cos(pr) - xo) ** 2 + (R * np.sin(pr) - yo) ** 2)
        ri = np.sqrt((R * np.cos(pi_) - xo) ** 2 + (R * np.sin(pi_) - yo) ** 2)
        ps += -np.exp(-rr ** 2) * 2.0 / (1.0 - X) ** 2 + 1j * (-np.exp(-ri ** 2) * 2.0 / (1.0 - X) ** 2)
        ch += -np.exp(-rr ** 2) / q / (1.0 - X) ** 2 + 1j * (-np.exp(-ri ** 2) / q / (1.0 - X) ** 2)
    a = np.zeros(dims, dtype=np.complex128, order="F")
    b = np.zeros(dims, dtype=np.complex128, order="F")
    a[: p.nr, :nph, :] = ps[:, :, None]
    b[: p.nr, :nph, :] = ch[:, :, None]
    return a, b


def uniform_ppp(p, dims, b):
    """uniform_z_fld (vortical_flow_3d.f90:328-351): b in every physical sample."""
    e = np.zeros(dims, dtype=np.complex128, order="F")
    e[: p.nr, : max(p.np // 2, 1), :] = b + 1j * b
    return e
