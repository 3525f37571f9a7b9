"""The 3-D vortex application (src/apps/vortical_flow_3d.f90) written against the operator API.

`kit` is any object exposing the reference's operator names (mlegs_gb300.Kit on the GPU; the CPU
oracle exposes the same names for the parity tests).  The sequence of calls follows the reference's
main program: initial condition (qvort_dist_tp, :258-326), Richardson bootstrap (:116-147), then the
main loop (:160-180) whose body is one `vortex_step` call.
"""
import numpy as np

from . import fields


class VortexState:
    names = ("psi", "chi", "nlpsi", "nlchi", "psi_p", "chi_p", "nlpsi_p", "nlchi_p", "uz")

    def __init__(self, kit):
        self.kit = kit
        for n in self.names:
            setattr(self, n, kit.scalar())
        self.gains = [0.0, 0.0]

    def args(self):
        return [getattr(self, n) for n in self.names]

    def free(self):
        for n in self.names:
            getattr(self, n).free()


def qvort_init(kit, st, q=1.0, centers=((0.0, 0.0),), uz_b=0.0, pert=None):
    """qvort_dist_tp + uniform_z_fld (vortical_flow_3d.f90:258-351).

    pert: optional (psi_fff, chi_fff) host arrays added to the spectral coefficients after the
    recipe (the seeded stand-in for the reference's rand() noise)."""
    p = kit.params
    r = kit.kit_get("r")
    x = kit.kit_get("x")
    src_psi, src_chi = fields.qvort_ppp(p, kit.dims, r, x, q=q, centers=centers)
    for s, src in ((st.psi, src_psi), (st.chi, src_chi)):
        s.set(src, 0.0, "PPP")
        kit.trans(s, "FFF")
        kit.idelsqp(s)
        kit.zeroat1(s)
    if pert is not None:
        for s, add in ((st.psi, pert[0]), (st.chi, pert[1])):
            e, ln, sp, _ = s.get()
            s.set(e + add, ln, sp)
    st.uz.set(fields.uniform_ppp(p, kit.dims, uz_b), 0.0, "PPP")
    for n in ("nlpsi", "nlchi", "psi_p", "chi_p", "nlpsi_p", "nlchi_p"):
        getattr(st, n).set(np.zeros(kit.dims, dtype=np.complex128, order="F"), 0.0, "FFF")


def bootstrap(kit, st, dt, rich_psi=None, rich_chi=None):
    """Richardson extrapolation start-up (vortical_flow_3d.f90:116-147)."""
    k = kit
    k.advection_rhs(st.psi, st.chi, st.nlpsi, st.nlchi, st.uz)
    st.psi_p.copy_from(st.psi); st.nlpsi_p.copy_from(st.nlpsi)
    st.chi_p.copy_from(st.chi); st.nlchi_p.copy_from(st.nlchi)
    pr = rich_psi or k.scalar()
    cr = rich_chi or k.scalar()
    pr.copy_from(st.psi)
    cr.copy_from(st.chi)
    k.advection_rhs(pr, cr, st.nlpsi, st.nlchi, st.uz)
    k.febe(pr, st.nlpsi, dt)
    k.febe(cr, st.nlchi, dt)
    for _ in range(2):
        k.advection_rhs(st.psi, st.chi, st.nlpsi, st.nlchi, st.uz)
        k.febe(st.psi, st.nlpsi, dt / 2.0)
        k.febe(st.chi, st.nlchi, dt / 2.0)
    k.axpby(st.psi, 2.0, st.psi, -1.0, pr)
    k.axpby(st.chi, 2.0, st.chi, -1.0, cr)
    k.dealias(st.psi); k.dealias(st.chi)
    st.gains[0] = k.svv_filter(st.psi, st.gains[0])
    st.gains[1] = k.svv_filter(st.chi, st.gains[1])
    k.zeroat1(st.psi); k.zeroat1(st.chi)
    k.advection_rhs(st.psi, st.chi, st.nlpsi, st.nlchi, st.uz)
    pr.free()
    cr.free()


def step(kit, st, dt):
    """One main-loop step (vortical_flow_3d.f90:168-180)."""
    kit.vortex_step(*st.args(), dt, st.gains)


def kinetic_energy_spectrum(e):
    """Per-(m) energy of a spectral field, sum over n and k of |c|^2 (diagnostic)."""
    return np.sum(np.abs(e) ** 2, axis=(0, 2))
