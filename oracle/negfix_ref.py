"""CPU restatement (numpy) of FElib's tracer negative fixer: test infrastructure, the checker of
fedg_trc_negative_fixer, used only by tests/.

atm_phy_mp_dgm_common_negative_fixer (FElib/src/microphysics/scale_atm_phy_mp_dgm_common.F90:429-556),
which the tracer driver runs after its step (fix_negative_val,
FElib/src/fluid_dyn_solver/scale_atm_dyn_dgm_driver_trcadv3d.F90:596-651).  The mixture's specific
heats are SCALE's ATMOS_THERMODYN_specific_heat (scale_atmos_thermodyn.F90 in SCALE, a dependency
the reference tree does not vendor), restated from its published mixing rule:
qdry = 1 - sum_q q MASS_q, Rtot = sum_q q R_q + qdry Rdry, CVtot and CPtot alike.

Parity unpinned against FElib itself (no Fortran compiler here and SCALE absent): the restatement is
pinned by the properties the routine exists for (tests/test_oracle_negfix.py): nonnegative species,
each species' element mass kept at max(M, 0), the element's internal energy kept (before the
potential-energy correction of the mass change), and a state without negative values left unchanged.
Arrays are (Ne, Np); the tracers (QA, Ne, Np)."""
import numpy as np

TRC_EPS = 1e-128  # scale_atm_phy_mp_dgm_common.F90:483 (double precision)


def specific_heat(q, mass, r, cv, cp, rdry, cvdry, cpdry):
    """ATMOS_THERMODYN_specific_heat: (Qdry, Rtot, CVtot, CPtot) of the mixing ratios q[iq]"""
    qdry = np.ones_like(q[0])
    rt = np.zeros_like(q[0])
    cvt = np.zeros_like(q[0])
    cpt = np.zeros_like(q[0])
    for iq in range(len(q)):
        qdry = qdry - q[iq] * mass[iq]
        rt = rt + q[iq] * r[iq]
        cvt = cvt + q[iq] * cv[iq]
        cpt = cpt + q[iq] * cp[iq]
    return qdry, rt + qdry * rdry, cvt + qdry * cvdry, cpt + qdry * cpdry


def negative_fixer(qtrc, ddens, pres, cvtot, cptot, rtot, dens_hyd, pres_hyd, drhot, int_w, zlev, qla, qia,
                   mass, r, cv, cp, grav, rdry, cvdry, cpdry, pres00):
    """One call of the fixer (scale_atm_phy_mp_dgm_common.F90:496-553); returns the new
    (qtrc, ddens, pres, cvtot, cptot, rtot, drhot) without touching the inputs.  int_w: Gsqrt J w of
    every node (Np,) or (Ne, Np); zlev: node heights (Ne, Np); drhot may be None."""
    qtrc = np.asarray(qtrc, dtype=np.float64)
    qa = qtrc.shape[0]
    w = np.broadcast_to(int_w, ddens.shape)
    dens = dens_hyd + ddens                                   # :502
    ddens0 = ddens.copy()                                     # :503
    ddens = ddens.copy()
    ien0 = cvtot * pres / rtot                                # :510
    temp = ien0 / (dens * cvtot)                              # :512
    ien = ien0.copy()                                         # :513
    m1 = np.zeros_like(qtrc)
    for iq in range(1 + qla + qia):                           # :516-527
        m0 = dens * qtrc[iq]
        t = np.maximum(TRC_EPS, m0)
        M0 = np.sum(w * m0, axis=1, keepdims=True)
        M1 = np.sum(w * t, axis=1, keepdims=True)
        t = np.maximum(M0, 0.0) / M1 * t
        ddens = ddens + (t - m0)
        ien = ien + (t - m0) * cv[iq] * temp
        m1[iq] = t
    dens = dens_hyd + ddens                                   # :531
    qnew = m1 / dens[None]                                    # :532-535 (QA = 1 + QLA + QIA)
    E0 = np.sum(w * ien0, axis=1, keepdims=True)              # :537-539
    E1 = np.sum(w * ien, axis=1, keepdims=True)
    ien = E0 / E1 * ien
    _, rt, cvt, cpt = specific_heat(qnew, mass, r, cv, cp, rdry, cvdry, cpdry)  # :541-544
    ien = ien - (ddens - ddens0) * grav * zlev                # :546
    p = ien * rt / cvt                                        # :547
    dr = None
    if drhot is not None:                                     # :549-552
        dr = pres00 / rt * (p / pres00) ** (cvt / cpt) - pres00 / rdry * (pres_hyd / pres00) ** (cvdry / cpdry)
    return qnew, ddens, p, cvt, cpt, rt, dr


def specific_heat_pressure(qtrc, drhot, pres_hyd, therm_hyd, mass, r, cv, cp, rdry, cvdry, cpdry, pres00):
    """update_pressure_specific_heat (FElib/src/fluid_dyn_solver/scale_atm_dyn_dgm_driver_trcadv3d.F90:
    653-716): the mixture's (Rtot, CVtot, CPtot) and, through atm_dyn_dgm_nonhydro3d_common_DRHOT2PRES
    (nonhydro3d_common.F90:470-474), PRES = P00 (Rtot / P00 (THERM_hyd + DRHOT))^(CPtot / CVtot) and
    DPRES = PRES - PRES_hyd.  qtrc: (QA, ...) or an empty list (the dry constants)."""
    shape = np.shape(drhot)
    q = np.asarray(qtrc, dtype=np.float64).reshape((len(qtrc),) + shape) if len(qtrc) else np.zeros((1,) + shape)
    tabs = (mass, r, cv, cp) if len(qtrc) else ([0.0], [0.0], [0.0], [0.0])
    _, rt, cvt, cpt = specific_heat(q, *tabs, rdry, cvdry, cpdry)
    rhot = therm_hyd + drhot
    pres = pres00 * (rt * (1.0 / pres00) * rhot) ** (cpt / cvt)
    return rt, cvt, cpt, pres, pres - pres_hyd
