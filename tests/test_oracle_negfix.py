"""The tracer negative fixer's CPU restatement (oracle/negfix_ref.py), pinned by the properties
FElib's routine (scale_atm_phy_mp_dgm_common.F90:429-556) is built to have, since neither FElib nor
SCALE's thermodynamics can be run here:
  - every water species ends nonnegative, with its element mass max(M, 0);
  - DDENS changes by the sum of the species' mass changes;
  - the element's internal energy CVtot PRES / Rtot is kept once the potential energy of the mass
    change (DDENS - DDENS0) g z is added back;
  - a state without negative values is left unchanged (to rounding);
  - DRHOT is the one of the new PRES with the mixture's exponent."""
import numpy as np

from fedg import cases
from negfix_ref import negative_fixer, specific_heat
from negfix_states import CP, CV, MASS, QIA, QLA, R, geometry, moist_state


def _case():
    return cases.C2().scaled(2, 2, 3, porder=3)


def _run(case, st):
    qtrc, ddens, pres, cvtot, cptot, rtot, dh, ph, drhot = st
    int_w, z = geometry(case)
    out = negative_fixer(qtrc, ddens, pres, cvtot, cptot, rtot, dh, ph, drhot, int_w, z, QLA, QIA, MASS, R, CV, CP,
                         case.grav, cases.RDRY, cases.CVDRY, cases.CPDRY, cases.PRES00)
    return out, int_w, z


def test_species_masses_and_density():
    case = _case()
    st = moist_state(case, seed=1, neg_elems=(3,))
    (qn, ddn, pn, cvn, cpn, rn, _), int_w, _ = _run(case, st)
    qtrc, ddens, _, _, _, _, dh, _, _ = st
    assert (qn >= 0).all()
    dens0, dens1 = dh + ddens, dh + ddn
    dm = np.zeros_like(ddens)
    for iq in range(qtrc.shape[0]):
        M0 = np.sum(int_w * dens0 * qtrc[iq], axis=1)
        M1 = np.sum(int_w * dens1 * qn[iq], axis=1)
        np.testing.assert_allclose(M1, np.maximum(M0, 0.0), rtol=1e-12, atol=1e-14 * np.abs(M0).max())
        dm += dens1 * qn[iq] - dens0 * qtrc[iq]
    np.testing.assert_allclose(ddn - ddens, dm, rtol=1e-9, atol=1e-18)
    assert np.all(qn[1][3] == 0.0)  # the element whose first condensate had a negative mass
    assert np.any(qtrc[1:] < 0)     # the state did have undershoots to fix


def test_internal_energy_and_pressure():
    case = _case()
    st = moist_state(case, seed=2)
    (qn, ddn, pn, cvn, cpn, rn, drn), int_w, z = _run(case, st)
    qtrc, ddens, pres, cvtot, cptot, rtot, dh, ph, _ = st
    e0 = np.sum(int_w * cvtot * pres / rtot, axis=1)
    e1 = np.sum(int_w * (cvn * pn / rn + (ddn - ddens) * case.grav * z), axis=1)
    np.testing.assert_allclose(e1, e0, rtol=1e-12)
    _, r2, cv2, cp2 = specific_heat(qn, MASS, R, CV, CP, cases.RDRY, cases.CVDRY, cases.CPDRY)
    np.testing.assert_array_equal(rn, r2)
    rhot = cases.PRES00 / rn * (pn / cases.PRES00) ** (cvn / cpn)
    rhot_hyd = cases.PRES00 / cases.RDRY * (ph / cases.PRES00) ** (cases.CVDRY / cases.CPDRY)
    np.testing.assert_allclose(drn, rhot - rhot_hyd, rtol=1e-12, atol=1e-9)


def test_state_without_negatives_is_kept():
    case = _case()
    st = moist_state(case, seed=3, neg_frac=0.0)
    (qn, ddn, pn, cvn, cpn, rn, drn), _, _ = _run(case, st)
    qtrc, ddens, pres, cvtot, cptot, rtot, _, _, drhot = st
    np.testing.assert_allclose(qn, qtrc, rtol=1e-14, atol=0)
    np.testing.assert_allclose(ddn, ddens, rtol=0, atol=1e-15 * np.abs(ddens).max() + 1e-17)
    np.testing.assert_allclose(pn, pres, rtol=1e-13)
    np.testing.assert_allclose(rn, rtot, rtol=1e-14)
    np.testing.assert_allclose(drn, drhot, rtol=0, atol=1e-9 * np.abs(drhot).max() + 1e-9)


def test_specific_heat_pressure_restates_the_dry_and_moist_forms():
    """update_pressure_specific_heat's restatement: with no tracers it is the dry DRHOT -> PRES of the
    dynamics oracle; with the moist state's tracers it gives back the mixture and the pressure the
    state was built from (PRES = P00 (Rtot RHOT / P00)^(CPtot / CVtot))."""
    import oracle as orc
    from negfix_ref import specific_heat_pressure

    case = _case()
    qtrc, ddens, pres, cvtot, cptot, rtot, dh, ph, drhot = moist_state(case, seed=4)
    therm_hyd = cases.PRES00 / cases.RDRY * (ph / cases.PRES00) ** (cases.CVDRY / cases.CPDRY)
    consts = (cases.RDRY, cases.CVDRY, cases.CPDRY, cases.PRES00)
    rt, cvt, cpt, p, dp = specific_heat_pressure(qtrc, drhot, ph, therm_hyd, MASS, R, CV, CP, *consts)
    np.testing.assert_array_equal(rt, rtot)
    np.testing.assert_array_equal(cvt, cvtot)
    np.testing.assert_allclose(p, pres, rtol=1e-14)
    np.testing.assert_allclose(dp, p - ph, rtol=0, atol=0)
    rt0, cvt0, cpt0, p0, dp0 = specific_heat_pressure([], drhot, ph, therm_hyd, MASS, R, CV, CP, *consts)
    assert np.all(rt0 == cases.RDRY) and np.all(cvt0 == cases.CVDRY) and np.all(cpt0 == cases.CPDRY)
    o = orc.Oracle(case.porder, case.NeX, case.NeY, case.NeZ, case.dom)
    o.set_base_state(dh, ph)
    pres_dry, dpres_dry = o.drhot2pres(drhot)
    np.testing.assert_allclose(p0, np.asarray(pres_dry).reshape(p0.shape), rtol=1e-13)
