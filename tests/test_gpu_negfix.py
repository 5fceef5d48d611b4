"""GPU parity of the tracer negative fixer (fedg_trc_negative_fixer, the C ABI) against its CPU
restatement oracle/negfix_ref.py (FElib/src/microphysics/scale_atm_phy_mp_dgm_common.F90:429-556).
Both are FP64; only the summation order of the element integrals (and the pow of CUDA against the
host's) differs: 1e-12 relative, DRHOT (a difference of two RHOT-sized terms) 1e-13 of RHOT."""
import numpy as np
import pytest

from conftest import have_gpu

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not have_gpu(), reason="needs a CUDA GPU")]

from fedg import cases  # noqa: E402
from fedg import lib as fl  # noqa: E402
from negfix_ref import negative_fixer  # noqa: E402
from negfix_states import CP, CV, MASS, QIA, QLA, R, geometry, moist_state  # noqa: E402

TOL = 1e-12


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("porder,dims,with_drhot", [(3, (3, 2, 4), True), (7, (2, 2, 2), True), (7, (2, 1, 2), False)])
def test_negative_fixer_matches_oracle(porder, dims, with_drhot):
    case = cases.C2().scaled(*dims, porder=porder)
    st = moist_state(case, seed=porder, neg_elems=(1,))
    qtrc, ddens, pres, cvtot, cptot, rtot, dh, ph, drhot = st
    int_w, z = geometry(case)
    want = negative_fixer(qtrc, ddens, pres, cvtot, cptot, rtot, dh, ph, drhot if with_drhot else None, int_w, z,
                          QLA, QIA, MASS, R, CV, CP, case.grav, cases.RDRY, cases.CVDRY, cases.CPDRY, cases.PRES00)
    ctx = fl.Context(case)
    t = ctx.tensor
    qd = [t(a) for a in qtrc]
    dd, pd, cvd, cpd, rd, dhd, phd = t(ddens), t(pres), t(cvtot), t(cptot), t(rtot), t(dh), t(ph)
    drd = t(drhot) if with_drhot else None
    ctx.trc_negative_fixer(qd, QLA, QIA, MASS, R, CV, CP, dd, pd, cvd, cpd, rd, dhd, phd, drd, dt=1.0)
    got_q = np.stack([a.cpu().numpy() for a in qd])
    for iq in range(qtrc.shape[0]):
        assert rel(got_q[iq], want[0][iq]) <= TOL, iq
    assert (got_q >= 0).all()
    for name, g, w in (("DDENS", dd, want[1]), ("PRES", pd, want[2]), ("CVtot", cvd, want[3]), ("CPtot", cpd, want[4]),
                       ("Rtot", rd, want[5])):
        assert rel(g.cpu().numpy(), w) <= TOL, name
    if with_drhot:
        # DRHOT is the difference of two RHOT-sized terms (~3e2): its rounding is measured against them
        rhot = cases.PRES00 / want[5] * (want[2] / cases.PRES00) ** (want[3] / want[4])
        assert np.abs(drd.cpu().numpy() - want[6]).max() <= 1e-13 * np.abs(rhot).max(), "DRHOT"

    ctx.close()


def test_negative_fixer_refusals():
    case = cases.C2().scaled(2, 2, 2, porder=3)
    st = moist_state(case)
    qtrc, ddens, pres, cvtot, cptot, rtot, dh, ph, _ = st
    ctx = fl.Context(case)
    t = ctx.tensor
    args = [t(ddens), t(pres), t(cvtot), t(cptot), t(rtot), t(dh), t(ph)]
    with pytest.raises(fl.FedgError, match="1 \\+ QLA \\+ QIA"):
        ctx.trc_negative_fixer([t(a) for a in qtrc], 1, 3, MASS, R, CV, CP, *args)  # 5 species for 6 tracers
    ctx.close()


@pytest.mark.parametrize("moist", [True, False])
def test_specific_heat_pressure_matches_oracle(moist):
    """fedg_trc_specific_heat_pressure (update_pressure_specific_heat) against its restatement:
    the mixture exactly up to FMA contraction, PRES and DPRES to 1e-13 relative."""
    from negfix_ref import specific_heat_pressure

    case = cases.C2().scaled(3, 2, 4, porder=3)
    qtrc, _, _, _, _, _, dh, ph, drhot = moist_state(case, seed=11)
    therm_hyd = cases.PRES00 / cases.RDRY * (ph / cases.PRES00) ** (cases.CVDRY / cases.CPDRY)
    tr = list(qtrc) if moist else []
    want = specific_heat_pressure(tr, drhot, ph, therm_hyd, MASS, R, CV, CP, cases.RDRY, cases.CVDRY, cases.CPDRY,
                                  cases.PRES00)
    ctx = fl.Context(case)
    t = ctx.tensor
    outs = [ctx.empty() for _ in range(5)]
    ctx.trc_specific_heat_pressure([t(a) for a in tr], MASS, R, CV, CP, t(drhot), t(ph), t(therm_hyd), *outs)
    for name, g, w, tol in zip(("Rtot", "CVtot", "CPtot", "PRES", "DPRES"), outs, want,
                               (1e-15, 1e-15, 1e-15, 1e-13, 1e-13)):
        got = g.cpu().numpy()
        scale = np.abs(want[3]).max() if name == "DPRES" else np.abs(w).max()  # DPRES: against PRES
        assert np.abs(got - w).max() <= tol * scale, name
    ctx.close()
