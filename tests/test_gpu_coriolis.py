"""The Coriolis term on an f-plane (FElib's CORIOLIS field of AUX_VARS2D, constant; heve.F90 and
hevi.F90 add f MOMY to the MOMX tendency and -f MOMX to the MOMY tendency) in every path, against
the oracle with the same f.

f = 0.05 s^-1, 500 times a mid-latitude value, so that a few steps turn the 10 m/s mean wind of the
C2 slice measurably (dMOMY/dt = -f DENS u, about -0.5 kg m^-2 s^-2): a wrong sign or a term left
out shows at the 1e-3 level, far above every tolerance below.

Tolerances (relative L2 per variable, momentum against at least 1 m/s of hydrostatic momentum):
the tendency 1e-11 (the bar of the f = 0 tendency parity); whole FP64 and float-pair steps 1e-9; the FP32 explicit mode 1e-6.
"""
import numpy as np
import pytest

from conftest import have_gpu

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not have_gpu(), reason="needs a CUDA GPU")]

import oracle as orc  # noqa: E402
from fedg import cases  # noqa: E402
from fedg import lib as fl  # noqa: E402
from test_gpu_parity import VARS, perturbed, relerr, state_floors, to_np  # noqa: E402

F = 0.05


def setup(case):
    q, b = cases.initial_state(case)
    o = orc.Oracle(case.porder, case.NeX, case.NeY, case.NeZ, case.dom, coriolis_f=F,
                   filter_on=case.filter_on)
    o.set_base_state(b["dens_hyd"], b["pres_hyd"])
    ctx = fl.Context(case)
    ctx.set_base_state(b["dens_hyd"], b["pres_hyd"], b["therm_hyd"], coriolis_f=F)
    return q, b, o, ctx


def full_errs(got, ref, b):
    """full fields (DENS, momentum, RHOT): momentum against at least 1 m/s of hydrostatic momentum"""
    dn = np.linalg.norm(b["dens_hyd"])
    hyd = [b["dens_hyd"], 0.0, 0.0, 0.0, b["therm_hyd"]]
    return [float(np.linalg.norm(g - r) / max(np.linalg.norm(r + h), dn)) for g, r, h in zip(got, ref, hyd)]


@pytest.mark.parametrize("hevi", [False, True])
def test_cal_tend_coriolis(hevi):
    """on a randomly perturbed state, so that every tendency is O(1) (the C2 initial state has a
    horizontally uniform RHOT and hence an RHOT tendency that is zero up to roundoff)"""
    case = cases.C2().scaled(4, 4, 4)
    _, b, o, ctx = setup(case)
    q, _ = perturbed(case, 3)
    ref = o.cal_tend(q, hevi)
    got = to_np(ctx.cal_tend_ex([ctx.tensor(a) for a in q], fl.HEVI if hevi else fl.HEVE))
    errs = [relerr(g, r) for g, r in zip(got, ref)]
    assert max(errs) < 1e-11, dict(zip(VARS, errs))
    # the term is there: MOMY's tendency carries -f MOMX of the mean wind
    o0 = orc.Oracle(case.porder, case.NeX, case.NeY, case.NeZ, case.dom, filter_on=case.filter_on)
    o0.set_base_state(b["dens_hyd"], b["pres_hyd"])
    ref0 = o0.cal_tend(q, hevi)
    assert relerr(ref0[2], ref[2]) > 1e-3


def test_update_fp64_coriolis():
    case = cases.C2().scaled(4, 4, 4)
    q, b, o, ctx = setup(case)
    dt, nst = 0.04, 10
    ref, rfail, _ = o.step_hevi(q, dt, nst, max_iter=10, tol=1e-12)
    qd = [ctx.tensor(a) for a in q]
    nf, _ = ctx.update(qd, nst, eqs=fl.HEVI, dt=dt, max_iter=10, tol=1e-12)
    assert nf == 0 and rfail == 0
    errs = [relerr(g, r, f) for g, r, f in zip(to_np(qd), ref, state_floors(b))]
    assert max(errs) < 1e-9, dict(zip(VARS, errs))
    heve = cases.replace(case, eqs="HEVE")
    q, b, o, ctx = setup(heve)
    ref = o.step_heve(q, 0.01, 10)
    qd = [ctx.tensor(a) for a in q]
    ctx.update(qd, 10, eqs=fl.HEVE, dt=0.01)
    errs = [relerr(g, r, f) for g, r, f in zip(to_np(qd), ref, state_floors(b))]
    assert max(errs) < 1e-9, dict(zip(VARS, errs))


@pytest.mark.parametrize("eqs", ["HEVI", "HEVE"])
def test_update_pair_coriolis(eqs):
    case = cases.replace(cases.C2().scaled(4, 4, 4), eqs=eqs)
    q, b, o, ctx = setup(case)
    qd = [ctx.tensor(a) for a in q]
    if eqs == "HEVI":
        ref, rfail, _ = o.step_hevi(q, 0.04, 10, max_iter=30, tol=1e-13)
        nf, _ = ctx.update(qd, 10, eqs=fl.HEVI, prec=fl.PREC_PAIR, dt=0.04, max_iter=30, tol=1e-13)
        assert rfail == 0
    else:
        ref = o.step_heve(q, 0.01, 10)
        nf, _ = ctx.update(qd, 10, eqs=fl.HEVE, prec=fl.PREC_PAIR, dt=0.01)
    assert nf == 0
    errs = full_errs(to_np(qd), ref, b)
    assert max(errs) < 1e-9, dict(zip(VARS, errs))


def test_update_mixed_coriolis():
    case = cases.C2().scaled(4, 4, 4)
    q, b, o, ctx = setup(case)
    ref, rfail, _ = o.step_hevi(q, 0.04, 10, max_iter=30, tol=1e-13)
    qd = [ctx.tensor(a) for a in q]
    nf, _ = ctx.update(qd, 10, eqs=fl.HEVI, prec=fl.PREC_MIXED, dt=0.04, max_iter=30, tol=1e-10)
    assert nf == 0 and rfail == 0
    errs = full_errs(to_np(qd), ref, b)
    assert max(errs) < 1e-6, dict(zip(VARS, errs))
