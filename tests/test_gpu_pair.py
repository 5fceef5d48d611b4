"""The float-pair precision mode (FEDG_PREC_PAIR: explicit operator, Newton residual and RK
accumulation in float pairs of about 48 bits) against the FP64 references, with the Newton
tolerance tightened to 1e-13 so that both sides converge the implicit stages to roundoff.

Tolerances (relative L2 per variable): full fields <= 1e-9 against the FP64 oracle after 10-20
steps and <= 1e-8 against the FP64 GPU path after 450 steps of the density current (two to three
orders of magnitude inside the 1e-6 bar); deviation fields <= 1e-7.
"""
import pytest

from conftest import have_gpu

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not have_gpu(), reason="needs a CUDA GPU")]

import oracle as orc  # noqa: E402
from fedg import cases  # noqa: E402
from fedg import lib as fl  # noqa: E402
from test_gpu_mixed import report  # noqa: E402
from test_gpu_parity import to_np  # noqa: E402

FULL_TOL = 1e-9
FULL_TOL_LONG = 1e-8
DEV_TOL = 1e-7
NEWTON_TOL = 1e-13


@pytest.mark.parametrize("name,case,dt,nst", [
    ("p7_C2_4x4x4", cases.C2().scaled(4, 4, 4), 0.04, 10),
    ("p3_C1", cases.C1(), 0.02, 20),
    ("p7_C5_4x4x8", cases.C5().scaled(4, 4, 8), 0.005, 10),
    # 27 elements: the last block of four p=3 elements is partly empty
    ("p3_C1_3x3x3_ragged", cases.replace(cases.C1().scaled(3, 3, 3), eqs="HEVI"), 0.02, 10),
])
def test_pair_vs_oracle(name, case, dt, nst):
    q, b = cases.initial_state(case)
    o = orc.Oracle(case.porder, case.NeX, case.NeY, case.NeZ, case.dom)
    o.set_base_state(b["dens_hyd"], b["pres_hyd"])
    ref, rfail, _ = o.step_hevi(q, dt, nst, max_iter=30, tol=NEWTON_TOL)
    ctx = fl.Context(case)
    ctx.set_base_state(b["dens_hyd"], b["pres_hyd"], b["therm_hyd"])
    qd = [ctx.tensor(a) for a in q]
    nfail, its = ctx.update(qd, nst, eqs=fl.HEVI, prec=fl.PREC_PAIR, dt=dt, max_iter=30, tol=NEWTON_TOL)
    fe, de = report("pair " + name, to_np(qd), ref, b)
    assert nfail == 0 and rfail == 0
    assert max(fe) < FULL_TOL, fe
    assert max(de) < DEV_TOL, de


def test_pair_vs_fp64_gpu_density_current():
    """450 HEVI steps (18 s) of the -15 K density current on an 8x8x8 slice of the p=7 mesh, the
    flow on which the FP32 mode drifts by ~4e-8 of the state per step."""
    case = cases.C2().scaled(8, 8, 8)
    q, b = cases.initial_state(case)
    ctx = fl.Context(case)
    ctx.set_base_state(b["dens_hyd"], b["pres_hyd"], b["therm_hyd"])
    q64 = [ctx.tensor(a) for a in q]
    qp = [ctx.tensor(a) for a in q]
    dt = 0.04
    f64, _ = ctx.update(q64, 450, eqs=fl.HEVI, prec=fl.PREC_FP64, dt=dt, max_iter=30, tol=NEWTON_TOL)
    fp, _ = ctx.update(qp, 450, eqs=fl.HEVI, prec=fl.PREC_PAIR, dt=dt, max_iter=30, tol=NEWTON_TOL)
    assert f64 == 0 and fp == 0
    fe, de = report("pair density current 450 steps", to_np(qp), to_np(q64), b)
    assert max(fe) < FULL_TOL_LONG, fe
    assert max(de) < DEV_TOL, de


@pytest.mark.parametrize("name,case,dt,nst", [
    ("p3_C1", cases.C1(), 0.02, 20),
    ("p7_C2_4x4x4", cases.replace(cases.C2().scaled(4, 4, 4), eqs="HEVE"), 0.01, 10),
    ("p3_C1_3x3x3_ragged", cases.C1().scaled(3, 3, 3), 0.02, 10),
])
def test_pair_heve_vs_oracle(name, case, dt, nst):
    """HEVE (explicit ERK_SSP_3s3o) in float pairs against the oracle's FP64 HEVE steps; the C2
    slice carries a 10 m/s mean wind, so the reference-wind deviations are exercised."""
    q, b = cases.initial_state(case)
    o = orc.Oracle(case.porder, case.NeX, case.NeY, case.NeZ, case.dom)
    o.set_base_state(b["dens_hyd"], b["pres_hyd"])
    ref = o.step_heve(q, dt, nst)
    ctx = fl.Context(case)
    ctx.set_base_state(b["dens_hyd"], b["pres_hyd"], b["therm_hyd"])
    qd = [ctx.tensor(a) for a in q]
    nfail, _ = ctx.update(qd, nst, eqs=fl.HEVE, prec=fl.PREC_PAIR, dt=dt)
    fe, de = report("pair HEVE " + name, to_np(qd), ref, b)
    assert nfail == 0
    assert max(fe) < FULL_TOL, fe
    assert max(de) < DEV_TOL, de


def test_pair_heve_vs_fp64_gpu_long():
    """1500 HEVE steps (30 s) of the C1 thermal against the FP64 GPU path, at dt = 0.02 s (the
    largest step that stays stable for this mesh with ERK_SSP_3s3o is between 0.025 and 0.03 s)."""
    case = cases.C1()
    q, b = cases.initial_state(case)
    ctx = fl.Context(case)
    ctx.set_base_state(b["dens_hyd"], b["pres_hyd"], b["therm_hyd"])
    q64 = [ctx.tensor(a) for a in q]
    qp = [ctx.tensor(a) for a in q]
    ctx.update(q64, 1500, eqs=fl.HEVE, prec=fl.PREC_FP64, dt=0.02)
    nf, _ = ctx.update(qp, 1500, eqs=fl.HEVE, prec=fl.PREC_PAIR, dt=0.02)
    assert nf == 0
    fe, de = report("pair HEVE C1 1500 steps", to_np(qp), to_np(q64), b)
    assert max(fe) < FULL_TOL_LONG, fe
    assert max(de) < DEV_TOL, de


def test_pair_heve_rejects_guess_and_mixed():
    case = cases.C1().scaled(2, 2, 2)
    q, b = cases.initial_state(case)
    ctx = fl.Context(case)
    ctx.set_base_state(b["dens_hyd"], b["pres_hyd"], b["therm_hyd"])
    qd = [ctx.tensor(a) for a in q]
    with pytest.raises(fl.FedgError, match="HEVE"):
        ctx.update(qd, 1, eqs=fl.HEVE, prec=fl.PREC_MIXED, dt=case.dt)
    with pytest.raises(fl.FedgError, match="use_guess"):
        ctx.update(qd, 1, eqs=fl.HEVE, prec=fl.PREC_PAIR, dt=case.dt, use_guess=True)
