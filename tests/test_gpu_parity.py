"""GPU parity of the FP64 CUDA path against the FP64 CPU oracle, through the C ABI.

Tolerances (relative L2 per variable, ||gpu - oracle|| / ||oracle||):
  * single operator calls (cal_tend_ex, cal_vi, modal filter, DRHOT2PRES): 1e-11
  * whole time steps (HEVE SSP-RK3, HEVI ARK232): 1e-9, the plain-FP64 parity bar
"""
import numpy as np
import pytest

from conftest import have_gpu

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not have_gpu(), reason="needs a CUDA GPU")]

import oracle as orc  # noqa: E402
import timeint_ref  # noqa: E402
from fedg import cases  # noqa: E402
from fedg import lib as fl  # noqa: E402

VARS = ("DDENS", "MOMX", "MOMY", "MOMZ", "DRHOT")


def relerr(a, b, floor=0.0):
    a = np.asarray(a)
    b = np.asarray(b)
    nb = max(np.linalg.norm(b), floor)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def state_floors(b):
    """Denominator floors of the per-variable relative L2 for whole-step parity: a variable
    that starts at zero (MOMY, MOMZ) is measured against 1 m/s of hydrostatic momentum,
    DDENS/DRHOT against 1e-6 of their hydrostatic fields, so roundoff on a near-empty
    field is not reported as a relative error of order one."""
    dn = np.linalg.norm(b["dens_hyd"])
    return [1e-6 * dn, dn, dn, dn, 1e-6 * np.linalg.norm(b["therm_hyd"])]


def small_cases():
    return {
        "p3_C1": cases.C1(),
        "p7_C2_4x4x4": cases.C2().scaled(4, 4, 4),
        "p7_C5_4x4x4": cases.C5().scaled(4, 4, 4),
        "p2_3x2x5": cases.C1().scaled(3, 2, 5, porder=2),
        # 27 columns: the FP64 column solve's two-columns-per-warp mapping leaves the last half-warp
        # without a column of its own
        "p2_3x1x4_odd_columns": cases.C1().scaled(3, 1, 4, porder=2),
    }


def perturbed(case, seed, amp=1.0):
    q, b = cases.initial_state(case)
    rng = np.random.default_rng(seed)
    sc = [1e-3 * b["dens_hyd"], 2.0, 2.0, 1.0, 0.3]
    q = [q[v] + amp * sc[v] * rng.standard_normal(q[v].shape) for v in range(5)]
    return q, b


def make(case, filter_on=None):
    o = orc.Oracle(case.porder, case.NeX, case.NeY, case.NeZ, case.dom,
                   filter_on=case.filter_on if filter_on is None else filter_on)
    ctx = fl.Context(case, filter_on=filter_on)
    return o, ctx


def to_np(ts):
    return [t.cpu().numpy() for t in ts]


@pytest.mark.parametrize("name", list(small_cases()))
@pytest.mark.parametrize("hevi", [0, 1])
def test_cal_tend_ex(name, hevi):
    case = small_cases()[name]
    q, b = perturbed(case, 1)
    o, ctx = make(case)
    o.set_base_state(b["dens_hyd"], b["pres_hyd"])
    ctx.set_base_state(b["dens_hyd"], b["pres_hyd"], b["therm_hyd"])
    ref = o.cal_tend(q, hevi)
    qd = [ctx.tensor(a) for a in q]
    _, dp = ctx.drhot2pres(qd[4])
    got = to_np(ctx.cal_tend_ex(qd, hevi, dpres=dp))
    errs = [relerr(g, r) for g, r in zip(got, ref)]
    assert max(errs) < 1e-11, dict(zip(VARS, errs))
    # DPRES formed inside the call when not passed
    got2 = to_np(ctx.cal_tend_ex(qd, hevi, dpres=None))
    assert max(relerr(g, r) for g, r in zip(got2, ref)) < 1e-11


@pytest.mark.parametrize("name", ["p3_C1", "p7_C2_4x4x4", "p7_C5_4x4x4", "p2_3x2x5"])
def test_drhot2pres_and_filter(name):
    case = small_cases()[name]
    q, b = perturbed(case, 2)
    o, ctx = make(case)
    o.set_base_state(b["dens_hyd"], b["pres_hyd"])
    ctx.set_base_state(b["dens_hyd"], b["pres_hyd"], b["therm_hyd"])
    pr, dp = o.drhot2pres(q[4])
    gpr, gdp = ctx.drhot2pres(ctx.tensor(q[4]))
    assert relerr(gpr.cpu().numpy(), pr) < 1e-14
    assert relerr(gdp.cpu().numpy(), dp) < 1e-11
    ref = o.modalfilter(q)
    qd = [ctx.tensor(a) for a in q]
    got = to_np(ctx.modalfilter(qd))
    assert max(relerr(g, r) for g, r in zip(got, ref)) < 1e-13


@pytest.mark.parametrize("name", ["p3_C1", "p7_C2_4x4x4", "p7_C5_4x4x4", "p2_3x2x5", "p2_3x1x4_odd_columns"])
@pytest.mark.parametrize("mode", ["ref1", "iter", "zero"])
def test_cal_vi(name, mode):
    case = small_cases()[name]
    q0, b = perturbed(case, 3, amp=0.3)
    rng = np.random.default_rng(4)
    # stage input = var0 + a small explicit increment
    q = [a + 0.05 * np.std(a) * rng.standard_normal(a.shape) for a in q0]
    o, ctx = make(case)
    o.set_base_state(b["dens_hyd"], b["pres_hyd"])
    ctx.set_base_state(b["dens_hyd"], b["pres_hyd"], b["therm_hyd"])
    gam = 1.0 - 1.0 / np.sqrt(2.0)
    dt = case.dt if case.porder > 3 else 0.02
    impl_fac = 0.0 if mode == "zero" else gam * dt
    max_iter, tol = (1, 0.0) if mode != "iter" else (20, 1e-10)
    ref, rfail, rits = o.cal_vi(q, q0, impl_fac, dt, max_iter, tol, want_iters=True)
    qd = [ctx.tensor(a) for a in q]
    q0d = [ctx.tensor(a) for a in q0]
    got, nfail, st = ctx.cal_vi(qd, q0d, impl_fac, dt, max_iter, tol, want_status=True)
    got = to_np(got)
    errs = [relerr(g, r) for g, r in zip(got, ref)]
    assert max(errs) < 1e-10, dict(zip(VARS, errs))
    assert nfail == rfail == 0
    st = st.cpu().numpy()
    if mode == "iter":
        assert np.all(st >= 1) and np.all(st <= 6)
        # same stopping rule on both sides: at most a handful of columns may differ by one
        # solve where the residual lands within roundoff of tol
        assert np.mean(st != rits) <= 0.01 and np.max(np.abs(st - rits)) <= 1


@pytest.mark.parametrize("scheme,name", [(fl.IMEX_ARK232, "IMEX_ARK232"), (fl.SSP_RK3, "ERK_SSP_3s3o")])
def test_timeint_rk_stage_methods(scheme, name):
    """The damped oscillator of test_timeint_rk.f90 driven through the device RK methods matches
    the host restatement of timeint_rk stage by stage."""
    case = cases.C1().scaled(1, 1, 1, porder=1)
    ctx = fl.Context(case)
    import torch

    dt = 0.01
    t = fl.TimeInt(ctx, scheme, dt)
    ref = timeint_ref.TimeIntRK(name, dt, (2,))
    qh = np.array([1.0, 0.0])
    qd = [torch.full(ctx.shape, x, dtype=torch.float64, device=ctx.dev) for x in (1.0, 0.0, 0.0, 0.0, 0.0)]
    omg, r = 2 * np.pi, 0.1
    for n in range(50):
        for s in range(1, 4):
            buf = s - 1 if scheme == fl.IMEX_ARK232 else 0
            if scheme == fl.IMEX_ARK232:
                fac = ref.implicit_diagfac(s)
                assert abs(fac - t.implicit_diagfac(s)) < 1e-16
                if fac != 0:
                    coef = fac * omg
                    ui = (qh[0] + coef * qh[1]) / (1 + coef ** 2)
                    vi = (qh[1] - coef * qh[0]) / (1 + coef ** 2)
                    tim = [(ui - qh[0]) / fac, (vi - qh[1]) / fac]
                else:
                    tim = [omg * qh[1], -omg * qh[0]]
                ref.tend_im[buf] = tim
                t.tend_im(s, 0).fill_(tim[0])
                t.tend_im(s, 1).fill_(tim[1])
                ref.store_implicit(s, qh)
                t.store_implicit(s, qd)
                tex = [-r * qh[0], 0.0]
            else:
                tex = [omg * qh[1] - r * qh[0], -omg * qh[0]]
            ref.tend_ex[buf] = tex
            t.tend_ex(s, 0).fill_(tex[0])
            t.tend_ex(s, 1).fill_(tex[1])
            ref.advance(s, qh)
            t.advance(s, qd)
            ctx.sync()
            assert abs(qd[0][0, 0].item() - qh[0]) <= 1e-14 and abs(qd[1][0, 0].item() - qh[1]) <= 1e-14


def test_update_heve_ssprk3():
    case = cases.C1()
    q, b = cases.initial_state(case)
    o, ctx = make(case)
    o.set_base_state(b["dens_hyd"], b["pres_hyd"])
    ctx.set_base_state(b["dens_hyd"], b["pres_hyd"], b["therm_hyd"])
    dt, nst = 0.02, 20
    ref = o.step_heve(q, dt, nst)
    qd = [ctx.tensor(a) for a in q]
    ctx.update(qd, nst, eqs=fl.HEVE, dt=dt)
    fl_ = state_floors(b)
    errs = [relerr(g, r, f) for g, r, f in zip(to_np(qd), ref, fl_)]
    assert max(errs) < 1e-9, dict(zip(VARS, errs))


@pytest.mark.parametrize("name,max_iter", [("p7_C2_4x4x4", 1), ("p7_C2_4x4x4", 10), ("p3_C1", 1),
                                           ("p7_C5_4x4x4", 10)])
def test_update_hevi_ark232(name, max_iter):
    case = small_cases()[name]
    q, b = cases.initial_state(case)
    o, ctx = make(case)
    o.set_base_state(b["dens_hyd"], b["pres_hyd"])
    ctx.set_base_state(b["dens_hyd"], b["pres_hyd"], b["therm_hyd"])
    dt = {"p7_C2_4x4x4": 0.04, "p3_C1": 0.02, "p7_C5_4x4x4": 0.005}[name]
    nst = 10
    tol = 1e-10 if max_iter > 1 else 0.0
    ref, rfail, rits = o.step_hevi(q, dt, nst, max_iter=max_iter, tol=tol)
    qd = [ctx.tensor(a) for a in q]
    nfail, its = ctx.update(qd, nst, eqs=fl.HEVI, dt=dt, max_iter=max_iter, tol=tol)
    fl_ = state_floors(b)
    errs = [relerr(g, r, f) for g, r, f in zip(to_np(qd), ref, fl_)]
    assert max(errs) < 1e-9, dict(zip(VARS, errs))
    assert nfail == 0 and rfail == 0
    if max_iter > 1:
        assert abs(its - rits) < 0.05
