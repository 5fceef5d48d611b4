"""The CUDA path through the analytic known answers of tests/test_oracle_physics.py, called through
the C ABI: the same states, the same measurements, the answers from analysis (physics_states.py),
for the FP64 path (FElib's arithmetic), the float-pair path and, where its FP32 arithmetic can
resolve the effect, the FP32 mode.

Tolerances: as in the CPU tests for FP64 and float pairs; the FP32 mode's explicit arithmetic
rounds at ~6e-8 of the quantities it differences, so its bars are wider and say so.
"""
from dataclasses import replace

import numpy as np
import pytest

from conftest import have_gpu

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not have_gpu(), reason="needs a CUDA GPU")]

import oracle as orc  # noqa: E402
import physics_states as ps  # noqa: E402
from fedg import cases  # noqa: E402
from fedg import lib as fl  # noqa: E402

PATHS = {"fp64": (fl.PREC_FP64, 1e-12), "pair": (fl.PREC_PAIR, 1e-13), "fp32": (fl.PREC_MIXED, 1e-10)}


def ctx_for(case, b):
    ctx = fl.Context(case)
    ctx.set_base_state(b["dens_hyd"], b["pres_hyd"], b["therm_hyd"])
    return ctx


def run(ctx, q, nsteps, eqs, path, dt, max_iter=20):
    prec, tol = PATHS[path]
    qd = [ctx.tensor(a) for a in q]
    nf, _ = ctx.update(qd, nsteps, eqs=fl.HEVE if eqs == "HEVE" else fl.HEVI, prec=prec, dt=dt,
                       max_iter=max_iter, tol=tol)
    assert nf == 0
    return [t.cpu().numpy() for t in qd]


def scaled_max(a, s):
    return float(np.max(np.abs(a)) / s)


@pytest.mark.parametrize("porder", [3, 7])
@pytest.mark.parametrize("U", [0.0, 10.0])
def test_hydrostatic_balance_has_zero_tendency(porder, U):
    """cal_tend_ex (HEVE, HEVI) and the implicit operator (cal_vi with impl_fac = 0 returns A(var0))
    of the balanced state: below 1e-9 of the gravity term."""
    case = ps.hydro_case(porder=porder, NeZ=4, filter_on=False)
    q, b, info = ps.hydrostatic_state(case, seed=1, U=U)
    ctx = ctx_for(case, b)
    qd = [ctx.tensor(a) for a in q]
    for eqs in (fl.HEVE, fl.HEVI):
        t = [a.cpu().numpy() for a in ctx.cal_tend_ex(qd, eqs)]
        assert max(scaled_max(a, info["gterm"]) for a in t) <= 1e-9, (eqs, [scaled_max(a, info["gterm"]) for a in t])
    A = [a.cpu().numpy() for a in ctx.cal_vi(qd, qd, 0.0, 0.1)]
    assert max(scaled_max(a, info["gterm"]) for a in A) <= 1e-9


@pytest.mark.parametrize("porder,dt", [(3, 0.01), (7, 0.02)])
@pytest.mark.parametrize("eqs,path", [("HEVE", "fp64"), ("HEVE", "pair"), ("HEVI", "fp64"), ("HEVI", "pair"),
                                      ("HEVI", "fp32")])
def test_hydrostatic_balance_stays_at_rest(porder, dt, eqs, path):
    """Twenty steps from the balanced state with a 10 m/s wind, modal filter off.  Bar: 1e-10 of
    each variable's size (FP64, float pairs); 1e-6 in the FP32 mode, whose pressure gradient and
    gravity cancel only to FP32 rounding."""
    case = ps.hydro_case(porder=porder, NeZ=4, filter_on=False)
    q, b, _ = ps.hydrostatic_state(case, seed=2, U=10.0)
    ctx = ctx_for(case, b)
    sc = [np.max(np.abs(q[0])), np.max(b["dens_hyd"]), np.max(b["dens_hyd"]), np.max(b["dens_hyd"]), np.max(np.abs(q[4]))]
    q1 = run(ctx, q, 20, eqs, path, dt)
    d = [scaled_max(q1[v] - q[v], sc[v]) for v in range(5)]
    assert max(d) <= (1e-6 if path == "fp32" else 1e-10), d
    if eqs == "HEVI" and path == "fp64":  # FElib's single linearised solve
        q1 = run(ctx, q, 20, eqs, path, dt, max_iter=1)
        assert max(scaled_max(q1[v] - q[v], sc[v]) for v in range(5)) <= 1e-10


@pytest.mark.parametrize("name", ["p3", "p7"])
def test_heve_equals_hevi_explicit_plus_implicit(name):
    """cal_tend_ex(HEVE) = cal_tend_ex(HEVI) + A(q) with A from cal_vi(impl_fac = 0, var0 = q):
    rel L2 per variable below 1e-12."""
    case = cases.C1().scaled(3, 3, 4) if name == "p3" else cases.C2().scaled(3, 3, 4)
    q, b = cases.initial_state(case)
    rng = np.random.default_rng(3)
    sc = [1e-3 * b["dens_hyd"], 2.0, 2.0, 1.0, 0.3]
    q = [q[v] + sc[v] * rng.standard_normal(q[v].shape) for v in range(5)]
    ctx = ctx_for(case, b)
    qd = [ctx.tensor(a) for a in q]
    te = [a.cpu().numpy() for a in ctx.cal_tend_ex(qd, fl.HEVE)]
    ti = [a.cpu().numpy() for a in ctx.cal_tend_ex(qd, fl.HEVI)]
    A = [a.cpu().numpy() for a in ctx.cal_vi(qd, qd, 0.0, 0.1)]
    err = [float(np.linalg.norm(te[v] - ti[v] - A[v]) / np.linalg.norm(te[v])) for v in range(5)]
    assert max(err) <= 1e-12, err


def _phase(ctx, q, phase, nrep, nst, eqs, path, dt):
    ph0, a0 = phase(q)
    phs, qq = [ph0], q
    for _ in range(nrep):
        qq = run(ctx, qq, nst, eqs, path, dt)
        ph, a = phase(qq)
        phs.append(ph)
    d = np.unwrap(np.array(phs))
    return d[-1] - d[0], a / a0, qq


@pytest.mark.parametrize("eqs,path", [("HEVE", "fp64"), ("HEVE", "pair"), ("HEVI", "fp64"), ("HEVI", "pair"),
                                      ("HEVI", "fp32")])
def test_lamb_wave_speed(eqs, path):
    """Lamb wave over 0.75 of its period, dt 0.1 s: phase speed sqrt(gamma R T) to 1e-5, amplitude
    within 1e-4, w' below 1e-6 of u'.  The FP32 mode resolves deviations only down to ~1e-7 of the
    base state (a 1e-7 wave comes out 0.3 % slow and 4 % damped), so it runs the wave at 1e-5 of
    the surface pressure instead of 1e-7, with w' below 1e-5 of u'."""
    dt = 0.1
    case = ps.lamb_case(eqs=eqs)
    q, b = ps.lamb_state(case, eps=1e-5 if path == "fp32" else 1e-7)
    ctx = ctx_for(case, b)
    c = ps.lamb_speed(case)
    k = 2.0 * np.pi / (case.dom[1] - case.dom[0])
    nst = int(round(0.25 * 2.0 * np.pi / (c * k) / dt))
    dph, amp, q1 = _phase(ctx, q, lambda s: ps.lamb_phase(case, s, b), 3, nst, eqs, path, dt)
    cnum = -dph / (k * 3 * nst * dt)
    assert abs(cnum / c - 1.0) <= 1e-5, (cnum, c)
    assert abs(amp - 1.0) <= 1e-4, amp
    assert np.max(np.abs(q1[3])) <= (1e-5 if path == "fp32" else 1e-6) * np.max(np.abs(q1[1]))


@pytest.mark.parametrize("eqs,path", [("HEVE", "fp64"), ("HEVE", "pair"), ("HEVI", "fp64"), ("HEVI", "pair"),
                                      ("HEVI", "fp32")])
def test_vertical_acoustic_frequency(eqs, path):
    """Standing acoustic mode between the lids, no gravity, dt 0.05 s, 0.75 of a period: frequency
    c pi / Z to 1e-6 (HEVE) and 1e-5 (HEVI, second order in time; FP32 mode 1e-4)."""
    dt = 0.05
    case = ps.vacoustic_case(eqs=eqs)
    q, b = ps.vacoustic_state(case)
    ctx = ctx_for(case, b)
    om, _ = ps.vacoustic_omega(case)
    nst = int(round(0.25 * 2.0 * np.pi / om / dt))
    dph, amp, _ = _phase(ctx, q, lambda s: ps.vacoustic_phase(case, s, b), 3, nst, eqs, path, dt)
    onum = dph / (3 * nst * dt)
    bar = 1e-6 if eqs == "HEVE" else (1e-4 if path == "fp32" else 1e-5)
    assert abs(onum / om - 1.0) <= bar, (onum, om)
    assert abs(amp - 1.0) <= (1e-4 if path == "fp32" else 1e-5), amp


def ark232_stability(z):
    g, d = 1.0 - 1.0 / np.sqrt(2.0), 1.0 / (2.0 * np.sqrt(2.0))
    y2 = (1.0 + g * z) / (1.0 - g * z)
    return (1.0 + d * z + d * z * y2) / (1.0 - g * z)


@pytest.mark.parametrize("path", ["fp64", "pair"])
@pytest.mark.parametrize("dt", [0.25, 0.5])
def test_hevi_vertical_acoustic_at_large_courant_number(path, dt):
    """Vertical Courant number 2 to 4: HEVI's phase per step and amplitude equal ARK232's implicit
    stability function R(i w dt) to 1e-6 and 1e-5."""
    case = replace(ps.vacoustic_case(eqs="HEVI", Ztop=1000.0), dom=(0.0, 1e5, 0.0, 1e5, 0.0, 1000.0))
    q, b = ps.vacoustic_state(case)
    ctx = ctx_for(case, b)
    om, _ = ps.vacoustic_omega(case)
    dph, amp, _ = _phase(ctx, q, lambda s: ps.vacoustic_phase(case, s, b), 8, 2, "HEVI", path, dt)
    r = ark232_stability(1j * om * dt)
    assert abs(dph / 16 / np.angle(r) - 1.0) <= 1e-6, (dph / 16, np.angle(r), om * dt)
    assert abs(amp / abs(r) ** 16 - 1.0) <= 1e-5, (amp, abs(r) ** 16)


@pytest.mark.parametrize("eqs,path", [("HEVE", "fp64"), ("HEVE", "pair"), ("HEVI", "fp64"), ("HEVI", "pair"),
                                      ("HEVI", "fp32")])
def test_conservation(eqs, path):
    """Twenty steps of a perturbed flow with wind, modal filter on: the integrals of DDENS, MOMX,
    MOMY and DRHOT change by at most 1e-12 of the L1 size of the deviation fields and of the
    horizontal momentum.  The float-pair path solves MOMX/MOMY iteratively to the Newton tolerance
    (1e-13 of 340 m/s of hydrostatic momentum), which bounds its momentum drift; the FP32 mode's
    explicit fluxes round at FP32 precision, so it is held to 1e-7 of the total mass, momentum and
    RHOT instead (its deviation integrals drift at ~1e-6 of their own size)."""
    if eqs == "HEVE":
        case, dt = replace(cases.C1().scaled(4, 4, 4), u0=10.0, v0=-5.0), 0.02
    else:
        case, dt = cases.C2().scaled(3, 3, 4), 0.04
    q, b = cases.initial_state(case)
    rng = np.random.default_rng(2)
    sc = [1e-4 * b["dens_hyd"], 0.5, 0.5, 0.5, 0.03]
    q = [q[v] + sc[v] * rng.standard_normal(q[v].shape) for v in range(5)]
    ctx = ctx_for(case, b)
    I0, A0 = ps.integrals(case, q, b if path == "fp32" else None)
    q1 = run(ctx, q, 20, eqs, path, dt)
    I1, _ = ps.integrals(case, q1)
    assert np.max(np.abs(I1 - I0) / A0) <= (1e-7 if path == "fp32" else 1e-12), (I1 - I0) / A0
    assert max(np.linalg.norm(q1[v] - q[v]) / np.linalg.norm(q[v]) for v in range(5)) > 1e-2


def newton_case(name):
    case = cases.C2().scaled(2, 2, 4) if name == "p7" else cases.C1().scaled(2, 2, 5)
    q, b = cases.initial_state(case)
    rng = np.random.default_rng(7)
    sc = [1e-3 * b["dens_hyd"], 2.0, 2.0, 1.0, 0.3]
    qs = [q[v] + sc[v] * rng.standard_normal(q[v].shape) for v in range(5)]
    z0 = [qs[v] + 0.3 * sc[v] * rng.standard_normal(q[v].shape) for v in range(5)]
    dmax = float(np.max(b["dens_hyd"]))
    scales = [dmax, 10 * dmax, 10 * dmax, 340 * dmax, float(np.max(b["therm_hyd"]))]
    impl = 0.1 if name == "p7" else 0.02
    return case, b, qs, z0, scales, impl


@pytest.mark.parametrize("name", ["p3", "p7"])
def test_newton_step_matches_finite_difference_jacobian(name):
    """fedg_cal_vi with max_iter = 1 (FElib's single solve) against the Newton step built from a
    central-difference Jacobian of the implicit operator (evaluated on the CPU by the oracle's
    operator routine) and a dense solve: 1e-9 of the step."""
    case, b, qs, z0, scales, impl = newton_case(name)
    o = orc.Oracle(case.porder, case.NeX, case.NeY, case.NeZ, case.dom)
    o.set_base_state(b["dens_hyd"], b["pres_hyd"])
    P1 = ps.newton_step_fd(case, o.vi_operator, qs, z0, impl, scales)
    ctx = ctx_for(case, b)
    tend = [t.cpu().numpy() for t in ctx.cal_vi([ctx.tensor(a) for a in qs], [ctx.tensor(a) for a in z0], impl, 0.1,
                                                 max_iter=1)]
    Pg = [qs[v] + impl * tend[v] for v in range(5)]
    err = [float(np.linalg.norm(Pg[v] - P1[v]) / np.linalg.norm(P1[v] - z0[v])) for v in range(5)]
    assert max(err) <= 1e-9, err


@pytest.mark.parametrize("name", ["p3", "p7"])
def test_converged_solve_satisfies_the_implicit_equation(name):
    """fedg_cal_vi iterated to tol 1e-13: P - q* - impl_fac A(P) = 0, with A, its Rusanov speed frozen
    at var0, evaluated on the CPU by the oracle's operator routine: below 1e-12 of each scale."""
    case, b, qs, z0, scales, impl = newton_case(name)
    ctx = ctx_for(case, b)
    out, nf, _ = ctx.cal_vi([ctx.tensor(a) for a in qs], [ctx.tensor(a) for a in z0], impl, 0.1, max_iter=30,
                            tol=1e-13, want_status=True)
    assert nf == 0
    P = [qs[v] + impl * t.cpu().numpy() for v, t in enumerate(out)]
    o = orc.Oracle(case.porder, case.NeX, case.NeY, case.NeZ, case.dom)
    o.set_base_state(b["dens_hyd"], b["pres_hyd"])
    A = o.vi_operator(P, z0)
    res = [scaled_max(P[v] - qs[v] - impl * A[v], scales[v]) for v in range(5)]
    assert max(res) <= 1e-12, res
