"""Known answers for the dynamics oracle that come from analysis, not from the oracle itself.

The reference's own tests pin only the element operators and the RK orders (test_oracle_kat.py).
These tests pin the rest of the restated dynamics step (oracle/fedg_oracle.cpp: the flux build,
the pressure gradient and gravity, the Rusanov faces, the HEVI operator split, the Newton
Jacobian and block LU, ARK232 and SSP-RK3) against answers known without running any
implementation (tests/physics_states.py derives each one):

  * a discretely hydrostatic deviation state has zero tendency and stays at rest (HEVE, HEVI);
  * the HEVE operator equals the HEVI explicit operator plus the HEVI implicit operator with its
    Rusanov speed frozen at the state itself (FElib's IMEX split is a split of one operator);
  * a Lamb wave travels at sqrt(gamma R T) under gravity; the vertical acoustic mode between the
    lids oscillates at c pi / Z, and at large vertical Courant numbers HEVI advances it by exactly
    ARK232's implicit stability function;
  * the integrals of DDENS, MOMX, MOMY and DRHOT are conserved with periodic sides and slip lids;
  * one cal_vi Newton step equals the Newton step built from a finite-difference Jacobian of the
    implicit operator, and the converged solve satisfies the implicit equation.

Tolerances are written per test; each is far below the size of the effect a wrong term would have.
"""
from dataclasses import replace

import numpy as np
import pytest

import oracle as orc
import physics_states as ps
from fedg import cases


def make(case):
    return orc.Oracle(case.porder, case.NeX, case.NeY, case.NeZ, case.dom, grav=case.grav, filter_on=case.filter_on)


def scaled_max(a, s):
    return float(np.max(np.abs(a)) / s)


@pytest.mark.parametrize("porder", [3, 7])
@pytest.mark.parametrize("U", [0.0, 10.0])
def test_hydrostatic_balance_has_zero_tendency(porder, U):
    """Pressure gradient and gravity cancel node by node; the degree-p mode of DDENS exerts no
    force (VPOrdM1); a uniform wind advects nothing.  Bar: 1e-9 of the gravity term (roundoff of
    the equation of state is ~1e-10); a gravity term without VPOrdM1 would leave 1e-2."""
    case = ps.hydro_case(porder=porder, NeZ=4, filter_on=False)
    q, b, info = ps.hydrostatic_state(case, seed=1, U=U)
    o = make(case)
    o.set_base_state(b["dens_hyd"], b["pres_hyd"])
    for hevi in (0, 1):
        t = o.cal_tend(q, hevi)
        assert max(scaled_max(a, info["gterm"]) for a in t) <= 1e-9, (hevi, [scaled_max(a, info["gterm"]) for a in t])
    A = o.vi_operator(q, q)
    assert max(scaled_max(a, info["gterm"]) for a in A) <= 1e-9


@pytest.mark.parametrize("porder,dt", [(3, 0.01), (7, 0.02)])
def test_hydrostatic_balance_stays_at_rest(porder, dt):
    """Twenty HEVE (SSP-RK3) and HEVI (ARK232, Newton to 1e-12 and FElib's single solve) steps
    from the balanced state, modal filter off.  Bar: 1e-10 of each variable's size."""
    case = ps.hydro_case(porder=porder, NeZ=4, filter_on=False)
    q, b, _ = ps.hydrostatic_state(case, seed=2, U=10.0)
    o = make(case)
    o.set_base_state(b["dens_hyd"], b["pres_hyd"])
    sc = [np.max(np.abs(q[0])), np.max(b["dens_hyd"]), np.max(b["dens_hyd"]), np.max(b["dens_hyd"]), np.max(np.abs(q[4]))]
    runs = {"HEVE": o.step_heve(q, dt, 20),
            "HEVI": o.step_hevi(q, dt, 20, max_iter=20, tol=1e-12)[0],
            "HEVI_1": o.step_hevi(q, dt, 20, max_iter=1)[0]}
    for name, q1 in runs.items():
        d = [scaled_max(q1[v] - q[v], sc[v]) for v in range(5)]
        assert max(d) <= 1e-10, (name, d)


@pytest.mark.parametrize("name", ["p3", "p7"])
def test_heve_equals_hevi_explicit_plus_implicit(name):
    """FElib's HEVI split of the operator: the explicit HEVI tendency plus the implicit operator
    (Rusanov speed frozen at the state) is the HEVE tendency.  Bar: 1e-13 rel L2 per variable."""
    case = cases.C1().scaled(3, 3, 4) if name == "p3" else cases.C2().scaled(3, 3, 4)
    q, b = cases.initial_state(case)
    rng = np.random.default_rng(3)
    sc = [1e-3 * b["dens_hyd"], 2.0, 2.0, 1.0, 0.3]
    q = [q[v] + sc[v] * rng.standard_normal(q[v].shape) for v in range(5)]
    o = make(case)
    o.set_base_state(b["dens_hyd"], b["pres_hyd"])
    te, ti, A = o.cal_tend(q, 0), o.cal_tend(q, 1), o.vi_operator(q, q)
    err = [float(np.linalg.norm(te[v] - ti[v] - A[v]) / np.linalg.norm(te[v])) for v in range(5)]
    assert max(err) <= 1e-13, err


def _phase_run(stepper, phase, q, nrep, nst):
    ph0, a0 = phase(q)
    phs, qq = [ph0], q
    for _ in range(nrep):
        qq = stepper(qq, nst)
        ph, a = phase(qq)
        phs.append(ph)
    d = np.unwrap(np.array(phs))
    return d[-1] - d[0], a / a0, qq


@pytest.mark.parametrize("eqs,dt", [("HEVE", 0.1), ("HEVI", 0.1)])
def test_lamb_wave_speed(eqs, dt):
    """A Lamb wave (p' ~ exp(-z/(gamma H)) cos kx, w' = 0) over 0.75 of its period: phase speed
    sqrt(gamma R T) to 1e-5, amplitude within 1e-4, w' stays below 1e-6 of u'."""
    case = ps.lamb_case(eqs=eqs)
    q, b = ps.lamb_state(case)
    o = make(case)
    o.set_base_state(b["dens_hyd"], b["pres_hyd"])
    c = ps.lamb_speed(case)
    k = 2.0 * np.pi / (case.dom[1] - case.dom[0])
    nst = int(round(0.25 * 2.0 * np.pi / (c * k) / dt))
    if eqs == "HEVE":
        step = lambda s, n: o.step_heve(s, dt, n)  # noqa: E731
    else:
        step = lambda s, n: o.step_hevi(s, dt, n, max_iter=20, tol=1e-12)[0]  # noqa: E731
    dph, amp, q1 = _phase_run(step, lambda s: ps.lamb_phase(case, s, b), q, 3, nst)
    cnum = -dph / (k * 3 * nst * dt)
    assert abs(cnum / c - 1.0) <= 1e-5, (cnum, c)
    assert abs(amp - 1.0) <= 1e-4, amp
    assert np.max(np.abs(q1[3])) <= 1e-6 * np.max(np.abs(q1[1]))


@pytest.mark.parametrize("eqs,dt", [("HEVE", 0.05), ("HEVI", 0.05)])
def test_vertical_acoustic_frequency(eqs, dt):
    """The standing acoustic mode between the lids (no gravity) over 0.75 of its period: HEVE at
    c pi / Z to 1e-6; HEVI (ARK232, second order) to 1e-5."""
    case = ps.vacoustic_case(eqs=eqs)
    q, b = ps.vacoustic_state(case)
    o = make(case)
    o.set_base_state(b["dens_hyd"], b["pres_hyd"])
    om, _ = ps.vacoustic_omega(case)
    nst = int(round(0.25 * 2.0 * np.pi / om / dt))
    if eqs == "HEVE":
        step = lambda s, n: o.step_heve(s, dt, n)  # noqa: E731
    else:
        step = lambda s, n: o.step_hevi(s, dt, n, max_iter=20, tol=1e-12)[0]  # noqa: E731
    dph, amp, _ = _phase_run(step, lambda s: ps.vacoustic_phase(case, s, b), q, 3, nst)
    onum = dph / (3 * nst * dt)
    assert abs(onum / om - 1.0) <= (1e-6 if eqs == "HEVE" else 1e-5), (onum, om)
    assert abs(amp - 1.0) <= 1e-5, amp


def ark232_stability(z):
    """Stability function of ARK232's implicit tableau (first stage explicit, then gamma, gamma;
    delta, delta, gamma; stiffly accurate) for y' = lambda y, z = lambda dt."""
    g, d = 1.0 - 1.0 / np.sqrt(2.0), 1.0 / (2.0 * np.sqrt(2.0))
    y2 = (1.0 + g * z) / (1.0 - g * z)
    return (1.0 + d * z + d * z * y2) / (1.0 - g * z)


@pytest.mark.parametrize("dt", [0.25, 0.5])
def test_hevi_vertical_acoustic_at_large_courant_number(dt):
    """Vertical Courant number 2 to 4 (250 m elements; HEVE blows up at these steps): HEVI's
    phase per step and amplitude equal ARK232's implicit stability function R(i w dt) (phase to
    1e-6 relative, amplitude to 1e-5), not the exact w dt they differ from by 0.3 to 1.2 %."""
    case = replace(ps.vacoustic_case(eqs="HEVI", Ztop=1000.0), dom=(0.0, 1e5, 0.0, 1e5, 0.0, 1000.0))
    q, b = ps.vacoustic_state(case)
    o = make(case)
    o.set_base_state(b["dens_hyd"], b["pres_hyd"])
    om, _ = ps.vacoustic_omega(case)
    dph, amp, _ = _phase_run(lambda s, n: o.step_hevi(s, dt, n, max_iter=20, tol=1e-13)[0],
                             lambda s: ps.vacoustic_phase(case, s, b), q, 8, 2)
    r = ark232_stability(1j * om * dt)
    assert abs(dph / 16 / np.angle(r) - 1.0) <= 1e-6, (dph / 16, np.angle(r), om * dt)
    assert abs(amp / abs(r) ** 16 - 1.0) <= 1e-5, (amp, abs(r) ** 16)
    qe = o.step_heve(q, dt, 16)
    assert not all(np.isfinite(a).all() for a in qe)  # the explicit scheme cannot take this step


@pytest.mark.parametrize("eqs", ["HEVE", "HEVI"])
def test_conservation(eqs):
    """Twenty steps of a perturbed flow with wind (modal filter on): the integrals of DDENS, MOMX,
    MOMY and DRHOT change by at most 1e-12 of the L1 size of the deviation fields and of the
    horizontal momentum while the fields change by O(1)."""
    if eqs == "HEVE":
        case, dt = replace(cases.C1().scaled(4, 4, 4), u0=10.0, v0=-5.0), 0.02
    else:
        case, dt = cases.C2().scaled(3, 3, 4), 0.04
    q, b = cases.initial_state(case)
    rng = np.random.default_rng(2)
    sc = [1e-4 * b["dens_hyd"], 0.5, 0.5, 0.5, 0.03]
    q = [q[v] + sc[v] * rng.standard_normal(q[v].shape) for v in range(5)]
    o = make(case)
    o.set_base_state(b["dens_hyd"], b["pres_hyd"])
    I0, A0 = ps.integrals(case, q)
    q1 = o.step_heve(q, dt, 20) if eqs == "HEVE" else o.step_hevi(q, dt, 20, max_iter=20, tol=1e-10)[0]
    I1, _ = ps.integrals(case, q1)
    assert np.max(np.abs(I1 - I0) / A0) <= 1e-12, (I1 - I0) / A0
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
    """FElib's single linearised solve (cal_vi, max_iter = 1, guess var0) is one Newton step of
    P - q* - impl_fac A(P) = 0: it equals the step built from a central-difference Jacobian of the
    oracle's implicit operator and a dense solve, to 1e-9 of the step (the difference quotients
    are accurate to ~1e-11).  This pins construct_matbnd, block-Thomas and the block LU."""
    case, b, qs, z0, scales, impl = newton_case(name)
    o = make(case)
    o.set_base_state(b["dens_hyd"], b["pres_hyd"])
    P1 = ps.newton_step_fd(case, o.vi_operator, qs, z0, impl, scales)
    tend = o.cal_vi(qs, z0, impl, 0.1, max_iter=1)
    Po = [qs[v] + impl * tend[v] for v in range(5)]
    err = [float(np.linalg.norm(Po[v] - P1[v]) / np.linalg.norm(P1[v] - z0[v])) for v in range(5)]
    assert max(err) <= 1e-9, err


@pytest.mark.parametrize("name", ["p3", "p7"])
def test_converged_solve_satisfies_the_implicit_equation(name):
    """The iterated solve (tol 1e-13) returns P with P - q* - impl_fac A(P) = 0 for the operator
    evaluated on its own: residual below 1e-12 of each variable's scale."""
    case, b, qs, z0, scales, impl = newton_case(name)
    o = make(case)
    o.set_base_state(b["dens_hyd"], b["pres_hyd"])
    tend, nf, _ = o.cal_vi(qs, z0, impl, 0.1, max_iter=30, tol=1e-13, want_iters=True)
    assert nf == 0
    P = [qs[v] + impl * tend[v] for v in range(5)]
    A = o.vi_operator(P, z0)
    res = [scaled_max(P[v] - qs[v] - impl * A[v], scales[v]) for v in range(5)]
    assert max(res) <= 1e-12, res
