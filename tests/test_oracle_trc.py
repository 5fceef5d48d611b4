"""CPU checks of the tracer-advection oracle (FElib's trcadvect3d_heve + tracer driver restated).

FElib's tests hold no tracer known answers, so the restatement is pinned by properties the
scheme has by construction:

* free-stream preservation: a uniform mixing ratio in a uniform flow has zero tendency
  (trcadvect3d_heve.F90:149-231 with the Rusanov flux of :554-674);
* transport direction and accuracy: a smooth profile in a uniform wind moves with the wind
  (exact solution q(x - u t)) to the discretisation error;
* conservation: without the limiter the tracer mass integral(dens q) of the exact-mass DG
  scheme is conserved to roundoff over steps (periodic x/y, no flux through the slip lids);
* limiter: FCT + TMAR (Light and Durran 2016; :234-340) keep a step profile non-negative
  where the unlimited scheme undershoots, and TMAR keeps each element's LGL-weighted mass;
* mass-flux averaging (save_massflux, :343-401): the stage-weighted sums of a steady state
  reproduce its mass flux and Rusanov coefficient.
"""
import numpy as np
import pytest

import oracle as orc
import timeint_ref
from fedg import cases


def _setup(case, nthreads=None):
    q, b = cases.initial_state(case)
    o = orc.Oracle(case.porder, case.NeX, case.NeY, case.NeZ, case.dom, grav=case.grav)
    o.set_base_state(b["dens_hyd"], b["pres_hyd"])
    return o, q, b


def _mass_exact(o, dens, Q):
    """integral of dens*Q with the exact (non-lumped) mass matrix of the tensor-product element"""
    ops = o.operators_1d()
    M1 = np.linalg.inv(ops["Minv"])
    n1 = o.N1
    f = (dens * Q).reshape(o.Ne, n1, n1, n1)  # (ke, k, j, i)
    s = np.einsum("ekji,ia,jb,kc->ekjc", f, M1, M1, M1)  # M applied along i, j, k; then sum
    return float(s.sum())


def _small_t1(ne=(6, 6, 3)):
    return cases.T1().scaled(*ne)


def test_free_stream_preserved():
    case = _small_t1()
    o, q, b = _setup(case)
    ddens = q[0]
    aM, aP = o.trc_alphdens_advtest(ddens, q[1], q[2], q[3])
    Q = np.ones(o.shape)
    fct = np.ones(o.shape)
    t = o.trc_cal_tend(Q, [q[1], q[2], q[3]], aM, aP, fct)
    scale = np.max(np.abs(q[1])) / (case.dom[1] / case.NeX)
    assert np.max(np.abs(t)) < 1e-12 * scale
    Q1 = o.trc_step(Q, [q[1], q[2], q[3]], aM, aP, ddens, ddens, case.dt, nsteps=5)
    assert np.max(np.abs(Q1 - 1.0)) < 1e-13


def test_transport_follows_the_wind():
    """sin profile in x, u = 10 m/s, 8 p=3 elements per wavelength: after 100 s the oracle matches
    sin(2 pi (x - u t)/L) to the p=3 discretisation error, and not the profile moved upwind."""
    case = cases.Case("trc_x", 3, 8, 2, 2, (0.0, 8000.0, 0.0, 2000.0, 0.0, 2000.0), "HEVE", dt=1.0, nsteps=100,
                      base="constPT", grav=0.0, u0=10.0, filter_on=False)
    o, q, b = _setup(case)
    x = b["x"]
    L = case.dom[1]
    Q0 = 1.0 + 0.5 * np.sin(2 * np.pi * x / L)
    aM, aP = o.trc_alphdens_advtest(q[0], q[1], q[2], q[3])
    Q = o.trc_step(Q0, [q[1], q[2], q[3]], aM, aP, q[0], q[0], case.dt, nsteps=100, limiter=False)
    exact = 1.0 + 0.5 * np.sin(2 * np.pi * (x - 10.0 * 100.0) / L)
    wrong = 1.0 + 0.5 * np.sin(2 * np.pi * (x + 10.0 * 100.0) / L)
    err = np.max(np.abs(Q - exact))
    assert err < 2e-3, err
    assert np.max(np.abs(Q - wrong)) > 0.5


def test_mass_conserved_without_limiter():
    case = _small_t1()
    o, q, b = _setup(case)
    dens = b["dens_hyd"] + q[0]
    Q0 = cases.tracer_state(case)
    aM, aP = o.trc_alphdens_advtest(q[0], q[1], q[2], q[3])
    m0 = _mass_exact(o, dens, Q0)
    Q = o.trc_step(Q0, [q[1], q[2], q[3]], aM, aP, q[0], q[0], case.dt, nsteps=20, limiter=False)
    m1 = _mass_exact(o, dens, Q)
    assert abs(m1 - m0) < 1e-13 * abs(m0)
    assert np.max(np.abs(Q - Q0)) > 1e-3  # it did move


def test_limiter_keeps_step_profile_nonnegative():
    """A one-element block of tracer in a fast diagonal wind: the unlimited scheme undershoots,
    FCT + TMAR keep q >= 0 (to roundoff) and TMAR keeps the element's LGL-weighted mass."""
    case = _small_t1((6, 6, 3))
    o, q, b = _setup(case)
    Q0 = np.zeros(o.shape)
    ke = 2 + 6 * 2 + 36 * 1
    Q0[ke] = 1.0
    mf = [q[1], q[2], q[3]]
    aM, aP = o.trc_alphdens_advtest(q[0], q[1], q[2], q[3])
    Qn = o.trc_step(Q0, mf, aM, aP, q[0], q[0], case.dt, nsteps=10, limiter=False)
    Ql = o.trc_step(Q0, mf, aM, aP, q[0], q[0], case.dt, nsteps=10, limiter=True, tmar=True)
    assert Qn.min() < -1e-3
    assert Ql.min() >= -1e-14
    # TMAR alone: element mass with LGL weights is kept, negatives removed
    w = o.operators_1d()["w"]
    w3 = (w[None, None, :] * w[None, :, None] * w[:, None, None]).reshape(-1)
    dens = b["dens_hyd"] + q[0]
    Qt = o.trc_tmar(Qn, q[0])
    m_before = ((dens * Qn) * w3).sum(axis=1)
    m_after = ((dens * Qt) * w3).sum(axis=1)
    pos = m_before > 1e-12
    assert np.allclose(m_after[pos], m_before[pos], rtol=1e-12, atol=0)
    # non-negative wherever the element's mass is (the FCT step is what guarantees that)
    assert Qt[m_before >= 0.0].min() >= 0.0


def test_fct_coefficient_bounds_outflow():
    """calc_fct_coef: 1 where the element holds enough tracer for its outflow, within [0, 1],
    and 0 for an empty element (no mass to give); one value per element."""
    case = _small_t1((6, 6, 3))
    o, q, b = _setup(case)
    mf = [q[1], q[2], q[3]]
    aM, aP = o.trc_alphdens_advtest(q[0], q[1], q[2], q[3])
    Q = np.full(o.shape, 1.0)
    fct = o.trc_fct_coef(Q, mf, aM, aP, q[0], q[0], 0.0, case.dt)
    assert np.all(fct == 1.0)
    Q2 = np.zeros(o.shape)
    Q2[0] = 1.0
    fct2 = o.trc_fct_coef(Q2, mf, aM, aP, q[0], q[0], 0.0, case.dt)
    assert np.all((fct2 >= 0.0) & (fct2 <= 1.0))
    assert np.all(fct2[0] == 1.0) and np.all(fct2[1:] == 0.0)
    assert np.all(fct2 == fct2[:, :1])  # one value per element
    # no flow: the tracer-holding element keeps coefficient 1
    still = o.trc_fct_coef(Q2, [np.zeros(o.shape)] * 3, np.zeros(o.face_shape), np.zeros(o.face_shape), q[0], q[0],
                           0.0, case.dt)
    assert np.all(still[0] == 1.0) and np.all(still[1:] == 0.0)


def test_save_massflux_of_steady_state():
    """Stage weights b = (1/6, 1/6, 2/3) of SSP-RK3 over a steady state give back MOM and the
    dynamics' Rusanov coefficient alpha * dens (alphdens_dyn)."""
    case = cases.C1().scaled(4, 4, 4)
    o, q, b = _setup(case)
    q[1] = q[1] + 3.0 * (b["dens_hyd"] + q[0])
    q[3] = q[3] + 0.5 * np.sin(b["x"] / 100.0) * (b["dens_hyd"] + q[0])
    mf = [np.zeros(o.shape) for _ in range(3)]
    aM, aP = np.zeros(o.face_shape), np.zeros(o.face_shape)
    for s, w in enumerate((1 / 6, 1 / 6, 2 / 3), start=1):
        o.trc_save_massflux(s, q, w, w, 0, mf, aM, aP)
    assert np.allclose(mf[0], q[1], rtol=1e-14, atol=1e-14)
    assert np.allclose(mf[2], q[3], rtol=1e-14, atol=1e-14)
    aM1, aP1 = np.zeros(o.face_shape), np.zeros(o.face_shape)
    m1 = [np.zeros(o.shape) for _ in range(3)]
    o.trc_save_massflux(1, q, 1.0, 1.0, 0, m1, aM1, aP1)
    assert np.allclose(aM, aM1, rtol=1e-14) and np.allclose(aP, aP1, rtol=1e-14)
    # HEVI: no sound speed on the vertical faces -> alpha = |w| there
    aMh, aPh = np.zeros(o.face_shape), np.zeros(o.face_shape)
    o.trc_save_massflux(1, q, 1.0, 1.0, 1, m1, aMh, aPh)
    assert np.all(aMh[:, :4] == aM1[:, :4])
    assert np.all(aMh[:, 4:] < aM1[:, 4:])


def test_tracer_filter_preserves_mean_and_constant():
    case = _small_t1((4, 4, 2))
    o, q, b = _setup(case)
    Q = cases.tracer_state(case) + 0.3
    Qf = o.trc_filter(Q, q[0])
    ones = o.trc_filter(np.ones(o.shape), q[0])
    assert np.max(np.abs(ones - 1.0)) < 1e-14
    dens = b["dens_hyd"] + q[0]
    assert abs(_mass_exact(o, dens, Qf) - _mass_exact(o, dens, Q)) < 1e-13 * _mass_exact(o, dens, Q)
    assert np.max(np.abs(Qf - Q)) > 0.0


def test_ssp3_tables_consistent():
    """the Shu-Osher tables of ERK_SSP_3s3o reproduce the Butcher nodes c = (0, 1, 1/2)"""
    tb = timeint_ref.tables("ERK_SSP_3s3o")
    sig, gam = tb["sig"], tb["gam"]
    ns = tb["nstage"]
    A = np.zeros((ns + 1, ns))
    for i in range(1, ns + 1):
        for j in range(ns):
            A[i, j] = gam[i, j] + sum(sig[i, k] * A[k, j] for k in range(i))
    assert np.allclose(A[:ns].sum(axis=1), tb["c"], atol=1e-15)


# ---- numerical diffusion (nonhydro3d_numdiff.F90) and sponge layer (dgm_spongelayer.F90) ----
def _nd_case(porder=3, ne=(8, 2, 4)):
    return cases.Case("nd", porder, *ne, (0.0, 8000.0, 0.0, 2000.0, 0.0, 4000.0), "HEVE", dt=1.0, nsteps=1,
                      base="constPT", grav=0.0, filter_on=False)


def _nd_setup(case):
    q, b = cases.initial_state(case)
    o = orc.Oracle(case.porder, case.NeX, case.NeY, case.NeZ, case.dom, grav=case.grav)
    o.set_base_state(b["dens_hyd"], b["pres_hyd"])
    return o, q, b


@pytest.mark.parametrize("nlap,porder", [(1, 5), (2, 7)])
def test_numdiff_damps_a_fourier_mode_at_its_rate(nlap, porder):
    """(-1)^(n+1) coef nabla^(2n) on sin(2 pi x / L): one application multiplies the mode by
    1 - coef dt (2 pi / L)^(2n) (uniform density, 8 elements per wavelength).  The iterated
    operator needs the higher order: the one-sided LDG Laplacian's nodal error sits in high modes,
    which the second application amplifies."""
    case = _nd_case(porder=porder)
    o, q, b = _nd_setup(case)
    L = case.dom[1]
    kx = 2 * np.pi / L
    dt = 1.0
    coef = 0.02 / (kx ** (2 * nlap) * dt)  # 2 % damping per application
    q[4] = 0.5 * np.sin(kx * b["x"])
    out = o.numdiff_apply(q, nlap, coef, coef, dt)
    ratio = (out[4] * q[4]).sum() / (q[4] * q[4]).sum()
    assert abs(ratio - (1.0 - 0.02)) < (1e-5 if nlap == 1 else 5e-5), ratio
    # the other variables (uniform momentum in x only, zero elsewhere) do not move
    for v in (0, 1, 2, 3):
        assert np.max(np.abs(out[v] - q[v])) < 1e-12 * max(1.0, np.max(np.abs(q[v])))


def test_numdiff_biharmonic_is_the_laplacian_twice():
    """ND_LAPLACIAN_NUM = 2 applies the one-sided LDG Laplacian twice (apply_numfilter's loop,
    numdiff.F90:313-357), with the sign (-1)^(n+1): B u = -L(L u) for a smooth x-mode"""
    case = _nd_case(porder=3, ne=(8, 2, 2))
    o, q, b = _nd_setup(case)
    u = 0.5 * np.sin(2 * np.pi * b["x"] / case.dom[1])
    q[4] = u
    Lu = o.numdiff_apply(q, 1, 1.0, 1.0, 1.0)[4] - u
    q2 = list(q)
    q2[4] = Lu
    LLu = o.numdiff_apply(q2, 1, 1.0, 1.0, 1.0)[4] - Lu
    Bu = o.numdiff_apply(q, 2, 1.0, 1.0, 1.0)[4] - u
    assert np.max(np.abs(Bu + LLu)) < 1e-5 * np.max(np.abs(LLu))


def test_numdiff_conserves_and_is_dissipative():
    """random fields: the exact-mass integrals of DRHOT and DDENS are kept (zero flux through the
    periodic faces and the lids), and the L2 norm of DRHOT decreases"""
    case = _nd_case(porder=3, ne=(4, 3, 3))
    o, q, b = _nd_setup(case)
    rng = np.random.default_rng(0)
    q[4] = rng.standard_normal(o.shape)
    q[0] = 1e-3 * rng.standard_normal(o.shape)
    q[3] = rng.standard_normal(o.shape)
    ones = np.zeros(o.shape)
    for nlap in (1, 2):
        out = o.numdiff_apply(q, nlap, 1.0e3 if nlap == 1 else 1.0e5, 1.0e3 if nlap == 1 else 1.0e5, 0.05)
        for v in (0, 4):
            m0 = _mass_exact(o, np.ones(o.shape), q[v])
            m1 = _mass_exact(o, np.ones(o.shape), out[v])
            assert abs(m1 - m0) < 1e-12 * np.abs(q[v]).sum() * (o.Np ** 0), (v, m0, m1)
        assert np.linalg.norm(out[4]) < np.linalg.norm(q[4])
    del ones


def test_numdiff_constant_state_unchanged():
    case = _nd_case(porder=3, ne=(3, 3, 3))
    o, q, b = _nd_setup(case)
    q[4] = q[4] + 7.0
    q[1] = 3.0 * (b["dens_hyd"] + q[0])  # constant velocity: MOMX/dens is uniform
    out = o.numdiff_apply(q, 2, 1e5, 1e5, 0.1)
    for v in range(5):
        assert np.max(np.abs(out[v] - q[v])) < 1e-11 * max(1.0, np.max(np.abs(q[v])))


def test_sponge_matches_formula():
    case = _nd_case(porder=3, ne=(2, 2, 6))
    o, q, b = _nd_setup(case)
    rng = np.random.default_rng(1)
    mom = [rng.standard_normal(o.shape) for _ in range(3)]
    tend = [rng.standard_normal(o.shape) for _ in range(3)]
    tau, h = 30.0, 2500.0
    ztop = case.dom[5]
    z = b["z"]
    c = 0.25 / tau * (1.0 + np.where(z - h >= 0, 1.0, -1.0)) * (1.0 - np.cos(np.pi * (z - h) / (ztop - h)))
    for hv in (False, True):
        out = o.sponge_add_tend(tend, mom, tau, h, hv)
        s = 1.0 if hv else 0.0
        assert np.allclose(out[2], tend[2] - c * mom[2], rtol=1e-14, atol=1e-14)
        assert np.allclose(out[0], tend[0] - s * c * mom[0], rtol=1e-14, atol=1e-14)
    assert np.all(c[z < h] == 0.0) and c.max() > 0
