"""GPU parity of the tracer-advection path against the FP64 CPU oracle, through the C ABI.

Restated routines: FElib/src/fluid_dyn_solver/scale_atm_dyn_dgm_trcadvect3d_heve.F90 (Rusanov
coefficients, mass-flux averaging, FCT coefficient, tendency, TMAR), the tracer modal filter
(..._dgm_modalfilter.F90:232-270) and one tracer's RK steps (..._driver_trcadv3d.F90:420-545,
scale_timeint_rk.F90:1390-1498).

Tolerances (FP64 on both sides; only the summation order of the element and face integrals
differs): single operator calls 1e-13 relative (max norm against the field's max); whole tracer
steps 1e-12 relative L2.
"""
import numpy as np
import pytest

from conftest import have_gpu

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not have_gpu(), reason="needs a CUDA GPU")]

import oracle as orc  # noqa: E402
from fedg import cases  # noqa: E402
from fedg import lib as fl  # noqa: E402

OP_TOL = 1e-13
STEP_TOL = 1e-12


def rel_max(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


def rel_l2(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300))


def setup(case, seed=None, wobble=0.0):
    """Oracle and GPU context with the case's base state, its state q (uniform wind) and the
    initial tracer; wobble > 0 adds a seeded divergent perturbation to the momentum and DDENS."""
    q, b = cases.initial_state(case)
    if wobble:
        rng = np.random.default_rng(seed)
        for v, s in ((0, 1e-3 * b["dens_hyd"]), (1, 3.0), (2, 3.0), (3, 1.0)):
            q[v] = q[v] + wobble * s * rng.standard_normal(q[v].shape)
    o = orc.Oracle(case.porder, case.NeX, case.NeY, case.NeZ, case.dom, grav=case.grav)
    o.set_base_state(b["dens_hyd"], b["pres_hyd"])
    ctx = fl.Context(case)
    ctx.set_base_state(b["dens_hyd"], b["pres_hyd"], b["therm_hyd"])
    Q = cases.tracer_state(case) if case.tracer else np.zeros_like(q[0])
    return o, ctx, q, b, Q


def np_(t):
    return t.cpu().numpy()


def t1(ne=(6, 6, 3), porder=None):
    return cases.T1().scaled(*ne, porder=porder)


@pytest.mark.parametrize("porder", [3, 7])
def test_alphdens_advtest(porder):
    case = t1((4, 4, 3), porder)
    o, ctx, q, b, Q = setup(case, seed=1, wobble=1.0)
    aM, aP = o.trc_alphdens_advtest(q[0], q[1], q[2], q[3])
    qd = [ctx.tensor(a) for a in q]
    gM, gP = ctx.trc_alphdens_advtest(qd[0], qd[1], qd[2], qd[3])
    assert rel_max(np_(gM), aM) < OP_TOL and rel_max(np_(gP), aP) < OP_TOL


@pytest.mark.parametrize("hevi", [0, 1])
def test_save_massflux_three_stages(hevi):
    """three dynamics stages with weights (1/6, 1/6, 2/3) accumulated on the GPU and in the oracle;
    DPRES passed in for stages 1-2 and formed from DRHOT for stage 3"""
    case = cases.C1().scaled(4, 4, 3)
    o, ctx, q, b, _ = setup(case, seed=2, wobble=1.0)
    mf_o = [np.zeros(o.shape) for _ in range(3)]
    aM_o, aP_o = np.zeros(o.face_shape), np.zeros(o.face_shape)
    mf_g = [ctx.empty() for _ in range(3)]
    aM_g, aP_g = ctx.empty_face(), ctx.empty_face()
    rng = np.random.default_rng(5)
    for s, w in enumerate((1 / 6, 1 / 6, 2 / 3), start=1):
        qs = [a + (0.1 * s) * rng.standard_normal(a.shape) * (1e-3 * b["dens_hyd"] if v in (0,) else 1.0)
              for v, a in enumerate(q)]
        _, dp = o.drhot2pres(qs[4])
        o.trc_save_massflux(s, qs, w, w * 0.9, hevi, mf_o, aM_o, aP_o, dpres=dp if s < 3 else None)
        qd = [ctx.tensor(a) for a in qs]
        dpd = ctx.tensor(dp) if s < 3 else None
        ctx.trc_save_massflux(s, qd, w, w * 0.9, hevi, mf_g, aM_g, aP_g, dpres=dpd)
    for d in range(3):
        assert rel_max(np_(mf_g[d]), mf_o[d]) < OP_TOL
    assert rel_max(np_(aM_g), aM_o) < 1e-12 and rel_max(np_(aP_g), aP_o) < 1e-12


@pytest.mark.parametrize("porder", [3, 7])
def test_fct_coef(porder):
    case = t1((4, 4, 3), porder)
    o, ctx, q, b, Q = setup(case)
    mf = [q[1], q[2], q[3]]
    aM, aP = o.trc_alphdens_advtest(q[0], q[1], q[2], q[3])
    qd = [ctx.tensor(a) for a in q]
    mfd = [qd[1], qd[2], qd[3]]
    aMd, aPd = ctx.tensor(aM), ctx.tensor(aP)
    # smooth positive tracer: coefficient 1 almost everywhere
    Qs = Q + 0.1
    ref = o.trc_fct_coef(Qs, mf, aM, aP, q[0], q[0], 0.0, case.dt)
    got = np_(ctx.trc_fct_coef(ctx.tensor(Qs), mfd, aMd, aPd, qd[0], qd[0], 0.0, case.dt))
    assert np.max(np.abs(got - ref)) < 1e-13
    # two loaded elements in an empty domain and a step 400x longer than the stable one, so that
    # their outflow exceeds their mass: coefficients strictly inside (0, 1)
    Qb = np.zeros(o.shape)
    Qb[5] = 1.0
    Qb[6] = 0.02
    ref = o.trc_fct_coef(Qb, mf, aM, aP, q[0], q[0], 0.5, 400 * case.dt)
    got = np_(ctx.trc_fct_coef(ctx.tensor(Qb), mfd, aMd, aPd, qd[0], qd[0], 0.5, 400 * case.dt))
    assert np.max(np.abs(got - ref)) < 1e-13
    assert ((ref > 0) & (ref < 1)).any()


@pytest.mark.parametrize("porder", [3, 7])
@pytest.mark.parametrize("with_fct", [False, True])
def test_cal_tend(porder, with_fct):
    case = t1((4, 4, 3), porder)
    o, ctx, q, b, Q = setup(case, seed=3, wobble=0.5)
    mf = [q[1], q[2], q[3]]
    aM, aP = o.trc_alphdens_advtest(q[0], q[1], q[2], q[3])
    rng = np.random.default_rng(4)
    rhoq = 1e-4 * rng.standard_normal(o.shape)
    fct = o.trc_fct_coef(Q, mf, aM, aP, q[0], q[0], 0.0, 400 * case.dt) if with_fct else None
    ref = o.trc_cal_tend(Q, mf, aM, aP, fct if with_fct else np.ones(o.shape), rhoq)
    qd = [ctx.tensor(a) for a in q]
    got = np_(ctx.trc_cal_tend(ctx.tensor(Q), [qd[1], qd[2], qd[3]], ctx.tensor(aM), ctx.tensor(aP),
                               ctx.tensor(fct) if with_fct else None, ctx.tensor(rhoq)))
    assert rel_max(got, ref) < 1e-12


@pytest.mark.parametrize("porder", [3, 7])
def test_tmar_and_filter(porder):
    case = t1((4, 4, 3), porder)
    o, ctx, q, b, Q = setup(case, seed=6, wobble=0.5)
    rng = np.random.default_rng(7)
    Qn = Q + 0.05 * rng.standard_normal(o.shape)  # negative undershoots to truncate
    ref = o.trc_tmar(Qn, q[0])
    got = np_(ctx.trc_tmar(ctx.tensor(Qn), ctx.tensor(q[0])))
    pos = (((b["dens_hyd"] + q[0]) * Qn).sum(axis=1) > 0)
    assert rel_max(got[pos], ref[pos]) < 1e-13
    ref = o.trc_filter(Qn, q[0], 0.6, 30.0, 12, 0.5, 20.0, 8)
    got = np_(ctx.trc_modalfilter(ctx.tensor(Qn), ctx.tensor(q[0]), 0.6, 30.0, 12, 0.5, 20.0, 8))
    assert rel_max(got, ref) < 1e-13


@pytest.mark.parametrize("porder,ne,steps", [(3, (6, 6, 3), 20), (7, (3, 3, 2), 6), (2, (5, 4, 3), 10)])
@pytest.mark.parametrize("limiter", [True, False])
def test_update_advection_test(porder, ne, steps, limiter):
    """the advection-test configuration (ONLY_TRACERADV_FLAG): fixed wind and density"""
    case = t1(ne, porder)
    o, ctx, q, b, Q = setup(case)
    mf = [q[1], q[2], q[3]]
    aM, aP = o.trc_alphdens_advtest(q[0], q[1], q[2], q[3])
    ref = o.trc_step(Q, mf, aM, aP, q[0], q[0], case.dt, nsteps=steps, limiter=limiter, tmar=True)
    qd = [ctx.tensor(a) for a in q]
    Qd = ctx.tensor(Q)
    ctx.trc_update(Qd, [qd[1], qd[2], qd[3]], ctx.tensor(aM), ctx.tensor(aP), qd[0], qd[0], case.dt, nsteps=steps,
                   limiter=limiter, tmar=True)
    got = np_(Qd)
    assert rel_l2(got, ref) < STEP_TOL
    assert np.max(np.abs(got - Q)) > 1e-3  # the tracer moved
    if limiter:
        assert got.min() >= -1e-14


def test_update_coupled_densities_filter_and_source():
    """the coupled configuration: time-averaged mass flux and Rusanov coefficients of three dynamics
    stages, DDENS_TRC != DDENS0_TRC != DDENS, a physics source RHOQ_tp and the tracer filter"""
    case = cases.C1().scaled(4, 4, 3)
    case = cases.replace(case, tracer=dict(qmax=2.0, rx=200.0, ry=200.0, rz=150.0, xc=250.0, yc=250.0, zc=180.0))
    o, ctx, q, b, Q = setup(case, seed=8, wobble=0.3)
    rng = np.random.default_rng(9)
    mf_o = [np.zeros(o.shape) for _ in range(3)]
    aM, aP = np.zeros(o.face_shape), np.zeros(o.face_shape)
    for s, w in enumerate((1 / 6, 1 / 6, 2 / 3), start=1):
        qs = [a.copy() for a in q]
        qs[1] = qs[1] + 2.0 * s
        o.trc_save_massflux(s, qs, w, w, 0, mf_o, aM, aP)
    ddens0 = q[0]
    ddens_trc = q[0] + 1e-4 * b["dens_hyd"] * rng.standard_normal(o.shape)
    ddens = q[0] + 2e-4 * b["dens_hyd"] * rng.standard_normal(o.shape)
    rhoq = 1e-5 * np.abs(rng.standard_normal(o.shape))
    filt = dict(etac_h=2.0 / 3.0, alpha_h=36.0, ord_h=16, etac_v=0.5, alpha_v=30.0, ord_v=12)
    ref = o.trc_step(Q, mf_o, aM, aP, ddens_trc, ddens0, 0.02, nsteps=8, ddens=ddens, rhoq_tp=rhoq, limiter=True,
                     tmar=True, filter=filt)
    Qd = ctx.tensor(Q)
    ctx.trc_update(Qd, [ctx.tensor(m) for m in mf_o], ctx.tensor(aM), ctx.tensor(aP), ctx.tensor(ddens_trc),
                   ctx.tensor(ddens0), 0.02, nsteps=8, ddens=ctx.tensor(ddens), rhoq_tp=ctx.tensor(rhoq),
                   limiter=True, tmar=True, filter=filt)
    assert rel_l2(np_(Qd), ref) < STEP_TOL


def test_update_properties_at_size():
    """p=7, 24x24x8 elements (2.4 M nodes): without the limiter the exact-mass tracer integral is
    conserved to roundoff; with FCT + TMAR a one-element block stays non-negative."""
    case = t1((24, 24, 8), 7)
    _, ctx, q, b, Q = setup(case)
    o = orc.Oracle(case.porder, 1, 1, 1, (0.0, 1.0, 0.0, 1.0, 0.0, 1.0))
    M1 = np.linalg.inv(o.operators_1d()["Minv"])
    dx, dy, dz = [(case.dom[2 * i + 1] - case.dom[2 * i]) / n for i, n in enumerate((case.NeX, case.NeY, case.NeZ))]

    def mass(Qn):
        f = ((b["dens_hyd"] + q[0]) * Qn).reshape(case.Ne, 8, 8, 8)
        return float(np.einsum("ekji,ia,jb,kc->", f, M1, M1, M1)) * dx * dy * dz / 8

    qd = [ctx.tensor(a) for a in q]
    aM, aP = ctx.trc_alphdens_advtest(qd[0], qd[1], qd[2], qd[3])
    mf = [qd[1], qd[2], qd[3]]
    Qd = ctx.tensor(Q)
    ctx.trc_update(Qd, mf, aM, aP, qd[0], qd[0], case.dt, nsteps=10, limiter=False)
    m0, m1 = mass(Q), mass(np_(Qd))
    assert abs(m1 - m0) < 1e-12 * abs(m0)
    Qb = np.zeros_like(Q)
    Qb[case.NeX * case.NeY * 3 + case.NeX * 5 + 7] = 1.0
    Qbd = ctx.tensor(Qb)
    ctx.trc_update(Qbd, mf, aM, aP, qd[0], qd[0], case.dt, nsteps=10, limiter=True, tmar=True)
    got = np_(Qbd)
    assert got.min() >= -1e-14 and got.max() > 0.01


# ---- the float-pair tracer step (fedg_trc_opts.prec = FEDG_PREC_PAIR) ----
PAIR_TOL = 1e-11  # FP64-class float pairs (relative rounding ~1e-14 per operation) against the FP64 oracle


@pytest.mark.parametrize("porder,ne,steps", [(3, (6, 6, 3), 20), (7, (3, 3, 2), 6), (2, (5, 4, 3), 10)])
@pytest.mark.parametrize("limiter", [True, False])
def test_update_pair_advection_test(porder, ne, steps, limiter):
    case = t1(ne, porder)
    o, ctx, q, b, Q = setup(case)
    mf = [q[1], q[2], q[3]]
    aM, aP = o.trc_alphdens_advtest(q[0], q[1], q[2], q[3])
    ref = o.trc_step(Q, mf, aM, aP, q[0], q[0], case.dt, nsteps=steps, limiter=limiter, tmar=True)
    qd = [ctx.tensor(a) for a in q]
    Qd = ctx.tensor(Q)
    ctx.trc_update(Qd, [qd[1], qd[2], qd[3]], ctx.tensor(aM), ctx.tensor(aP), qd[0], qd[0], case.dt, nsteps=steps,
                   limiter=limiter, tmar=True, prec=fl.PREC_PAIR)
    got = np_(Qd)
    assert rel_l2(got, ref) < PAIR_TOL, rel_l2(got, ref)
    if limiter:
        assert got.min() >= -1e-14


def test_update_pair_coupled_densities_filter_and_source():
    case = cases.C1().scaled(4, 4, 3)
    case = cases.replace(case, tracer=dict(qmax=2.0, rx=200.0, ry=200.0, rz=150.0, xc=250.0, yc=250.0, zc=180.0))
    o, ctx, q, b, Q = setup(case, seed=8, wobble=0.3)
    rng = np.random.default_rng(9)
    mf_o = [np.zeros(o.shape) for _ in range(3)]
    aM, aP = np.zeros(o.face_shape), np.zeros(o.face_shape)
    for s, w in enumerate((1 / 6, 1 / 6, 2 / 3), start=1):
        qs = [a.copy() for a in q]
        qs[1] = qs[1] + 2.0 * s
        o.trc_save_massflux(s, qs, w, w, 0, mf_o, aM, aP)
    ddens0 = q[0]
    ddens_trc = q[0] + 1e-4 * b["dens_hyd"] * rng.standard_normal(o.shape)
    ddens = q[0] + 2e-4 * b["dens_hyd"] * rng.standard_normal(o.shape)
    rhoq = 1e-5 * np.abs(rng.standard_normal(o.shape))
    filt = dict(etac_h=2.0 / 3.0, alpha_h=36.0, ord_h=16, etac_v=0.5, alpha_v=30.0, ord_v=12)
    ref = o.trc_step(Q, mf_o, aM, aP, ddens_trc, ddens0, 0.02, nsteps=8, ddens=ddens, rhoq_tp=rhoq, limiter=True,
                     tmar=True, filter=filt)
    Qd = ctx.tensor(Q)
    ctx.trc_update(Qd, [ctx.tensor(m) for m in mf_o], ctx.tensor(aM), ctx.tensor(aP), ctx.tensor(ddens_trc),
                   ctx.tensor(ddens0), 0.02, nsteps=8, ddens=ctx.tensor(ddens), rhoq_tp=ctx.tensor(rhoq),
                   limiter=True, tmar=True, filter=filt, prec=fl.PREC_PAIR)
    assert rel_l2(np_(Qd), ref) < PAIR_TOL


@pytest.mark.parametrize("hevi", [0, 1])
def test_update_accumulates_tracer_flux(hevi):
    """fedg_update (FP64) with fedg_update_set_tracer_flux: the stage-weighted mass flux, the dynamics'
    Rusanov coefficients, DDENS_TRC and DDENS0_TRC of the last step, against the oracle's dynamics
    step with the same outputs (driver_nonhydro3d.F90:900-935)"""
    case = cases.C2().scaled(2, 2, 3) if hevi else cases.C1().scaled(3, 3, 3)
    dt = 0.04 if hevi else 0.02
    o, ctx, q, b, _ = setup(case, seed=12, wobble=0.5)
    outs_o = [np.zeros(o.shape) for _ in range(3)] + [np.zeros(o.face_shape) for _ in range(2)] + \
             [np.zeros(o.shape) for _ in range(2)]
    o.set_trc_flux(outs_o)
    if hevi:
        ref, _, _ = o.step_hevi(q, dt, 2, max_iter=1)
    else:
        ref = o.step_heve(q, dt, 2)
    o.set_trc_flux(None)
    outs_g = [ctx.empty() for _ in range(3)] + [ctx.empty_face() for _ in range(2)] + [ctx.empty() for _ in range(2)]
    ctx.set_tracer_flux(outs_g)
    qd = [ctx.tensor(a) for a in q]
    ctx.update(qd, 2, eqs=fl.HEVI if hevi else fl.HEVE, dt=dt, max_iter=1)
    ctx.set_tracer_flux(None)
    names = ["MFLX_x", "MFLX_y", "MFLX_z", "alph_M", "alph_P", "DDENS_TRC", "DDENS0_TRC"]
    for nm, g, r in zip(names, outs_g, outs_o):
        e = rel_max(np_(g), r)
        assert e < 1e-10, (nm, e)
    # the dynamics state itself is unchanged by the registration
    assert rel_max(np_(qd[3]), ref[3]) < 1e-9


@pytest.mark.parametrize("eqs,prec,bar", [("HEVI", "pair", 1e-9), ("HEVE", "pair", 1e-9), ("HEVI", "mixed", 1e-6)])
def test_update_tracer_flux_fast_paths(eqs, prec, bar):
    """The float-pair (HEVI and HEVE) and FP32 updates with registered tracer-flux outputs: the
    stage-weighted mass flux and Rusanov coefficients from the stage states they hold as deviations,
    DDENS_TRC written by the fused stage-3 kernel before its modal filter, DDENS0_TRC; against the
    oracle's converged steps with the same outputs.  Maximum error relative to the field's maximum,
    with floors: the mass fluxes against at least 1 m/s of hydrostatic momentum (a component that
    stays near zero, MFLX_y of a flow along x, is not measured against its own roundoff), the DDENS
    fields against the hydrostatic density."""
    hevi = eqs == "HEVI"
    case = cases.C2().scaled(2, 2, 3) if hevi else cases.C1().scaled(3, 3, 3)
    dt = 0.04 if hevi else 0.02
    o, ctx, q, b, _ = setup(case)
    outs_o = [np.zeros(o.shape) for _ in range(3)] + [np.zeros(o.face_shape) for _ in range(2)] + \
             [np.zeros(o.shape) for _ in range(2)]
    o.set_trc_flux(outs_o)
    if hevi:
        ref, rfail, _ = o.step_hevi(q, dt, 2, max_iter=30, tol=1e-13)
        assert rfail == 0
    else:
        ref = o.step_heve(q, dt, 2)
    o.set_trc_flux(None)
    outs_g = [ctx.empty() for _ in range(3)] + [ctx.empty_face() for _ in range(2)] + [ctx.empty() for _ in range(2)]
    ctx.set_tracer_flux(outs_g)
    qd = [ctx.tensor(a) for a in q]
    p = fl.PREC_PAIR if prec == "pair" else fl.PREC_MIXED
    nf, _ = ctx.update(qd, 2, eqs=fl.HEVI if hevi else fl.HEVE, prec=p, dt=dt, max_iter=30,
                       tol=1e-13 if prec == "pair" else 1e-10)
    ctx.set_tracer_flux(None)
    assert nf == 0
    names = ["MFLX_x", "MFLX_y", "MFLX_z", "alph_M", "alph_P", "DDENS_TRC", "DDENS0_TRC"]
    dmax = float(np.max(np.abs(b["dens_hyd"])))
    for nm, g, r in zip(names, outs_g, outs_o):
        g = np_(g)
        floor = dmax if (nm.startswith("DDENS") or nm.startswith("MFLX")) else 0.0
        e = float(np.max(np.abs(g - r))) / max(np.max(np.abs(r)), floor, 1e-300)
        assert e < bar, (nm, e)
