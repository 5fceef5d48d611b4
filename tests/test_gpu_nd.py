"""GPU parity of the numerical diffusion (FElib's hyperdiffusion filter,
FElib/src/fluid_dyn_solver/scale_atm_dyn_dgm_nonhydro3d_numdiff.F90:214-721 with the lid values of
..._dgm_bnd.F90:370-508) and of the sponge layer (..._dgm_spongelayer.F90:134-219) against the FP64
CPU oracle, through the C ABI.

Tolerance: the change each call makes to a field, relative (max norm) to the largest change, 1e-11
(FP64 on both sides; only the summation order inside the contractions differs); sponge 1e-14.
"""
import numpy as np
import pytest

from conftest import have_gpu

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not have_gpu(), reason="needs a CUDA GPU")]

import oracle as orc  # noqa: E402
from fedg import cases  # noqa: E402
from fedg import lib as fl  # noqa: E402

VARS = ("DDENS", "MOMX", "MOMY", "MOMZ", "DRHOT")


def setup(case, seed):
    q, b = cases.initial_state(case)
    rng = np.random.default_rng(seed)
    sc = [1e-3 * b["dens_hyd"], 2.0, 2.0, 1.0, 0.3]
    q = [q[v] + sc[v] * rng.standard_normal(q[v].shape) for v in range(5)]
    o = orc.Oracle(case.porder, case.NeX, case.NeY, case.NeZ, case.dom, grav=case.grav)
    o.set_base_state(b["dens_hyd"], b["pres_hyd"])
    ctx = fl.Context(case)
    ctx.set_base_state(b["dens_hyd"], b["pres_hyd"], b["therm_hyd"])
    return o, ctx, q, b


@pytest.mark.parametrize("porder,ne", [(3, (4, 3, 4)), (7, (2, 2, 3)), (2, (3, 4, 3))])
@pytest.mark.parametrize("nlap", [1, 2, 3])
def test_numdiff_apply(porder, ne, nlap):
    case = cases.C1().scaled(*ne, porder=porder)
    o, ctx, q, b = setup(case, seed=10 + nlap)
    coef = {1: 2.0e2, 2: 5.0e5, 3: 1.0e9}[nlap]
    ref = o.numdiff_apply(q, nlap, coef, 0.5 * coef, 0.01)
    qd = [ctx.tensor(a) for a in q]
    ctx.numdiff_apply(qd, nlap, coef, 0.5 * coef, 0.01)
    for v in range(5):
        got = qd[v].cpu().numpy()
        dref = ref[v] - q[v]
        err = np.max(np.abs((got - q[v]) - dref)) / max(np.max(np.abs(dref)), 1e-300)
        assert err < 1e-11, (VARS[v], err)


def test_sponge_add_tend():
    case = cases.C1().scaled(3, 3, 8)
    o, ctx, q, b = setup(case, seed=3)
    rng = np.random.default_rng(4)
    tend = [rng.standard_normal(o.shape) for _ in range(3)]
    mom = [q[1], q[2], q[3]]
    for hv in (False, True):
        ref = o.sponge_add_tend(tend, mom, 20.0, 600.0, hv)
        td = [ctx.tensor(a) for a in tend]
        ctx.sponge_add_tend(td, [ctx.tensor(a) for a in mom], 20.0, 600.0, hv)
        for d in range(3):
            got = td[d].cpu().numpy()
            assert np.max(np.abs(got - ref[d])) <= 1e-14 * max(1.0, np.max(np.abs(ref[d]))), (d, hv)


@pytest.mark.parametrize("hevi", [0, 1])
def test_update_with_sponge(hevi):
    """fedg_update (FP64) with the sponge layer on (fedg_update_set_sponge) against the oracle's steps
    with the same sponge: whole-step parity bar 1e-9"""
    case = cases.C2().scaled(2, 2, 4) if hevi else cases.C1().scaled(3, 3, 4)
    dt = 0.04 if hevi else 0.02
    o, ctx, q, b = setup(case, seed=21)
    ztop = case.dom[5]
    o.set_sponge(50 * dt, 0.5 * ztop, True)
    ctx.set_sponge(50 * dt, 0.5 * ztop, True)
    if hevi:
        ref, _, _ = o.step_hevi(q, dt, 2, max_iter=1)
    else:
        ref = o.step_heve(q, dt, 2)
    qd = [ctx.tensor(a) for a in q]
    ctx.update(qd, 2, eqs=fl.HEVI if hevi else fl.HEVE, dt=dt, max_iter=1)
    o.set_sponge(0.0)
    ctx.set_sponge(0.0)
    dn = np.linalg.norm(b["dens_hyd"])
    floors = [1e-6 * dn, dn, dn, dn, 1e-6 * np.linalg.norm(b["therm_hyd"])]
    for v in range(5):
        got = qd[v].cpu().numpy()
        e = np.linalg.norm(got - ref[v]) / max(np.linalg.norm(ref[v]), floors[v])
        assert e < 1e-9, (VARS[v], e)
    # and the sponge did something: the same steps without it differ
    ref0 = o.step_hevi(q, dt, 2, max_iter=1)[0] if hevi else o.step_heve(q, dt, 2)
    assert np.max(np.abs(ref0[3] - ref[3])) > 1e-6 * max(1.0, np.max(np.abs(ref[3])))


@pytest.mark.parametrize("eqs,prec,bar", [("HEVI", "pair", 1e-9), ("HEVE", "pair", 1e-9), ("HEVI", "mixed", 1e-6)])
def test_update_with_sponge_fast_paths(eqs, prec, bar):
    """The float-pair and FP32 update paths with the sponge layer (applied inside their stage
    kernels) against the oracle's converged steps with the same sponge; full fields, momentum
    against at least 1 m/s of hydrostatic momentum"""
    hevi = eqs == "HEVI"
    case = cases.C2().scaled(2, 2, 4) if hevi else cases.C1().scaled(3, 3, 4)
    dt = 0.04 if hevi else 0.02
    o, ctx, _, b = setup(case, seed=22)
    q, _ = cases.initial_state(case)  # unperturbed: the FP32 mode's bar is for smooth states
    ztop = case.dom[5]
    o.set_sponge(50 * dt, 0.5 * ztop, True)
    ctx.set_sponge(50 * dt, 0.5 * ztop, True)
    p = fl.PREC_PAIR if prec == "pair" else fl.PREC_MIXED
    qd = [ctx.tensor(a) for a in q]
    if hevi:
        ref, rfail, _ = o.step_hevi(q, dt, 3, max_iter=30, tol=1e-13)
        nf, _ = ctx.update(qd, 3, eqs=fl.HEVI, prec=p, dt=dt, max_iter=30, tol=1e-13 if prec == "pair" else 1e-10)
        assert rfail == 0 and nf == 0
    else:
        ref = o.step_heve(q, dt, 3)
        ctx.update(qd, 3, eqs=fl.HEVE, prec=p, dt=dt)
    o.set_sponge(0.0)
    ctx.set_sponge(0.0)
    dn = np.linalg.norm(b["dens_hyd"])
    hyd = [b["dens_hyd"], 0.0, 0.0, 0.0, b["therm_hyd"]]
    errs = [float(np.linalg.norm(g.cpu().numpy() - r) / max(np.linalg.norm(r + h), dn)) for g, r, h in zip(qd, ref, hyd)]
    assert max(errs) < bar, dict(zip(VARS, errs))


@pytest.mark.parametrize("porder,ne", [(3, (4, 3, 4)), (7, (2, 2, 3)), (2, (3, 4, 3))])
@pytest.mark.parametrize("nlap", [1, 2, 3])
def test_numdiff_apply_pair(porder, ne, nlap):
    """the float-pair passes (FEDG_PREC_PAIR) against the FP64 oracle: the change of each field,
    relative to the largest change, <= 1e-10 (FP64-class pairs)"""
    case = cases.C1().scaled(*ne, porder=porder)
    o, ctx, q, b = setup(case, seed=30 + nlap)
    coef = {1: 2.0e2, 2: 5.0e5, 3: 1.0e9}[nlap]
    ref = o.numdiff_apply(q, nlap, coef, 0.5 * coef, 0.01)
    qd = [ctx.tensor(a) for a in q]
    ctx.numdiff_apply(qd, nlap, coef, 0.5 * coef, 0.01, prec=fl.PREC_PAIR)
    for v in range(5):
        got = qd[v].cpu().numpy()
        dref = ref[v] - q[v]
        err = np.max(np.abs((got - q[v]) - dref)) / max(np.max(np.abs(dref)), 1e-300)
        assert err < 1e-10, (VARS[v], err)
