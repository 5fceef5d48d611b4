"""The mixed-precision fused HEVI path (FP32 explicit arithmetic on deviations, FP64 Newton
residual / update / RK accumulation) against the FP64 references.

Tolerance: relative L2 per variable <= 1e-6 against the FP64 oracle / the FP64 GPU path
(the precision-form bar), with the denominator floors of test_gpu_parity.state_floors.
"""
import numpy as np
import pytest

from conftest import have_gpu

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not have_gpu(), reason="needs a CUDA GPU")]

import oracle as orc  # noqa: E402
from fedg import cases  # noqa: E402
from fedg import lib as fl  # noqa: E402
from test_gpu_parity import VARS, relerr, state_floors, to_np  # noqa: E402

TOL = 1e-6


def full_errors(got, ref, b):
    """rel L2 per variable of the full fields DENS, MOMX, MOMY, MOMZ, RHOT (the variables the
    precision bar is stated on): DENS = DENS_hyd + DDENS, RHOT = THERM_hyd + DRHOT.  The momentum
    components are measured against at least 1 m/s of hydrostatic momentum, so a component that
    is still near zero (MOMY, MOMZ early in a run) does not turn roundoff into an O(1) ratio."""
    add = [b["dens_hyd"], 0.0, 0.0, 0.0, b["therm_hyd"]]
    mfloor = float(np.linalg.norm(b["dens_hyd"]))
    out = []
    for v in range(5):
        r = ref[v] + add[v]
        den = np.linalg.norm(r) if v in (0, 4) else max(np.linalg.norm(r), mfloor)
        out.append(float(np.linalg.norm(got[v] - ref[v]) / max(den, 1e-300)))
    return out


def report(tag, got, ref, b):
    fe = full_errors(got, ref, b)
    de = [relerr(g, r, f) for g, r, f in zip(got, ref, state_floors(b))]
    print(f"\n[{tag}] full-field rel L2 " + " ".join(f"{n}={e:.2e}" for n, e in zip(("DENS", "MOMX", "MOMY", "MOMZ", "RHOT"), fe))
          + " | deviation rel L2 " + " ".join(f"{n}={e:.2e}" for n, e in zip(VARS, de)))
    return fe, de


@pytest.mark.parametrize("name,case,dt,nst", [
    ("p7_C2_4x4x4", cases.C2().scaled(4, 4, 4), 0.04, 10),
    ("p3_C1", cases.C1(), 0.02, 20),
    ("p7_C5_4x4x8", cases.C5().scaled(4, 4, 8), 0.005, 10),
])
def test_mixed_vs_oracle(name, case, dt, nst):
    q, b = cases.initial_state(case)
    o = orc.Oracle(case.porder, case.NeX, case.NeY, case.NeZ, case.dom)
    o.set_base_state(b["dens_hyd"], b["pres_hyd"])
    ref, rfail, rits = o.step_hevi(q, dt, nst, max_iter=20, tol=1e-10)
    ctx = fl.Context(case)
    ctx.set_base_state(b["dens_hyd"], b["pres_hyd"], b["therm_hyd"])
    qd = [ctx.tensor(a) for a in q]
    nfail, its = ctx.update(qd, nst, eqs=fl.HEVI, prec=fl.PREC_MIXED, dt=dt, max_iter=20, tol=1e-10)
    fe, de = report(name, to_np(qd), ref, b)
    assert nfail == 0 and rfail == 0
    assert max(fe) < TOL, fe
    assert max(de) < 1e-4, de
    assert 1.0 <= its <= 3.0


def test_mixed_vs_fp64_gpu_long():
    """300 HEVI steps of the p=3 bubble (6 s simulated) side by side with the FP64 GPU path."""
    case = cases.C1()
    q, b = cases.initial_state(case)
    ctx = fl.Context(case)
    ctx.set_base_state(b["dens_hyd"], b["pres_hyd"], b["therm_hyd"])
    q64 = [ctx.tensor(a) for a in q]
    qmx = [ctx.tensor(a) for a in q]
    dt = 0.02
    for _ in range(3):
        f64, _ = ctx.update(q64, 100, eqs=fl.HEVI, prec=fl.PREC_FP64, dt=dt, max_iter=20, tol=1e-10)
        fmx, _ = ctx.update(qmx, 100, eqs=fl.HEVI, prec=fl.PREC_MIXED, dt=dt, max_iter=20, tol=1e-10)
        assert f64 == 0 and fmx == 0
    fe, de = report("C1 300 steps", to_np(qmx), to_np(q64), b)
    assert max(fe) < TOL, fe
    assert max(de) < 1e-4, de


def test_mixed_rejects_heve_and_low_order():
    case = cases.C1()
    q, b = cases.initial_state(case)
    ctx = fl.Context(case)
    ctx.set_base_state(b["dens_hyd"], b["pres_hyd"], b["therm_hyd"])
    qd = [ctx.tensor(a) for a in q]
    with pytest.raises(fl.FedgError):
        ctx.update(qd, 1, eqs=fl.HEVE, prec=fl.PREC_MIXED, dt=0.02)
    c2 = cases.C1().scaled(2, 2, 2, porder=2)
    q2, b2 = cases.initial_state(c2)
    ctx2 = fl.Context(c2)
    ctx2.set_base_state(b2["dens_hyd"], b2["pres_hyd"], b2["therm_hyd"])
    with pytest.raises(fl.FedgError):
        ctx2.update([ctx2.tensor(a) for a in q2], 1, eqs=fl.HEVI, prec=fl.PREC_MIXED, dt=0.02)


def test_tensor_core_wait_limit_reports_error_and_context_recovers():
    """The FP32 mode's stage kernels differentiate the fluxes on the tensor cores and wait on the MMA
    barrier with a bounded poll count.  With a limit of zero polls every wait runs out at once: the
    kernels drain their MMAs with the full limit, raise the error flag, and fedg_update returns < 0
    with the error text; with the default limit restored the same context steps normally."""
    import torch

    case = cases.C2().scaled(2, 2, 4)
    q, b = cases.initial_state(case)
    ctx = fl.Context(case)
    ctx.set_base_state(b["dens_hyd"], b["pres_hyd"], b["therm_hyd"])
    qd = [ctx.tensor(a) for a in q]
    ctx.set_wait_limit(0)
    with pytest.raises(fl.FedgError, match="tensor-core contraction timed out"):
        ctx.update(qd, 1, prec=fl.PREC_MIXED, dt=0.04, max_iter=20, tol=1e-10)
    torch.cuda.synchronize()
    ctx.set_wait_limit(1 << 20)
    qd = [ctx.tensor(a) for a in q]
    nf, _ = ctx.update(qd, 1, prec=fl.PREC_MIXED, dt=0.04, max_iter=20, tol=1e-10)
    assert nf == 0
    assert all(bool(torch.isfinite(t).all()) for t in qd)
