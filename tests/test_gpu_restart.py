"""Restart files through the C ABI (fedg_restart_write / fedg_restart_read): the library's files
and the numpy writer's are the same format, and a run split by a save, a new context and a restore
continues bit for bit, in FElib's FP64 arithmetic and in the float-pair path (whose reference wind
the file carries)."""
import numpy as np
import pytest

from conftest import have_gpu

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not have_gpu(), reason="needs a CUDA GPU")]

from fedg import cases  # noqa: E402
from fedg import lib as fl  # noqa: E402
from fedg import restart as rs  # noqa: E402


def _ctx(case, b):
    ctx = fl.Context(case)
    ctx.set_base_state(b["dens_hyd"], b["pres_hyd"], b["therm_hyd"])
    return ctx


def test_library_and_numpy_files_agree(tmp_path):
    case = cases.C2().scaled(2, 2, 3)
    q, b = cases.initial_state(case)
    ctx = _ctx(case, b)
    qd = [ctx.tensor(a) for a in q]
    ctx.restart_write(tmp_path / "lib.rst", qd, step=7, time=0.28, dt=0.04, scheme="IMEX_ARK232")
    r = rs.read(tmp_path / "lib.rst")
    assert (r.step, r.time, r.dt, r.scheme, r.ref_wind) == (7, 0.28, 0.04, "IMEX_ARK232", None)
    for nm, a in zip(rs.NAMES[:5], q):
        assert np.array_equal(r.fields[nm], a), nm
    for nm, key in (("DENS_hyd", "dens_hyd"), ("PRES_hyd", "pres_hyd"), ("THERM_hyd", "therm_hyd")):
        assert np.array_equal(r.fields[nm], b[key]), nm
    # numpy-written file read by the library
    rng = np.random.default_rng(1)
    r.fields = {nm: a + 1e-4 * rng.standard_normal(a.shape) for nm, a in r.fields.items()}
    r.step, r.scheme = 11, "ERK_SSP_3s3o"
    rs.write(tmp_path / "np.rst", r)
    out = [ctx.empty() for _ in range(5)]
    base = [ctx.empty() for _ in range(3)]
    step, t, dt, scheme = ctx.restart_read(tmp_path / "np.rst", out, base)
    assert (step, t, dt, scheme) == (11, 0.28, 0.04, "ERK_SSP_3s3o")
    for nm, a in zip(rs.NAMES, out + base):
        assert np.array_equal(a.cpu().numpy(), r.fields[nm]), nm


def test_restart_rejects_another_mesh(tmp_path):
    case = cases.C2().scaled(2, 2, 3)
    q, b = cases.initial_state(case)
    ctx = _ctx(case, b)
    ctx.restart_write(tmp_path / "a.rst", [ctx.tensor(a) for a in q])
    other = cases.C2().scaled(2, 2, 4)
    q2, b2 = cases.initial_state(other)
    ctx2 = _ctx(other, b2)
    with pytest.raises(fl.FedgError, match="does not match"):
        ctx2.restart_read(tmp_path / "a.rst", [ctx2.empty() for _ in range(5)])


@pytest.mark.parametrize("eqs,prec,tol", [(fl.HEVI, fl.PREC_FP64, 1e-10), (fl.HEVE, fl.PREC_FP64, 0.0),
                                          (fl.HEVI, fl.PREC_PAIR, 1e-13), (fl.HEVE, fl.PREC_PAIR, 0.0)])
def test_run_split_by_restart_is_bit_exact(tmp_path, eqs, prec, tol):
    """3 + 3 steps in one context == 3 steps, a restart file, a new context, 3 steps."""
    case = cases.C2().scaled(2, 2, 4)
    q, b = cases.initial_state(case)
    dt = 0.04
    opts = dict(eqs=eqs, prec=prec, dt=dt, max_iter=30 if tol else 1, tol=tol)
    ca = _ctx(case, b)
    qa = [ca.tensor(a) for a in q]
    ca.update(qa, 3, **opts)
    ca.update(qa, 3, **opts)
    cb = _ctx(case, b)
    qb = [cb.tensor(a) for a in q]
    cb.update(qb, 3, **opts)
    cb.restart_write(tmp_path / "mid.rst", qb, step=3, time=3 * dt, dt=dt)
    del cb
    cc = fl.Context(case)
    qc = [cc.empty() for _ in range(5)]
    base = [cc.empty() for _ in range(3)]
    step, _, _, _ = cc.restart_read(tmp_path / "mid.rst", qc, base)
    assert step == 3
    bh = [t.cpu().numpy() for t in base]
    cc.set_base_state(bh[0], bh[1], bh[2])
    cc.update(qc, 3, **opts)
    for v in range(5):
        assert np.array_equal(qa[v].cpu().numpy(), qc[v].cpu().numpy()), v
