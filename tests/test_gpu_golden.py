"""The CUDA path against the committed golden vectors (tests/golden/, the oracle's outputs; see
tests/golden/make_golden.py): the FP64 and float-pair updates of the HEVE and HEVI cases and
the FP64 and float-pair tracer steps, through the C ABI, without running the oracle.

Tolerances: whole dynamics steps 1e-9 relative L2 of the full fields (momentum against at least
1 m/s of hydrostatic momentum, the bar of the oracle parity tests); tracer steps 1e-12 (FP64)
and 1e-11 (float pairs).
"""
import os

import numpy as np
import pytest

from conftest import ROOT, have_gpu

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not have_gpu(), reason="needs a CUDA GPU")]

from fedg import cases  # noqa: E402
from fedg import lib as fl  # noqa: E402

GOLD = os.path.join(ROOT, "tests", "golden")


def _mg():
    import importlib.util

    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLD, "make_golden.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def full_errs(got, ref, b):
    dn = np.linalg.norm(b["dens_hyd"])
    hyd = [b["dens_hyd"], 0.0, 0.0, 0.0, b["therm_hyd"]]
    return [float(np.linalg.norm(g - r) / max(np.linalg.norm(r + h), dn)) for g, r, h in zip(got, ref, hyd)]


@pytest.mark.parametrize("name", ["heve_C1_3x3x3", "hevi_C1_3x3x3", "hevi_C2_2x2x2"])
@pytest.mark.parametrize("prec", ["fp64", "pair"])
def test_update_matches_golden(name, prec):
    spec = _mg().golden_cases()[name]
    case = spec["case"]
    ref = np.load(os.path.join(GOLD, name + ".npz"))["q"]
    q, b = cases.initial_state(case)
    ctx = fl.Context(case)
    ctx.set_base_state(b["dens_hyd"], b["pres_hyd"], b["therm_hyd"])
    qd = [ctx.tensor(a) for a in q]
    p = fl.PREC_PAIR if prec == "pair" else fl.PREC_FP64
    if spec["eqs"] == "HEVE":
        ctx.update(qd, spec["nsteps"], eqs=fl.HEVE, prec=p, dt=spec["dt"])
    else:
        nf, _ = ctx.update(qd, spec["nsteps"], eqs=fl.HEVI, prec=p, dt=spec["dt"], max_iter=spec["max_iter"],
                           tol=spec["tol"])
        assert nf == 0
    errs = full_errs([t.cpu().numpy() for t in qd], list(ref), b)
    assert max(errs) < 1e-9, errs


@pytest.mark.parametrize("prec,bar", [("fp64", 1e-12), ("pair", 1e-11)])
def test_tracer_matches_golden(prec, bar):
    spec = _mg().golden_cases()["trc_T1_4x4x3"]
    case = spec["case"]
    g = np.load(os.path.join(GOLD, "trc_T1_4x4x3.npz"))
    q, b = cases.initial_state(case)
    ctx = fl.Context(case)
    ctx.set_base_state(b["dens_hyd"], b["pres_hyd"], b["therm_hyd"])
    qd = [ctx.tensor(a) for a in q]
    aM, aP = ctx.trc_alphdens_advtest(qd[0], qd[1], qd[2], qd[3])
    assert np.linalg.norm(aM.cpu().numpy() - g["aM"]) <= 1e-13 * np.linalg.norm(g["aM"])
    Qd = ctx.tensor(cases.tracer_state(case))
    ctx.trc_update(Qd, qd[1:4], aM, aP, qd[0], qd[0], case.dt, nsteps=spec["nsteps"],
                   prec=fl.PREC_PAIR if prec == "pair" else fl.PREC_FP64)
    e = float(np.linalg.norm(Qd.cpu().numpy() - g["Q"]) / np.linalg.norm(g["Q"]))
    assert e < bar, e
