"""fedg_update_host: the update for fields in page-locked host memory (FElib's CPU build keeps its
fields on the host).  The float-pair paths store the result into the host arrays from their last
stage kernel; the FP64 path copies it back.  Either way the host arrays must end bit-identical to
the device-array update of the same state."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("eqs,prec,tol,dt", [("HEVI", "pair", 1e-13, 0.04), ("HEVE", "pair", 0.0, 0.02),
                                             ("HEVI", "fp64", 1e-10, 0.04)])
def test_host_update_equals_device_update(eqs, prec, tol, dt):
    import torch

    from fedg import cases, lib as fl

    case = cases.C2().scaled(4, 2, 4)
    q, b = cases.initial_state(case)
    opts = dict(eqs=fl.HEVI if eqs == "HEVI" else fl.HEVE, prec=fl.PREC_PAIR if prec == "pair" else fl.PREC_FP64,
                dt=dt, max_iter=30 if tol else 1, tol=tol)
    ca = fl.Context(case)
    ca.set_base_state(b["dens_hyd"], b["pres_hyd"], b["therm_hyd"])
    qd = [ca.tensor(a) for a in q]
    nf_a, it_a = ca.update(qd, 3, **opts)
    cb = fl.Context(case)
    cb.set_base_state(b["dens_hyd"], b["pres_hyd"], b["therm_hyd"])
    qh = [torch.from_numpy(np.ascontiguousarray(a)).pin_memory() for a in q]
    nf_b, it_b = cb.update_host(qh, 3, **opts)
    assert (nf_a, it_a) == (nf_b, it_b)
    for v in range(5):
        assert np.array_equal(qh[v].numpy(), qd[v].cpu().numpy()), v
    # the host arrays are the state: a second call continues from them
    ca.update(qd, 2, **opts)
    cb.update_host(qh, 2, **opts)
    for v in range(5):
        assert np.array_equal(qh[v].numpy(), qd[v].cpu().numpy()), v
    ca.close()
    cb.close()


def test_host_update_refuses_pageable_memory():
    from fedg import cases, lib as fl
    import torch

    case = cases.C2().scaled(2, 2, 2)
    q, b = cases.initial_state(case)
    c = fl.Context(case)
    c.set_base_state(b["dens_hyd"], b["pres_hyd"], b["therm_hyd"])
    qh = [torch.from_numpy(np.ascontiguousarray(a)) for a in q]  # not page-locked
    with pytest.raises(fl.FedgError, match="page-locked"):
        c.update_host(qh, 1, eqs=fl.HEVI, prec=fl.PREC_PAIR, dt=0.04, max_iter=30, tol=1e-13)
    c.close()
