"""Slab decomposition on one GPU: the library's face-layer packing and its halo reads in the FP64
and float-pair stage kernels.  Two slab contexts of one domain (split along x) run their updates in
two host threads; their exchange function copies each slab's packed layers into the other's receive
buffers (device copies, both threads meeting at a barrier: no kernel waits on another).  The result
must equal the single-domain context bit for bit: every node's arithmetic is the same, only where
its exterior values are read from changes.  The multi-rank transport itself (fedg.slabs.HaloExchange
over torch.distributed) is tested with gloo ranks on the CPU (tests/test_slabs_gloo.py)."""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

WIND = (10.0, 0.0)


def _case():
    from fedg import cases

    return cases.C2().scaled(4, 2, 4)  # p = 7, the density current


def _full(fl, case, b, q, opts, nsteps):
    ctx = fl.Context(case)
    ctx.set_base_state(b["dens_hyd"], b["pres_hyd"], b["therm_hyd"])
    ctx.set_ref_wind(*WIND)
    qd = [ctx.tensor(a) for a in q]
    ctx.update(qd, nsteps, **opts)
    out = [t.cpu().numpy() for t in qd]
    ctx.close()
    return out


def _slabs(fl, case, b, q, opts, nsteps, nranks=2):
    import torch

    from fedg import slabs

    ctxs, qs, bufs = [], [], []
    for r in range(nranks):
        sc = slabs.slab_case(case, r, nranks, weak=False)
        c = fl.Context(sc, periodic_x=fl.HALO)
        c.set_base_state(*[slabs.slab_of(b[k], case, r, nranks) for k in ("dens_hyd", "pres_hyd", "therm_hyd")])
        c.set_ref_wind(*WIND)
        nb = c.halo_bytes()
        send = [torch.empty(nb, dtype=torch.uint8, device=c.dev) for _ in range(2)]
        recv = [torch.zeros(nb, dtype=torch.uint8, device=c.dev) for _ in range(2)]
        ctxs.append(c)
        bufs.append((send, recv))
        qs.append([c.tensor(slabs.slab_of(a, case, r, nranks)) for a in q])
    bar = threading.Barrier(nranks, timeout=60)
    calls = [[] for _ in range(nranks)]

    def make_exchange(r):
        def exchange(stage):
            calls[r].append(stage)
            bar.wait()  # every slab has packed this stage
            send = bufs[r][0]
            right, left = (r + 1) % nranks, (r - 1) % nranks
            bufs[right][1][0].copy_(send[1])
            bufs[left][1][1].copy_(send[0])
            torch.cuda.synchronize()
            bar.wait()  # every slab's receive buffers are complete
        return exchange

    for r in range(nranks):
        ctxs[r].set_halo(bufs[r][0], bufs[r][1], make_exchange(r))
    torch.cuda.synchronize()
    errs = [None] * nranks

    def run(r):
        try:
            ctxs[r].update(qs[r], nsteps, sync=False, **opts)
        except Exception as e:  # noqa: BLE001
            errs[r] = e
            bar.abort()

    th = [threading.Thread(target=run, args=(r,)) for r in range(nranks)]
    for t in th:
        t.start()
    for t in th:
        t.join(300)
    assert errs == [None] * nranks, errs
    nst = 3 * nsteps
    assert all(c == [1, 2, 3] * nsteps for c in calls) and len(calls[0]) == nst
    parts = [[t.cpu().numpy() for t in qq] for qq in qs]
    for c in ctxs:
        c.close()
    nx = case.NeX // nranks
    return [np.concatenate([parts[r][v].reshape(case.NeZ, case.NeY, nx, -1) for r in range(nranks)],
                           axis=2).reshape(case.Ne, -1) for v in range(5)]


@pytest.mark.parametrize("eqs,prec,tol", [("HEVI", "fp64", 1e-10), ("HEVE", "fp64", 0.0),
                                          ("HEVI", "pair", 1e-13), ("HEVE", "pair", 0.0)])
def test_two_slabs_equal_one_domain(eqs, prec, tol):
    from fedg import cases, lib as fl

    case = _case()
    q, b = cases.initial_state(case)
    opts = dict(eqs=fl.HEVI if eqs == "HEVI" else fl.HEVE, prec=fl.PREC_FP64 if prec == "fp64" else fl.PREC_PAIR,
                dt=0.04 if eqs == "HEVI" else 0.02, max_iter=30 if tol else 1, tol=tol)
    want = _full(fl, case, b, q, opts, 3)
    got = _slabs(fl, case, b, q, opts, 3)
    for v in range(5):
        assert np.array_equal(got[v], want[v]), (v, np.abs(got[v] - want[v]).max())


def test_one_slab_exchanging_with_itself_is_the_periodic_domain():
    """periodic_x = FEDG_HALO with the exchange copying the slab's own layers (fedg.slabs.HaloExchange
    with one rank) is the periodic mesh; also the single-call fedg_cal_tend_ex after fedg_halo_pack."""
    import torch

    from fedg import cases, lib as fl, slabs

    case = _case()
    q, b = cases.initial_state(case)
    opts = dict(eqs=fl.HEVI, prec=fl.PREC_PAIR, dt=0.04, max_iter=30, tol=1e-13)
    want = _full(fl, case, b, q, opts, 2)
    c = fl.Context(case, periodic_x=fl.HALO)
    c.set_base_state(b["dens_hyd"], b["pres_hyd"], b["therm_hyd"])
    c.set_ref_wind(*WIND)
    nb = c.halo_bytes()
    send = [torch.empty(nb, dtype=torch.uint8, device=c.dev) for _ in range(2)]
    recv = [torch.zeros(nb, dtype=torch.uint8, device=c.dev) for _ in range(2)]
    ex = slabs.HaloExchange(send, recv, 0, 1)
    c.set_halo(send, recv, ex)
    qd = [c.tensor(a) for a in q]
    c.update(qd, 2, **opts)
    assert ex.calls == 6
    for v in range(5):
        assert np.array_equal(qd[v].cpu().numpy(), want[v]), v
    # cal_tend_ex on the slab after the caller's pack + exchange == the periodic context's
    p = fl.Context(case)
    p.set_base_state(b["dens_hyd"], b["pres_hyd"], b["therm_hyd"])
    qd = [p.tensor(a) for a in q]
    tp = p.cal_tend_ex(qd, fl.HEVI)
    c.halo_pack(qd)
    ex()
    tc = c.cal_tend_ex(qd, fl.HEVI)
    for v in range(5):
        assert torch.equal(tp[v], tc[v]), v
    c.close()
    p.close()


def test_slab_refusals():
    import torch

    from fedg import cases, lib as fl

    case = _case()
    q, b = cases.initial_state(case)
    c = fl.Context(case, periodic_x=fl.HALO)
    c.set_base_state(b["dens_hyd"], b["pres_hyd"], b["therm_hyd"])
    qd = [c.tensor(a) for a in q]
    with pytest.raises(fl.FedgError, match="halo"):  # no buffers registered
        c.update(qd, 1, eqs=fl.HEVI, prec=fl.PREC_FP64, dt=0.04, max_iter=30, tol=1e-10)
    nb = c.halo_bytes()
    bufs = [[torch.zeros(nb, dtype=torch.uint8, device=c.dev) for _ in range(2)] for _ in range(2)]
    c.set_halo(bufs[0], bufs[1], lambda stage: None)
    with pytest.raises(fl.FedgError, match="reference wind"):
        c.update(qd, 1, eqs=fl.HEVI, prec=fl.PREC_PAIR, dt=0.04, max_iter=30, tol=1e-13)
    c.set_ref_wind(*WIND)
    with pytest.raises(fl.FedgError, match="FP32 mode"):
        c.update(qd, 1, eqs=fl.HEVI, prec=fl.PREC_MIXED, dt=0.04, max_iter=30, tol=1e-10)
    with pytest.raises(fl.FedgError, match="slab"):
        c.numdiff_apply(qd, 1, 1.0, 1.0, 0.04)

    def failing(stage):
        raise RuntimeError("transport down")

    c.set_halo(bufs[0], bufs[1], failing)
    with pytest.raises(fl.FedgError, match="exchange function failed"):
        c.update(qd, 1, eqs=fl.HEVI, prec=fl.PREC_FP64, dt=0.04, max_iter=30, tol=1e-10)
    assert "transport down" in str(c.halo_error)
    # a periodic context has no halo
    p = fl.Context(case)
    with pytest.raises(fl.FedgError, match="periodic"):
        p.set_halo(bufs[0], bufs[1], lambda stage: None)
    p.close()
    c.close()
