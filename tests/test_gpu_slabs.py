"""Domain decomposition on one GPU: the library's face-layer packing and its halo reads in the FP64
float-pair and FP32-mode stage kernels.  The part contexts of one domain (split along x, along y, or both)
run their updates in host threads; their exchange function copies each part's packed layers into
its neighbours' receive buffers (device copies, the threads meeting at a barrier: no kernel waits on
another).  The result must equal the single-domain context bit for bit: every node's arithmetic is
the same, only where its exterior values are read from changes.  The multi-rank transport itself (fedg.slabs.HaloExchange
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


def _bufs(torch, c):
    send = [torch.empty(n, dtype=torch.uint8, device=c.dev) if n else None for n in map(c.halo_bytes, range(4))]
    recv = [torch.zeros(n, dtype=torch.uint8, device=c.dev) if n else None for n in map(c.halo_bytes, range(4))]
    return send, recv


def _slabs(fl, case, b, q, opts, nsteps, dims=(2, 1)):
    import torch

    from fedg import slabs

    nranks = dims[0] * dims[1]
    pxf, pyf = slabs.periodic_flags(nranks, dims, fl.HALO)
    ctxs, qs, bufs, peers = [], [], [], []
    for r in range(nranks):
        sc = slabs.slab_case(case, r, nranks, weak=False, dims=dims)
        c = fl.Context(sc, periodic_x=pxf, periodic_y=pyf)
        c.set_base_state(*[slabs.slab_of(b[k], case, r, nranks, dims) for k in ("dens_hyd", "pres_hyd", "therm_hyd")])
        c.set_ref_wind(*WIND)
        ctxs.append(c)
        bufs.append(_bufs(torch, c))
        peers.append(slabs.HaloExchange(None, None, r, nranks, dims=dims).peers)
        qs.append([c.tensor(slabs.slab_of(a, case, r, nranks, dims)) for a in q])
    bar = threading.Barrier(nranks, timeout=60)
    calls = [[] for _ in range(nranks)]

    def make_exchange(r):
        def exchange(stage):
            calls[r].append(stage)
            bar.wait()  # every part has packed this stage
            send = bufs[r][0]
            for sd, opp in ((1, 0), (0, 1), (3, 2), (2, 3)):  # my side sd lands on the neighbour's side opp
                if send[sd] is not None:
                    bufs[peers[r][sd]][1][opp].copy_(send[sd])
            torch.cuda.synchronize()
            bar.wait()  # every part's receive buffers are complete
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
    assert all(c == [1, 2, 3] * nsteps for c in calls)
    parts = [[t.cpu().numpy() for t in qq] for qq in qs]
    for c in ctxs:
        c.close()
    return [slabs.assemble([parts[r][v] for r in range(nranks)], case, dims) for v in range(5)]


@pytest.mark.parametrize("eqs,prec,tol,dims", [("HEVI", "fp64", 1e-10, (2, 1)), ("HEVE", "fp64", 0.0, (2, 1)),
                                               ("HEVI", "pair", 1e-13, (2, 1)), ("HEVE", "pair", 0.0, (2, 1)),
                                               ("HEVI", "pair", 1e-13, (1, 2)), ("HEVI", "fp64", 1e-10, (2, 2)),
                                               ("HEVI", "pair", 1e-13, (2, 2)), ("HEVI", "fp32", 1e-10, (2, 1)),
                                               ("HEVI", "fp32", 1e-10, (2, 2))])
def test_parts_equal_one_domain(eqs, prec, tol, dims):
    from fedg import cases, lib as fl

    case = cases.C2().scaled(4, 4, 4)  # p = 7, the density current
    q, b = cases.initial_state(case)
    precs = {"fp64": fl.PREC_FP64, "pair": fl.PREC_PAIR, "fp32": fl.PREC_MIXED}
    opts = dict(eqs=fl.HEVI if eqs == "HEVI" else fl.HEVE, prec=precs[prec],
                dt=0.04 if eqs == "HEVI" else 0.02, max_iter=30 if tol else 1, tol=tol)
    want = _full(fl, case, b, q, opts, 3)
    got = _slabs(fl, case, b, q, opts, 3, dims)
    for v in range(5):
        assert np.array_equal(got[v], want[v]), (v, np.abs(got[v] - want[v]).max())


def test_one_slab_exchanging_with_itself_is_the_periodic_domain():
    """periodic_x = periodic_y = FEDG_HALO with the exchange copying the part's own layers
    (fedg.slabs.HaloExchange with one rank) is the periodic mesh; also the single-call fedg_cal_tend_ex
    after fedg_halo_pack."""
    import torch

    from fedg import cases, lib as fl, slabs

    case = _case()
    q, b = cases.initial_state(case)
    opts = dict(eqs=fl.HEVI, prec=fl.PREC_PAIR, dt=0.04, max_iter=30, tol=1e-13)
    want = _full(fl, case, b, q, opts, 2)
    c = fl.Context(case, periodic_x=fl.HALO, periodic_y=fl.HALO)
    c.set_base_state(b["dens_hyd"], b["pres_hyd"], b["therm_hyd"])
    c.set_ref_wind(*WIND)
    send, recv = _bufs(torch, c)
    ex = slabs.HaloExchange(send, recv, 0, 1, dims=(1, 1))
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
    bufs = _bufs(torch, c)
    c.set_halo(bufs[0], bufs[1], lambda stage: None)
    with pytest.raises(fl.FedgError, match="reference wind"):
        c.update(qd, 1, eqs=fl.HEVI, prec=fl.PREC_PAIR, dt=0.04, max_iter=30, tol=1e-13)
    c.set_ref_wind(*WIND)
    with pytest.raises(fl.FedgError, match="decomposed"):
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
        p.set_halo([None] * 4, [None] * 4, lambda stage: None)
    p.close()
    c.close()
