"""Slab decomposition on the CPU: two gloo ranks, each running the FP64 oracle on its half of the
domain (split along x) with the face-layer exchange of fedg.slabs before every tendency, reproduce
the single-domain oracle steps (HEVI ARK232 with the Newton solve, and HEVE SSP-RK3).  This is the
host side of the multi-GPU path: the same exchange object moves device buffers over NCCL in
bench.py --gpus N; the library's own pack and halo reads are tested on one GPU in
tests/test_gpu_slabs.py."""
import os
import socket

import numpy as np
import pytest

DT = 0.05
STEPS = 2


def _case():
    from fedg import cases

    # the density current on a p = 3 mesh of 4 x 2 x 4 elements: the bubble spans both slabs
    return cases.C2().scaled(4, 2, 4, porder=3)


def _oracle(orc, case):
    return orc.Oracle(case.porder, case.NeX, case.NeY, case.NeZ, case.dom, filter_on=case.filter_on)


def _worker(rank, nranks, port, tmp, eqs):
    import sys
    from datetime import timedelta

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for p in (os.path.join(root, "fe-project_gb300"), os.path.join(root, "oracle")):
        sys.path.insert(0, p)
    import torch
    import torch.distributed as dist

    import oracle as orc
    from fedg import cases, slabs

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=nranks, timeout=timedelta(seconds=120))
    orc.set_num_threads(2)
    case = _case()
    q, b = cases.initial_state(case)
    sc = slabs.slab_case(case, rank, nranks, weak=False)
    o = _oracle(orc, sc)
    o.set_base_state(slabs.slab_of(b["dens_hyd"], case, rank, nranks),
                     slabs.slab_of(b["pres_hyd"], case, rank, nranks))
    ex = slabs.HaloExchange(None, None, rank, nranks)
    log = []

    def exchange(stage, send, recv):
        log.append(stage)
        ex(stage, [torch.from_numpy(send[0]), torch.from_numpy(send[1])],
           [torch.from_numpy(recv[0]), torch.from_numpy(recv[1])])

    o.set_halo(exchange)
    ql = [slabs.slab_of(a, case, rank, nranks) for a in q]
    if eqs == "HEVI":
        out, nfail, _ = o.step_hevi(ql, DT, STEPS, max_iter=30, tol=1e-10)
        assert nfail == 0
    else:
        out = o.step_heve(ql, DT, STEPS)
    assert not o.halo_errors, o.halo_errors
    assert log == [1, 2, 3] * STEPS  # one exchange before every stage's tendency
    np.save(os.path.join(tmp, f"{eqs}_r{rank}.npy"), np.stack(out))
    dist.destroy_process_group()


@pytest.mark.parametrize("eqs", ["HEVI", "HEVE"])
def test_two_slabs_match_the_single_domain_oracle(tmp_path, eqs):
    import torch.multiprocessing as mp

    import oracle as orc
    from fedg import cases, slabs

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_worker, args=(r, 2, port, str(tmp_path), eqs)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(300)
    for p in procs:
        if p.exitcode is None:
            p.kill()
        assert p.exitcode == 0
    case = _case()
    q, b = cases.initial_state(case)
    o = _oracle(orc, case)
    o.set_base_state(b["dens_hyd"], b["pres_hyd"])
    if eqs == "HEVI":
        ref, nfail, _ = o.step_hevi(q, DT, STEPS, max_iter=30, tol=1e-10)
        assert nfail == 0
    else:
        ref = o.step_heve(q, DT, STEPS)
    parts = [np.load(os.path.join(tmp_path, f"{eqs}_r{r}.npy")) for r in range(2)]
    for v in range(5):
        got = np.concatenate([parts[r][v].reshape(case.NeZ, case.NeY, case.NeX // 2, -1) for r in range(2)],
                             axis=2).reshape(case.Ne, -1)
        want = np.asarray(ref[v]).reshape(case.Ne, -1)
        scale = max(np.abs(want).max(), 1e-300)
        assert np.abs(got - want).max() <= 1e-12 * scale, (v, np.abs(got - want).max() / scale)
    # the decomposition moved something: the slabs differ from a periodic run of one slab alone
    sc = slabs.slab_case(case, 0, 2, weak=False)
    o1 = _oracle(orc, sc)
    o1.set_base_state(slabs.slab_of(b["dens_hyd"], case, 0, 2), slabs.slab_of(b["pres_hyd"], case, 0, 2))
    q0 = [slabs.slab_of(a, case, 0, 2) for a in q]
    alone = o1.step_hevi(q0, DT, STEPS, max_iter=30, tol=1e-10)[0] if eqs == "HEVI" else o1.step_heve(q0, DT, STEPS)
    assert np.abs(np.asarray(alone[1]) - parts[0][1]).max() > 1e-9 * np.abs(parts[0][1]).max()


def test_slab_helpers():
    from fedg import cases, slabs

    case = cases.C2().scaled(4, 2, 3, porder=2)
    a = np.arange(case.Ne * case.Np, dtype=np.float64).reshape(case.Ne, case.Np)
    parts = [slabs.slab_of(a, case, r, 2) for r in range(2)]
    assert parts[0].shape == (case.Ne // 2, case.Np)
    back = np.concatenate([p.reshape(case.NeZ, case.NeY, 2, -1) for p in parts], axis=2).reshape(case.Ne, -1)
    assert np.array_equal(back, a)
    s1 = slabs.slab_case(case, 1, 2, weak=False)
    assert s1.NeX == 2 and s1.dom[0] == case.dom[0] + 0.5 * (case.dom[1] - case.dom[0])
    w2 = slabs.slab_case(case, 2, 4, weak=True)
    assert w2.NeX == case.NeX and w2.dom[0] == case.dom[0] + 2 * (case.dom[1] - case.dom[0])
    with pytest.raises(ValueError):
        slabs.slab_case(case, 0, 3, weak=False)
