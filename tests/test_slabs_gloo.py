"""Domain decomposition on the CPU: gloo ranks, each running the FP64 oracle on its part of the
domain (split along x, along y, or both) with the face-layer exchange of fedg.slabs before every
tendency, reproduce the single-domain oracle steps (HEVI ARK232 with the Newton solve, and HEVE
SSP-RK3).  This is the host side of the multi-GPU path: the same exchange object moves device
buffers over NCCL in bench.py --gpus N; the library's own pack and halo reads are tested on one GPU
in tests/test_gpu_slabs.py."""
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


def _worker(rank, nranks, port, tmp, eqs, dims):
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
    sc = slabs.slab_case(case, rank, nranks, weak=False, dims=dims)
    o = _oracle(orc, sc)
    o.set_base_state(slabs.slab_of(b["dens_hyd"], case, rank, nranks, dims),
                     slabs.slab_of(b["pres_hyd"], case, rank, nranks, dims))
    sides = tuple(sd for sd in range(4) if dims[sd // 2] > 1)
    ex = slabs.HaloExchange(None, None, rank, nranks, dims=dims)
    log = []

    def exchange(stage, send, recv):
        log.append(stage)
        ex(stage, [torch.from_numpy(send[sd]) if sd in send else None for sd in range(4)],
           [torch.from_numpy(recv[sd]) if sd in recv else None for sd in range(4)])

    o.set_halo(exchange, sides)
    ql = [slabs.slab_of(a, case, rank, nranks, dims) for a in q]
    if eqs == "HEVI":
        out, nfail, _ = o.step_hevi(ql, DT, STEPS, max_iter=30, tol=1e-10)
        assert nfail == 0
    else:
        out = o.step_heve(ql, DT, STEPS)
    assert not o.halo_errors, o.halo_errors
    assert log == [1, 2, 3] * STEPS  # one exchange before every stage's tendency
    np.save(os.path.join(tmp, f"{eqs}_r{rank}.npy"), np.stack(out))
    dist.destroy_process_group()


def _run(tmp_path, eqs, dims):
    import torch.multiprocessing as mp

    nranks = dims[0] * dims[1]
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_worker, args=(r, nranks, port, str(tmp_path), eqs, dims)) for r in range(nranks)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(300)
    for p in procs:
        if p.exitcode is None:
            p.kill()
        assert p.exitcode == 0
    return [np.load(os.path.join(tmp_path, f"{eqs}_r{r}.npy")) for r in range(nranks)]


def _reference(eqs):
    import oracle as orc
    from fedg import cases

    case = _case()
    q, b = cases.initial_state(case)
    o = _oracle(orc, case)
    o.set_base_state(b["dens_hyd"], b["pres_hyd"])
    if eqs == "HEVI":
        ref, nfail, _ = o.step_hevi(q, DT, STEPS, max_iter=30, tol=1e-10)
        assert nfail == 0
    else:
        ref = o.step_heve(q, DT, STEPS)
    return case, q, b, ref


@pytest.mark.parametrize("eqs,dims", [("HEVI", (2, 1)), ("HEVE", (2, 1)), ("HEVI", (1, 2)), ("HEVI", (2, 2))])
def test_parts_match_the_single_domain_oracle(tmp_path, eqs, dims):
    import oracle as orc
    from fedg import slabs

    parts = _run(tmp_path, eqs, dims)
    case, q, b, ref = _reference(eqs)
    for v in range(5):
        got = slabs.assemble([p[v] for p in parts], case, dims)
        want = np.asarray(ref[v]).reshape(case.Ne, -1)
        scale = max(np.abs(want).max(), 1e-300)
        assert np.abs(got - want).max() <= 1e-12 * scale, (v, np.abs(got - want).max() / scale)
    # the decomposition moved something: rank 0's part differs from a periodic run of that part alone
    nranks = dims[0] * dims[1]
    sc = slabs.slab_case(case, 0, nranks, weak=False, dims=dims)
    o1 = _oracle(orc, sc)
    o1.set_base_state(slabs.slab_of(b["dens_hyd"], case, 0, nranks, dims), slabs.slab_of(b["pres_hyd"], case, 0, nranks, dims))
    q0 = [slabs.slab_of(a, case, 0, nranks, dims) for a in q]
    alone = o1.step_hevi(q0, DT, STEPS, max_iter=30, tol=1e-10)[0] if eqs == "HEVI" else o1.step_heve(q0, DT, STEPS)
    v = 1 if dims[0] > 1 else 2  # the momentum across the split
    assert np.abs(np.asarray(alone[v]) - parts[0][v]).max() > 1e-9 * np.abs(parts[0][v]).max()


def test_slab_helpers():
    from fedg import cases, slabs

    case = cases.C2().scaled(4, 2, 3, porder=2)
    a = np.arange(case.Ne * case.Np, dtype=np.float64).reshape(case.Ne, case.Np)
    for dims in ((2, 1), (1, 2), (2, 2), (4, 1)):
        n = dims[0] * dims[1]
        parts = [slabs.slab_of(a, case, r, n, dims) for r in range(n)]
        assert parts[0].shape == (case.Ne // n, case.Np)
        assert np.array_equal(slabs.assemble(parts, case, dims), a)
    s1 = slabs.slab_case(case, 1, 2, weak=False)
    assert s1.NeX == 2 and s1.dom[0] == case.dom[0] + 0.5 * (case.dom[1] - case.dom[0])
    s3 = slabs.slab_case(case, 3, 4, weak=False, dims=(2, 2))
    assert (s3.NeX, s3.NeY) == (2, 1) and s3.dom[2] == case.dom[2] + 0.5 * (case.dom[3] - case.dom[2])
    w2 = slabs.slab_case(case, 2, 4, weak=True)
    assert w2.NeX == case.NeX and w2.dom[0] == case.dom[0] + 2 * (case.dom[1] - case.dom[0])
    with pytest.raises(ValueError):
        slabs.slab_case(case, 0, 3, weak=False)
    assert slabs.periodic_flags(4, (4, 1)) == (2, 1) and slabs.periodic_flags(4, (2, 2)) == (2, 2)
    ex = slabs.HaloExchange(None, None, 3, 4, dims=(2, 2))  # rank 3 = (1, 1)
    assert ex.peers == [2, 2, 1, 1]
