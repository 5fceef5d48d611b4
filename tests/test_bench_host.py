"""Host-side arithmetic of bench.py that needs no GPU: the issue-rate roofline of the dominant kernel."""
import importlib.util
import os

from conftest import ROOT


def _bench():
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def test_issue_roofline_arithmetic():
    b = _bench()
    ipn = b.NCU_INST_PER_NODE["pair"]["vi_mixed"]
    nodes = 134217728
    r = b.issue_roofline("vi_mixed", "pair", nodes, 78.0, 2070.0, 152)
    assert r["bound"] == "issue" and r["unit"] == "warp instructions/s"
    assert abs(r["achieved"] - ipn * nodes / 0.078) < 1e-6 * r["achieved"]
    assert abs(r["peak"] - 4 * 152 * 2070e6) < 1.0
    assert 0.0 < r["frac"] < 1.0
    # a kernel or path without an ncu instruction count has no issue roofline
    assert b.issue_roofline("stage_mixed", "pair", nodes, 10.0, 2070.0, 152) is None
    assert b.issue_roofline("vi_mixed", "fp64", nodes, 10.0, 2070.0, 152) is None
    # no clock sample: the maximum SM clock
    assert b.issue_roofline("vi_mixed", "pair", nodes, 78.0, None, 152)["sm_mhz"] == 2070.0


def _replica(rank, world, port, out):
    import os as _os

    import torch.distributed as dist

    _os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    b = _bench()
    ms = b.max_over_ranks(10.0 + 5.0 * rank, world, "cpu")  # rank 1 is the slower replica
    out[rank] = (ms, b.replica_throughput(1000, 3, ms, world))
    dist.destroy_process_group()


def test_replicas_take_the_slowest_rank_gloo():
    """bench.py --gpus N runs N independent replicas; the timed region is the max over ranks and the
    throughput counts all ranks' units (two gloo ranks on the CPU)."""
    import socket

    import torch.multiprocessing as mp

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    procs = [ctx.Process(target=_replica, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    for r in range(2):
        ms, v = out[r]
        assert ms == 15.0
        assert abs(v - 1000 * 3 * 2 / 0.015) < 1e-6 * v
    b = _bench()
    assert b.max_over_ranks(7.0, 1, "cpu") == 7.0
