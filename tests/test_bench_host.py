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
