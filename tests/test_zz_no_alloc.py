"""fedg_cal_tend_ex_noalloc: the explicit tendency for callers that cannot allocate device memory
after their set-up (a Fortran model whose device memory belongs to its OpenACC runtime, or a
host whose allocator has already claimed the GPU).  It must give the same tendencies as
fedg_cal_tend_ex on two calls in a row, and refuse meshes larger than its static scratch.

Tolerance: relative L2 per variable <= 1e-11, as for the other single-operator parity tests
(both entry points run the same kernels, so the results are expected to be identical).
"""
import ctypes

import numpy as np
import pytest

from conftest import have_gpu

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not have_gpu(), reason="needs a CUDA GPU")]

from fedg import cases  # noqa: E402
from fedg import lib as fl  # noqa: E402


def _inputs(ctx, q):
    b = ctx._base
    return (ctypes.c_void_p * 16)(*[t.data_ptr() for t in q], None, b[0].data_ptr(), b[1].data_ptr(), None,
                                  b[2].data_ptr(), None, None, None, None, None, None)


@pytest.mark.parametrize("name,case,eqs", [("p3_C1", cases.C1(), fl.HEVE), ("p7_C2_4x4x4", cases.C2().scaled(4, 4, 4), fl.HEVI)])
def test_noalloc_matches_cal_tend_ex_twice(name, case, eqs):
    import torch

    q, b = cases.initial_state(case)
    rng = np.random.default_rng(21)
    sc = [1e-3 * b["dens_hyd"], 2.0, 2.0, 1.0, 0.3]
    ctx = fl.Context(case)
    ctx.set_base_state(b["dens_hyd"], b["pres_hyd"], b["therm_hyd"])
    for call in range(2):
        qd = [ctx.tensor(q[v] + (call * 0.1) * sc[v] * rng.standard_normal(q[v].shape)) for v in range(5)]
        ref = [t.cpu().numpy() for t in ctx.cal_tend_ex(qd, eqs)]  # the allocating entry point
        out = [ctx.empty() for _ in range(5)]
        torch.cuda.synchronize()
        rc = ctx.lib.fedg_cal_tend_ex_noalloc(ctx.h, _inputs(ctx, qd), fl._p5(out), int(eqs))
        assert rc == 0, fl.last_error()
        ctx.sync()
        for v in range(5):
            g = out[v].cpu().numpy()
            err = np.linalg.norm(g - ref[v]) / max(np.linalg.norm(ref[v]), 1e-300)
            assert err <= 1e-11, (name, call, v, err)


def test_noalloc_rejects_meshes_beyond_its_scratch():
    import torch

    case = cases.C2().scaled(16, 16, 17)  # 4352 elements x 512 nodes > 2,097,152 nodes
    q, b = cases.initial_state(case)
    ctx = fl.Context(case)
    ctx.set_base_state(b["dens_hyd"], b["pres_hyd"], b["therm_hyd"])
    qd = [ctx.tensor(a) for a in q]
    out = [ctx.empty() for _ in range(5)]
    torch.cuda.synchronize()
    rc = ctx.lib.fedg_cal_tend_ex_noalloc(ctx.h, _inputs(ctx, qd), fl._p5(out), int(fl.HEVI))
    assert rc < 0 and "static scratch" in fl.last_error()


def test_noalloc_first_on_a_fresh_context_allocates_nothing():
    """On a context that has never run the allocating entry point, two calls leave the device's
    free memory unchanged (a fallback to the context's cudaMalloc'd scratch would take at least
    the 1 MiB DPRES field of this mesh), and both match fedg_cal_tend_ex afterwards."""
    import torch

    case = cases.C2().scaled(8, 8, 4)  # 256 elements x 512 nodes: DPRES is 1 MiB
    q, b = cases.initial_state(case)
    rng = np.random.default_rng(5)
    ctx = fl.Context(case)
    ctx.set_base_state(b["dens_hyd"], b["pres_hyd"], b["therm_hyd"])
    sc = [1e-3 * b["dens_hyd"], 2.0, 2.0, 1.0, 0.3]
    qs = [[ctx.tensor(q[v] + 0.1 * (call + 1) * sc[v] * rng.standard_normal(q[v].shape)) for v in range(5)]
          for call in range(2)]
    outs = [[ctx.empty() for _ in range(5)] for _ in range(2)]
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for call in range(2):
        rc = ctx.lib.fedg_cal_tend_ex_noalloc(ctx.h, _inputs(ctx, qs[call]), fl._p5(outs[call]), int(fl.HEVI))
        assert rc == 0, fl.last_error()
        ctx.sync()
        free1, _ = torch.cuda.mem_get_info()
        assert free1 == free0, (call, free0, free1)
    for call in range(2):
        ref = [t.cpu().numpy() for t in ctx.cal_tend_ex(qs[call], fl.HEVI)]
        for v in range(5):
            g = outs[call][v].cpu().numpy()
            err = np.linalg.norm(g - ref[v]) / max(np.linalg.norm(ref[v]), 1e-300)
            assert err <= 1e-11, (call, v, err)
