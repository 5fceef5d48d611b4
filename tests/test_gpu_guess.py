"""The learned Newton initial iterate: the network's GPU forward/backward against the numpy
oracle, training on the GPU, and what the trained network gains over the plain guess var0.

Tolerances: gradients rel L2 <= 2e-4 (FP32 kernels vs FP64 reference on the same BF16 weights);
tensor-core inference rel L2 <= 2e-2 (BF16 activations between layers).
"""
import numpy as np
import pytest

from conftest import have_gpu

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not have_gpu(), reason="needs a CUDA GPU")]

import mlp_ref  # noqa: E402
from fedg import cases, guess  # noqa: E402
from fedg import lib as fl  # noqa: E402


def _rand_net(levels, hidden, seed):
    net = fl.Guess(levels, hidden)
    net.init_params(seed)
    rng = np.random.default_rng(seed + 1)
    p = net.get_params()
    p += 0.01 * rng.standard_normal(p.size).astype(np.float32)  # non-zero biases
    net.set_params(p)
    return net, net.get_params()


@pytest.mark.parametrize("levels,hidden,batch", [(4, 64, 37), (64, 256, 300)])
def test_guess_gradient_vs_oracle(levels, hidden, batch):
    import torch

    net, p = _rand_net(levels, hidden, 3)
    rng = np.random.default_rng(5)
    X = rng.standard_normal((batch, net.din)).astype(np.float32)
    T = rng.standard_normal((batch, net.dout)).astype(np.float32)
    loss, g = net.loss_grad(torch.tensor(X, device="cuda"), torch.tensor(T, device="cuda"))
    rl, rg, _ = mlp_ref.loss_grad(p, X, T, net.din, net.hidden, net.dout)
    assert abs(loss - rl) <= 1e-5 * abs(rl)
    assert np.linalg.norm(g - rg) <= 2e-4 * np.linalg.norm(rg)


def test_guess_tensor_core_inference_vs_oracle():
    import torch

    net, p = _rand_net(64, 256, 7)
    rng = np.random.default_rng(9)
    X = rng.standard_normal((1000, net.din)).astype(np.float32)
    Y = net.predict(torch.tensor(X, device="cuda")).cpu().numpy()
    _, _, Yr = mlp_ref.loss_grad(p, X, np.zeros((1000, net.dout)), net.din, net.hidden, net.dout)
    assert np.linalg.norm(Y - Yr) <= 2e-2 * np.linalg.norm(Yr)


def test_guess_training_reduces_loss():
    import torch

    net, _ = _rand_net(8, 64, 11)
    rng = np.random.default_rng(12)
    W = rng.standard_normal((net.din, net.dout)) / np.sqrt(net.din)
    X = rng.standard_normal((8192, net.din))
    T = np.tanh(X @ W)
    Xd = torch.tensor(X, dtype=torch.float32, device="cuda")
    Td = torch.tensor(T, dtype=torch.float32, device="cuda")
    hist = guess.train(net, Xd, Td, 400, batch=1024, lr=1e-3)
    assert np.mean(hist[-20:]) < 0.1 * hist[0]


def test_learned_guess_gain_c4_geometry():
    """C4 recipe on a 4x4x8-element slice of the C2 geometry (64 levels -> 193 inputs, 192
    outputs): train on pairs from the plain solver for 6 seeds, then on a held-out seed the
    learned iterate needs fewer Newton solves and reaches the same converged state."""
    import torch

    base = cases.C2().scaled(4, 4, 8)
    dt = 0.04
    net, info = guess.build_guess(base, dt, seeds=range(6), nsteps=3, train_steps=1500, batch=2048)
    assert net.din == 193 and net.dout == 192
    assert info["loss_last"] < 0.05 * info["loss_first"], info
    rng = np.random.default_rng(1000)
    case = guess.random_case(base, rng)
    q, b = cases.initial_state(case)
    ctx = fl.Context(case)
    ctx.set_base_state(b["dens_hyd"], b["pres_hyd"], b["therm_hyd"])
    qa = [ctx.tensor(a) for a in q]
    qb = [ctx.tensor(a) for a in q]
    nfa, plain = ctx.update(qa, 4, prec=fl.PREC_MIXED, dt=dt, max_iter=20, tol=1e-10)
    net.attach(ctx)
    nfb, learned = ctx.update(qb, 4, prec=fl.PREC_MIXED, dt=dt, max_iter=20, tol=1e-10, use_guess=True)
    print(f"\n[C4 slice] plain mean Newton solves {plain:.3f}, learned {learned:.3f}, training {info}")
    assert nfa == 0 and nfb == 0
    assert learned <= plain + 1e-9
    dn = float(np.linalg.norm(b["dens_hyd"]))
    for v in range(5):
        d = float(torch.linalg.norm(qa[v] - qb[v]).item())
        assert d <= 1e-8 * dn, (v, d)


def test_guess_wait_limit_reports_error_and_context_recovers():
    """The tensor-core GEMMs' bounded barrier waits: with a wait limit of zero polls every wait of
    the normal path runs out at once, the kernels drain their MMAs with the full limit, skip their
    stores and raise the error flag, and fedg_update returns < 0 with the error text.  With the
    default limit restored the same context steps normally."""
    import torch

    case = cases.C2().scaled(2, 2, 8)
    q, b = cases.initial_state(case)
    ctx = fl.Context(case)
    ctx.set_base_state(b["dens_hyd"], b["pres_hyd"], b["therm_hyd"])
    net = fl.Guess(case.NeZ * case.N1, 64)
    net.set_params(np.zeros(net.n, np.float32))  # guess Q = q*: a valid iterate, whatever the training
    net.attach(ctx)
    qd = [ctx.tensor(a) for a in q]
    net.set_wait_limit(0)
    with pytest.raises(fl.FedgError, match="timed out waiting on its barrier"):
        ctx.update(qd, 1, prec=fl.PREC_MIXED, dt=0.04, max_iter=20, tol=1e-10, use_guess=True)
    torch.cuda.synchronize()
    net.set_wait_limit(1 << 20)
    qd = [ctx.tensor(a) for a in q]
    nf, it = ctx.update(qd, 1, prec=fl.PREC_MIXED, dt=0.04, max_iter=20, tol=1e-10, use_guess=True)
    assert nf == 0 and it >= 1.0
    assert all(bool(torch.isfinite(t).all()) for t in qd)
