"""Learned initial iterate of the HEVI column Newton solve.

Training pairs come from the plain method itself: :func:`capture_pairs` drives the time step
stage by stage through the FElib-facing C ABI exactly as FElib's driver does
(AtmDynDGMDriver_nonhydro3d_update, FElib/src/fluid_dyn_solver/scale_atm_dyn_dgm_driver_nonhydro3d.F90:
727-922: cal_vi -> StoreImplicit -> cal_tend_ex -> Advance), and at every implicit stage records
each column's stage input q* (DDENS, MOMZ, DRHOT at all levels) with impl_fac, and the converged
increment Q - q* of the plain Newton solve (tol 1e-10).  The network is then trained on the GPU
with the library's own forward/backward/Adam kernels (:class:`fedg.lib.Guess`).
"""
from __future__ import annotations

import dataclasses
import time

import numpy as np

from . import cases
from . import lib as fl


def column_index(case, device):
    """(ncol, L) flat indices into an (Ne, Np) field: column c = (ex, ey, i, j), level l = (ez, k)."""
    import torch

    N1, Np = case.N1, case.Np
    NF = N1 * N1
    ncol = case.NeX * case.NeY * NF
    L = case.NeZ * N1
    c = torch.arange(ncol, device=device)
    ij, exy = c % NF, c // NF
    ci, cj = ij % N1, ij // N1
    l = torch.arange(L, device=device)
    ez, k = l // N1, l % N1
    nxy = case.NeX * case.NeY
    g = ((ez[None, :] * nxy + exy[:, None]) * Np + (ci + N1 * cj)[:, None] + NF * k[None, :])
    return g


@dataclasses.dataclass
class PairSet:
    X: object  # (n, 3L+1) raw features: DDENS', MOMZ, DRHOT' per level, impl_fac
    Y: object  # (n, 3L) raw targets: Q - q*
    solves_plain: float


def capture_pairs(case, q0, base, dt, nsteps, max_iter=20, tol=1e-10, every=1, keep=None, seed=0):
    """Runs nsteps HEVI ARK232 steps through cal_vi / cal_tend_ex / timeint_rk and returns the
    (stage input -> converged increment) column pairs of the implicit stages."""
    import torch

    ctx = fl.Context(case)
    ctx.set_base_state(base["dens_hyd"], base["pres_hyd"], base["therm_hyd"])
    q = [ctx.tensor(a) for a in q0]
    tint = fl.TimeInt(ctx, fl.IMEX_ARK232, dt)
    gidx = column_index(case, ctx.dev)
    Xs, Ys = [], []
    nsolve, ncnt = 0, 0
    gen = torch.Generator(device=ctx.dev)
    gen.manual_seed(seed)
    for step in range(nsteps):
        tint.store_var0(q)
        ctx.sync()
        for s in range(1, 4):
            fac = tint.implicit_diagfac(s)
            var0 = [tint.var0(v) for v in range(5)]
            tim, nfail, st = ctx.cal_vi(q, var0, fac, dt, max_iter, tol, want_status=True)
            if nfail:
                raise RuntimeError(f"plain Newton failed in {nfail} columns while generating training data")
            if fac > 0:
                nsolve += int(st.sum().item())
                ncnt += int(st.numel())
                if step % every == 0:
                    feats = [q[v].reshape(-1)[gidx] for v in (0, 3, 4)]
                    incr = [tim[v].reshape(-1)[gidx] * fac for v in (0, 3, 4)]
                    X = torch.cat(feats + [torch.full((gidx.shape[0], 1), fac, device=ctx.dev, dtype=torch.float64)], 1)
                    Y = torch.cat(incr, 1)
                    if keep is not None and keep < X.shape[0]:
                        sel = torch.randperm(X.shape[0], generator=gen, device=ctx.dev)[:keep]
                        X, Y = X[sel], Y[sel]
                    Xs.append(X.float())
                    Ys.append(Y.float())
            for v in range(5):
                tint.tend_im(s, v).copy_(tim[v])
            torch.cuda.synchronize()
            tint.store_implicit(s, q)
            ctx.sync()
            tex = ctx.cal_tend_ex(q, fl.HEVI)
            for v in range(5):
                tint.tend_ex(s, v).copy_(tex[v])
            torch.cuda.synchronize()
            tint.advance(s, q)
            ctx.sync()
        if case.filter_on:
            ctx.modalfilter(q)
    tint.close()
    ctx.close()
    return PairSet(torch.cat(Xs), torch.cat(Ys), nsolve / max(ncnt, 1))


def random_case(base_case, rng):
    """C4 recipe: bubble amplitude U(-20, 5) K, radius U(1, 5) km (horizontal; half vertically),
    centre uniform in the domain, background wind U(-15, 15) m/s."""
    xmin, xmax, ymin, ymax, zmin, zmax = base_case.dom
    r = rng.uniform(1000.0, 5000.0)
    b = dict(amp=rng.uniform(-20.0, 5.0), rx=r, ry=r, rz=0.5 * r, xc=rng.uniform(xmin, xmax),
             yc=rng.uniform(ymin, ymax), zc=rng.uniform(zmin + 0.2 * (zmax - zmin), zmax - 0.2 * (zmax - zmin)))
    return dataclasses.replace(base_case, bubble=b, u0=rng.uniform(-15.0, 15.0))


def generate(base_case, seeds, dt, nsteps, per_stage_keep, spinup=0):
    """Pairs from len(seeds) randomised initial states of base_case geometry."""
    import torch

    Xs, Ys, sp = [], [], []
    for sd in seeds:
        rng = np.random.default_rng(sd)
        if base_case.bubble:
            case = random_case(base_case, rng)
        else:  # noise-driven workloads: new noise field, amplitude and background wind per seed
            case = dataclasses.replace(base_case, u0=rng.uniform(0.0, 10.0),
                                       noise=dict(base_case.noise, seed=int(sd),
                                                  amp=base_case.noise.get("amp", 0.1) * rng.uniform(0.5, 2.0)))
        q, b = cases.initial_state(case)
        ps = capture_pairs(case, q, b, dt, nsteps, keep=per_stage_keep, seed=int(sd))
        Xs.append(ps.X)
        Ys.append(ps.Y)
        sp.append(ps.solves_plain)
    return torch.cat(Xs), torch.cat(Ys), float(np.mean(sp))


def scales_from(X, Y, L, dt):
    """Per-variable feature/target scales (1/std), impl_fac scaled by 1/dt."""
    def inv_std(a):
        s = float(a.std().item())
        return 1.0 / s if s > 0 else 1.0
    ins = [inv_std(X[:, v * L:(v + 1) * L]) for v in range(3)] + [1.0 / dt]
    outs = [inv_std(Y[:, v * L:(v + 1) * L]) for v in range(3)]
    return ins, outs


def normalise(X, Y, L, ins, outs):
    import torch

    Xn = X.clone()
    Yn = Y.clone()
    for v in range(3):
        Xn[:, v * L:(v + 1) * L] *= ins[v]
        Yn[:, v * L:(v + 1) * L] *= outs[v]
    Xn[:, 3 * L] *= ins[3]
    return Xn.contiguous(), Yn.contiguous()


def train(net, Xn, Yn, steps, batch=4096, lr=1e-3, seed=0, log_every=0):
    """Adam on the GPU with the library's kernels; returns the loss history."""
    import torch

    g = torch.Generator(device=Xn.device)
    g.manual_seed(seed)
    n = Xn.shape[0]
    hist = []
    for it in range(steps):
        idx = torch.randint(0, n, (min(batch, n),), generator=g, device=Xn.device)
        xb = Xn[idx].contiguous()
        yb = Yn[idx].contiguous()
        loss = net.train_step(xb, yb, lr)
        hist.append(loss)
        if log_every and it % log_every == 0:
            print(f"  step {it:5d} loss {loss:.4e}", flush=True)
    return hist


def build_guess(base_case, dt, seeds=range(20), nsteps=3, per_stage_keep=None, train_steps=2000, hidden=256,
                batch=4096, lr=1e-3, log_every=0):
    """Generate pairs with the plain solver, fit scales, train the network; returns (net, info)."""
    t0 = time.time()
    L = base_case.NeZ * base_case.N1
    X, Y, sp = generate(base_case, list(seeds), dt, nsteps, per_stage_keep)
    t1 = time.time()
    ins, outs = scales_from(X, Y, L, dt)
    Xn, Yn = normalise(X, Y, L, ins, outs)
    net = fl.Guess(L, hidden)
    net.set_scales(ins, outs)
    net.init_params(0)
    hist = train(net, Xn, Yn, train_steps, batch, lr, log_every=log_every)
    t2 = time.time()
    info = dict(pairs=int(X.shape[0]), plain_solves_in_data=sp, gen_s=t1 - t0, train_s=t2 - t1,
                loss_first=hist[0], loss_last=float(np.mean(hist[-20:])))
    return net, info
