"""One-hour precision run: the learned-guess HEVI paths in the float-pair and FP32 precision modes
against the plain FP64 path, all on the GPU from the same initial state.  It reports the relative
L2 error per variable at checkpoints.

Workload: the density current on the p = 7 mesh with 800 m elements. This is the recipe of the
medium HEVI case run in the precision form:

  - isothermal 300 K base state;
  - -15 K cosine bubble of 4 km x 2 km radius at z = 3 km;
  - u = 10 m/s;
  - periodic in x and y, slip lids;
  - 8 vertical elements, i.e. 64-level columns.

The default horizontal extent is 8 x 8 elements (6.4 km), so the four paths finish the hour in
about half an hour of GPU time (almost all of it in the two FP64 paths).  The time step is dt = 0.04 s. It is the stable step for this mesh: 0.08 s
diverges, and the 0.5 s of the original recipe exceeds the horizontal acoustic limit of p = 7
elements of 800 m. One simulated hour is therefore 90,000 steps.

Paths (all from the same initial state; the four HEVI paths at the same dt):

  plain_fp64_tol1e-14   FP64 fused update (FElib's algorithm), Newton to tol 1e-14: the
                        implicit stages converged to roundoff; the reference of the comparison.
  plain_fp64_tol1e-13   the same at tol 1e-13 (its distance from the tol 1e-14 run is how far a
                        1e-13 Newton tolerance alone carries a state over the run).
  plain_fp64_tol1e-10   the same at the plain method's tolerance 1e-10.
  learned_pair_tol1e-13 float-pair precision mode (FEDG_PREC_PAIR: explicit operator, Newton
                        residual and RK accumulation in float pairs, FP32 Jacobian/LU), Newton from
                        the column-guess MLP to tol 1e-13.
  learned_fp32_tol1e-10 FP32 explicit mode (FEDG_PREC_MIXED), Newton from the MLP to tol 1e-10.
  pair_tol1e-13/1e-14,  the float-pair and FP32 modes from FElib's guess var0 (no MLP).
  fp32_tol1e-10

Each path is compared with each of the plain FP64 runs that ran (tol 1e-14, 1e-13, 1e-10).

The MLP follows the learned-guess recipe:
  - 193 -> 256 -> 256 -> 192;
  - trained on the GPU on pairs the plain solver generates from 20 random density-current seeds,
    on 4 x 4 x 8 slices of the same mesh.

Errors are computed on the full fields DENS, MOMX, MOMY, MOMZ, RHOT, with momentum measured against
at least 1 m/s of hydrostatic momentum. The deviation fields DDENS and DRHOT are also reported
against their own norms.

With --case C1 --eqs HEVE the warm bubble runs with its own explicit HEVE scheme (ERK_SSP_3s3o),
plain FP64 (plain_fp64_heve) against the float-pair mode (pair_heve).

With --case C5 the stably stratified C5 workload (p = 7, 100 m elements, 16 vertical elements)
runs on --nex x --ney x --nez elements at dt 0.005 s, e.g. a 720-step window on 32 x 32 x 16.

Usage (from the repository root):  PYTHONPATH=fe-project_gb300 python -m fedg.precision [--nex 8 ...]
"""
from __future__ import annotations

import argparse
import json
import sys
import time

import numpy as np

from . import cases
from . import guess as fguess
from . import lib as fl

VARS = ("DENS", "MOMX", "MOMY", "MOMZ", "RHOT")


def _errors(torch, got, ref, dens_hyd, therm_hyd):
    full, dev = {}, {}
    mfloor = float(dens_hyd.norm().item())
    for v, nm in enumerate(VARS):
        d = float((got[v] - ref[v]).norm().item())
        if v == 0:
            den = float((ref[0] + dens_hyd).norm().item())
        elif v == 4:
            den = float((ref[4] + therm_hyd).norm().item())
        else:
            den = max(float(ref[v].norm().item()), mfloor)
        full[nm] = d / den
    for v, nm in ((0, "DDENS"), (4, "DRHOT")):
        dev[nm] = float((got[v] - ref[v]).norm().item()) / max(float(ref[v].norm().item()), 1e-300)
    return full, dev


PATHS = {
    "plain_fp64_tol1e-14": (fl.PREC_FP64, 1e-14, False),
    "plain_fp64_tol1e-13": (fl.PREC_FP64, 1e-13, False),
    "plain_fp64_tol1e-10": (fl.PREC_FP64, 1e-10, False),
    "learned_pair_tol1e-13": (fl.PREC_PAIR, 1e-13, True),
    "learned_pair_tol1e-12": (fl.PREC_PAIR, 1e-12, True),
    "learned_pair_tol1e-11": (fl.PREC_PAIR, 1e-11, True),
    "learned_fp32_tol1e-10": (fl.PREC_MIXED, 1e-10, True),
    "pair_tol1e-14": (fl.PREC_PAIR, 1e-14, False),
    "pair_tol1e-13": (fl.PREC_PAIR, 1e-13, False),
    "fp32_tol1e-10": (fl.PREC_MIXED, 1e-10, False),
}
REFS = ("plain_fp64_tol1e-14", "plain_fp64_tol1e-13", "plain_fp64_tol1e-10")
# HEVE (explicit ERK_SSP_3s3o, no implicit solve): FP64 against float pairs
HEVE_PATHS = {
    "plain_fp64_heve": (fl.PREC_FP64, 0.0, False),
    "pair_heve": (fl.PREC_PAIR, 0.0, False),
}
HEVE_REFS = ("plain_fp64_heve",)


def run(nex=8, ney=8, nez=8, dt=0.04, hours=1.0, checkpoint_min=10.0, chunk=250, paths=tuple(PATHS), seeds=20,
        train_steps=2000, case_name="C2", eqs="HEVI", out=sys.stdout, steps=None, concurrent=False, max_iter=30):
    import dataclasses

    import torch

    # C2: the density current (default); C1: the +2 K warm bubble of the small case, run with the
    # HEVI IMEX scheme of the precision form or (eqs="HEVE") with its own explicit HEVE scheme
    heve = eqs == "HEVE"
    table, refs = (HEVE_PATHS, HEVE_REFS) if heve else (PATHS, REFS)
    if case_name == "C1":
        base = dataclasses.replace(cases.C1(), eqs=eqs)
    else:
        base = cases.C2() if case_name == "C2" else cases.C5()
    case = base.scaled(nex, ney, nez)
    nsteps = steps if steps else int(round(hours * 3600.0 / dt))
    ck_every = max(1, int(round(checkpoint_min * 60.0 / dt)))
    scheme = "HEVE ERK_SSP_3s3o" if heve else "HEVI IMEX-ARK232"
    info = {"workload": f"{case_name} recipe p={case.porder} {nex}x{ney}x{nez} elements, {scheme}",
            "dt": dt, "steps": nsteps, "simulated_s": nsteps * dt, "paths": list(paths), "max_iter": max_iter}
    net = None
    if any(table[p][2] for p in paths):
        t0 = time.perf_counter()
        # learned-guess recipe: about 200k (stage input, converged increment) pairs from 20 seeds
        # of 4x4x8 slices; 5 steps x 2 implicit stages x 1024 columns per seed
        net, ginfo = fguess.build_guess(base.scaled(4, 4, nez), dt, seeds=range(seeds), nsteps=5,
                                        per_stage_keep=None, train_steps=train_steps, batch=4096, lr=1e-3)
        ginfo["build_s"] = time.perf_counter() - t0
        info["guess_training"] = ginfo
    q, b = cases.initial_state(case)
    ctx = fl.Context(case)
    ctx.set_base_state(b["dens_hyd"], b["pres_hyd"], b["therm_hyd"])
    dens_hyd = ctx.tensor(b["dens_hyd"])
    therm_hyd = ctx.tensor(b["therm_hyd"])
    q0 = [ctx.tensor(a) for a in q]
    states = {p: [t.clone() for t in q0] for p in paths}
    # concurrent: one context (own stream and scratch) and one host thread per path, so that the
    # small launch-bound cases of different paths share the GPU; ms_per_step is then wall time
    # under that sharing, not a per-path speed
    ctxs = {p: ctx for p in paths}
    if concurrent and sum(1 for p in paths if table[p][2]) > 1:
        raise ValueError("concurrent paths share one guess network: run at most one learned path")
    if concurrent:
        for p in paths[1:]:
            c2 = fl.Context(case)
            c2.set_base_state(b["dens_hyd"], b["pres_hyd"], b["therm_hyd"])
            ctxs[p] = c2
    info["concurrent_paths"] = bool(concurrent)
    if net is not None:
        for c2 in {id(c): c for c in ctxs.values()}.values():
            net.attach(c2)
    stats = {p: {"s": 0.0, "fail": 0, "its": 0.0} for p in paths}
    done = 0
    print(json.dumps({"setup": info}), file=out, flush=True)
    rec = None

    def advance(p, n):
        prec, tol, guess = table[p]
        t0 = time.perf_counter()
        nf, its = ctxs[p].update(states[p], n, eqs=fl.HEVE if heve else fl.HEVI, prec=prec, dt=dt, max_iter=max_iter,
                                 tol=tol, use_guess=guess, sync=not concurrent)
        ctxs[p].sync()
        s = stats[p]
        s["s"] += time.perf_counter() - t0
        s["fail"] += nf
        s["its"] += its * n

    while done < nsteps:
        n = min(chunk, nsteps - done, ck_every - done % ck_every)
        torch.cuda.synchronize()
        if concurrent:
            import concurrent.futures as cf

            with cf.ThreadPoolExecutor(max_workers=len(paths)) as ex:
                for fut in [ex.submit(advance, p, n) for p in paths]:
                    fut.result()
        else:
            for p in paths:
                advance(p, n)
        torch.cuda.synchronize()
        done += n
        if done % ck_every == 0 or done == nsteps:
            finite = all(bool(torch.isfinite(t).all().item()) for st in states.values() for t in st)
            rec = {"step": done, "t_s": done * dt, "finite": finite, "errors": {}}
            for ref in refs:
                if ref not in states:
                    continue
                for p in paths:
                    if p == ref:
                        continue
                    full, dev = _errors(torch, states[p], states[ref], dens_hyd, therm_hyd)
                    rec["errors"][f"{p} vs {ref}"] = {"rel_l2_full": full, "rel_l2_deviation": dev}
            rec["ms_per_step"] = {p: 1e3 * stats[p]["s"] / done for p in paths}
            rec["mean_solves"] = {p: stats[p]["its"] / done for p in paths}
            rec["nonconverged"] = {p: stats[p]["fail"] for p in paths}
            print(json.dumps(rec), file=out, flush=True)
            if not finite:
                break
    for c2 in {id(c): c for c in ctxs.values()}.values():
        c2.close()
    return rec


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--case", choices=["C2", "C1", "C5"], default="C2")
    ap.add_argument("--eqs", choices=["HEVI", "HEVE"], default="HEVI",
                    help="HEVE: C1 with its explicit scheme, paths " + ", ".join(HEVE_PATHS))
    ap.add_argument("--nex", type=int, default=8)
    ap.add_argument("--ney", type=int, default=8)
    ap.add_argument("--nez", type=int, default=8)
    ap.add_argument("--dt", type=float, default=0.04)
    ap.add_argument("--hours", type=float, default=1.0)
    ap.add_argument("--steps", type=int, default=None, help="number of steps (overrides --hours)")
    ap.add_argument("--max-iter", type=int, default=30, help="Newton solves per implicit stage at most")
    ap.add_argument("--concurrent", action="store_true",
                    help="run the paths at the same time, one context and host thread each")
    ap.add_argument("--checkpoint-min", type=float, default=10.0)
    ap.add_argument("--chunk", type=int, default=250)
    ap.add_argument("--paths", default=None, help="comma-separated subset of " + ", ".join(PATHS))
    ap.add_argument("--seeds", type=int, default=20)
    ap.add_argument("--train-steps", type=int, default=2000)
    a = ap.parse_args(argv)
    import __graft_entry__ as ge  # noqa: F401  (repository root on sys.path when run from it)

    ge.build()
    table = HEVE_PATHS if a.eqs == "HEVE" else PATHS
    if a.eqs == "HEVE" and a.case != "C1":
        ap.error("--eqs HEVE runs the C1 case")
    paths = tuple(p for p in (a.paths or ",".join(table)).split(",") if p)
    unknown = [p for p in paths if p not in table]
    if unknown:
        ap.error(f"unknown paths {unknown}")
    run(a.nex, a.ney, a.nez, a.dt, a.hours, a.checkpoint_min, a.chunk, paths, a.seeds, a.train_steps, a.case, a.eqs,
        steps=a.steps, concurrent=a.concurrent, max_iter=a.max_iter)
    return 0


if __name__ == "__main__":
    sys.path.insert(0, ".")
    sys.exit(main())
