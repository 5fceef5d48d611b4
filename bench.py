#!/usr/bin/env python
"""Benchmark of the SCALE-DG nonhydrostatic 3D DG dynamics step on one GB300.

Workload (default): p=7, 128x128x16 elements over 12.8 x 12.8 x 3.2 km, periodic in x/y,
slip lids, constant Brunt-Vaisala base state (N = 0.01 1/s, theta_sfc = 300 K), i.i.d.
+-0.1 K potential-temperature noise below 500 m (seed 0), u = 5 m/s, HEVI with IMEX
ARK(2,3,2) and the column Newton solve (tol per path, below).  134,217,728 nodes x 5 variables.

A "step" is one full time step (3 RK stages) of the whole domain; the metric is
DOF-stage updates per second = 5 * Np * Ne * 3 * steps / time.

Paths (--path):
  pair   (default) the learned Newton guess with the FP32-pipe float-pair arithmetic
         (FEDG_PREC_PAIR) and the Newton solve to tol 1e-13: the path that stays within 1e-6
         relative L2 of converged FP64 over a simulated hour;
  mixed  the learned guess with FP32 explicit arithmetic (FEDG_PREC_MIXED), Newton tol 1e-10;
  fp64   FElib's algorithm in FP64 on the GPU, Newton tol 1e-10.
The default run also times learned+FP32, the headline path without the guess and the plain
FP64 path on the same state, and reports the error of each against plain FP64; then HEVE (FP64
and float pairs), the tracer advection and the numerical diffusion / sponge on the same mesh.

  python bench.py [--steps K] [--warmup W] [--path pair|mixed|fp64] [--impl fedg|reference]

--impl reference times the CPU implementation of the same step (the FP64 oracle port of
FElib's routines, all host cores) on a bounded sample of the workload.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for p in (os.path.join(ROOT, "fe-project_gb300"), os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

METRIC = "DOF-stage/s on 1 GB300: learned+FP32 vs plain FP64 HEVI, rel L2 err <=1e-6"
UNIT = "DOF-stage/s"
DT_STABLE = 0.005  # C5 geometry (h = 100 m, p = 7): the oracle is stable at 0.005 s, not at 0.01 s

# precision mode (fedg.lib PREC_*), Newton tolerance and iteration cap of each path
PATH_PREC = {"pair": 2, "mixed": 1, "fp64": 0}
PATH_TOL = {"pair": 1e-13, "mixed": 1e-10, "fp64": 1e-10}
PATH_ITER = {"pair": 30, "mixed": 20, "fp64": 20}
PATH_NAME = {"pair": "pair", "mixed": "fp32", "fp64": "plain_fp64"}
# FP64 flops of the plain column solve per node and launch, counted on FElib's algorithm (dense
# block LU with partial pivoting of the 3N1 x 3N1 element blocks, hevi_common_linalgebra.F90:2296-2445):
# per element column (n = 24 at p = 7) 2n^3/3 for the factorisation plus 4 right-hand sides x 2n^2
# for the substitutions, per node (/ N1); the MOMX/MOMY element solves (N1 x N1, 3 right-hand sides)
# and two residual evaluations (Dz of three fluxes, VPOrdM1, Lift: ~100 flop per node each)
def fp64_vi_flops_per_node(N1):
    n = 3 * N1
    return (2 * n ** 3 / 3 + 4 * 2 * n * n) / N1 + (2 * N1 ** 3 / 3 + 3 * 2 * N1 * N1) / N1 + 2 * 100
PATH_DTYPE = {"pair": "f32x2", "mixed": "f32+f32x2", "fp64": "f64"}
# DRAM bytes per node of one launch of the dominant kernel, measured by ncu (dram__bytes_read.sum +
# dram__bytes_write.sum on the 32x32x16-element slice, 8,388,608 nodes; the mean of the step's two
# launches, one per implicit stage), per path
NCU_BYTES_PER_NODE = {
    "pair": {"vi_mixed": ((1126.824704e6 + 656.262912e6) + (1039.029504e6 + 647.403264e6)) / 2 / (32 * 32 * 16 * 512)},
}


# warp instructions per node of one launch of the dominant kernel, measured by ncu
# (smsp__inst_executed.sum on the 32x32x16-element slice, the mean of the step's two launches), per path
NCU_INST_PER_NODE = {
    "pair": {"vi_mixed": (1.841753748e9 + 1.782838923e9) / 2 / (32 * 32 * 16 * 512)},
}


def issue_roofline(kname, path, nodes, avg_ms, sm_mhz, n_sm):
    """The dominant kernel against the SM issue rate, the ceiling of a latency-bound kernel: ncu's
    warp instructions per node times the nodes of one launch over the CUDA-event launch time,
    against 4 schedulers x SMs x the SM clock sampled during the timed region."""
    ipn = NCU_INST_PER_NODE.get(path, {}).get(kname)
    if ipn is None or not avg_ms or avg_ms <= 0:
        return None
    mhz = sm_mhz or 2070.0
    achieved = ipn * nodes / (avg_ms * 1e-3)
    peak = 4.0 * n_sm * mhz * 1e6
    return {"bound": "issue", "kernel": kname, "achieved": achieved, "peak": peak, "unit": "warp instructions/s",
            "frac": achieved / peak, "inst_per_node": ipn, "sm_mhz": mhz, "sms": n_sm,
            "source": "ncu smsp__inst_executed.sum on the 32x32x16 slice, scaled by nodes; peak = 4 x SMs x SM clock"}


def max_over_ranks(value, world, device):
    """The largest of the ranks' values (the slowest replica's time); one rank: the value."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist

    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(units_per_rank, steps, ms_max, world):
    """Whole-job throughput of N independent replicas: the units all ranks processed over the
    slowest rank's time."""
    return units_per_rank * steps * world / (ms_max * 1e-3)


def _env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(
        os.environ.get("LOCAL_RANK", "0"))


# ----------------------------------------------------------------------------------------
# clocks during the timed region
# ----------------------------------------------------------------------------------------
class Clocks:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = max(mx, float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


# ----------------------------------------------------------------------------------------
# CPU leg: the FP64 oracle on a bounded sample of the workload
# ----------------------------------------------------------------------------------------
def cpu_sample(path_kind, seconds_target=15.0):
    """Times the oracle's HEVI ARK232 step on an 8x8x16-element sample of the C5 workload
    (same p, same column depth, same base state and noise); returns DOF-stage/s."""
    import oracle as orc
    from fedg import cases

    case = cases.C5().scaled(8, 8, 16)
    q, b = cases.initial_state(case)
    o = orc.Oracle(case.porder, case.NeX, case.NeY, case.NeZ, case.dom)
    o.set_base_state(b["dens_hyd"], b["pres_hyd"])
    threads = orc.num_threads()
    max_iter, tol = (20, 1e-10)
    t0 = time.perf_counter()
    o.step_hevi(q, DT_STABLE, 1, max_iter=max_iter, tol=tol)
    t1 = time.perf_counter()
    nsteps = max(1, int(seconds_target / max(t1 - t0, 1e-3)))
    nsteps = min(nsteps, 400)
    t2 = time.perf_counter()
    o.step_hevi(q, DT_STABLE, nsteps, max_iter=max_iter, tol=tol)
    t3 = time.perf_counter()
    value = case.dofs * 3 * nsteps / (t3 - t2)
    return {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"FP64 oracle (C++/OpenMP restatement of FElib), HEVI ARK232 Newton tol 1e-10, "
                      f"{nsteps} steps of an 8x8x16-element p=7 sample of the 128x128x16 workload "
                      f"({case.dofs} DOF), {t3 - t2:.1f} s"}


# ----------------------------------------------------------------------------------------
def run_reference(args):
    rank, world, _ = _env_rank()
    if rank != 0:
        return 0
    cb = cpu_sample("reference", seconds_target=max(5.0, 10.0 * max(args.steps, 1) / 5.0))
    line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "C5 p=7 128x128x16 HEVI IMEX-ARK232 (8x8x16-element sample on the host cores)",
                       "dt": DT_STABLE},
            "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def fp64_dgemm_tflops(torch, dev):
    """Measured FP64 matrix throughput (cuBLAS DGEMM 4096^3, best of 3) -- the FP64 roofline."""
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device=dev)
    b = torch.randn(n, n, dtype=torch.float64, device=dev)
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e30
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    del a, b
    return 2.0 * n ** 3 / (best * 1e-3) / 1e12


def c4_guess_bench(np, torch, fl, cases, stream, nsteps=10):
    """The learned-guess workload (C4): the C2 geometry (p = 7, 800 m elements, 64 levels per
    column: 193 -> 256 -> 256 -> 192), trained with Adam (lr 1e-3, batch 4096) on 204,800 (column state,
    converged increment) pairs that the plain solver generates from 20 seeds of random bubbles and
    winds; then, on a held-out seed, the mean Newton solves per implicit column solve and ms per step
    with and without the learned iterate, in the FP32 mode (tol 1e-10) and the float-pair mode (tol
    1e-13), on a 16x16x8-element slice at dt 0.04 s (the stable step of this mesh)."""
    from fedg import guess

    dt = 0.04
    base = cases.C2().scaled(8, 8, 8)
    t0 = time.perf_counter()
    net, info = guess.build_guess(base, dt, seeds=range(20), nsteps=2, per_stage_keep=2560, train_steps=2000,
                                  batch=4096, lr=1e-3)
    info["build_s"] = time.perf_counter() - t0
    case = guess.random_case(cases.C2().scaled(16, 16, 8), np.random.default_rng(1000))
    q, b = cases.initial_state(case)
    ctx = fl.Context(case)
    ctx.set_base_state(b["dens_hyd"], b["pres_hyd"], b["therm_hyd"])
    net.attach(ctx)
    out = {"training": info, "workload": f"C2 geometry, {case.NeX}x{case.NeY}x{case.NeZ} elements, dt {dt} s, "
                                          f"{nsteps} steps, held-out seed", "paths": {}}
    for name, prec, tol in (("fp32", fl.PREC_MIXED, 1e-10), ("pair", fl.PREC_PAIR, 1e-13)):
        for g in (False, True):
            qd = [ctx.tensor(a) for a in q]
            ctx.update(qd, 1, prec=prec, dt=dt, max_iter=30, tol=tol, use_guess=g)
            ms, nf, its = _timed_update(ctx, torch, torch.cuda.ExternalStream(ctx.stream_handle), qd, nsteps,
                                        dict(prec=prec, dt=dt, max_iter=30, tol=tol, use_guess=g))
            out["paths"][name + ("_learned" if g else "_plain")] = {
                "mean_newton_solves": its, "ms_per_step": ms / nsteps, "nonconverged_columns": nf, "newton_tol": tol}
    ctx.close()
    return out


def _timed_update(ctx, torch, stream, qd, steps, opts):
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    nfail, its = ctx.update(qd, steps, sync=False, **opts)
    e1.record(stream)
    ctx.sync()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1), nfail, its


def _full_field_errors(np, got, ref, dens_hyd_norm_sq, dens_hyd, therm_hyd):
    """rel L2 per variable of DENS, MOMX, MOMY, MOMZ, RHOT (momentum against at least 1 m/s of
    hydrostatic momentum) between two device states, computed on the device."""
    out = {}
    names = ["DENS", "MOMX", "MOMY", "MOMZ", "RHOT"]
    for v, nm in enumerate(names):
        d = float((got[v] - ref[v]).double().norm().item())
        if v == 0:
            den = float((ref[0] + dens_hyd).norm().item())
        elif v == 4:
            den = float((ref[4] + therm_hyd).norm().item())
        else:
            den = max(float(ref[v].norm().item()), dens_hyd_norm_sq ** 0.5)
        out[nm] = d / den
    return out


TRC_DT = 0.5  # tracer step on the C5 mesh: |u| ~ 6 m/s, element 100 m at p = 7 (stable up to ~1 s)


def tracer_bench(args, torch, np, fl, cases, peaks, peak_src, steps, warmup):
    """Tracer advection (FElib's trcadvect3d_heve + tracer driver; the advection-test configuration
    ONLY_TRACERADV_FLAG) on the bench mesh: one cosine-bell tracer carried by the mass flux of the C5
    state with (u, v) = (5, -3) m/s, FCT + TMAR, ERK_SSP_3s3o, FP64.  DOF = one tracer value per node."""
    from dataclasses import replace

    base = cases.C5().scaled(32, 32, 16) if args.small else cases.C5()
    x0, x1, y0, y1, z0, z1 = base.dom
    case = replace(base, v0=-3.0, filter_on=False,
                   tracer=dict(qmax=1.0, rx=0.25 * (x1 - x0), ry=0.25 * (y1 - y0), rz=0.3 * (z1 - z0),
                               xc=0.5 * (x0 + x1), yc=0.5 * (y0 + y1), zc=0.35 * (z1 - z0)))
    q, b = cases.initial_state(case)
    Q = cases.tracer_state(case)
    ctx = fl.Context(case)
    ctx.set_base_state(b["dens_hyd"], b["pres_hyd"], b["therm_hyd"])
    qd = [ctx.tensor(a) for a in q[:4]]
    del q
    Qh = torch.from_numpy(np.ascontiguousarray(Q)).pin_memory()
    Qd = ctx.tensor(Q)
    mf = qd[1:4]
    aM, aP = ctx.trc_alphdens_advtest(qd[0], qd[1], qd[2], qd[3])
    stream = torch.cuda.ExternalStream(ctx.stream_handle)

    def timed(prec, Qt):
        ctx.trc_update(Qt, mf, aM, aP, qd[0], qd[0], TRC_DT, nsteps=warmup, prec=prec)
        fl.prof_reset(ctx)
        fl.prof_enable(ctx, True)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ctx.trc_update(Qt, mf, aM, aP, qd[0], qd[0], TRC_DT, nsteps=steps, sync=False, prec=prec)
        e1.record(stream)
        ctx.sync()
        torch.cuda.synchronize()
        fl.prof_enable(ctx, False)
        pr = {k: v for k, v in fl.prof_read(ctx).items() if k.startswith("trc") and v[1]}
        return e0.elapsed_time(e1), pr

    # FP64 (FElib's arithmetic) on a copy, then the float-pair path on Qd: same state, same steps
    Q64 = Qd.clone()
    ms64, prof64 = timed(fl.PREC_FP64, Q64)
    ms, prof = timed(fl.PREC_PAIR, Qd)
    pair_vs_fp64 = float((Qd - Q64).norm().item() / max(Q64.norm().item(), 1e-300))
    del Q64
    nodes = case.Np * case.Ne
    value = nodes * 3 * steps / (ms * 1e-3)
    nf_per_node = 6 * case.N1 ** 2 / case.Np  # face nodes per volume node
    # algorithmic bytes per node of one launch (one read or write per array element; pairs and FP64
    # values are both 8 bytes):
    #   trc_fct:   Q, MFLX x3, DDENS_TRC, DDENS0_TRC + alph_dens M/P on the faces
    #   trc_stage: the same inputs, the stage output, and var0 / varTmp (mean of the three stages)
    algo = {"trc_fct": 8 * 6 + 16 * nf_per_node, "trc_stage": 8 * 6 + 16 * nf_per_node + (24 + 16 + 16) / 3}

    def kern_table(pr):
        out = {}
        for k, (kms, kn) in pr.items():
            avg = kms / kn
            ach = algo.get(k, 0.0) * nodes / (avg * 1e-3) / 1e9
            out[k] = {"ms": kms, "launches": kn, "avg_launch_ms": avg, "algorithmic_bytes_per_node": algo.get(k),
                      "achieved_gbs": ach, "frac_of_hbm": ach / peaks.get("hbm_gbs", 6800.0)}
        return out

    kern = kern_table(prof)
    top = max(kern, key=lambda k: kern[k]["ms"]) if kern else None
    roof = None
    if top:
        roof = {"bound": "hbm", "kernel": top, "achieved": kern[top]["achieved_gbs"], "peak": peaks.get("hbm_gbs", 6800.0),
                "unit": "GB/s", "frac": kern[top]["frac_of_hbm"], "peak_source": peak_src,
                "note": "float-pair tracer kernels"}
    # end to end: the step's inputs (QTRC, MFLX x3, alph_dens M/P, DDENS_TRC, DDENS0_TRC) from pinned host
    # memory, one tracer step, QTRC back to the host
    e2e = None
    if not args.no_e2e:
        hs = [Qh] + [t.cpu().pin_memory() for t in (mf[0], mf[1], mf[2], aM, aP, qd[0], qd[0])]
        ds = [torch.empty_like(Qd)] + [torch.empty_like(t) for t in (mf[0], mf[1], mf[2], aM, aP, qd[0], qd[0])]
        ke = max(1, min(steps, 3))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(ke):
            for d_, h_ in zip(ds, hs):
                d_.copy_(h_, non_blocking=True)
            torch.cuda.synchronize()
            ctx.trc_update(ds[0], ds[1:4], ds[4], ds[5], ds[6], ds[7], TRC_DT, nsteps=1, sync=False,
                           prec=fl.PREC_PAIR)
            ctx.sync()
            Qh.copy_(ds[0], non_blocking=True)
            torch.cuda.synchronize()
        t1 = time.perf_counter()
        e2e = {"value": nodes * 3 * ke / (t1 - t0), "unit": UNIT,
               "h2d_bytes_per_step": int(sum(h.numel() * 8 for h in hs)), "d2h_bytes_per_step": int(Qd.numel() * 8),
               "steps": ke}
        del hs, ds
    finite = bool(torch.isfinite(Qd).all().item())
    qmin = float(Qd.min().item())
    cb = None
    if not args.no_cpu:
        import oracle as orc

        sc = case.scaled(8, 8, 16)
        qs, bs = cases.initial_state(sc)
        o = orc.Oracle(sc.porder, sc.NeX, sc.NeY, sc.NeZ, sc.dom)
        o.set_base_state(bs["dens_hyd"], bs["pres_hyd"])
        am, ap = o.trc_alphdens_advtest(qs[0], qs[1], qs[2], qs[3])
        Qs = cases.tracer_state(sc)
        t0 = time.perf_counter()
        o.trc_step(Qs, qs[1:4], am, ap, qs[0], qs[0], TRC_DT, nsteps=1)
        t1 = time.perf_counter()
        ns = max(1, min(400, int(8.0 / max(t1 - t0, 1e-3))))
        t2 = time.perf_counter()
        o.trc_step(Qs, qs[1:4], am, ap, qs[0], qs[0], TRC_DT, nsteps=ns)
        t3 = time.perf_counter()
        cb = {"value": sc.Np * sc.Ne * 3 * ns / (t3 - t2), "unit": UNIT, "cores": orc.num_threads(), "kind": "port",
              "sample": f"FP64 oracle tracer step (FCT + TMAR, SSP-RK3), {ns} steps of an 8x8x16-element p=7 "
                        f"sample of the same workload, {t3 - t2:.1f} s"}
    ctx.close()
    return {"metric": "tracer DOF-stage/s (one tracer, FCT + TMAR, ERK_SSP_3s3o)", "value": value, "unit": UNIT,
            "ms_per_step": ms / steps, "steps": steps, "dt": TRC_DT, "dtype": "f32x2", "path": "float pairs",
            "fp64": {"value": nodes * 3 * steps / (ms64 * 1e-3), "ms_per_step": ms64 / steps,
                     "kernels": kern_table(prof64)},
            "rel_l2_pair_vs_fp64": pair_vs_fp64,
            "workload": f"C5 mesh p=7 {case.NeX}x{case.NeY}x{case.NeZ}, cosine-bell tracer, (u, v) = (5, -3) m/s",
            "kernels": kern, "roofline": roof, "e2e": e2e, "cpu_baseline": cb, "finite": finite, "min_q": qmin,
            "gpu_launches": sum(v[1] for v in prof.values())}


def heve_bench(args, torch, np, fl, ctx, q_host, dofs_stage, dnorm2, dens_hyd, therm_hyd):
    """The HEVE scheme (config 1's explicit SSP-RK3 with the vertical terms explicit) on the bench
    workload: plain FP64 against the float-pair mode, from the same state, dt half the HEVI step.
    DOF-stage/s as for the headline (3 stages per step); the full-field relative L2 of the pair
    path against FP64 after the timed steps."""
    stream = torch.cuda.ExternalStream(ctx.stream_handle)
    dt = 0.5 * DT_STABLE
    out = {"dt": dt, "steps": args.steps}
    qs = {}
    for name, prec in (("fp64", fl.PREC_FP64), ("pair", fl.PREC_PAIR)):
        q = [torch.empty(h.shape, dtype=h.dtype, device=ctx.dev) for h in q_host]
        for a, h in zip(q, q_host):
            a.copy_(h)
        o = dict(eqs=fl.HEVE, prec=prec, dt=dt)
        ctx.update(q, 1, **o)  # warm-up step (also allocates the pair scratch)
        for a, h in zip(q, q_host):
            a.copy_(h)
        fl.prof_reset(ctx)
        fl.prof_enable(ctx, True)
        ms, _, _ = _timed_update(ctx, torch, stream, q, args.steps, o)
        fl.prof_enable(ctx, False)
        launches = sum(v[1] for v in fl.prof_read(ctx).values())
        out[name] = {"value": dofs_stage * args.steps / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms / args.steps,
                     "gpu_launches_per_step": launches / args.steps}
        qs[name] = q
    out["speedup_pair_vs_fp64"] = out["pair"]["value"] / out["fp64"]["value"]
    out["pair_rel_l2_vs_fp64"] = _full_field_errors(np, qs["pair"], qs["fp64"], dnorm2, dens_hyd, therm_hyd)
    del qs
    return out


def numdiff_bench(args, torch, np, fl, ctx, qd, peaks, peak_src, case):
    """Numerical diffusion (FElib's hyperdiffusion filter, nonhydro3d_numdiff.F90) and the sponge layer
    (dgm_spongelayer.F90) on the bench state: one application each, FP64.  DOF = one value of one
    prognostic variable; the filter touches 5 variables per application."""
    stream = torch.cuda.ExternalStream(ctx.stream_handle)
    nodes = case.Np * case.Ne
    out = {}
    q = [t.clone() for t in qd]
    for nlap, coef, prec in ((1, 1.0e2, fl.PREC_FP64), (2, 1.0e5, fl.PREC_FP64), (1, 1.0e2, fl.PREC_PAIR),
                             (2, 1.0e5, fl.PREC_PAIR)):
        ctx.numdiff_apply(q, nlap, coef, coef, 1e-3, prec=prec)  # warm-up (allocates the scratch)
        fl.prof_reset(ctx)
        fl.prof_enable(ctx, True)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            ctx.lib.fedg_numdiff_apply_prec(ctx.h, fl._p5(q), nlap, coef, coef, 1e-3, prec)
        e1.record(stream)
        ctx.sync()
        torch.cuda.synchronize()
        fl.prof_enable(ctx, False)
        ms = e0.elapsed_time(e1) / args.steps
        launches = fl.prof_read(ctx)["numdiff"][1] // args.steps
        # algorithmic bytes per node and variable: gradient pass reads q (+ DDENS) and writes G (3);
        # each extra Laplacian pass reads G (3), writes 2, reads 2, writes 3; the tendency pass reads
        # G (3) + DDENS and updates q (read + write)
        bpn = 8 * ((2 + 3) + (nlap - 1) * (3 + 2 + 2 + 3) + (3 + 1 + 2))
        gbs = 5 * bpn * nodes / (ms * 1e-3) / 1e9
        out[f"nlap{nlap}_{'pair' if prec == fl.PREC_PAIR else 'fp64'}"] = {
                              "value": 5 * nodes / (ms * 1e-3), "unit": "DOF/s", "ms_per_apply": ms,
                              "launches_per_apply": launches, "algorithmic_bytes_per_node_var": bpn,
                              "achieved_gbs": gbs, "frac_of_hbm": gbs / peaks.get("hbm_gbs", 6800.0),
                              "peak_source": peak_src}
    del q
    tend = [torch.zeros_like(qd[1]) for _ in range(3)]
    ztop = case.dom[5]
    ctx.sponge_add_tend(tend, qd[1:4], 30.0, 0.5 * ztop, True)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        ctx.lib.fedg_sponge_add_tend(ctx.h, (fl.ctypes.c_void_p * 3)(*[x.data_ptr() for x in tend]),
                                     (fl.ctypes.c_void_p * 3)(*[x.data_ptr() for x in qd[1:4]]), 30.0, 0.5 * ztop, 1)
    e1.record(stream)
    ctx.sync()
    ms = e0.elapsed_time(e1) / args.steps
    gbs = 8 * 9 * nodes / (ms * 1e-3) / 1e9  # 3 tendencies read + written, 3 momenta read
    out["sponge"] = {"ms_per_call": ms, "achieved_gbs": gbs, "frac_of_hbm": gbs / peaks.get("hbm_gbs", 6800.0)}
    del tend
    return out


def run_fedg(args):
    import numpy as np
    import torch

    import __graft_entry__ as ge
    rank, world, local = _env_rank()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    if rank == 0:
        ge.build()
    if world > 1:
        dist.barrier()
    from fedg import cases
    from fedg import lib as fl

    case = cases.C5()
    if args.small:
        case = case.scaled(32, 32, 16)
    if world > 1:
        # one slab of a domain split along x (weak scaling: every rank holds a whole C5 mesh, the
        # domain is world times as long in x); the x faces are exchanged over NCCL before every stage
        from fedg import slabs

        case = slabs.slab_case(case, rank, world, weak=True)
    side = rank == 0 and world == 1  # the side measurements run on one GPU only
    path = args.path
    prec = PATH_PREC[path]
    use_guess = path != "fp64" and bool(args.guess)
    guess_side = path != "fp64" and not use_guess and not args.no_guess_side and side
    net, ginfo = None, None
    if use_guess or guess_side:
        # the C5 column network (128 levels: 385 -> 256 -> 256 -> 384), trained on the GPU with the
        # library's kernels on (stage input, converged increment) pairs of the plain solver on a
        # 16x16x16-element slice of the same geometry, 8 noise/wind seeds
        from fedg import guess

        t0 = time.perf_counter()
        net, ginfo = guess.build_guess(cases.C5().scaled(16, 16, 16), DT_STABLE, seeds=range(100, 108), nsteps=3,
                                       per_stage_keep=4096, train_steps=args.train_steps, batch=4096, lr=1e-3)
        ginfo["build_s"] = time.perf_counter() - t0
    q, b = cases.initial_state(case)
    ctx = fl.Context(case, device=local, periodic_x=fl.HALO if world > 1 else 1)
    ctx.set_base_state(b["dens_hyd"], b["pres_hyd"], b["therm_hyd"])
    halo = None
    if world > 1:
        # the slabs share the case's mean wind as the reference of the momentum deviations
        ctx.set_ref_wind(case.u0, case.v0)
        # slabs along x: halo buffers on the x- and x+ sides only
        hsend = [torch.empty(ctx.halo_bytes(sd), dtype=torch.uint8, device=ctx.dev) if sd < 2 else None
                 for sd in range(4)]
        hrecv = [torch.zeros(ctx.halo_bytes(sd), dtype=torch.uint8, device=ctx.dev) if sd < 2 else None
                 for sd in range(4)]
        halo = slabs.HaloExchange(hsend, hrecv, rank, world)
        ctx.set_halo(hsend, hrecv, halo)
    dens_hyd = ctx.tensor(b["dens_hyd"])
    therm_hyd = ctx.tensor(b["therm_hyd"])
    dnorm2 = float((dens_hyd * dens_hyd).sum().item())
    del b
    qd = [ctx.tensor(a) for a in q]
    q_host = [torch.from_numpy(np.ascontiguousarray(a)).pin_memory() for a in q]
    del q
    if net is not None:
        net.attach(ctx)  # used by the headline only with --guess 1; otherwise by the with_guess side run
    stream = torch.cuda.ExternalStream(ctx.stream_handle)
    if args.tol is not None:
        PATH_TOL[path] = args.tol
    opts = dict(prec=prec, dt=DT_STABLE, max_iter=PATH_ITER[path], tol=PATH_TOL[path], use_guess=use_guess)

    # warm-up
    ctx.update(qd, args.warmup, **opts)
    # timed region: K steps of the whole domain; the inputs (FP64 state 5.4 GB) are larger than L2
    fl.prof_reset(ctx)
    fl.prof_enable(ctx, True)
    clk = Clocks(local)
    clk.start()
    if world > 1:
        dist.barrier()
    ms, nfail, its = _timed_update(ctx, torch, stream, qd, args.steps, opts)
    clocks = clk.stop()
    fl.prof_enable(ctx, False)
    prof = fl.prof_read(ctx)
    ms = max_over_ranks(ms, world, "cuda")
    dofs_stage = case.dofs * 3
    value = replica_throughput(dofs_stage, args.steps, ms, world)

    # dominant kernel and its roofline
    peaks, peak_src = measured_peaks()
    kname = max(prof, key=lambda k: prof[k][0])
    ktime, klaunch = prof[kname]
    nodes = case.Np * case.Ne
    # algorithmic bytes per node per launch (one read/write of each array element)
    bytes_per_node = {
        "vi_fp64": 8 * (5 + 5 + 5),          # q*, var0 in; tend_im out
        "tend_fp64": 8 * (6 + 5),            # 5 fields + DPRES in; 5 tendencies out
        "rk": 8 * 20,                        # general IMEX advance (upper bound of the stage kinds)
        # fused stage kernels, mean of the three (FP32 deviation state in, FP64 q^n / q* ):
        # S1 q^n(f32) + q^n(f64) in -> q*_2, S3, SF out; S2 Q_2(f32), t_im, q^n, S3, SF in -> q*_3, SF out;
        # S3 Q_3(f32), t_im, q^n, SF in -> q^n+1 (f64) + its f32 copy out; S1 also writes A(q^n) of
        # DENS, MOMZ, RHOT (3 pairs) for the column solve's first residual
        "stage_mixed": (20 + 40 + 40 + 20 + 20 + 20 + 20 + 40 + 20 + 20 + 40 + 20 + 20 + 40 + 20 + 40 + 20 + 24) / 3,
        # column solve: q* (float pairs) and var0 (FP64) in -> Q and t_im out, FP32 in the FP32 mode and
        # float pairs in the pair mode; plus the three guess fields (FP32) when the guess is on, else
        # the stage-1 kernel's A(var0) of DENS, MOMZ, RHOT (pairs) for the first residual
        "vi_mixed": 8 * 5 + 8 * 5 + (8 if prec == fl.PREC_PAIR else 4) * 10 + (12 if use_guess else 24),
        "filter": 8 * 10, "drhot2pres": 8 * 2, "mlp": 0, "aux": 0,
    }
    avg_ms = ktime / max(klaunch, 1)
    achieved = bytes_per_node.get(kname, 0) * nodes / (avg_ms * 1e-3) / 1e9 if avg_ms > 0 else 0.0
    # DRAM bytes per node of one launch measured by ncu (dram__bytes_read.sum + dram__bytes_write.sum
    # of the kernel on the 32x32x16-element slice), scaled to this workload's node count
    ncu_bytes_per_node = NCU_BYTES_PER_NODE.get(path, {})
    traffic = ncu_bytes_per_node[kname] * nodes / 1e9 if kname in ncu_bytes_per_node else None
    roof = {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": peaks.get("hbm_gbs", 6800.0),
            "unit": "GB/s", "frac": achieved / peaks.get("hbm_gbs", 6800.0), "traffic": traffic,
            "traffic_unit": "GB per launch (ncu DRAM read+write of the same path on the 32x32x16 slice, scaled by nodes)",
            "peak_source": peak_src, "avg_launch_ms": avg_ms, "algorithmic_bytes_per_node": bytes_per_node.get(kname)}
    n_sm = torch.cuda.get_device_properties(ctx.dev).multi_processor_count
    roof_issue = issue_roofline(kname, path, nodes, avg_ms, (clocks or {}).get("sm_mhz"), n_sm)
    fp64_tf = fp64_dgemm_tflops(torch, ctx.dev) if rank == 0 else 0.0
    gpu_launches = sum(v[1] for v in prof.values())

    # end to end through the public API with host buffers (fedg_update_host): per step the H2D of the
    # state from the pinned host arrays, the step, and the result back in the host arrays (stored by the
    # last stage kernel in the float-pair path).  It starts from the state the timed region ended at
    # (the same point of the same simulation); the comparisons below start from there too.
    for h_, t_ in zip(q_host, qd):
        h_.copy_(t_)
    e2e = None
    if not args.no_e2e:  # every rank: each slab's state crosses its own host link
        ke = max(1, min(args.steps, 3))
        nb = sum(t.numel() * 8 for t in qd)
        ctx.update_host(q_host, 1, **opts)  # one untimed call first, identical to the timed ones
        each = []
        if world > 1:
            dist.barrier()
        t0 = time.perf_counter()
        for _ in range(ke):
            ta = time.perf_counter()
            ctx.update_host(q_host, 1, **opts)
            each.append(1e3 * (time.perf_counter() - ta))
        t1 = time.perf_counter()
        e2e_ms = max_over_ranks(1e3 * (t1 - t0), world, "cuda")
        e2e = {"value": replica_throughput(dofs_stage, ke, e2e_ms, world), "unit": UNIT, "h2d_bytes_per_step": nb,
               "d2h_bytes_per_step": nb, "steps": ke, "ms_each": each,
               "api": "fedg_update_host (H2D copies, the step, the result stored into the pinned host arrays "
                      + ("by the last stage kernel)" if prec == fl.PREC_PAIR else "by D2H copies after the step)")}
        if side:
            # the same with the copies outside the library: H2D, the device-array update, D2H, each timed
            q_e = [torch.empty_like(t) for t in qd]
            ph = [0.0, 0.0, 0.0]
            for it in range(ke + 1):  # the first round trip untimed
                ta = time.perf_counter()
                for dst, src in zip(q_e, q_host):
                    dst.copy_(src, non_blocking=True)
                torch.cuda.synchronize()
                tb = time.perf_counter()
                ctx.update(q_e, 1, sync=False, **opts)
                ctx.sync()
                tc = time.perf_counter()
                for dst, src in zip(q_host, q_e):
                    dst.copy_(src, non_blocking=True)
                torch.cuda.synchronize()
                td = time.perf_counter()
                if it:
                    ph[0] += tb - ta
                    ph[1] += tc - tb
                    ph[2] += td - tc
            e2e["separate_copies"] = {
                "value": dofs_stage * ke / sum(ph), "ms_per_step": {"h2d": 1e3 * ph[0] / ke, "update": 1e3 * ph[1] / ke,
                                                                   "d2h": 1e3 * ph[2] / ke},
                "copy_gbs": {"h2d": nb * ke / max(ph[0], 1e-9) / 1e9, "d2h": nb * ke / max(ph[2], 1e-9) / 1e9}}
            del q_e

    # the headline path without the learned guess, the other precision mode, and the plain FP64 path, on
    # the same state
    noguess, withguess, plain, acc, other = None, None, None, None, None
    if side and use_guess:
        o2 = dict(opts, use_guess=False)
        ms2, nf2, its2 = _timed_update(ctx, torch, stream, qd, args.steps, o2)
        noguess = {"value": dofs_stage * args.steps / (ms2 * 1e-3), "unit": UNIT, "ms_per_step": ms2 / args.steps,
                   "newton_tol": opts["tol"], "mean_newton_solves": its2, "nonconverged_columns": nf2}
    if side and guess_side:
        # the headline path with the learned initial iterate, on the same state
        o2 = dict(opts, use_guess=True)
        ctx.update(qd, 1, **o2)
        fl.prof_reset(ctx)
        fl.prof_enable(ctx, True)
        ms2, nf2, its2 = _timed_update(ctx, torch, stream, qd, args.steps, o2)
        fl.prof_enable(ctx, False)
        pg = fl.prof_read(ctx)
        withguess = {"value": dofs_stage * args.steps / (ms2 * 1e-3), "unit": UNIT, "ms_per_step": ms2 / args.steps,
                     "newton_tol": opts["tol"], "mean_newton_solves": its2, "nonconverged_columns": nf2,
                     "guess_network_ms_per_step": pg["mlp"][0] / args.steps,
                     "column_solve_ms_per_step": pg["vi_mixed"][0] / args.steps}
    c4 = None
    if side and path != "fp64" and not args.no_c4:
        c4 = c4_guess_bench(np, torch, fl, cases, stream)
    other_path = {"pair": "mixed", "mixed": "pair"}.get(path)
    if side and other_path and not args.no_other:
        op_ = dict(opts, prec=PATH_PREC[other_path], tol=PATH_TOL[other_path], max_iter=PATH_ITER[other_path])
        ctx.update(qd, 1, **op_)
        mso, nfo, itso = _timed_update(ctx, torch, stream, qd, args.steps, op_)
        other = {"value": dofs_stage * args.steps / (mso * 1e-3), "unit": UNIT, "ms_per_step": mso / args.steps,
                 "newton_tol": op_["tol"], "mean_newton_solves": itso, "nonconverged_columns": nfo,
                 "path": ("learned+" if use_guess else "") + PATH_NAME[other_path]}
    if side and prec != fl.PREC_FP64 and not args.no_plain:
        # FElib's algorithm in FP64 on the GPU from the same initial state, and the error of each
        # precision mode against it after the same number of steps
        q_ref = [torch.empty_like(t) for t in qd]
        q_mix = [torch.empty_like(t) for t in qd]
        for a, h in zip(q_ref, q_host):
            a.copy_(h)
        for a, h in zip(q_mix, q_host):
            a.copy_(h)
        ncmp = args.compare_steps
        o64 = dict(opts, prec=fl.PREC_FP64, use_guess=False, tol=1e-10, max_iter=20)
        ctx.update(q_ref, max(ncmp - 2, 0), **o64)
        fl.prof_reset(ctx)
        fl.prof_enable(ctx, True)
        pms, nf64, its64 = _timed_update(ctx, torch, stream, q_ref, 2, o64)
        fl.prof_enable(ctx, False)
        p64 = fl.prof_read(ctx)
        plain = {"value": dofs_stage * 2 / (pms * 1e-3), "unit": UNIT, "ms_per_step": pms / 2, "steps": 2,
                 "newton_tol": 1e-10, "mean_newton_solves": its64, "nonconverged_columns": nf64,
                 "kernels": {k: {"ms": v[0], "launches": v[1]} for k, v in p64.items() if v[1]}}
        vt, vn = p64.get("vi_fp64", (0.0, 0))
        if vn and fp64_tf > 0:
            fpn = fp64_vi_flops_per_node(case.N1) * max(its64, 1.0)
            ach = fpn * nodes / (vt / vn * 1e-3) / 1e12
            plain["roofline_fp64_column_solve"] = {
                "bound": "fp64", "kernel": "vi_fp64", "achieved_tflops": ach, "peak_tflops": fp64_tf,
                "frac": ach / fp64_tf, "flop_per_node": fpn, "avg_launch_ms": vt / vn,
                "flop_count": "FElib's dense block LU with partial pivoting, its substitutions and the residuals, "
                              "per Newton solve; the kernel itself skips the DENS rows' structural zeros"}
        ctx.update(q_mix, ncmp, **opts)
        acc = {"steps": ncmp, "rel_l2_vs_plain_fp64": _full_field_errors(np, q_mix, q_ref, dnorm2, dens_hyd, therm_hyd)}
        if other is not None:
            for a, h in zip(q_mix, q_host):
                a.copy_(h)
            ctx.update(q_mix, ncmp, **dict(opts, prec=PATH_PREC[other_path], tol=PATH_TOL[other_path],
                                           max_iter=PATH_ITER[other_path]))
            other["rel_l2_vs_plain_fp64"] = _full_field_errors(np, q_mix, q_ref, dnorm2, dens_hyd, therm_hyd)
        del q_ref, q_mix

    cb = None
    if side and not args.no_cpu:
        cb = cpu_sample(path)
    trc = None
    if side and not args.no_tracer:
        trc = tracer_bench(args, torch, np, fl, cases, peaks, peak_src, args.steps, args.warmup)
    ndf = None
    if side and not args.no_numdiff:
        ndf = numdiff_bench(args, torch, np, fl, ctx, qd, peaks, peak_src, case)
    hv = None
    if side and not args.no_heve:
        hv = heve_bench(args, torch, np, fl, ctx, q_host, dofs_stage, dnorm2, dens_hyd, therm_hyd)

    finite = all(bool(torch.isfinite(t).all().item()) for t in qd)
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": PATH_DTYPE[path], "data": "synthetic",
            "config": {"workload": f"{case.name}: p=7 {case.NeX}x{case.NeY}x{case.NeZ} elements, HEVI IMEX-ARK232, "
                                   f"constBVFreq N=0.01, +-0.1K noise below 500 m, u=5 m/s",
                       "path": ("learned+" if use_guess else "") + PATH_NAME[path],
                       "one_hour_accuracy": "fe-project_gb300/fedg/precision.py (C1 warm bubble and C2 density current)",
                       "dt": DT_STABLE, "dt_baseline": 0.5, "newton_tol": opts["tol"], "newton_max_iter": opts["max_iter"],
                       "mean_newton_solves": its, "nonconverged_columns": nfail, "finite": finite,
                       "l2": "inputs larger than L2 (FP64 state %.1f GB)" % (case.dofs * 8 / 1e9),
                       "parallelism": "slabs" if world > 1 else "single",
                       "halo_bytes_sent_per_stage": 2 * halo.send[0].numel() if halo else 0},
            "roofline": roof,
            "roofline_issue": roof_issue,
            "roofline_fp64": {"bound": "fp64", "peak_tflops": fp64_tf, "peak_source": "measured cuBLAS DGEMM 4096^3"},
            "kernels": {k: {"ms": v[0], "launches": v[1]} for k, v in prof.items() if v[1]},
            "cpu_baseline": cb, "e2e": e2e, "gpu_launches": gpu_launches, "clocks": clocks,
            "guess_training": ginfo,
            "without_guess": noguess,
            "with_guess": withguess,
            "learned_guess_c4": c4,
            ("fp32_mode" if other_path == "mixed" else "pair_mode"): other,
            "plain_fp64": plain,
            "speedup_vs_plain_fp64": (value / plain["value"]) if plain else None,
            "accuracy": acc,
            "tracer_advection": trc,
            "numdiff_sponge": ndf,
            "heve": hv,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["fedg", "reference"], default="fedg")
    ap.add_argument("--path", choices=["pair", "mixed", "fp64"], default=os.environ.get("FEDG_BENCH_PATH", "pair"))
    ap.add_argument("--guess", type=int, default=0, help="1: the headline path uses the learned Newton iterate")
    ap.add_argument("--no-guess-side", action="store_true", help="skip the with_guess side measurement")
    ap.add_argument("--no-c4", action="store_true", help="skip the C4 learned-guess measurement")
    ap.add_argument("--tol", type=float, default=None, help="Newton tolerance of the timed path (default per path)")
    ap.add_argument("--train-steps", type=int, default=2000)
    ap.add_argument("--compare-steps", type=int, default=4,
                    help="steps of the accuracy comparison against the plain FP64 path")
    ap.add_argument("--small", action="store_true", help="32x32x16 elements instead of 128x128x16 (profiling)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-heve", action="store_true", help="skip the HEVE (FP64 vs float pairs) side measurement")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain FP64 comparison run")
    ap.add_argument("--no-other", action="store_true", help="skip the run of the other precision mode")
    ap.add_argument("--no-tracer", action="store_true", help="skip the tracer-advection measurement")
    ap.add_argument("--no-numdiff", action="store_true", help="skip the numerical-diffusion / sponge measurement")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_fedg(args)


if __name__ == "__main__":
    sys.exit(main())
