"""Writes the golden input/output vectors of tests/golden/ from the FP64 oracle.

FElib itself cannot be built or imported here (Fortran 2008 + MPI + LAPACK + the SCALE library,
none of them in this image), so the goldens are the oracle's outputs on small seeded cases; the
oracle is pinned to FElib's own known-answer tests (tests/test_oracle_kat.py).  They let the
CPU suite catch any drift of the oracle (tests/test_golden.py) and let the GPU suite compare the
CUDA path against stored vectors without running the oracle (tests/test_gpu_golden.py).

Cases (inputs = the cases.py initial states, so only the outputs are stored):
  heve_C1_3x3x3   p=3, 27 elements, HEVE SSP-RK3, dt 0.02 s, 10 steps
  hevi_C1_3x3x3   the same mesh, HEVI IMEX ARK232, Newton to tol 1e-13 (max 30), 10 steps
  hevi_C2_2x2x2   p=7, 8 elements of the density-current mesh (u = 10 m/s), HEVI, dt 0.04 s, 5 steps
  trc_T1_4x4x3    p=3 tracer advection test (fixed wind and density), FCT + TMAR, 3 steps

Usage (from the repository root, after __graft_entry__.build()):
    python tests/golden/make_golden.py
"""
import dataclasses
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (os.path.join(ROOT, "fe-project_gb300"), os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

import oracle as orc  # noqa: E402
from fedg import cases  # noqa: E402


def golden_cases():
    c1 = cases.C1().scaled(3, 3, 3)
    return {
        "heve_C1_3x3x3": dict(case=c1, eqs="HEVE", dt=0.02, nsteps=10),
        "hevi_C1_3x3x3": dict(case=dataclasses.replace(c1, eqs="HEVI"), eqs="HEVI", dt=0.02, nsteps=10,
                              max_iter=30, tol=1e-13),
        "hevi_C2_2x2x2": dict(case=cases.C2().scaled(2, 2, 2), eqs="HEVI", dt=0.04, nsteps=5, max_iter=30,
                              tol=1e-13),
        "trc_T1_4x4x3": dict(case=cases.T1().scaled(4, 4, 3), eqs="TRC", dt=None, nsteps=3),
    }


def oracle_outputs(spec):
    """The oracle's outputs of one golden case (a dict of arrays)."""
    case = spec["case"]
    q, b = cases.initial_state(case)
    o = orc.Oracle(case.porder, case.NeX, case.NeY, case.NeZ, case.dom, grav=case.grav, filter_on=case.filter_on)
    o.set_base_state(b["dens_hyd"], b["pres_hyd"])
    if spec["eqs"] == "HEVE":
        out = o.step_heve(q, spec["dt"], spec["nsteps"])
        return {"q": np.stack(out)}
    if spec["eqs"] == "HEVI":
        out, nfail, _ = o.step_hevi(q, spec["dt"], spec["nsteps"], max_iter=spec["max_iter"], tol=spec["tol"])
        assert nfail == 0
        return {"q": np.stack(out)}
    Q0 = cases.tracer_state(case)
    aM, aP = o.trc_alphdens_advtest(q[0], q[1], q[2], q[3])
    Q = o.trc_step(Q0, q[1:4], aM, aP, q[0], q[0], case.dt, nsteps=spec["nsteps"])
    return {"Q": Q, "aM": aM, "aP": aP}


def main():
    for name, spec in golden_cases().items():
        out = oracle_outputs(spec)
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **out)
        print(name, {k: v.shape for k, v in out.items()}, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
